"""Generates tests/golden/tri.npz: triangle fixtures from the reference's own code.

Run in the container that has the reference tree (after ``make -C oracle/ref``):
    python tests/golden/make_tri_golden.py
Outputs come from oracle/_ref/libithaca_ref.so: Polylib.cpp (zwglj/Dglj, zwgrjm/Dgrjm)
and the MatrixFree triangle kernel templates (BwdTransTriKernel, IProductTriKernel,
PhysDerivTriKernel, PhysDerivTensor2DKernel) compiled in place and driven as the
reference operators drive them (oracle/ref/ref_kernels.cpp). Contents:
  * t{n}_*        tables of the n-mode triangle expansion, n = 2..12: z0 w0 D0 B0 DB0
                  (GLL, ModifiedA) and z1 w1 D1 B1 DB1 (Gauss-Radau alpha 1 beta 0, ModifiedB)
  * unit_*        the MatrixFree cases of library/UnitTests/Collections/TestTriCollection.cpp:
                  BwdTrans (:322-382, standard triangle, 4 modes, coefficients 1),
                  IProductWRTBase (:959-1100, sin(x) cos(y), v2 = (-1, 1) and (-1, 2)),
                  PhysDeriv (:1668-1808, 2 modes, same fields),
                  Helmholtz (:2805-2896, v0 = (-1.5, -1.5), 10 elements, lambda 1.5, coefficients 1)
  * mesh_*        a curved, jittered 3 x 2 TriMesh (12 triangles, 6 modes), per-point
                  geometry: every operator on seeded inputs
  * reg_*         the same mesh straight (per-element geometry), 5 modes
Geometry inputs (jac, df) come from the oracle's triangle GeomFactors restatement.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300")]

from ithaca_gpu.mesh import TriMesh  # noqa: E402
from oracle import refbind  # noqa: E402
from oracle import tri as otri  # noqa: E402


def straight_coords(tb, verts):
    """Coordinates (2, 1, nq) of one straight triangle at the collapsed points."""
    e0, e1 = np.meshgrid(tb.z0, tb.z1, indexing="xy")
    xi0 = 0.5 * (1.0 + e0) * (1.0 - e1) - 1.0
    xi1 = e1
    W = np.stack([-0.5 * (xi0 + xi1), 0.5 * (1.0 + xi0), 0.5 * (1.0 + xi1)])
    return np.einsum("vji,vc->cji", W, np.asarray(verts, float)).reshape(2, 1, -1)


def main():
    out = {}
    for n in range(2, 13):
        a, b = refbind.tri_tables(n)
        for name, v in zip(("z0", "w0", "D0", "B0", "DB0"), a):
            out[f"t{n}_{name}"] = v
        for name, v in zip(("z1", "w1", "D1", "B1", "DB1"), b):
            out[f"t{n}_{name}"] = v

    # unit tests of TestTriCollection.cpp
    std = [(-1.0, -1.0), (1.0, -1.0), (-1.0, 1.0)]
    tall = [(-1.0, -1.0), (1.0, -1.0), (-1.0, 2.0)]
    n = 4
    tb = otri.TriBasis(n)
    out["unit_bwd_in"] = np.ones(tb.nc)
    out["unit_bwd_out"] = refbind.tri_bwdtrans(n, 1, out["unit_bwd_in"])
    for tag, verts in (("undeformed", std), ("deformed", tall)):
        X = straight_coords(tb, verts)
        J, df = otri.straight_tri_geometry(np.asarray(verts)[None])
        f = (np.sin(X[0]) * np.cos(X[1])).reshape(-1)
        out[f"unit_ipr_{tag}_jac"], out[f"unit_ipr_{tag}_df"], out[f"unit_ipr_{tag}_f"] = J, df, f
        out[f"unit_ipr_{tag}_out"] = refbind.tri_iproduct(n, 1, J, False, f)
    n2 = 2
    tb2 = otri.TriBasis(n2)
    for tag, verts in (("undeformed", std), ("deformed", tall)):
        X = straight_coords(tb2, verts)
        J, df = otri.straight_tri_geometry(np.asarray(verts)[None])
        f = (np.sin(X[0]) * np.cos(X[1])).reshape(-1)
        out[f"unit_deriv_{tag}_df"], out[f"unit_deriv_{tag}_f"] = df, f
        out[f"unit_deriv_{tag}_out"] = np.stack(refbind.tri_physderiv(n2, 1, df, False, f))
    E = 10
    verts = [(-1.5, -1.5), (1.0, -1.0), (-1.0, 1.0)]
    J, df = otri.straight_tri_geometry(np.repeat(np.asarray(verts)[None], E, axis=0))
    u = np.ones(E * tb.nc)
    out["unit_helm_jac"], out["unit_helm_df"], out["unit_helm_lambda"] = J, df, 1.5
    out["unit_helm_out"] = refbind.tri_helmholtz(n, E, J, df, False, 1.5, u)

    # seeded meshes
    rng = np.random.default_rng(31)
    for tag, mesh, n, deformed in (("mesh", TriMesh(3, 2, jitter=0.15, seed=5, rotate=np.arange(12) % 3,
                                                    curve_amp=0.05), 6, True),
                                   ("reg", TriMesh(3, 2, jitter=0.15, seed=5, rotate=(np.arange(12) * 2) % 3),
                                    5, False)):
        tb = otri.TriBasis(n)
        E = mesh.E
        X = mesh.coords(n)
        if deformed:
            J, df = otri.geom_factors(tb, X)
        else:
            J, df = otri.straight_tri_geometry(mesh.V[mesh.EV])
        u = rng.uniform(-1, 1, E * tb.nc)
        f = rng.uniform(-1, 1, E * tb.nq)
        g = rng.uniform(-1, 1, E * tb.nq)
        out.update({f"{tag}_n": n, f"{tag}_X": X, f"{tag}_jac": J.reshape(-1), f"{tag}_df": df, f"{tag}_u": u,
                    f"{tag}_f": f, f"{tag}_g": g,
                    f"{tag}_bwd": refbind.tri_bwdtrans(n, E, u),
                    f"{tag}_iprod": refbind.tri_iproduct(n, E, J.reshape(-1), deformed, f),
                    f"{tag}_deriv": np.stack(refbind.tri_physderiv(n, E, df, deformed, f)),
                    f"{tag}_iprd": refbind.tri_iproduct_deriv(n, E, J.reshape(-1), df, deformed, f, g),
                    f"{tag}_helm": refbind.tri_helmholtz(n, E, J.reshape(-1), df, deformed, 1.3, u)})
    np.savez_compressed(os.path.join(HERE, "tri.npz"), **out)
    print("tri.npz written to", HERE)


if __name__ == "__main__":
    main()
