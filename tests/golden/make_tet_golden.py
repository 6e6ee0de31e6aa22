"""Generates tests/golden/tet.npz: tetrahedron fixtures from the reference's own code.

Run in the container that has the reference tree (after ``make -C oracle/ref``):
    python tests/golden/make_tet_golden.py
Outputs come from oracle/_ref/libithaca_ref.so: Polylib.cpp (zwglj/Dglj, zwgrjm/Dgrjm with
alpha 1 and 2) and the MatrixFree tetrahedron kernel templates (BwdTransTetKernel,
IProductTetKernel, PhysDerivTetKernel, PhysDerivTensor3DKernel) compiled in place and
composed as HelmholtzTetImpl and IProductWRTDerivBaseTetImpl compose them
(oracle/ref/ref_kernels.cpp). Contents:
  * t{n}_*        tables n = 2..10: z0 w0 D0 B0 DB0, z1 w1 D1 B1 DB1, z2 w2 D2 B2 DB2
  * unit_*        MatrixFree cases of library/UnitTests/Collections/TestTetCollection.cpp:
                  BwdTrans (:640-715, standard tet, 4 modes, coefficients 1), IProductWRTBase
                  (:1070-1236, sin(x) cos(y) sin(z) on the standard tet and on v0 = (-2,-3,-4)),
                  Helmholtz (:2325-2430, standard tet, 10 elements, lambda 0, coefficients 1)
  * mesh_*        a curved, jittered 1 x 1 x 2 TetMesh (12 tetrahedra, 5 modes), per-point
                  geometry: every operator on seeded inputs
  * reg_*         the same mesh straight (per-element geometry), 4 modes
Geometry inputs come from the oracle's tetrahedron GeomFactors restatement.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300")]

from ithaca_gpu.mesh import TetMesh  # noqa: E402
from oracle import refbind  # noqa: E402
from oracle import tet as otet  # noqa: E402


def straight_coords(tb, verts):
    xi0, xi1, xi2 = otet.collapsed_to_xi(tb.z0, tb.z1, tb.z2)
    W = np.stack([-0.5 * (1 + xi0 + xi1 + xi2), 0.5 * (1 + xi0), 0.5 * (1 + xi1), 0.5 * (1 + xi2)])
    return np.einsum("vkji,vc->ckji", W, np.asarray(verts, float)).reshape(3, 1, -1)


def main():
    out = {}
    names = ("z0", "w0", "D0", "B0", "DB0", "z1", "w1", "D1", "B1", "DB1", "z2", "w2", "D2", "B2", "DB2")
    for n in range(2, 11):
        a, b, c = refbind.tet_tables(n)
        for name, v in zip(names, a + b + c):
            out[f"t{n}_{name}"] = v
    std = [(-1.0, -1.0, -1.0), (1.0, -1.0, -1.0), (-1.0, 1.0, -1.0), (-1.0, -1.0, 1.0)]
    far = [(-2.0, -3.0, -4.0), (1.0, -1.0, -1.0), (-1.0, 1.0, -1.0), (-1.0, -1.0, 1.0)]
    n = 4
    tb = otet.TetBasis(n)
    out["unit_bwd_in"] = np.ones(tb.nc)
    out["unit_bwd_out"] = refbind.tet_bwdtrans(n, 1, out["unit_bwd_in"])
    for tag, verts in (("undeformed", std), ("deformed", far)):
        X = straight_coords(tb, verts)
        J, df = otet.straight_tet_geometry(np.asarray(verts)[None])
        f = (np.sin(X[0]) * np.cos(X[1]) * np.sin(X[2])).reshape(-1)
        out[f"unit_ipr_{tag}_jac"], out[f"unit_ipr_{tag}_df"], out[f"unit_ipr_{tag}_f"] = J, df, f
        out[f"unit_ipr_{tag}_out"] = refbind.tet_iproduct(n, 1, J, False, f)
        out[f"unit_deriv_{tag}_out"] = np.stack(refbind.tet_physderiv(n, 1, df, False, f))
    E = 10
    J, df = otet.straight_tet_geometry(np.repeat(np.asarray(std)[None], E, axis=0))
    out["unit_helm_jac"], out["unit_helm_df"], out["unit_helm_lambda"] = J, df, 0.0
    out["unit_helm_out"] = refbind.tet_helmholtz(n, E, J, df, False, 0.0, np.ones(E * tb.nc))
    rng = np.random.default_rng(41)
    for tag, mesh, n, deformed in (("mesh", TetMesh(1, 1, 2, jitter=0.2, seed=3, curve_amp=0.03), 5, True),
                                   ("reg", TetMesh(1, 1, 2, jitter=0.2, seed=3), 4, False)):
        tb = otet.TetBasis(n)
        E = mesh.E
        X = mesh.coords(n)
        if deformed:
            J, df = otet.geom_factors(tb, X)
        else:
            J, df = otet.straight_tet_geometry(mesh.V[mesh.EV])
        u = rng.uniform(-1, 1, E * tb.nc)
        f, g, h = (rng.uniform(-1, 1, E * tb.nq) for _ in range(3))
        out.update({f"{tag}_n": n, f"{tag}_jac": J.reshape(-1), f"{tag}_df": df, f"{tag}_u": u, f"{tag}_f": f,
                    f"{tag}_g": g, f"{tag}_h": h,
                    f"{tag}_bwd": refbind.tet_bwdtrans(n, E, u),
                    f"{tag}_iprod": refbind.tet_iproduct(n, E, J.reshape(-1), deformed, f),
                    f"{tag}_deriv": np.stack(refbind.tet_physderiv(n, E, df, deformed, f)),
                    f"{tag}_iprd": refbind.tet_iproduct_deriv(n, E, J.reshape(-1), df, deformed, f, g, h),
                    f"{tag}_helm": refbind.tet_helmholtz(n, E, J.reshape(-1), df, deformed, 1.3, u)})
    np.savez_compressed(os.path.join(HERE, "tet.npz"), **out)
    print("tet.npz written to", HERE)


if __name__ == "__main__":
    main()
