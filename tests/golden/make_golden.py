"""Generates the golden fixtures in tests/golden/*.npz from the reference's own code.

Run in the container that has the reference tree (after ``make -C oracle/ref``):
    python tests/golden/make_golden.py
Outputs are computed by oracle/_ref/libithaca_ref.so, i.e. the reference's
Polylib.cpp and MatrixFreeOps kernel templates compiled in place (scalar tinysimd),
driven as the reference operators drive them (oracle/ref/ref_kernels.cpp). Inputs:
  * basis.npz         GLL points/weights/D and ModifiedA B/DB for n = 2..10, Q = n + 1.
  * unit_quad.npz     the Helmholtz MatrixFree collection tests of
                      library/UnitTests/Collections/TestQuadCollection.cpp:2612-2782
                      (10 copies of one quad, 5 modes, 6 GLL points, coefficients 1;
                      regular square with lambda 1.5, deformed quad with lambda 0).
  * unit_hex.npz      TestHexCollection.cpp:3649-3746 (trilinear hex with v6 = (2,3,4),
                      4 modes, 5 points, coefficients 1, lambda 0).
  * mesh_quad.npz     3x2 jittered quads, 7 modes: all four operators on seeded inputs.
  * mesh_hex.npz      2x2x1 curved hexes, 5 modes: all four operators.
  * cg_quad.npz       4x4 jittered quads, 5 modes, homogeneous Dirichlet: the reference
                      CG recurrence (NekLinSysIterCG) on an assembled right-hand side.
Geometry inputs (jac, df) come from the oracle's GeomFactors restatement.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300")]

from ithaca_gpu.mesh import HexMesh, QuadMesh, gll_points  # noqa: E402
from oracle import basis as obasis  # noqa: E402
from oracle import geom as ogeom  # noqa: E402
from oracle import refbind  # noqa: E402
from oracle import solve as osolve  # noqa: E402


def bilinear_coords(verts, Q):
    z = gll_points(Q)
    a, b = 0.5 * (1 - z), 0.5 * (1 + z)
    W = np.stack([np.outer(a, a), np.outer(a, b), np.outer(b, b), np.outer(b, a)])  # [v, j, i]
    return np.einsum("vji,vc->cji", W, np.asarray(verts, float)).reshape(2, 1, Q * Q)


def trilinear_coords(verts, Q):
    z = gll_points(Q)
    a, b = 0.5 * (1 - z), 0.5 * (1 + z)
    f = [(a, a, a), (b, a, a), (b, b, a), (a, b, a), (a, a, b), (b, a, b), (b, b, b), (a, b, b)]
    W = np.stack([np.einsum("k,j,i->kji", fz, fy, fx) for (fx, fy, fz) in f])
    return np.einsum("vkji,vc->ckji", W, np.asarray(verts, float)).reshape(3, 1, Q ** 3)


def replicate(X, E):
    return np.repeat(X, E, axis=1)


def main():
    out = {}
    for n in range(2, 11):
        Q = n + 1
        z, w, D = refbind.gll(Q)
        B, DB = refbind.modA(n, Q)
        out.update({f"z{n}": z, f"w{n}": w, f"D{n}": D, f"B{n}": B, f"DB{n}": DB})
    np.savez_compressed(os.path.join(HERE, "basis.npz"), **out)

    # quad unit tests
    res = {}
    n, Q, E = 5, 6, 10
    b = obasis.Basis1D(n, Q)
    for name, verts, lam, deformed in (("regular", [(-1, -1), (1, -1), (1, 1), (-1, 1)], 1.5, False),
                                        ("deformed", [(-1.5, -1.5), (1, -1), (1, 1), (-1, 1)], 0.0, True)):
        X = replicate(bilinear_coords(verts, Q), E)
        jac, df = ogeom.geom_factors(X, b.D2, 2)
        if not deformed:
            jac, df = jac[:, 0].copy(), df.reshape(4, E, Q * Q)[:, :, 0].copy()
        u = np.ones(E * n * n)
        res[f"{name}_jac"], res[f"{name}_df"], res[f"{name}_lambda"] = jac.reshape(-1), df, lam
        res[f"{name}_out"] = refbind.helmholtz(2, n, Q, E, jac, df, deformed, lam, u)
    np.savez_compressed(os.path.join(HERE, "unit_quad.npz"), **res)

    # hex unit test
    n, Q, E = 4, 5, 10
    b = obasis.Basis1D(n, Q)
    verts = [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (2, 3, 4), (-1, 1, 1)]
    X = replicate(trilinear_coords(verts, Q), E)
    jac, df = ogeom.geom_factors(X, b.D2, 3)
    u = np.ones(E * n ** 3)
    np.savez_compressed(os.path.join(HERE, "unit_hex.npz"), jac=jac.reshape(-1), df=df, lam=0.0,
                        out=refbind.helmholtz(3, n, Q, E, jac, df, True, 0.0, u))

    # seeded meshes: every operator
    for fname, mesh, n, dim in (("mesh_quad.npz", QuadMesh(3, 2, jitter=0.1, seed=11), 7, 2),
                                ("mesh_hex.npz", HexMesh(2, 2, 1, curve_amp=0.05), 5, 3)):
        Q = n + 1
        b = obasis.Basis1D(n, Q)
        X = mesh.coords(Q)
        E = mesh.E
        jac, df = ogeom.geom_factors(X, b.D2, dim)
        rng = np.random.default_rng(21)
        u = rng.uniform(-1, 1, E * n ** dim)
        f = rng.uniform(-1, 1, E * Q ** dim)
        d = refbind.physderiv(dim, n, Q, E, df, True, f)
        np.savez_compressed(os.path.join(HERE, fname), X=X, jac=jac.reshape(-1), df=df, u=u, f=f,
                            bwd=refbind.bwdtrans(dim, n, Q, E, u),
                            iprod=refbind.iproduct(dim, n, Q, E, jac, True, f),
                            deriv=np.stack(d), helm=refbind.helmholtz(dim, n, Q, E, jac, df, True, 1.0, u))

    # reference CG on a small quad mesh
    mesh = QuadMesh(4, 4, jitter=0.1, seed=0)
    n, Q = 5, 6
    b = obasis.Basis1D(n, Q)
    X = mesh.coords(Q)
    jac, df = ogeom.geom_factors(X, b.D2, 2)
    amap = mesh.assembly(n)
    fphys = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1])).reshape(-1)
    m = osolve.Map.of(amap)
    rhs = -m.assemble(refbind.iproduct(2, n, Q, mesh.E, jac, True, fphys))
    dinv = osolve.jacobi_inverse(b, 2, jac, df, 1.0, m)
    x, it, eps = refbind.cg_solve(2, n, Q, mesh.E, jac, df, True, 1.0, amap.l2g, amap.sign, amap.nglobal,
                                  amap.ndir, dinv, rhs, 1e-12, 5000)
    np.savez_compressed(os.path.join(HERE, "cg_quad.npz"), l2g=amap.l2g, sign=amap.sign, nglobal=amap.nglobal,
                        ndir=amap.ndir, jac=jac.reshape(-1), df=df, rhs=rhs, dinv=dinv, x=x, iterations=it, eps=eps,
                        fphys=fphys)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
