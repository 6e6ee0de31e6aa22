"""Parity at the benchmark's own sizes (not toy meshes).

* 32 x 32 jittered quads, P = 6 (0.1 h jitter, seed 0), lambda = 1: the four FP64
  operators on coefficients U[-1, 1] (seed 1) against the oracle to 1e-12, and HelmSolve
  of f = sin(pi x) sin(pi y) by Jacobi PCG to 1e-12 against the oracle's restatement of
  the reference recurrence: iterations within one, solution to 1e-10.
* The same mesh at P = 6 and P = 8, lambda in {0.1, 1, 10}: mixed-precision solves (FP32
  inner PCG in FP64 refinement) to 1e-10; each run's error against the FP64 oracle is
  printed and bounded by 1e-8 (relative max-norm).
* 32^3 curved hexes at P = 4, 6, 8 (Q = P + 2): BwdTrans, IProductWRTBase, PhysDeriv and
  Helmholtz in FP64 against the compiled CPU port of the reference kernels (oracle/cport,
  pinned to the reference build by tests/test_cport_golden.py) to 1e-12; at P = 4 the
  Jacobi PCG to 1e-12 against the port's recurrence (iterations within one, solution to 1e-10).
* The 256-solve parametric batch (lambda = 10^U(-2, 2), E ~ U{500..8000}, P ~ U{3..9}):
  every solve reaches 1e-10 in FP64 and mixed mode; four seeded solves are checked
  against the port's FP64 recurrence (solution to 1e-9, mixed to 1e-8).
Relative errors are max-norm of the difference over max-norm of the oracle, the
semantics of TestQuadCollection.cpp:2612-2782.
"""
import os

import numpy as np
import pytest

from cases import rel_err

pytestmark = pytest.mark.gpu
NTH = os.cpu_count() or 1


@pytest.fixture(scope="module")
def ctx():
    from ithaca_gpu.operators import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def cport():
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.run(["make", "-s", "-C", os.path.join(root, "oracle", "cport")], check=True)
    from oracle import cportbind
    return cportbind


def _quad(ctx, P):
    from ithaca_gpu.mesh import QuadMesh
    from ithaca_gpu.operators import Collection, GlobalLinSysIterativeFullGPU
    from oracle import basis as obasis
    from oracle import geom as ogeom
    n, Q = P + 1, P + 2
    mesh = QuadMesh(32, 32, jitter=0.1, seed=0)
    X = mesh.coords(Q)
    b = obasis.Basis1D(n, Q)
    jac, df = ogeom.geom_factors(X, b.D2, 2)
    coll = Collection(ctx, "quad", n, Q, mesh.E, jac.reshape(-1), df)
    amap = mesh.assembly(n)
    return dict(mesh=mesh, X=X, b=b, jac=jac, df=df, coll=coll, amap=amap, n=n, Q=Q,
                sys=GlobalLinSysIterativeFullGPU(coll, amap))


def test_quad32_p6_operators_and_cg(ctx):
    from oracle import ops as oops
    from oracle import solve as osolve
    w = _quad(ctx, 6)
    b, jac, df, coll, E, n = w["b"], w["jac"], w["df"], w["coll"], w["mesh"].E, w["n"]
    u = np.random.default_rng(1).uniform(-1, 1, E * n * n)
    phys = oops.bwdtrans(b, 2, u).reshape(-1)
    assert rel_err(coll.bwdtrans(u), phys) < 1e-12
    assert rel_err(coll.iproduct(phys), oops.iproduct(b, 2, jac, phys).reshape(-1)) < 1e-12
    d = coll.physderiv(phys)
    for k, ref in enumerate(oops.physderiv(b, 2, df, phys)):
        assert rel_err(d[k], ref.reshape(-1)) < 1e-12
    assert rel_err(coll.helmholtz(1.0, u), oops.helmholtz(b, 2, jac, df, 1.0, u).reshape(-1)) < 1e-12
    X = w["X"]
    f = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1])).reshape(-1)
    xg, res = w["sys"].helmsolve(1.0, f, tol=1e-12)
    xo, it_o = osolve.helmsolve(b, 2, jac, df, 1.0, w["amap"], f, tol=1e-12)
    assert abs(res.iterations - it_o) <= 1, (res.iterations, it_o)
    assert rel_err(xg, xo.reshape(-1)) < 1e-10


@pytest.mark.parametrize("P", [6, 8])
def test_quad32_mixed_lambda_sweep_vs_fp64_oracle(ctx, P):
    from oracle import solve as osolve
    w = _quad(ctx, P)
    b, jac, df, amap = w["b"], w["jac"], w["df"], w["amap"]
    X = w["X"]
    f = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1])).reshape(-1)
    m = osolve.Map.of(amap)
    from oracle import ops as oops
    rhs = -m.assemble(oops.iproduct(b, 2, jac, f))
    for lam in (0.1, 1.0, 10.0):
        xo, it_o, _, _ = osolve.solve(b, 2, jac, df, lam, m, rhs, tol=1e-12)
        x, res = w["sys"].solve(lam, rhs, tol=1e-10, mode="mixed")
        err = rel_err(x[amap.ndir:], xo[amap.ndir:])
        print(f"P={P} lambda={lam}: mixed rel residual {res.rel_residual:.2e}, "
              f"{res.iterations} inner / {res.outer_iterations} outer; error vs FP64 oracle {err:.2e} "
              f"(oracle {it_o} iterations)")
        assert res.rel_residual < 1e-10
        assert err < 1e-8


@pytest.mark.parametrize("P", [4, 6, 8])
def test_hex32_fp64_operators_vs_cport(ctx, cport, P):
    import torch
    from ithaca_gpu.mesh import HexMesh
    from ithaca_gpu.operators import Collection, geom_factors
    n, Q = P + 1, P + 2
    mesh = HexMesh(32, 32, 32, curve_amp=0.05)
    E = mesh.E
    X = torch.from_numpy(mesh.coords(Q)).cuda()
    jac, df = geom_factors(ctx, "hex", Q, X)
    del X
    coll = Collection(ctx, "hex", n, Q, E, jac, df, deformed=True, precision="fp64")
    jh, dh = jac.cpu().numpy(), df.cpu().numpy()
    gen = torch.Generator(device="cuda").manual_seed(2)
    u = torch.rand(E * n ** 3, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
    uh = u.cpu().numpy()
    phys = coll.bwdtrans(u)
    ph = cport.bwdtrans(3, n, Q, E, uh, NTH)
    assert rel_err(phys.cpu().numpy(), ph) < 1e-12
    assert rel_err(coll.iproduct(phys).cpu().numpy(), cport.iproduct(3, n, Q, E, jh, True, ph, NTH)) < 1e-12
    dg = coll.physderiv(phys)
    dc = cport.physderiv(3, n, Q, E, dh, True, ph, NTH)
    for k in range(3):
        assert rel_err(dg[k].cpu().numpy(), dc[k]) < 1e-12
    del dg, phys
    hg = coll.helmholtz(1.0, u).cpu().numpy()
    assert rel_err(hg, cport.helmholtz(3, n, Q, E, jh, dh, True, 1.0, uh, NTH)) < 1e-12
    coll.close()
    del jac, df, u
    torch.cuda.empty_cache()


def test_hex32_p4_cg_vs_cport(ctx, cport):
    import torch
    from ithaca_gpu.workload import hex_workload
    w = hex_workload(32, 4)
    sysg, amap = w["system"], w["amap"]
    b = w["b"]
    x, res = sysg.solve(1.0, b, tol=1e-12)
    dinv = 1.0 / sysg.diagonal(1.0)
    jh, dh = w["jac"].cpu().numpy(), w["df"].cpu().numpy()
    xc, it_c, _ = cport.cg_solve(3, w["n"], w["Q"], w["mesh"].E, jh, dh, True, 1.0, amap.l2g, amap.sign, amap.nglobal,
                                 amap.ndir, dinv, b.cpu().numpy(), 1e-12, 5000, NTH)
    assert it_c > 0 and abs(res.iterations - it_c) <= 1, (res.iterations, it_c)
    nd = amap.ndir
    assert rel_err(x.cpu().numpy()[nd:], xc[nd:]) < 1e-10
    w["ctx"].close()
    torch.cuda.empty_cache()


def test_parametric_batch_256(ctx, cport):
    from ithaca_gpu.batched import BatchedHelmholtz, parametric_quad_problems
    from oracle import basis as obasis
    from oracle import solve as osolve
    probs = parametric_quad_problems(ctx, nsolve=256)
    bt = BatchedHelmholtz(ctx, "quad", probs)
    r64 = bt.solve(mode="fp64", tol=1e-10)
    rmx = bt.solve(mode="mixed", tol=1e-10)
    assert np.all(r64["rel_residual"] < 1e-10) and np.all(rmx["rel_residual"] < 1e-10)
    for i in sorted(np.random.default_rng(8).choice(256, 4, replace=False)):
        p = probs[i]
        amap, E, n, Q = p["amap"], p["mesh"].E, p["nmodes"], p["npoints"]
        bas = obasis.Basis1D(n, Q)
        dinv = osolve.jacobi_inverse(bas, 2, p["jac"].reshape(E, -1), p["df"], p["lam"], amap)
        xc, it_c, _ = cport.cg_solve(2, n, Q, E, p["jac"], p["df"], True, p["lam"], amap.l2g, amap.sign,
                                     amap.nglobal, amap.ndir, dinv, p["rhs"], 1e-10, 5000, NTH)
        nd = amap.ndir
        assert abs(int(r64["iterations"][i]) - it_c) <= 1, (i, r64["iterations"][i], it_c)
        assert rel_err(r64["x"][i][nd:], xc[nd:]) < 1e-9
        assert rel_err(rmx["x"][i][nd:], xc[nd:]) < 1e-8
    bt.close()
