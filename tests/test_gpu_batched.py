"""Batched parametric solves vs one-at-a-time solves and the oracle.

FP64 mode: each solve of the batch follows the reference CG recurrence with its own
scalars, so its iteration count matches the single-system solver (within one) and the
solution agrees to 1e-10 relative; mixed mode must reach the FP64 relative residual.
"""
import numpy as np
import pytest

from cases import rel_err
from oracle import solve as osolve

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def family():
    from ithaca_gpu.batched import parametric_quad_problems
    from ithaca_gpu.operators import Context
    ctx = Context(0)
    probs = parametric_quad_problems(ctx, nsolve=14, e_range=(20, 90), p_range=(3, 9), seed=4)
    yield ctx, probs


def test_batched_fp64_matches_single_solves(family):
    from ithaca_gpu.batched import BatchedHelmholtz
    from ithaca_gpu.operators import Collection, GlobalLinSysIterativeFullGPU
    ctx, probs = family
    b = BatchedHelmholtz(ctx, "quad", probs)
    res = b.solve(mode="fp64", tol=1e-11)
    assert np.all(res["rel_residual"] < 1e-10)
    for i, p in enumerate(probs):
        coll = Collection(ctx, "quad", p["nmodes"], p["npoints"], p["mesh"].E, p["jac"], p["df"])
        sysg = GlobalLinSysIterativeFullGPU(coll, p["amap"])
        x, r = sysg.solve(p["lam"], p["rhs"], tol=1e-11)
        assert abs(int(res["iterations"][i]) - r.iterations) <= 1, (i, res["iterations"][i], r.iterations)
        nd = p["amap"].ndir
        assert rel_err(res["x"][i][nd:], x[nd:]) < 1e-10


def test_batched_matches_oracle(family):
    from ithaca_gpu.batched import BatchedHelmholtz
    from oracle import basis as obasis
    from oracle import geom as ogeom
    ctx, probs = family
    sub = probs[:4]
    b = BatchedHelmholtz(ctx, "quad", sub)
    res = b.solve(mode="fp64", tol=1e-12)
    for i, p in enumerate(sub):
        bas = obasis.Basis1D(p["nmodes"], p["npoints"])
        E = p["mesh"].E
        x, it, _, _ = osolve.solve(bas, 2, p["jac"].reshape(E, -1), p["df"], p["lam"], p["amap"], p["rhs"], tol=1e-12)
        nd = p["amap"].ndir
        assert rel_err(res["x"][i][nd:], x[nd:]) < 1e-10
        assert abs(int(res["iterations"][i]) - it) <= 1


def test_batched_mixed_reaches_fp64_residual(family):
    from ithaca_gpu.batched import BatchedHelmholtz
    ctx, probs = family
    b = BatchedHelmholtz(ctx, "quad", probs)
    ref = b.solve(mode="fp64", tol=1e-12)
    res = b.solve(mode="mixed", tol=1e-10)
    assert np.all(res["rel_residual"] < 1e-10), res["rel_residual"]
    assert np.all(res["outer"] >= 1)
    for i, p in enumerate(probs):
        nd = p["amap"].ndir
        assert rel_err(res["x"][i][nd:], ref["x"][i][nd:]) < 1e-8
