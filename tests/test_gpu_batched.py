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


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_one_launch_matches_host_checked_path(family, mode):
    """The whole solve as one graph launch (device-side loops) runs the same kernels in
    the same order as the host-checked chunk launches: identical iterations and
    solutions, bit for bit, on two solves in a row."""
    from ithaca_gpu.batched import BatchedHelmholtz
    ctx, probs = family
    b = BatchedHelmholtz(ctx, "quad", probs)
    b.set_one_launch(0)
    ref = b.solve(mode=mode, tol=1e-10)
    b.set_one_launch(1)
    l0 = ctx.launch_count()
    for _ in range(2):
        res = b.solve(mode=mode, tol=1e-10)
        assert np.array_equal(res["iterations"], ref["iterations"])
        assert np.array_equal(res["outer"], ref["outer"])
        for x, xr in zip(res["x"], ref["x"]):
            assert np.array_equal(x, xr)
        assert np.array_equal(res["rel_residual"], ref["rel_residual"])
    # one graph launch per solve, plus the final FP64 residual's few launches
    assert ctx.launch_count() - l0 < 2 * (1 + 3 * 8)


def test_one_launch_reports_iteration_limit(family):
    from ithaca_gpu._capi import ERR_NOT_CONVERGED, GpuError
    from ithaca_gpu.batched import BatchedHelmholtz
    ctx, probs = family
    b = BatchedHelmholtz(ctx, "quad", probs[:3])
    with pytest.raises(GpuError) as ei:
        b.solve(mode="fp64", tol=1e-12, max_iter=4)
    assert ei.value.code == ERR_NOT_CONVERGED
    with pytest.raises(GpuError) as ei:
        b.solve(mode="mixed", tol=1e-12, max_outer=1)
    assert ei.value.code == ERR_NOT_CONVERGED
    res = b.solve(mode="mixed", tol=1e-10)  # the batch stays usable
    assert np.all(res["rel_residual"] < 1e-10)


def test_autotuned_tile_shapes_keep_the_results(family):
    """The per-order tile-shape autotuner picks, for every order group and precision, the
    fastest element-kernel variant; the solves keep their FP64 residuals and iteration
    counts (within one: the variants sum in a different order)."""
    from ithaca_gpu.batched import BatchedHelmholtz
    ctx, probs = family
    b = BatchedHelmholtz(ctx, "quad", probs)
    ref = b.solve(mode="fp64", tol=1e-11)
    refm = b.solve(mode="mixed", tol=1e-10)
    choice = b.autotune(reps=3)
    assert sorted(choice) == sorted({p["nmodes"] for p in probs})
    for n, c in choice.items():
        for prec in ("fp32", "fp64"):
            v, times = c[prec]
            assert v in (0, 1, 2) and times[v] == min(times) and all(t > 0 for t in times)
    res = b.solve(mode="fp64", tol=1e-11)
    assert np.all(np.abs(res["iterations"] - ref["iterations"]) <= 1)
    for x, xr, p in zip(res["x"], ref["x"], probs):
        nd = p["amap"].ndir
        assert rel_err(x[nd:], xr[nd:]) < 1e-10
    resm = b.solve(mode="mixed", tol=1e-10)
    assert np.all(resm["rel_residual"] < 1e-10)
    for x, xr, p in zip(resm["x"], refm["x"], probs):
        nd = p["amap"].ndir
        assert rel_err(x[nd:], xr[nd:]) < 1e-8
