"""Persistent single-launch PCG for 2-D systems against the graph-captured kernels and
the oracle's restatement of the reference recurrence.

Both paths run NekLinSysIterCG's recurrence with the same summation structure, so the
FP64 iteration counts agree within one iteration and the solutions to 1e-10 relative;
the mixed mode must reach the requested FP64 residual on either path.
"""
import numpy as np
import pytest

from cases import quad_case, rel_err
from oracle import solve as osolve

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from ithaca_gpu.operators import Context
    c = Context(0)
    yield c
    c.close()


def _system(ctx, c, amap=None):
    from ithaca_gpu.operators import Collection, GlobalLinSysIterativeFullGPU
    coll = Collection(ctx, c.shape, c.n, c.Q, c.E, c.jac, c.df, deformed=c.deformed)
    amap = amap or c.mesh.assembly(c.n)
    return coll, amap, GlobalLinSysIterativeFullGPU(coll, amap)


def _rhs(amap, seed):
    rhs = np.random.default_rng(seed).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    return rhs


CASES = {
    "p2": lambda: quad_case(6, 5, 3),
    "p4": lambda: quad_case(8, 8, 5),
    "p6": lambda: quad_case(12, 10, 7),
    "p9": lambda: quad_case(5, 4, 10),
    "p6_regular": lambda: quad_case(6, 6, 7, jitter=0.0, deformed=False),
    "p4_rotated": lambda: quad_case(5, 4, 5, rotate=np.random.default_rng(9).integers(0, 4, 20)),
}


@pytest.mark.parametrize("name", list(CASES))
def test_persistent_matches_graph_and_oracle(ctx, name):
    c = CASES[name]()
    coll, amap, sys_ = _system(ctx, c)
    rhs = _rhs(amap, 5)
    sys_.set_persistent(0)
    l0 = ctx.launch_count()
    xg, rg = sys_.solve(1.0, rhs, tol=1e-11)
    graph_launches = ctx.launch_count() - l0
    sys_.set_persistent(1)
    l0 = ctx.launch_count()
    xp, rp = sys_.solve(1.0, rhs, tol=1e-11)
    persist_launches = ctx.launch_count() - l0
    # the persistent path is the one that ran: one launch for the whole recurrence
    assert persist_launches < 12 < graph_launches, (persist_launches, graph_launches)
    assert abs(rp.iterations - rg.iterations) <= 1, (rp.iterations, rg.iterations)
    assert rel_err(xp[amap.ndir:], xg[amap.ndir:]) < 1e-10
    assert rp.rel_residual < 1e-10
    xo, it_o, _, _ = osolve.solve(c.basis, 2, c.jac.reshape(c.E, -1), c.df, 1.0, amap, rhs, tol=1e-11)
    assert abs(rp.iterations - it_o) <= 1, (rp.iterations, it_o)
    assert rel_err(xp[amap.ndir:], xo[amap.ndir:]) < 1e-9


@pytest.mark.parametrize("lam", [0.1, 10.0])
def test_persistent_mixed(ctx, lam):
    c = quad_case(10, 10, 7)
    coll, amap, sys_ = _system(ctx, c)
    rhs = _rhs(amap, 6)
    sys_.set_persistent(1)
    x64, _ = sys_.solve(lam, rhs, tol=1e-12)
    x, res = sys_.solve(lam, rhs, tol=1e-10, mode="mixed")
    assert res.rel_residual < 1e-10 and res.outer_iterations >= 2
    assert rel_err(x[amap.ndir:], x64[amap.ndir:]) < 1e-8
    sys_.set_persistent(0)
    xg, resg = sys_.solve(lam, rhs, tol=1e-10, mode="mixed")
    assert abs(res.iterations - resg.iterations) <= 4, (res.iterations, resg.iterations)


def _merged_quad_map(amap):
    """Three interior vertices merged into one row of 12 local entries (longer than the
    ELL classes) and an edge dof into a vertex dof (6 entries)."""
    from ithaca_gpu.mesh import AssemblyMap
    l2g = amap.l2g.astype(np.int64).copy()
    cnt = np.bincount(l2g, minlength=amap.nglobal)
    free = np.arange(amap.ndir, amap.nglobal)
    v4, k2 = free[cnt[free] == 4], free[cnt[free] == 2]
    l2g[np.isin(l2g, v4[1:3])] = v4[0]
    l2g[l2g == k2[0]] = v4[3]
    ids = np.unique(l2g)
    return AssemblyMap(np.searchsorted(ids, l2g), amap.sign, ids.size, amap.ndir)


def test_persistent_long_rows(ctx):
    c = quad_case(6, 6, 5)
    amap = _merged_quad_map(c.mesh.assembly(c.n))
    counts = np.bincount(amap.l2g, minlength=amap.nglobal)
    assert counts.max() == 12 and 6 in counts
    coll, amap, sys_ = _system(ctx, c, amap)
    rhs = _rhs(amap, 7)
    sys_.set_persistent(1)
    x, res = sys_.solve(1.0, rhs, tol=1e-12)
    xo, it_o, _, _ = osolve.solve(c.basis, 2, c.jac.reshape(c.E, -1), c.df, 1.0, amap, rhs, tol=1e-12)
    assert abs(res.iterations - it_o) <= 1, (res.iterations, it_o)
    assert rel_err(x[amap.ndir:], xo[amap.ndir:]) < 1e-9
    xm, resm = sys_.solve(1.0, rhs, tol=1e-10, mode="mixed")
    assert resm.rel_residual < 1e-10


@pytest.mark.parametrize("mode", [0, 1])
def test_status_codes_on_both_paths(ctx, mode):
    from ithaca_gpu._capi import ERR_NOT_CONVERGED, ERR_NUMERIC, GpuError
    c = quad_case(4, 4, 5)
    coll, amap, sys_ = _system(ctx, c)
    sys_.set_persistent(mode)
    rhs = np.random.default_rng(1).uniform(-1, 1, amap.nglobal)
    with pytest.raises(GpuError) as ei:
        sys_.solve(1.0, rhs, tol=1e-14, max_iter=3)
    assert ei.value.code == ERR_NOT_CONVERGED
    bad = rhs.copy()
    bad[amap.ndir + 2] = np.nan
    with pytest.raises(GpuError) as ei:
        sys_.solve(1.0, bad)
    assert ei.value.code == ERR_NUMERIC
    x, res = sys_.solve(1.0, rhs, tol=1e-10)  # the context stays usable
    assert res.rel_residual < 1e-9


def test_set_persistent_rejects_bad_mode(ctx):
    from ithaca_gpu._capi import GpuError
    c = quad_case(2, 2, 3)
    coll, amap, sys_ = _system(ctx, c)
    with pytest.raises(GpuError):
        sys_.set_persistent(2)


def test_persistent_barrier_timeout_then_solves(ctx):
    """A CTA that never arrives at the grid barrier: every bounded wait runs out, the
    solve returns ERR_TIMEOUT, and the next solve on the same context converges."""
    from ithaca_gpu._capi import ERR_TIMEOUT, GpuError
    c = quad_case(12, 10, 7)
    coll, amap, sys_ = _system(ctx, c)
    rhs = _rhs(amap, 11)
    sys_.set_persistent(1)
    x0, r0 = sys_.solve(1.0, rhs, tol=1e-11)
    sys_.set_wait_test(barrier_polls=20000, drop_cta=0)  # ~1 ms waits
    with pytest.raises(GpuError) as ei:
        sys_.solve(1.0, rhs, tol=1e-11)
    assert ei.value.code == ERR_TIMEOUT
    sys_.set_wait_test()
    x1, r1 = sys_.solve(1.0, rhs, tol=1e-11)
    assert r1.iterations == r0.iterations and np.array_equal(x1, x0)


@pytest.mark.parametrize("delay_ns", [2000, 50000])
def test_persistent_partials_race_stress(ctx, delay_ns):
    """Every third CTA pauses after each grid barrier while the others run ahead into the
    next phase and write their next partial sums. All CTAs must still read the same
    partials: the solve is bitwise identical to an undisturbed one."""
    c = quad_case(32, 32, 7)
    coll, amap, sys_ = _system(ctx, c)
    rhs = _rhs(amap, 12)
    sys_.set_persistent(1)
    x0, r0 = sys_.solve(1.0, rhs, tol=1e-11)
    try:
        sys_.set_wait_test(delay_ns=delay_ns)
        for _ in range(3):
            x1, r1 = sys_.solve(1.0, rhs, tol=1e-11)
            assert r1.iterations == r0.iterations
            assert np.array_equal(x1, x0)
    finally:
        sys_.set_wait_test()


def test_wait_test_hook_rejects_bad_values(ctx):
    from ithaca_gpu._capi import GpuError
    c = quad_case(2, 2, 3)
    coll, amap, sys_ = _system(ctx, c)
    for kw in ({"barrier_polls": -1}, {"drop_cta": -2}, {"delay_ns": 2_000_000}):
        with pytest.raises(GpuError):
            sys_.set_wait_test(**kw)
