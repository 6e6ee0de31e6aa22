"""Successive right-hand sides: projection onto previous solutions
(GlobalLinSysIterative::DoProjection / UpdateKnownSolutions,
MultiRegions/GlobalLinSysIterative.cpp:156-482).

A sequence of right-hand sides from a slowly varying forcing (the time-dependent case the
projection is made for) is solved with the buffer on. The oracle's restatement must cut
the CG iterations and keep the residual at the solver's tolerance; the GPU solver must
take the oracle's iteration count on every solve (within one) and agree with the
oracle's solution to 1e-9 relative, in both basis modes, through buffer wrap-around.
"""
import numpy as np
import pytest

from cases import quad_case, rel_err
from oracle import ops as oops
from oracle import solve as osolve


def _sequence(c, amap, nsteps):
    m = osolve.Map.of(amap)
    X = c.X
    out = []
    for k in range(nsteps):
        t = 0.1 * k
        f = (np.sin(np.pi * X[0] * (1 + 0.1 * t)) * np.sin(np.pi * X[1]) * np.cos(t)).reshape(-1)
        out.append(-m.assemble(oops.iproduct(c.basis, 2, c.jac.reshape(c.E, -1), f)))
    return out


def _oracle_run(c, amap, lam, nsucc, rhss, tol):
    m = osolve.Map.of(amap)
    A = lambda v: osolve.global_apply(c.basis, 2, c.jac.reshape(c.E, -1), c.df, lam, m, v)
    dinv = osolve.jacobi_inverse(c.basis, 2, c.jac.reshape(c.E, -1), c.df, lam, m)
    P = osolve.SuccessiveRHS(nsucc)
    return [P.solve(A, dinv, r, m.ndir, tol) for r in rhss], A


@pytest.mark.parametrize("nsucc", [4, -4])
def test_oracle_projection_cuts_iterations(nsucc):
    c = quad_case(8, 8, 7)
    amap = c.mesh.assembly(c.n)
    rhss = _sequence(c, amap, 8)
    runs, A = _oracle_run(c, amap, 1.0, nsucc, rhss, 1e-10)
    its = [it for _, it in runs]
    assert its[0] > 100 and max(its[3:]) < its[0] / 3, its
    for (x, _), r in zip(runs, rhss):
        res = r[amap.ndir:] - A(x)[amap.ndir:]
        assert np.linalg.norm(res) < 1e-9  # absolute: the projected rhs falls under the 1e-6 magnitude floor


def test_oracle_ldlt_solve():
    rng = np.random.default_rng(0)
    B = rng.standard_normal((6, 6))
    M = B @ B.T + 6 * np.eye(6)
    y = rng.standard_normal(6)
    assert np.max(np.abs(osolve.ldlt_solve(M, y) - np.linalg.solve(M, y))) < 1e-12
    assert osolve.ldlt_solve(-np.eye(2), np.ones(2)) is None


@pytest.mark.gpu
@pytest.mark.parametrize("nsucc,nsteps", [(4, 8), (-4, 8), (3, 9)])
def test_gpu_projection_matches_oracle(nsucc, nsteps):
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU
    c = quad_case(8, 8, 7)
    amap = c.mesh.assembly(c.n)
    rhss = _sequence(c, amap, nsteps)
    runs, _ = _oracle_run(c, amap, 1.0, nsucc, rhss, 1e-10)
    ctx = Context(0)
    coll = Collection(ctx, "quad", c.n, c.Q, c.E, c.jac, c.df)
    sys_ = GlobalLinSysIterativeFullGPU(coll, amap)
    sys_.set_successive_rhs(nsucc)
    nd = amap.ndir
    for k, (r, (xo, it_o)) in enumerate(zip(rhss, runs)):
        x, res = sys_.solve(1.0, r, tol=1e-10)
        assert abs(res.iterations - it_o) <= 1, (k, res.iterations, it_o)
        assert rel_err(x[nd:], xo[nd:]) < 1e-9, k
    ctx.close()


@pytest.mark.gpu
def test_gpu_projection_mixed_and_operator_change():
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU
    c = quad_case(8, 8, 7)
    amap = c.mesh.assembly(c.n)
    rhss = _sequence(c, amap, 6)
    ctx = Context(0)
    coll = Collection(ctx, "quad", c.n, c.Q, c.E, c.jac, c.df)
    sys_ = GlobalLinSysIterativeFullGPU(coll, amap)
    ref = [sys_.solve(1.0, r, tol=1e-12)[0] for r in rhss]
    sys_.set_successive_rhs(5)
    its = []
    for r, xr in zip(rhss, ref):
        x, res = sys_.solve(1.0, r, tol=1e-10, mode="mixed")
        its.append(res.iterations)
        assert rel_err(x[amap.ndir:], xr[amap.ndir:]) < 1e-7
    assert max(its[2:]) < its[0], its
    # another lambda: the stored solutions of lambda = 1 are dropped, so a full solve follows
    x, res = sys_.solve(2.0, rhss[-1], tol=1e-10)
    x0, res0 = GlobalLinSysIterativeFullGPU(coll, amap).solve(2.0, rhss[-1], tol=1e-10)
    assert res.iterations == res0.iterations and np.array_equal(x, x0)
    ctx.close()
