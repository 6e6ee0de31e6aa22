"""Anisotropic variable coefficients (the eVarCoeffD00..D22 tensor of
StdRegions/StdExpansion.cpp:664-717) against the oracle's restatement of
LaplacianMatrixOp_MatFree(k1, k2) composed over k1, k2.

CPU: the tensor operator with K = kappa I equals the isotropic one, and the assembled
operator is symmetric. GPU: the library folds K into the per-point metric
(J w (dxi/dx)^T K (dxi/dx)); its global apply matches the oracle to 1e-12 and its CG
solve takes the oracle's iterations (within one) with the solution to 1e-10, on quads
and curved hexes.
"""
import numpy as np
import pytest

from cases import hex_case, quad_case, rel_err
from oracle import ops as oops
from oracle import solve as osolve


def _tensor(c, seed):
    rng = np.random.default_rng(seed)
    X = c.X
    g = [np.sin(np.pi * (rng.uniform(0.5, 2) * X[0] + rng.uniform(0, 1))) *
         np.cos(np.pi * (rng.uniform(0.5, 2) * X[1] + rng.uniform(0, 1))) for _ in range(6)]
    g = [x.reshape(-1) for x in g]
    if c.dim == 2:  # D00, D01, D11: SPD (diagonal >= 0.5, |off-diagonal| <= 0.3)
        return np.stack([1 + 0.5 * g[0], 0.3 * g[1], 1 + 0.4 * g[2]])
    return np.stack([1 + 0.5 * g[0], 0.2 * g[1], 0.1 * g[2], 1 + 0.4 * g[3], 0.2 * g[4], 1 + 0.3 * g[5]])


def _apply(c, amap, lam, K, x):
    m = osolve.Map.of(amap)
    xx = x.copy()
    xx[:m.ndir] = 0.0
    loc = oops.helmholtz_varcoeff_tensor(c.basis, c.dim, c.jac.reshape(c.E, -1), c.df, lam, K, m.gather(xx))
    return m.assemble(np.asarray(loc).reshape(-1))


def test_oracle_tensor_reduces_to_isotropic():
    c = quad_case(3, 3, 6)
    kappa = 1 + 0.5 * np.sin(np.pi * c.X[0]).reshape(-1)
    u = np.random.default_rng(2).uniform(-1, 1, c.E * c.nm)
    K = np.stack([kappa, 0 * kappa, kappa])
    a = oops.helmholtz_varcoeff_tensor(c.basis, 2, c.jac.reshape(c.E, -1), c.df, 0.7, K, u)
    b = oops.helmholtz_varcoeff(c.basis, 2, c.jac.reshape(c.E, -1), c.df, 0.7, kappa, u)
    assert rel_err(np.asarray(a).reshape(-1), np.asarray(b).reshape(-1)) < 1e-13


def test_oracle_tensor_operator_is_symmetric():
    c = quad_case(3, 2, 5)
    amap = c.mesh.assembly(c.n)
    K = _tensor(c, 1)
    rng = np.random.default_rng(3)
    u, v = rng.uniform(-1, 1, amap.nglobal), rng.uniform(-1, 1, amap.nglobal)
    u[:amap.ndir] = v[:amap.ndir] = 0
    a, b = v @ _apply(c, amap, 1.0, K, u), u @ _apply(c, amap, 1.0, K, v)
    assert abs(a - b) < 1e-12 * max(abs(a), 1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["quad", "hex"])
def test_gpu_tensor_coefficient_matches_oracle(case):
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU
    c = quad_case(6, 5, 6) if case == "quad" else hex_case(3, 2, 2, 5)
    amap = c.mesh.assembly(c.n)
    K = _tensor(c, 7)
    ctx = Context(0)
    coll = Collection(ctx, c.shape, c.n, c.Q, c.E, c.jac, c.df)
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    sysg.set_varcoeff_tensor(K)
    x = np.random.default_rng(4).uniform(-1, 1, amap.nglobal)
    x[:amap.ndir] = 0
    y = sysg.apply(1.0, x)
    ref = _apply(c, amap, 1.0, K, x)
    assert rel_err(y[amap.ndir:], ref[amap.ndir:]) < 1e-12
    rhs = np.random.default_rng(5).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    xs, res = sysg.solve(1.0, rhs, tol=1e-12)
    m = osolve.Map.of(amap)
    d = np.zeros(amap.nglobal)
    jac = c.jac.reshape(c.E, -1)
    # Jacobi diagonal of the tensor operator: the element diagonals by unit vectors
    nm = c.nm
    for j in range(nm):
        u = np.zeros((c.E, nm))
        u[:, j] = 1.0
        col = np.asarray(oops.helmholtz_varcoeff_tensor(c.basis, c.dim, jac, c.df, 1.0, K, u.reshape(-1))).reshape(c.E, nm)
        np.add.at(d, m.l2g.reshape(c.E, nm)[:, j], col[:, j])
    xo, it_o, _, _ = osolve.cg(lambda v: _apply(c, amap, 1.0, K, v), 1.0 / d[amap.ndir:], rhs, amap.ndir, 1e-12)
    # same recurrence; at tol 1e-12 rounding in the last digits may move the stop by an iteration or two
    assert abs(res.iterations - it_o) <= max(2, it_o // 50), (res.iterations, it_o)
    assert rel_err(xs[amap.ndir:], xo[amap.ndir:]) < 1e-10
    mixed, resm = sysg.solve(1.0, rhs, tol=1e-10, mode="mixed")
    assert resm.rel_residual < 1e-10
    sysg.set_varcoeff(None)  # back to K = I
    x1, r1 = sysg.solve(1.0, rhs, tol=1e-12)
    x2, r2 = GlobalLinSysIterativeFullGPU(coll, amap).solve(1.0, rhs, tol=1e-12)
    assert r1.iterations == r2.iterations and np.array_equal(x1, x2)
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_gpu_coefficient_set_after_a_solve(mode):
    """A coefficient set after a solve (its graph already captured with the old geometry
    buffer) must reach the next solve: same result as a system that had it from the start."""
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU
    c = quad_case(6, 5, 6)
    amap = c.mesh.assembly(c.n)
    ctx = Context(0)
    coll = Collection(ctx, c.shape, c.n, c.Q, c.E, c.jac, c.df)
    rhs = np.random.default_rng(5).uniform(-1, 1, amap.nglobal)
    rhs[:amap.ndir] = 0
    kappa = (1.0 + 0.5 * np.sin(3 * c.X[0]) * np.cos(2 * c.X[1])).reshape(-1)
    a = GlobalLinSysIterativeFullGPU(coll, amap)
    a.solve(1.0, rhs, tol=1e-10, mode=mode)
    a.set_varcoeff(kappa)
    xa, ra = a.solve(1.0, rhs, tol=1e-10, mode=mode)
    b = GlobalLinSysIterativeFullGPU(coll, amap)
    b.set_varcoeff(kappa)
    xb, rb = b.solve(1.0, rhs, tol=1e-10, mode=mode)
    assert ra.iterations == rb.iterations and np.array_equal(xa, xb)
    a.set_varcoeff_tensor(_tensor(c, 3))
    a.solve(1.0, rhs, tol=1e-10, mode=mode)
    a.set_varcoeff(None)
    xa, ra = a.solve(1.0, rhs, tol=1e-10, mode=mode)
    xc, rc = GlobalLinSysIterativeFullGPU(coll, amap).solve(1.0, rhs, tol=1e-10, mode=mode)
    assert ra.iterations == rc.iterations and np.array_equal(xa, xc)
    ctx.close()
