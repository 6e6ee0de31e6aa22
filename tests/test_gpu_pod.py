"""GPU POD offline / online vs the oracle (numpy SVD / eigh / dense LU, FP64).

POD parity is not pinned by a reference test for the Helmholtz operator; the checks
are subspace agreement with the thin SVD (principal angles), the reduced operators
against dense products of the oracle operator, the reduced solves against LU, and the
ROM-vs-FOM error at unseen parameters.
"""
import numpy as np
import pytest

from cases import quad_case, rel_err
from oracle import ops as oops
from oracle import pod as opod
from oracle import solve as osolve

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU
    ctx = Context(0)
    c = quad_case(8, 8, 5, jitter=0.1, seed=0)
    coll = Collection(ctx, "quad", c.n, c.Q, c.E, c.jac, c.df)
    amap = c.mesh.assembly(c.n)
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    f = (np.sin(np.pi * c.X[0]) * np.sin(np.pi * c.X[1]) + c.X[0] ** 2).reshape(-1)
    b = -osolve.Map.of(amap).assemble(oops.iproduct(c.basis, 2, c.jac.reshape(c.E, -1), f))
    lams = 10 ** np.random.default_rng(4).uniform(-2, 2, 24)
    snaps = []
    for lam in lams:
        x, res = sysg.solve(lam, b, tol=1e-13)
        snaps.append(x[amap.ndir:].copy())
    S = np.stack(snaps, axis=1)
    yield dict(ctx=ctx, c=c, sysg=sysg, amap=amap, b=b, S=S, lams=lams)


def test_gram(setup):
    from ithaca_gpu import pod
    S = setup["S"]
    assert rel_err(pod.gram(setup["ctx"], S), S.T @ S) < 1e-13


def test_offline_subspace_matches_svd(setup):
    from ithaca_gpu import pod
    S = setup["S"]
    V, sigma, r = pod.offline(setup["ctx"], S, 8)
    assert r == 8
    assert np.max(np.abs(V.T @ V - np.eye(r))) < 1e-12
    U, s = opod.pod_svd(S, nmodes=8)
    # singular values resolved well above the FP64 floor of S agree closely
    big = s[:8] > 1e-8 * s[0]
    assert np.max(np.abs(sigma[:8][big] - s[:8][big]) / s[:8][big]) < 1e-5
    cos = opod.principal_angle_cos(U, V)
    assert np.min(cos[:int(big.sum())]) > 1 - 1e-8
    # the method of snapshots and the oracle's snapshot variant span the same space
    Vo, _, _ = opod.pod_snapshots(S, 4)
    assert np.min(opod.principal_angle_cos(Vo, V[:, :4])) > 1 - 1e-10
    assert pod.rb_size(sigma, 0.9999) == opod.rb_size(sigma, 0.9999)


def test_project_and_online(setup):
    from ithaca_gpu import pod
    c, amap, sysg = setup["c"], setup["amap"], setup["sysg"]
    V, sigma, r = pod.offline(setup["ctx"], setup["S"], 8)
    A_L, A_M = pod.project(sysg, V)
    # oracle: apply L (lambda = 0) and M columns on the free dofs
    jac = c.jac.reshape(c.E, -1)
    m = osolve.Map.of(amap)
    full = np.zeros((amap.nglobal, r))
    full[amap.ndir:] = V
    LV = np.stack([osolve.global_apply(c.basis, 2, jac, c.df, 0.0, m, full[:, j])[amap.ndir:] for j in range(r)], 1)
    AV = np.stack([osolve.global_apply(c.basis, 2, jac, c.df, 1.0, m, full[:, j])[amap.ndir:] for j in range(r)], 1)
    oL, oM = opod.project(V, LV, AV - LV)
    assert rel_err(A_L, oL) < 1e-11
    assert rel_err(A_M, oM) < 1e-9
    f_r = V.T @ setup["b"][amap.ndir:]
    new = 10 ** np.random.default_rng(5).uniform(-2, 2, 40)
    X = pod.online(setup["ctx"], A_L, A_M, f_r, new)
    Xo = opod.online_lu(A_L, A_M, f_r, new)
    assert rel_err(X, Xo) < 1e-11
    assert rel_err(X, opod.online_qr(A_L, A_M, f_r, new)) < 1e-10
    U = pod.reconstruct(setup["ctx"], V, X[:3])
    assert rel_err(U, (V @ X[:3].T).T) < 1e-13
    # ROM vs FOM at an unseen lambda
    x, _ = sysg.solve(new[0], setup["b"], tol=1e-13)
    assert np.max(np.abs(U[0] - x[amap.ndir:])) / np.max(np.abs(x)) < 1e-6
