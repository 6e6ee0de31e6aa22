"""Adjoint gradient dJ/dkappa through torch.autograd vs the FP64 oracle and central FD.

Tolerances: J to 1e-10 relative; the adjoint gradient to 1e-8 relative (max-norm)
against the oracle's FP64 adjoint gradient (both solves at tol 1e-13); central finite
differences (h = 1e-6) to 1e-5 relative at seeded quadrature points.
"""
import numpy as np
import pytest

from cases import quad_case, rel_err
from oracle import adjoint as oadj
from oracle import ops as oops
from oracle import solve as osolve

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _problem(nx, n, seed_k=6, seed_t=7):
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU
    c = quad_case(nx, nx, n, jitter=0.1, seed=0)
    ctx = Context(0)
    coll = Collection(ctx, "quad", c.n, c.Q, c.E, c.jac, c.df)
    amap = c.mesh.assembly(c.n)
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    m = osolve.Map.of(amap)
    jac = c.jac.reshape(c.E, -1)
    kappa = (1 + 0.5 * oadj.smooth_field(c.X, seed_k)).reshape(-1)
    kt = (1 + 0.5 * oadj.smooth_field(c.X, seed_t)).reshape(-1)
    f = (np.sin(np.pi * c.X[0]) * np.sin(np.pi * c.X[1])).reshape(-1)
    rhs = -m.assemble(oops.iproduct(c.basis, 2, jac, f).reshape(-1))
    # target: solution with a different coefficient field (GPU solve)
    sysg.set_varcoeff(kt)
    xt, _ = sysg.solve(1.0, rhs, tol=1e-13)
    xt[:amap.ndir] = 0
    ut = oops.bwdtrans(c.basis, 2, m.gather(xt)).reshape(-1)
    return dict(c=c, ctx=ctx, sysg=sysg, m=m, jac=jac, kappa=kappa, rhs=rhs, ut=ut, amap=amap)


def _torch(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_gradient_matches_oracle_and_fd():
    from ithaca_gpu.adjoint import misfit
    P = _problem(6, 5)
    c = P["c"]
    k = _torch(P["kappa"]).requires_grad_(True)
    J = misfit(k, P["sysg"], 1.0, _torch(P["rhs"]), _torch(P["ut"]), 1e-13)
    J.backward()
    g = k.grad.cpu().numpy()
    Jo, go, _ = oadj.objective_and_gradient(c.basis, 2, P["jac"], c.df, 1.0, P["kappa"].reshape(c.E, -1), P["m"],
                                            P["rhs"], P["ut"])
    assert abs(J.item() - Jo) / Jo < 1e-10
    assert rel_err(g, go) < 1e-8
    rng = np.random.default_rng(11)
    h = 1e-6
    with torch.no_grad():
        for q in rng.choice(c.E * c.nq, 6, replace=False):
            kp = k.detach().clone()
            kp[q] += h
            km = k.detach().clone()
            km[q] -= h
            Jp = misfit(kp, P["sysg"], 1.0, _torch(P["rhs"]), _torch(P["ut"]), 1e-14).item()
            Jm = misfit(km, P["sysg"], 1.0, _torch(P["rhs"]), _torch(P["ut"]), 1e-14).item()
            fd = (Jp - Jm) / (2 * h)
            assert abs(fd - g[q]) <= 1e-5 * np.max(np.abs(g)), (q, fd, g[q])


def test_config5_gradient_fd_sample():
    """64x64 quads, P = 6, FP64: FD at 32 seeded quadrature points and the oracle gradient."""
    from ithaca_gpu.adjoint import misfit
    P = _problem(64, 7)
    c = P["c"]
    k = _torch(P["kappa"]).requires_grad_(True)
    J = misfit(k, P["sysg"], 1.0, _torch(P["rhs"]), _torch(P["ut"]), 1e-13)
    J.backward()
    g = k.grad.cpu().numpy()
    gmax = np.max(np.abs(g))
    rng = np.random.default_rng(6)
    h = 1e-6
    errs = []
    with torch.no_grad():
        for q in rng.choice(c.E * c.nq, 32, replace=False):
            kp = k.detach().clone()
            kp[q] += h
            km = k.detach().clone()
            km[q] -= h
            Jp = misfit(kp, P["sysg"], 1.0, _torch(P["rhs"]), _torch(P["ut"]), 1e-14).item()
            Jm = misfit(km, P["sysg"], 1.0, _torch(P["rhs"]), _torch(P["ut"]), 1e-14).item()
            errs.append(abs((Jp - Jm) / (2 * h) - g[q]) / gmax)
    assert max(errs) < 1e-4, max(errs)
    Jo, go, _ = oadj.objective_and_gradient(c.basis, 2, P["jac"], c.df, 1.0, P["kappa"].reshape(c.E, -1), P["m"],
                                            P["rhs"], P["ut"], tol=1e-12)
    assert abs(J.item() - Jo) / Jo < 1e-8
    assert rel_err(g, go) < 1e-6
