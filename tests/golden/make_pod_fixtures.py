"""Writes tests/golden/pod_eigen.npz: POD offline / online results of the reference's own
arithmetic (Eigen 3.3.7 BDCSVD and colPivHouseholderQr, as CoupledLinearNS_ROM.cpp:3925
and :4053 use them; oracle/_ref/libithaca_eigen.so built by oracle/ref/Makefile) at the
benchmark's POD scale: 256 snapshots over the free dofs of the 32 x 32 jittered-quad
P=6 mesh, 50 modes, 4096 online parameters.

The snapshot matrix is generated, not solved for, so that every machine rebuilds the same
matrix from the seed: S = G1 diag(sigma) G2^T with G1, G2 uniform in [-1, 1) and
sigma_k = 10^(-k/16), a separated spectrum over 256 values. The fixture keeps quantities
that do not depend on the sign or rotation of the modes within their span:
  sigma            all 256 singular values
  sketch           U^T R for R = 2 rng.random((N, 64)) - 1 (seed 32): a first-order check of
                   the 50-mode subspace (an orthogonal Procrustes fit of the tested basis)
  ritz_L, ritz_M   eigenvalues of A_L = U^T L U and A_M = U^T M U (L, M: the oracle's
                   stiffness and mass operators on the free dofs)
  xnorm            ||x_r(lambda)|| of the 4096 online solves (A_L + lambda A_M) x_r = U^T b
  usample          (U x_r)(lambda) at 64 seeded dofs for the first 64 lambdas
Run where the reference tree is present (after make -C oracle/ref):
    python tests/golden/make_pod_fixtures.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300"), os.path.join(ROOT, "tests")]

NS, NMODES, NLAM, NSKETCH = 256, 50, 4096, 64


def problem():
    """Mesh, operators and rhs of the POD fixture (shared with the tests)."""
    from cases import quad_case
    from oracle import ops as oops
    from oracle import solve as osolve
    c = quad_case(32, 32, 7)
    amap = c.mesh.assembly(c.n)
    m = osolve.Map.of(amap)
    jac = c.jac.reshape(c.E, -1)
    f = (np.sin(np.pi * c.X[0]) * np.sin(np.pi * c.X[1])).reshape(-1)
    b = -m.assemble(oops.iproduct(c.basis, 2, jac, f))
    N = amap.nglobal - amap.ndir
    rng = np.random.default_rng(30)
    G1 = 2 * rng.random((N, NS)) - 1
    G2 = 2 * rng.random((NS, NS)) - 1
    sig = 10.0 ** (-np.arange(NS) / 16.0)
    S = (G1 * sig[None, :]) @ G2.T
    R = 2 * np.random.default_rng(32).random((N, NSKETCH)) - 1
    lams = 10 ** np.random.default_rng(31).uniform(-2, 2, NLAM)
    idx = np.sort(np.random.default_rng(33).choice(N, 64, replace=False))
    return dict(c=c, amap=amap, m=m, jac=jac, b=b, S=S, R=R, lams=lams, idx=idx, N=N)


def apply_LM(p, V):
    """L V and M V on the free dofs (columns of V are free-dof vectors)."""
    from oracle import solve as osolve
    c, m, nd = p["c"], p["m"], p["amap"].ndir
    LV, MV = np.zeros_like(V), np.zeros_like(V)
    for j in range(V.shape[1]):
        x = np.zeros(p["amap"].nglobal)
        x[nd:] = V[:, j]
        l0 = osolve.global_apply(c.basis, 2, p["jac"], c.df, 0.0, m, x)[nd:]
        l1 = osolve.global_apply(c.basis, 2, p["jac"], c.df, 1.0, m, x)[nd:]
        LV[:, j], MV[:, j] = l0, l1 - l0
    return LV, MV


def main():
    from oracle import eigenbind
    p = problem()
    sigma, U = eigenbind.bdcsvd(p["S"], NMODES)
    LU, MU = apply_LM(p, U)
    A_L, A_M = U.T @ LU, U.T @ MU
    f_r = U.T @ p["b"][p["amap"].ndir:]
    xnorm = np.zeros(NLAM)
    usample = np.zeros((64, 64))
    for k, lam in enumerate(p["lams"]):
        x = eigenbind.colpivqr_solve(A_L + lam * A_M, f_r)
        xnorm[k] = np.linalg.norm(x)
        if k < 64:
            usample[k] = (U @ x)[p["idx"]]
    np.savez_compressed(os.path.join(HERE, "pod_eigen.npz"), sigma=sigma, sketch=U.T @ p["R"],
                        ritz_L=np.linalg.eigvalsh(0.5 * (A_L + A_L.T)), ritz_M=np.linalg.eigvalsh(0.5 * (A_M + A_M.T)),
                        xnorm=xnorm, usample=usample, fr_norm=np.linalg.norm(f_r))
    print("wrote pod_eigen.npz")


if __name__ == "__main__":
    main()
