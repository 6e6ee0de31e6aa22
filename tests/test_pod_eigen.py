"""POD offline / online against the reference's own arithmetic at the benchmark's POD
scale (256 snapshots, 50 modes, 4096 online parameters; the free dofs of the 32 x 32
quad P=6 mesh).

The fixture tests/golden/pod_eigen.npz holds the results of the reference's vendored
Eigen 3.3.7 (BDCSVD thin U, CoupledLinearNS_ROM.cpp:3925; colPivHouseholderQr solves,
:4053) on a snapshot matrix that every machine rebuilds from its seed
(tests/golden/make_pod_fixtures.py). Only basis-invariant quantities are compared:
singular values; the 50-mode subspace through a sketch U^T R fitted by an orthogonal
Procrustes rotation (first order in the principal angles); the Ritz values of
A_L = V^T L V and A_M = V^T M V; the norms of the 4096 reduced solutions; and
reconstructed ROM solutions at sampled dofs. The GPU computes the modes by the method of
snapshots (Gram matrix, eigen-decomposition, deflation) and the online solves by LU with
partial pivoting, the reference by the SVD and column-pivoted QR: tolerances are written
per quantity below.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_pod_fixtures as fx  # noqa: E402

G = np.load(os.path.join(HERE, "golden", "pod_eigen.npz"))
TOL_SIGMA = 1e-12      # |sigma - sigma_ref| / sigma_1 over the 50 modes
TOL_SUBSPACE = 1e-10   # Procrustes residual of the sketch, relative
TOL_RITZ = 1e-10       # Ritz values, relative to the largest
TOL_ONLINE = 1e-10     # reduced-solution norms and reconstructed samples, relative


@pytest.fixture(scope="module")
def prob():
    return fx.problem()


def subspace_residual(V, R, sketch):
    Gs = V.T @ R
    P, _, Qt = np.linalg.svd(sketch @ Gs.T)
    O = P @ Qt
    return np.linalg.norm(sketch - O @ Gs) / np.linalg.norm(sketch)


def check_all(p, sigma, V, A_L, A_M, online, reconstruct):
    s1 = G["sigma"][0]
    assert np.max(np.abs(sigma[:fx.NMODES] - G["sigma"][:fx.NMODES])) / s1 < TOL_SIGMA
    assert subspace_residual(V, p["R"], G["sketch"]) < TOL_SUBSPACE
    rL = np.linalg.eigvalsh(0.5 * (A_L + A_L.T))
    rM = np.linalg.eigvalsh(0.5 * (A_M + A_M.T))
    assert np.max(np.abs(rL - G["ritz_L"])) / np.max(np.abs(G["ritz_L"])) < TOL_RITZ
    assert np.max(np.abs(rM - G["ritz_M"])) / np.max(np.abs(G["ritz_M"])) < TOL_RITZ
    f_r = V.T @ p["b"][p["amap"].ndir:]
    assert abs(np.linalg.norm(f_r) - G["fr_norm"]) / G["fr_norm"] < TOL_ONLINE
    X = online(A_L, A_M, f_r, p["lams"])
    xn = np.linalg.norm(X, axis=1)
    assert np.max(np.abs(xn - G["xnorm"]) / G["xnorm"]) < TOL_ONLINE
    U = reconstruct(V, X[:64])
    assert np.max(np.abs(U[:, p["idx"]] - G["usample"])) / np.max(np.abs(G["usample"])) < TOL_ONLINE


def test_oracle_pod_matches_reference_eigen(prob):
    from oracle import pod as opod
    V, sigma = opod.pod_svd(prob["S"], nmodes=fx.NMODES)
    LV, MV = fx.apply_LM(prob, V)
    A_L, A_M = opod.project(V, LV, MV)
    check_all(prob, sigma, V, A_L, A_M, opod.online_lu, lambda V_, X: X @ V_.T)


@pytest.mark.skipif(not __import__("oracle.eigenbind", fromlist=["x"]).available(),
                    reason="oracle/_ref/libithaca_eigen.so not built (reference tree absent)")
def test_reference_eigen_reproduces_fixture(prob):
    from oracle import eigenbind
    sigma, U = eigenbind.bdcsvd(prob["S"], fx.NMODES)
    assert np.max(np.abs(sigma - G["sigma"])) / sigma[0] < 1e-14
    assert subspace_residual(U, prob["R"], G["sketch"]) < 1e-13


@pytest.mark.gpu
def test_gpu_pod_matches_reference_eigen(prob):
    from ithaca_gpu import pod
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU
    c, amap = prob["c"], prob["amap"]
    ctx = Context(0)
    coll = Collection(ctx, "quad", c.n, c.Q, c.E, c.jac, c.df)
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    V, sigma, r = pod.offline(ctx, prob["S"], fx.NMODES)
    assert r == fx.NMODES
    A_L, A_M = pod.project(sysg, V)
    check_all(prob, sigma, V, A_L, A_M, lambda L, M, f, lam: pod.online(ctx, L, M, f, lam),
              lambda V_, X: pod.reconstruct(ctx, V_, X))
    ctx.close()
