"""POD offline / online (oracle restatement, FP64).

Follows solvers/IncNavierStokesSolver/EquationSystems/CoupledLinearNS_ROM.cpp:
  * ROM_offline_phase (:3916-4001): thin SVD of the snapshot matrix (Eigen BDCSVD,
    :3924), reduced-basis size from the cumulative singular-value fraction against
    POD_tolerance (:3935-3944), POD modes = leading left singular vectors (:3953-3954),
    reduced operators RB^T X RB (:3661-3663, :3904-3911).
  * ROM_online_phase (:4003-4100): affine assembly A_r(mu) = A_const + mu A_1
    (gen_affine_mat_proj :4694-4703), reduced solve (colPivHouseholderQr, :4053),
    reconstruction RB x (:4054).
For the Helmholtz operator A(lambda) = L + lambda M the affine pieces are V^T L V and
V^T M V. The method of snapshots (eigen-decomposition of S^T S) spans the same space
as the SVD's U and is what the GPU path implements; both are provided here.
"""
import numpy as np


def rb_size(singular_values, pod_tolerance):
    """CoupledLinearNS_ROM.cpp:3935-3944: RBsize = 1 + (last i with cum(i) < tol) + 1."""
    s = np.asarray(singular_values, dtype=np.float64)
    cum = np.cumsum(s) / s.sum()
    size = 1
    for i, c in enumerate(cum):
        if c < pod_tolerance:
            size = i + 2
    return size


def pod_svd(S, nmodes=None, pod_tolerance=None):
    U, s, _ = np.linalg.svd(S, full_matrices=False)
    r = nmodes if nmodes is not None else rb_size(s, pod_tolerance)
    return U[:, :r], s


def pod_snapshots(S, nmodes):
    """Method of snapshots: C = S^T S = W diag(l) W^T, V = S W_r diag(l_r)^-1/2."""
    C = S.T @ S
    lam, W = np.linalg.eigh(C)
    order = np.argsort(lam)[::-1]
    lam, W = lam[order], W[:, order]
    r = nmodes
    V = S @ (W[:, :r] / np.sqrt(lam[:r]))
    return V, np.sqrt(np.maximum(lam, 0.0)), C


def principal_angle_cos(V1, V2):
    """Cosines of the principal angles between span(V1) and span(V2) (orthonormal bases)."""
    return np.linalg.svd(V1.T @ V2, compute_uv=False)


def project(V, LV, MV):
    """A_L = V^T L V, A_M = V^T M V (columns of LV / MV are L or M applied to V's columns)."""
    return V.T @ LV, V.T @ MV


def online_lu(A_L, A_M, f_r, lambdas):
    """Solve (A_L + lambda A_M) x = f_r for each lambda (LU with partial pivoting)."""
    return np.stack([np.linalg.solve(A_L + lam * A_M, f_r) for lam in lambdas])


def online_qr(A_L, A_M, f_r, lambdas):
    """Same systems through a Householder QR (the reference's colPivHouseholderQr family)."""
    out = []
    for lam in lambdas:
        Qm, R = np.linalg.qr(A_L + lam * A_M)
        out.append(np.linalg.solve(R, Qm.T @ f_r))
    return np.stack(out)
