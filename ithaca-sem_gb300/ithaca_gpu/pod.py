"""POD reduced basis on the GPU (ITHACA-SEM ROM offline / online, CoupledLinearNS_ROM.cpp).

* ``offline(ctx, S, nmodes)``      -- method-of-snapshots POD of the snapshot matrix
  S (N x ns, one snapshot per column): V (N x r orthonormal), singular values, r.
* ``offline_device(ctx, St, nmodes)`` -- the same for a snapshot matrix already on the
  device: a CUDA tensor St (ns, N) whose row k is snapshot k (fieldio.load_snapshots);
  V comes back on the device as (r, N), one mode per row.
* ``rb_size(sigma, tol)``          -- reduced-basis size from POD_tolerance (:3935-3944).
* ``project(system, V)``           -- A_L = V^T L V, A_M = V^T M V on the free dofs.
* ``online(ctx, A_L, A_M, f_r, lambdas)`` -- batched FP64 LU solves of
  (A_L + lambda A_M) x = f_r, returned as (nlambda, r).
* ``reconstruct(ctx, V, X)``       -- u = V x for each reduced solution.
"""
import ctypes

import numpy as np

from . import _capi as C


def _f64(a):
    return np.asfortranarray(a, dtype=np.float64)


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def gram(ctx, S):
    S = _f64(S)
    N, ns = S.shape
    Cm = np.zeros((ns, ns), order="F")
    C.call("ithaca_gpu_pod_gram", ctx.handle, N, ns, _p(S), _p(Cm), 0)
    return Cm


def offline(ctx, S, nmodes):
    S = _f64(S)
    N, ns = S.shape
    V = np.zeros((N, nmodes), order="F")
    sigma = np.zeros(ns)
    r = ctypes.c_int()
    C.call("ithaca_gpu_pod_offline", ctx.handle, N, ns, _p(S), nmodes, _p(V), _p(sigma), ctypes.byref(r), 0)
    return np.asfortranarray(V[:, :r.value]), sigma, r.value


def offline_device(ctx, St, nmodes):
    import torch
    if not getattr(St, "is_cuda", False) or St.dtype != torch.float64 or St.dim() != 2 or not St.is_contiguous():
        raise ValueError("St must be a contiguous FP64 CUDA tensor (nsnapshots, N)")
    ns, N = St.shape
    V = torch.zeros((nmodes, N), dtype=torch.float64, device=St.device)
    sigma = np.zeros(ns)
    r = ctypes.c_int()
    C.call("ithaca_gpu_pod_offline", ctx.handle, N, ns, ctypes.c_void_p(St.data_ptr()), nmodes,
           ctypes.c_void_p(V.data_ptr()), _p(sigma), ctypes.byref(r), 1)
    return V[:r.value], sigma, r.value


def rb_size(sigma, pod_tolerance):
    sigma = np.ascontiguousarray(sigma, dtype=np.float64)
    r = ctypes.c_int()
    C.call("ithaca_gpu_pod_rb_size", sigma.size, _p(sigma), ctypes.c_double(pod_tolerance), ctypes.byref(r))
    return r.value


def project(system, V):
    V = _f64(V)
    r = V.shape[1]
    A_L = np.zeros((r, r), order="F")
    A_M = np.zeros((r, r), order="F")
    C.call("ithaca_gpu_pod_project", system.handle, r, _p(V), _p(A_L), _p(A_M), 0)
    return A_L, A_M


def online(ctx, A_L, A_M, f_r, lambdas):
    A_L, A_M = _f64(A_L), _f64(A_M)
    r = A_L.shape[0]
    f_r = np.ascontiguousarray(f_r, dtype=np.float64)
    lambdas = np.ascontiguousarray(lambdas, dtype=np.float64)
    X = np.zeros((lambdas.size, r))
    C.call("ithaca_gpu_pod_online", ctx.handle, r, _p(A_L), _p(A_M), _p(f_r), lambdas.size, _p(lambdas), _p(X), 0)
    return X


def reconstruct(ctx, V, X):
    V = _f64(V)
    X = np.ascontiguousarray(X, dtype=np.float64)  # (nsol, r): column-major r x nsol
    N, r = V.shape
    U = np.zeros((X.shape[0], N))
    C.call("ithaca_gpu_pod_reconstruct", ctx.handle, N, r, _p(V), X.shape[0], _p(X), _p(U), 0)
    return U
