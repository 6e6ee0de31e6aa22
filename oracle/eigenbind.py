"""ctypes binding of oracle/_ref/libithaca_eigen.so: the reference's vendored Eigen 3.3.7
BDCSVD and colPivHouseholderQr, as CoupledLinearNS_ROM.cpp:3925 and :4053 call them.
Test infrastructure only (fixture generation and CPU checks where the reference tree is)."""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libithaca_eigen.so")
_lib = None
_dp = ctypes.POINTER(ctypes.c_double)


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(LIB_PATH)
    return _lib


def bdcsvd(S, nmodes):
    """(sigma (ns,), U (N, nmodes)) of the thin BDCSVD of S (N x ns)."""
    S = np.asfortranarray(S, dtype=np.float64)
    N, ns = S.shape
    sigma = np.zeros(min(N, ns))
    U = np.zeros((N, nmodes), order="F")
    rc = lib().ref_pod_bdcsvd(N, ns, S.ctypes.data_as(_dp), nmodes, sigma.ctypes.data_as(_dp), U.ctypes.data_as(_dp))
    if rc:
        raise RuntimeError(f"ref_pod_bdcsvd returned {rc}")
    return sigma, U


def colpivqr_solve(A, b):
    A = np.asfortranarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(A.shape[0])
    rc = lib().ref_pod_colpivqr_solve(A.shape[0], A.ctypes.data_as(_dp), b.ctypes.data_as(_dp), x.ctypes.data_as(_dp))
    if rc:
        raise RuntimeError(f"ref_pod_colpivqr_solve returned {rc}")
    return x
