"""ctypes binding of oracle/cport/libcport.so, the compiled CPU port of the reference path
(used as the CPU baseline where the reference tree itself cannot be compiled). Test
infrastructure / CPU baseline only."""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "cport", "libcport.so")
_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("oracle/cport/libcport.so is not built (make -C oracle/cport)")
        _lib = ctypes.CDLL(LIB_PATH)
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def helmholtz(dim, n, Q, E, jac, df, deformed, lam, coeffs, nthreads=1, out=None):
    out = np.zeros(E * n ** dim) if out is None else out
    j, jp = _d(jac)
    f, fp = _d(df)
    c, cp = _d(coeffs)
    rc = lib().cport_helmholtz(dim, n, Q, E, jp, fp, int(deformed), ctypes.c_double(lam), cp,
                               out.ctypes.data_as(_dp), nthreads)
    if rc != 0:
        raise RuntimeError(f"cport_helmholtz returned {rc}")
    return out


def bwdtrans(dim, n, Q, E, coeffs, nthreads=1):
    out = np.zeros(E * Q ** dim)
    c, cp = _d(coeffs)
    rc = lib().cport_bwdtrans(dim, n, Q, E, cp, out.ctypes.data_as(_dp), nthreads)
    if rc != 0:
        raise RuntimeError(f"cport_bwdtrans returned {rc}")
    return out


def iproduct(dim, n, Q, E, jac, deformed, phys, nthreads=1):
    out = np.zeros(E * n ** dim)
    j, jp = _d(jac)
    f, fp = _d(phys)
    rc = lib().cport_iproduct(dim, n, Q, E, jp, int(deformed), fp, out.ctypes.data_as(_dp), nthreads)
    if rc != 0:
        raise RuntimeError(f"cport_iproduct returned {rc}")
    return out


def physderiv(dim, n, Q, E, df, deformed, phys, nthreads=1):
    outs = [np.zeros(E * Q ** dim) for _ in range(3 if dim == 3 else 2)]
    f, fp = _d(df)
    u, up = _d(phys)
    ptrs = [o.ctypes.data_as(_dp) for o in outs] + ([None] if dim == 2 else [])
    rc = lib().cport_physderiv(dim, n, Q, E, fp, int(deformed), up, *ptrs, nthreads)
    if rc != 0:
        raise RuntimeError(f"cport_physderiv returned {rc}")
    return outs


def cg_solve(dim, n, Q, E, jac, df, deformed, lam, l2g, sign, nglobal, ndir, dinv, rhs, tol, max_iter, nthreads=1):
    x = np.zeros(nglobal)
    eps = ctypes.c_double(0.0)
    j, jp = _d(jac)
    f, fp = _d(df)
    s, sp = _d(sign)
    di, dp = _d(dinv)
    r, rp = _d(rhs)
    l = np.ascontiguousarray(l2g, dtype=np.int32)
    it = lib().cport_cg_solve(dim, n, Q, E, jp, fp, int(deformed), ctypes.c_double(lam), l.ctypes.data_as(_ip), sp,
                              nglobal, ndir, dp, rp, x.ctypes.data_as(_dp), ctypes.c_double(tol), max_iter, nthreads,
                              ctypes.byref(eps))
    return x, it, eps.value


def tri_helmholtz(tb, E, jac, df, deformed, lam, coeffs, nthreads=1, out=None):
    """Triangle Helmholtz apply through the compiled port; tb: oracle.tri.TriBasis."""
    out = np.zeros(E * tb.nc) if out is None else out
    held = [_d(a) for a in (tb.B0, tb.DB0, tb.D0, tb.w0, tb.z0, tb.B1, tb.DB1, tb.D1, tb.w1, tb.z1,
                            jac, df, coeffs)]
    ptr = [p for _, p in held]
    rc = lib().cport_tri_helmholtz(int(tb.n), E, *ptr[:10], ptr[10], ptr[11], int(deformed), ctypes.c_double(lam),
                                   ptr[12], out.ctypes.data_as(_dp), nthreads)
    if rc != 0:
        raise RuntimeError(f"cport_tri_helmholtz returned {rc}")
    return out
