"""ctypes binding of oracle/_ref/libithaca_ref.so (reference kernels compiled in place).

The library is built by ``oracle/ref/Makefile`` from the reference's Polylib.cpp and
MatrixFreeOps kernel headers; see oracle/ref/ref_kernels.cpp for the drivers.
Test infrastructure only.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libithaca_ref.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("oracle/_ref/libithaca_ref.so is not built (make -C oracle/ref)")
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.ref_cg_solve.restype = ctypes.c_int
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.flags.c_contiguous
    if a.dtype == np.int32:
        return a.ctypes.data_as(_ip)
    assert a.dtype == np.float64
    return a.ctypes.data_as(_dp)


def gll(Q):
    z, w, D = np.zeros(Q), np.zeros(Q), np.zeros(Q * Q)
    lib().ref_gll(Q, _p(z), _p(w), _p(D))
    return z, w, D


def modA(n, Q):
    B, DB = np.zeros(n * Q), np.zeros(n * Q)
    lib().ref_modA(n, Q, _p(B), _p(DB))
    return B, DB


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what}: reference driver returned {rc}")


def helmholtz(dim, n, Q, E, jac, df, deformed, lam, coeffs, nthreads=1):
    out = np.zeros(E * n ** dim)
    rc = lib().ref_helmholtz(dim, n, Q, E, _p(np.ascontiguousarray(jac, dtype=np.float64)),
                             _p(np.ascontiguousarray(df, dtype=np.float64)), int(deformed),
                             ctypes.c_double(lam), _p(np.ascontiguousarray(coeffs, dtype=np.float64)),
                             _p(out), nthreads)
    _check(rc, "ref_helmholtz")
    return out


def bwdtrans(dim, n, Q, E, coeffs, nthreads=1):
    out = np.zeros(E * Q ** dim)
    rc = lib().ref_bwdtrans(dim, n, Q, E, _p(np.ascontiguousarray(coeffs, dtype=np.float64)), _p(out), nthreads)
    _check(rc, "ref_bwdtrans")
    return out


def iproduct(dim, n, Q, E, jac, deformed, phys, nthreads=1):
    out = np.zeros(E * n ** dim)
    rc = lib().ref_iproduct(dim, n, Q, E, _p(np.ascontiguousarray(jac, dtype=np.float64)), int(deformed),
                            _p(np.ascontiguousarray(phys, dtype=np.float64)), _p(out), nthreads)
    _check(rc, "ref_iproduct")
    return out


def physderiv(dim, n, Q, E, df, deformed, phys, nthreads=1):
    outs = [np.zeros(E * Q ** dim) for _ in range(3)]
    rc = lib().ref_physderiv(dim, n, Q, E, _p(np.ascontiguousarray(df, dtype=np.float64)), int(deformed),
                             _p(np.ascontiguousarray(phys, dtype=np.float64)), _p(outs[0]), _p(outs[1]),
                             _p(outs[2]), nthreads)
    _check(rc, "ref_physderiv")
    return outs[:dim]


def cg_solve(dim, n, Q, E, jac, df, deformed, lam, l2g, sign, nglobal, ndir, dinv, rhs, tol, max_iter,
             nthreads=1, x0=None):
    x = np.zeros(nglobal) if x0 is None else np.array(x0, dtype=np.float64)
    eps = ctypes.c_double(0.0)
    it = lib().ref_cg_solve(dim, n, Q, E, _p(np.ascontiguousarray(jac, dtype=np.float64)),
                            _p(np.ascontiguousarray(df, dtype=np.float64)), int(deformed), ctypes.c_double(lam),
                            _p(np.ascontiguousarray(l2g, dtype=np.int32)),
                            _p(np.ascontiguousarray(sign, dtype=np.float64)), nglobal, ndir,
                            _p(np.ascontiguousarray(dinv, dtype=np.float64)),
                            _p(np.ascontiguousarray(rhs, dtype=np.float64)), _p(x), ctypes.c_double(tol),
                            max_iter, nthreads, ctypes.byref(eps))
    return x, it, eps.value


# ---- triangles (ref_tri_* drivers) ----
def tri_tables(n):
    """Reference tables: (z0, w0, D0, B0, DB0), (z1, w1, D1, B1, DB1); w1 as GetW() holds it."""
    Q0, Q1, nc = n + 1, n, n * (n + 1) // 2
    a = [np.zeros(Q0), np.zeros(Q0), np.zeros(Q0 * Q0), np.zeros(n * Q0), np.zeros(n * Q0)]
    b = [np.zeros(Q1), np.zeros(Q1), np.zeros(Q1 * Q1), np.zeros(nc * Q1), np.zeros(nc * Q1)]
    _check(lib().ref_tri_tables(n, *[_p(x) for x in a], *[_p(x) for x in b]), "ref_tri_tables")
    return a, b


def tri_bwdtrans(n, E, coeffs, nthreads=1):
    out = np.zeros(E * (n + 1) * n)
    _check(lib().ref_tri_bwdtrans(n, E, _p(np.ascontiguousarray(coeffs, dtype=np.float64)), _p(out), nthreads),
           "ref_tri_bwdtrans")
    return out


def tri_iproduct(n, E, jac, deformed, phys, nthreads=1):
    out = np.zeros(E * n * (n + 1) // 2)
    _check(lib().ref_tri_iproduct(n, E, _p(np.ascontiguousarray(jac, dtype=np.float64)), int(deformed),
                                  _p(np.ascontiguousarray(phys, dtype=np.float64)), _p(out), nthreads),
           "ref_tri_iproduct")
    return out


def tri_physderiv(n, E, df, deformed, phys, nthreads=1):
    nq = (n + 1) * n
    o0, o1 = np.zeros(E * nq), np.zeros(E * nq)
    _check(lib().ref_tri_physderiv(n, E, _p(np.ascontiguousarray(df, dtype=np.float64)), int(deformed),
                                   _p(np.ascontiguousarray(phys, dtype=np.float64)), _p(o0), _p(o1), nthreads),
           "ref_tri_physderiv")
    return o0, o1


def tri_helmholtz(n, E, jac, df, deformed, lam, coeffs, nthreads=1):
    out = np.zeros(E * n * (n + 1) // 2)
    _check(lib().ref_tri_helmholtz(n, E, _p(np.ascontiguousarray(jac, dtype=np.float64)),
                                   _p(np.ascontiguousarray(df, dtype=np.float64)), int(deformed),
                                   ctypes.c_double(lam), _p(np.ascontiguousarray(coeffs, dtype=np.float64)),
                                   _p(out), nthreads),
           "ref_tri_helmholtz")
    return out


def tri_iproduct_deriv(n, E, jac, df, deformed, in0, in1, nthreads=1):
    out = np.zeros(E * n * (n + 1) // 2)
    f = lambda a: _p(np.ascontiguousarray(a, dtype=np.float64))
    _check(lib().ref_tri_iproduct_deriv(n, E, f(jac), f(df), int(deformed), f(in0), f(in1), _p(out), nthreads),
           "ref_tri_iproduct_deriv")
    return out


# ---- tetrahedra (ref_tet_* drivers) ----
def tet_tables(n):
    Q0, Q, ncb, nct = n + 1, n, n * (n + 1) // 2, n * (n + 1) * (n + 2) // 6
    a = [np.zeros(Q0), np.zeros(Q0), np.zeros(Q0 * Q0), np.zeros(n * Q0), np.zeros(n * Q0)]
    b = [np.zeros(Q), np.zeros(Q), np.zeros(Q * Q), np.zeros(ncb * Q), np.zeros(ncb * Q)]
    c = [np.zeros(Q), np.zeros(Q), np.zeros(Q * Q), np.zeros(nct * Q), np.zeros(nct * Q)]
    _check(lib().ref_tet_tables(n, *[_p(x) for x in a + b + c]), "ref_tet_tables")
    return a, b, c


def _f(a):
    return _p(np.ascontiguousarray(a, dtype=np.float64))


def tet_bwdtrans(n, E, coeffs, nthreads=1):
    out = np.zeros(E * (n + 1) * n * n)
    _check(lib().ref_tet_bwdtrans(n, E, _f(coeffs), _p(out), nthreads), "ref_tet_bwdtrans")
    return out


def tet_iproduct(n, E, jac, deformed, phys, nthreads=1):
    out = np.zeros(E * n * (n + 1) * (n + 2) // 6)
    _check(lib().ref_tet_iproduct(n, E, _f(jac), int(deformed), _f(phys), _p(out), nthreads), "ref_tet_iproduct")
    return out


def tet_physderiv(n, E, df, deformed, phys, nthreads=1):
    nq = (n + 1) * n * n
    o = [np.zeros(E * nq) for _ in range(3)]
    _check(lib().ref_tet_physderiv(n, E, _f(df), int(deformed), _f(phys), *[_p(x) for x in o], nthreads),
           "ref_tet_physderiv")
    return o


def tet_helmholtz(n, E, jac, df, deformed, lam, coeffs, nthreads=1):
    out = np.zeros(E * n * (n + 1) * (n + 2) // 6)
    _check(lib().ref_tet_helmholtz(n, E, _f(jac), _f(df), int(deformed), ctypes.c_double(lam), _f(coeffs),
                                   _p(out), nthreads), "ref_tet_helmholtz")
    return out


def tet_iproduct_deriv(n, E, jac, df, deformed, in0, in1, in2, nthreads=1):
    out = np.zeros(E * n * (n + 1) * (n + 2) // 6)
    _check(lib().ref_tet_iproduct_deriv(n, E, _f(jac), _f(df), int(deformed), _f(in0), _f(in1), _f(in2), _p(out),
                                        nthreads), "ref_tet_iproduct_deriv")
    return out


# ---- prisms (ref_prism_* drivers); tables: directions 0 and 1 as ref_gll/ref_modA(n, n+1),
# direction 2 as tri_tables(n)[1] ----
def prism_bwdtrans(n, E, coeffs, nthreads=1):
    out = np.zeros(E * (n + 1) * (n + 1) * n)
    _check(lib().ref_prism_bwdtrans(n, E, _f(coeffs), _p(out), nthreads), "ref_prism_bwdtrans")
    return out


def prism_iproduct(n, E, jac, deformed, phys, nthreads=1):
    out = np.zeros(E * n * n * (n + 1) // 2)
    _check(lib().ref_prism_iproduct(n, E, _f(jac), int(deformed), _f(phys), _p(out), nthreads), "ref_prism_iproduct")
    return out


def prism_physderiv(n, E, df, deformed, phys, nthreads=1):
    nq = (n + 1) * (n + 1) * n
    o = [np.zeros(E * nq) for _ in range(3)]
    _check(lib().ref_prism_physderiv(n, E, _f(df), int(deformed), _f(phys), *[_p(x) for x in o], nthreads),
           "ref_prism_physderiv")
    return o


def prism_helmholtz(n, E, jac, df, deformed, lam, coeffs, nthreads=1):
    out = np.zeros(E * n * n * (n + 1) // 2)
    _check(lib().ref_prism_helmholtz(n, E, _f(jac), _f(df), int(deformed), ctypes.c_double(lam), _f(coeffs),
                                     _p(out), nthreads), "ref_prism_helmholtz")
    return out


def prism_iproduct_deriv(n, E, jac, df, deformed, in0, in1, in2, nthreads=1):
    out = np.zeros(E * n * n * (n + 1) // 2)
    _check(lib().ref_prism_iproduct_deriv(n, E, _f(jac), _f(df), int(deformed), _f(in0), _f(in1), _f(in2),
                                          _p(out), nthreads), "ref_prism_iproduct_deriv")
    return out


# ---- pyramids (ref_pyr_* drivers); directions 0 and 1 as ref_gll/ref_modA(n, n+1) ----
def pyr_tables(n):
    ncp = n * (n + 1) * (2 * n + 1) // 6
    c = [np.zeros(n), np.zeros(n), np.zeros(n * n), np.zeros(ncp * n), np.zeros(ncp * n)]
    _check(lib().ref_pyr_tables(n, *[_p(x) for x in c]), "ref_pyr_tables")
    return c


def pyr_bwdtrans(n, E, coeffs, nthreads=1):
    out = np.zeros(E * (n + 1) * (n + 1) * n)
    _check(lib().ref_pyr_bwdtrans(n, E, _f(coeffs), _p(out), nthreads), "ref_pyr_bwdtrans")
    return out


def pyr_iproduct(n, E, jac, deformed, phys, nthreads=1):
    out = np.zeros(E * n * (n + 1) * (2 * n + 1) // 6)
    _check(lib().ref_pyr_iproduct(n, E, _f(jac), int(deformed), _f(phys), _p(out), nthreads), "ref_pyr_iproduct")
    return out


def pyr_physderiv(n, E, df, deformed, phys, nthreads=1):
    nq = (n + 1) * (n + 1) * n
    o = [np.zeros(E * nq) for _ in range(3)]
    _check(lib().ref_pyr_physderiv(n, E, _f(df), int(deformed), _f(phys), *[_p(x) for x in o], nthreads),
           "ref_pyr_physderiv")
    return o


def pyr_helmholtz(n, E, jac, df, deformed, lam, coeffs, nthreads=1):
    out = np.zeros(E * n * (n + 1) * (2 * n + 1) // 6)
    _check(lib().ref_pyr_helmholtz(n, E, _f(jac), _f(df), int(deformed), ctypes.c_double(lam), _f(coeffs),
                                   _p(out), nthreads), "ref_pyr_helmholtz")
    return out


def pyr_iproduct_deriv(n, E, jac, df, deformed, in0, in1, in2, nthreads=1):
    out = np.zeros(E * n * (n + 1) * (2 * n + 1) // 6)
    _check(lib().ref_pyr_iproduct_deriv(n, E, _f(jac), _f(df), int(deformed), _f(in0), _f(in1), _f(in2),
                                        _p(out), nthreads), "ref_pyr_iproduct_deriv")
    return out
