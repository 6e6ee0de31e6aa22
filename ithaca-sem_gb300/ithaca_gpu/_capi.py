"""ctypes binding of lib/libithaca_gpu.so (the C ABI declared in include/ithaca_gpu.h).

The library must have been built (``python ithaca-sem_gb300/build.py``); there is no
CPU fallback: loading fails loudly when the shared object is missing.
"""
import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(_PKG)
LIB_PATH = os.path.join(ROOT, "lib", "libithaca_gpu.so")

OK = 0
ERR_ARG, ERR_UNSUPPORTED, ERR_CUDA, ERR_NOMEM = 1, 2, 3, 4
ERR_NOT_CONVERGED, ERR_GEOMETRY, ERR_TIMEOUT, ERR_NUMERIC = 5, 6, 7, 8
SHAPE_TRI, SHAPE_QUAD, SHAPE_TET, SHAPE_PYR, SHAPE_PRISM, SHAPE_HEX = 3, 4, 5, 6, 7, 8
FP64, FP32 = 0, 1
SOLVE_FP64, SOLVE_MIXED_FP32, SOLVE_MIXED_FP32_GEO16 = 0, 1, 2

_ERRNAMES = {1: "ERR_ARG", 2: "ERR_UNSUPPORTED", 3: "ERR_CUDA", 4: "ERR_NOMEM", 5: "ERR_NOT_CONVERGED",
             6: "ERR_GEOMETRY", 7: "ERR_TIMEOUT", 8: "ERR_NUMERIC"}


class GpuError(RuntimeError):
    """A non-zero status from the C ABI (the reference would raise NekError)."""

    def __init__(self, code, msg):
        super().__init__(f"{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


class CgOpts(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("max_iter", ctypes.c_int), ("mode", ctypes.c_int),
                ("inner_tol", ctypes.c_double), ("max_outer", ctypes.c_int), ("check_every", ctypes.c_int)]


class CgResult(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("outer_iterations", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("eps", ctypes.c_double), ("rhs_magnitude", ctypes.c_double)]


class SolveDesc(ctypes.Structure):
    """ithaca_gpu_solve_desc (one system of a batch)."""
    _fields_ = [("nmodes", ctypes.c_int), ("npoints", ctypes.c_int), ("nelmt", ctypes.c_int),
                ("jac", ctypes.c_void_p), ("df", ctypes.c_void_p), ("deformed", ctypes.c_int),
                ("l2g", ctypes.c_void_p), ("sign", ctypes.c_void_p), ("nglobal", ctypes.c_int),
                ("ndir", ctypes.c_int), ("lam", ctypes.c_double), ("rhs", ctypes.c_void_p)]


_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_pp = ctypes.POINTER(ctypes.c_void_p)

# name -> argtypes (all return int status)
SIGNATURES = {
    "ithaca_gpu_last_error": [ctypes.c_char_p, ctypes.c_size_t],
    "ithaca_gpu_version": [],
    "ithaca_gpu_ctx_create": [_i, _pp],
    "ithaca_gpu_ctx_destroy": [_vp],
    "ithaca_gpu_ctx_synchronize": [_vp],
    "ithaca_gpu_ctx_stream": [_vp, _pp],
    "ithaca_gpu_ctx_launch_count": [_vp, ctypes.POINTER(ctypes.c_longlong)],
    "ithaca_gpu_basis_modA": [_i, _i, _vp, _vp, _vp, _vp, _vp],
    "ithaca_gpu_basis_tri": [_i] + [_vp] * 10,
    "ithaca_gpu_basis_tet": [_i] + [_vp] * 5,
    "ithaca_gpu_basis_pyr": [_i] + [_vp] * 5,
    "ithaca_gpu_geom_factors": [_vp, _i, _i, _i, _vp, _vp, _vp, _i],
    "ithaca_gpu_op_create": [_vp, _i, _i, _i, _i, _vp, _vp, _i, _i, _i, _pp],
    "ithaca_gpu_op_destroy": [_vp],
    "ithaca_gpu_op_ndof": [_vp, ctypes.POINTER(ctypes.c_longlong)],
    "ithaca_gpu_bwdtrans": [_vp, _vp, _vp, _i],
    "ithaca_gpu_iproduct": [_vp, _vp, _vp, _i],
    "ithaca_gpu_physderiv": [_vp, _vp, _vp, _vp, _vp, _i],
    "ithaca_gpu_iproduct_deriv": [_vp, _vp, _vp, _vp, _vp, _i],
    "ithaca_gpu_helmholtz": [_vp, _d, _vp, _vp, _i],
    "ithaca_gpu_helmholtz_diag": [_vp, _d, _vp, _i],
    "ithaca_gpu_op_set_variant": [_vp, _i],
    "ithaca_gpu_op_set_variant64": [_vp, _i],
    "ithaca_gpu_op_autotune": [_vp, _i, ctypes.POINTER(ctypes.c_int), _vp],
    "ithaca_gpu_cg_create": [_vp, _vp, _vp, _i, _i, _pp],
    "ithaca_gpu_cg_destroy": [_vp],
    "ithaca_gpu_cg_set_persistent": [_vp, _i],
    "ithaca_gpu_cg_set_successive_rhs": [_vp, _i],
    "ithaca_gpu_cg_set_wait_test": [_vp, ctypes.c_longlong, _i, _i],
    "ithaca_gpu_cg_default_opts": [ctypes.POINTER(CgOpts)],
    "ithaca_gpu_cg_solve": [_vp, _d, _vp, _vp, ctypes.POINTER(CgOpts), ctypes.POINTER(CgResult), _i],
    "ithaca_gpu_cg_apply": [_vp, _d, _vp, _vp, _i],
    "ithaca_gpu_cg_diagonal": [_vp, _d, _vp, _i],
    "ithaca_gpu_cg_assemble": [_vp, _vp, _vp, _i],
    "ithaca_gpu_cg_global_to_local": [_vp, _vp, _vp, _i],
    "ithaca_gpu_helmsolve": [_vp, _d, _vp, _vp, ctypes.POINTER(CgOpts), ctypes.POINTER(CgResult), _i],
    "ithaca_gpu_helmsolve_dirichlet": [_vp, _d, _vp, _vp, _vp, ctypes.POINTER(CgOpts), ctypes.POINTER(CgResult), _i],
    "ithaca_gpu_vcs_solve_viscous": [_vp, _i, _pp, _pp, _d, _vp, _pp, _pp, ctypes.POINTER(CgOpts),
                                     ctypes.POINTER(CgResult), _i],
    "ithaca_gpu_cg_set_fused_update": [_vp, _i],
    "ithaca_gpu_vcs_solve_pressure": [_vp, _vp, _vp, _vp, ctypes.POINTER(CgOpts), ctypes.POINTER(CgResult), _i],
    "ithaca_gpu_sc_create": [_vp, _vp, _vp, _i, _i, _pp],
    "ithaca_gpu_sc_destroy": [_vp],
    "ithaca_gpu_sc_info": [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                           ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
    "ithaca_gpu_sc_solve": [_vp, _d, _vp, _vp, ctypes.POINTER(CgOpts), ctypes.POINTER(CgResult), _i],
    "ithaca_gpu_batch_create": [_vp, _i, _i, ctypes.POINTER(SolveDesc), _pp],
    "ithaca_gpu_batch_destroy": [_vp],
    "ithaca_gpu_batch_set_one_launch": [_vp, _i],
    "ithaca_gpu_batch_autotune": [_vp, _i, ctypes.POINTER(ctypes.c_int), _vp, _vp, _vp, _vp],
    "ithaca_gpu_batch_solve": [_vp, ctypes.POINTER(CgOpts), _vp, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_double)],
    "ithaca_gpu_cg_set_varcoeff": [_vp, _vp, _i],
    "ithaca_gpu_cg_set_varcoeff_tensor": [_vp, _vp, _i],
    "ithaca_gpu_misfit": [_vp, _vp, _vp, _vp, _vp, _i],
    "ithaca_gpu_kappa_gradient": [_vp, _vp, _vp, _vp, _i],
    "ithaca_gpu_pod_gram": [_vp, _i, _i, _vp, _vp, _i],
    "ithaca_gpu_pod_gram_noalloc": [_i, _i, _vp, _vp, _vp],
    "ithaca_gpu_pod_offline": [_vp, _i, _i, _vp, _i, _vp, _vp, ctypes.POINTER(ctypes.c_int), _i],
    "ithaca_gpu_pod_rb_size": [_i, _vp, _d, ctypes.POINTER(ctypes.c_int)],
    "ithaca_gpu_pod_project": [_vp, _i, _vp, _vp, _vp, _i],
    "ithaca_gpu_pod_online": [_vp, _i, _vp, _vp, _vp, _i, _vp, _vp, _i],
    "ithaca_gpu_pod_reconstruct": [_vp, _i, _i, _vp, _i, _vp, _vp, _i],
    "ithaca_gpu_measure_pipe_peaks": [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_double)],
    "ithaca_gpu_cg_profile_apply": [_vp, _i, _d, _i, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
}

_lib = None


def exported_symbols():
    """Names of every entry point the header declares (checked against the .so)."""
    return sorted(SIGNATURES)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with python ithaca-sem_gb300/build.py "
                               "(the GPU path has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = None if name == "ithaca_gpu_cg_default_opts" else ctypes.c_int
        _lib = L
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().ithaca_gpu_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc):
    if rc != OK:
        raise GpuError(rc, last_error())
    return rc


def call(name, *args):
    return check(getattr(lib(), name)(*args))
