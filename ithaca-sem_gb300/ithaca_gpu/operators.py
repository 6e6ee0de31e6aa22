"""Python mirror of the reference operator interfaces over the C ABI.

* ``Context``           -- a device + stream (ithaca_gpu_ctx).
* ``geom_factors``      -- GeomFactors::ComputeJac/ComputeDerivFactors on the GPU.
* ``Collection``        -- one collection of same-shape elements with the GPU
                           implementation of BwdTrans / IProductWRTBase / PhysDeriv /
                           Helmholtz (Collections/Collection.h:119-171 ApplyOperator).
* ``GlobalLinSysIterativeFullGPU`` -- the C0 global Helmholtz system solved by the
                           reference CG recurrence (MultiRegions/GlobalLinSysIterativeFull.cpp)
                           in FP64 or in mixed precision.

Arrays are numpy arrays (host; the library copies them) or CUDA tensors exposing
``data_ptr()`` and ``is_cuda`` (device; no copy). Element arrays use the reference
layouts (include/ithaca_gpu.h). Errors raise ``GpuError`` as the reference raises NekError.
"""
import ctypes

import numpy as np

from . import _capi as C

SHAPES = {"tri": C.SHAPE_TRI, "quad": C.SHAPE_QUAD, "tet": C.SHAPE_TET, "pyr": C.SHAPE_PYR,
          "prism": C.SHAPE_PRISM, "hex": C.SHAPE_HEX}
PRECISIONS = {"fp64": C.FP64, "fp32": C.FP32}
SOLVE_MODES = {"fp64": C.SOLVE_FP64, "mixed": C.SOLVE_MIXED_FP32, "mixed_geo16": C.SOLVE_MIXED_FP32_GEO16}


def _is_device(a):
    return getattr(a, "is_cuda", False)


def _ptr(a, dtype=None):
    """(pointer, on_device) for a numpy array or a CUDA tensor."""
    if a is None:
        return None, 1
    if _is_device(a):
        if not a.is_contiguous():
            raise ValueError("device tensors must be contiguous")
        return ctypes.c_void_p(a.data_ptr()), 1
    if not isinstance(a, np.ndarray) or not a.flags.c_contiguous:
        raise ValueError("host arrays must be C-contiguous numpy arrays")
    if dtype is not None and a.dtype != dtype:
        raise ValueError(f"expected {np.dtype(dtype)} array, got {a.dtype}")
    return ctypes.c_void_p(a.ctypes.data), 0


def _like(ref, size, dtype=np.float64):
    """A zeroed output buffer on the same side as `ref`: a CUDA tensor (same device)
    for a CUDA input, else a numpy array. One call passes one on_device flag for all
    its pointers, so outputs must live where the inputs live."""
    if _is_device(ref):
        import torch
        tdt = torch.float32 if np.dtype(dtype) == np.float32 else torch.float64
        return torch.zeros(size, dtype=tdt, device=ref.device)
    return np.zeros(size, dtype=dtype)


def _same_side(*arrays):
    """Rejects a call that mixes host arrays and CUDA tensors."""
    kinds = {_is_device(a) for a in arrays if a is not None}
    if len(kinds) > 1:
        raise ValueError("the arrays of one call must be all host numpy arrays or all CUDA tensors")


class Context:
    def __init__(self, device=0):
        h = ctypes.c_void_p()
        C.call("ithaca_gpu_ctx_create", device, ctypes.byref(h))
        self.handle = h
        self.device = device

    def synchronize(self):
        C.call("ithaca_gpu_ctx_synchronize", self.handle)

    @property
    def stream(self):
        s = ctypes.c_void_p()
        C.call("ithaca_gpu_ctx_stream", self.handle, ctypes.byref(s))
        return s.value

    def launch_count(self):
        n = ctypes.c_longlong()
        C.call("ithaca_gpu_ctx_launch_count", self.handle, ctypes.byref(n))
        return n.value

    def pipe_peaks(self):
        """Measured FP64 FMA, FP64 MMA (DMMA) and FP32 FMA throughput, TFLOP/s."""
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        C.call("ithaca_gpu_measure_pipe_peaks", self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return {"fp64_fma_tflops": a.value, "fp64_mma_tflops": b.value, "fp32_fma_tflops": c.value}

    def close(self):
        if self.handle:
            C.call("ithaca_gpu_ctx_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def basis_modA(nmodes, npoints):
    """(z, w, D, B, DB) host tables computed by the library (ModifiedA on GLL)."""
    z, w = np.zeros(npoints), np.zeros(npoints)
    D = np.zeros(npoints * npoints)
    B, DB = np.zeros(nmodes * npoints), np.zeros(nmodes * npoints)
    C.call("ithaca_gpu_basis_modA", nmodes, npoints, *[ctypes.c_void_p(a.ctypes.data) for a in (z, w, D, B, DB)])
    return z, w, D, B, DB


def basis_tri(nmodes):
    """Triangle tables computed by the library: (z0, w0, D0, B0, DB0) of ModifiedA on
    nmodes + 1 GLL points and (z1, w1, D1, B1, DB1) of ModifiedB on nmodes Gauss-Radau points."""
    Q0, Q1, nc = nmodes + 1, nmodes, nmodes * (nmodes + 1) // 2
    a = [np.zeros(Q0), np.zeros(Q0), np.zeros(Q0 * Q0), np.zeros(nmodes * Q0), np.zeros(nmodes * Q0)]
    b = [np.zeros(Q1), np.zeros(Q1), np.zeros(Q1 * Q1), np.zeros(nc * Q1), np.zeros(nc * Q1)]
    C.call("ithaca_gpu_basis_tri", nmodes, *[ctypes.c_void_p(x.ctypes.data) for x in a + b])
    return tuple(a), tuple(b)


def basis_tet(nmodes):
    """Direction 2 of the tetrahedron tables computed by the library: (z2, w2, D2, B2, DB2) of
    ModifiedC on nmodes Gauss-Radau (alpha 2) points; directions 0 and 1 are basis_tri's."""
    Q, nc = nmodes, nmodes * (nmodes + 1) * (nmodes + 2) // 6
    c = [np.zeros(Q), np.zeros(Q), np.zeros(Q * Q), np.zeros(nc * Q), np.zeros(nc * Q)]
    C.call("ithaca_gpu_basis_tet", nmodes, *[ctypes.c_void_p(x.ctypes.data) for x in c])
    return tuple(c)


def basis_pyr(nmodes):
    """Direction 2 of the pyramid tables computed by the library: (z2, w2, D2, B2, DB2) of
    ModifiedPyr_C on nmodes Gauss-Radau (alpha 2) points."""
    Q, nc = nmodes, nmodes * (nmodes + 1) * (2 * nmodes + 1) // 6
    c = [np.zeros(Q), np.zeros(Q), np.zeros(Q * Q), np.zeros(nc * Q), np.zeros(nc * Q)]
    C.call("ithaca_gpu_basis_pyr", nmodes, *[ctypes.c_void_p(x.ctypes.data) for x in c])
    return tuple(c)


def _npts(shape, npoints):
    """Quadrature points per element (triangles: npoints x (npoints - 1) collapsed points,
    tetrahedra npoints x (npoints - 1)^2)."""
    if shape == "tri":
        return npoints * (npoints - 1)
    if shape == "tet":
        return npoints * (npoints - 1) ** 2
    if shape in ("prism", "pyr"):
        return npoints * npoints * (npoints - 1)
    return npoints ** (2 if shape == "quad" else 3)


def geom_factors(ctx, shape, npoints, coords):
    """coords (d, E, nq) -> (jac (E*nq,), df (d*d, E*nq)) computed on the GPU, nq = Q^d
    (triangles: Q (Q - 1) collapsed points, Q the direction-0 count).
    Host numpy in -> host numpy out; CUDA tensor in -> CUDA tensors out."""
    dim = 3 if shape in ("hex", "tet", "prism", "pyr") else 2
    if _is_device(coords):
        import torch
        E = coords.shape[1]
        nq = _npts(shape, npoints)
        jac = torch.empty(E * nq, dtype=torch.float64, device=coords.device)
        df = torch.empty((dim * dim, E * nq), dtype=torch.float64, device=coords.device)
        C.call("ithaca_gpu_geom_factors", ctx.handle, SHAPES[shape], npoints, E, ctypes.c_void_p(coords.data_ptr()),
               ctypes.c_void_p(jac.data_ptr()), ctypes.c_void_p(df.data_ptr()), 1)
        return jac, df
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    E = coords.shape[1]
    nq = _npts(shape, npoints)
    jac = np.zeros(E * nq)
    df = np.zeros((dim * dim, E * nq))
    C.call("ithaca_gpu_geom_factors", ctx.handle, SHAPES[shape], npoints, E, ctypes.c_void_p(coords.ctypes.data),
           ctypes.c_void_p(jac.ctypes.data), ctypes.c_void_p(df.ctypes.data), 0)
    return jac, df


class Collection:
    """Element operators for one collection (ImplementationType "GPU")."""

    def __init__(self, ctx, shape, nmodes, npoints, nelmt, jac, df, deformed=True, precision="fp64"):
        self.ctx = ctx
        self.shape = shape
        self.dim = 3 if shape in ("hex", "tet", "prism", "pyr") else 2
        self.n, self.Q, self.E = nmodes, npoints, nelmt
        if shape == "tri":
            self.nm, self.nq = nmodes * (nmodes + 1) // 2, _npts(shape, npoints)
        elif shape == "tet":
            self.nm, self.nq = nmodes * (nmodes + 1) * (nmodes + 2) // 6, _npts(shape, npoints)
        elif shape == "prism":
            self.nm, self.nq = nmodes * nmodes * (nmodes + 1) // 2, _npts(shape, npoints)
        elif shape == "pyr":
            self.nm, self.nq = nmodes * (nmodes + 1) * (2 * nmodes + 1) // 6, _npts(shape, npoints)
        else:
            self.nm, self.nq = nmodes ** self.dim, npoints ** self.dim
        self.precision = precision
        self.dtype = np.float64 if precision == "fp64" else np.float32
        if not _is_device(jac):
            jac = np.ascontiguousarray(jac, dtype=np.float64)
            df = np.ascontiguousarray(df, dtype=np.float64)
        pj, on_dev = _ptr(jac)
        pd, _ = _ptr(df)
        h = ctypes.c_void_p()
        C.call("ithaca_gpu_op_create", ctx.handle, SHAPES[shape], nmodes, npoints, nelmt, pj, pd,
               int(bool(deformed)), PRECISIONS[precision], on_dev, ctypes.byref(h))
        self.handle = h

    def Ndof(self):
        n = ctypes.c_longlong()
        C.call("ithaca_gpu_op_ndof", self.handle, ctypes.byref(n))
        return n.value

    def _out(self, a, size, ref=None):
        if a is not None:
            _same_side(a, ref)
            return a
        return _like(ref, size, self.dtype)

    def bwdtrans(self, inp, out=None):
        out = self._out(out, self.E * self.nq, inp)
        pi, d = _ptr(inp, self.dtype if not _is_device(inp) else None)
        po, _ = _ptr(out)
        C.call("ithaca_gpu_bwdtrans", self.handle, pi, po, d)
        return out

    def iproduct(self, inp, out=None):
        out = self._out(out, self.E * self.nm, inp)
        pi, d = _ptr(inp, self.dtype if not _is_device(inp) else None)
        po, _ = _ptr(out)
        C.call("ithaca_gpu_iproduct", self.handle, pi, po, d)
        return out

    def physderiv(self, inp, outs=None):
        outs = outs or [self._out(None, self.E * self.nq, inp) for _ in range(self.dim)]
        _same_side(inp, *outs)
        pi, d = _ptr(inp, self.dtype if not _is_device(inp) else None)
        ps = [_ptr(o)[0] for o in outs] + [None] * (3 - len(outs))
        C.call("ithaca_gpu_physderiv", self.handle, pi, ps[0], ps[1], ps[2], d)
        return outs

    def iproduct_deriv(self, ins, out=None):
        """IProductWRTDerivBase: sum_k (d phi / d x_k, ins[k]) for the d physical components."""
        ins = list(ins)
        if len(ins) != self.dim:
            raise ValueError(f"expected {self.dim} components")
        out = self._out(out, self.E * self.nm, ins[0])
        _same_side(*ins, out)
        ps = []
        d = 0
        for a in ins:
            p, d = _ptr(a, self.dtype if not _is_device(a) else None)
            ps.append(p)
        ps += [None] * (3 - len(ps))
        po, _ = _ptr(out)
        C.call("ithaca_gpu_iproduct_deriv", self.handle, ps[0], ps[1], ps[2], po, d)
        return out

    def helmholtz(self, lam, inp, out=None):
        out = self._out(out, self.E * self.nm, inp)
        pi, d = _ptr(inp, self.dtype if not _is_device(inp) else None)
        po, _ = _ptr(out)
        C.call("ithaca_gpu_helmholtz", self.handle, ctypes.c_double(lam), pi, po, d)
        return out

    def set_variant(self, variant):
        """FP32 hex Helmholtz kernel: 0 shared-memory, 2/4 register-pencil with TMA-staged
        geometry (elements per CTA), 21/22 persistent pipelined pencil (1/2 elements per group,
        double geometry buffer), 31/32 the same with a single geometry buffer, 41/42 = 31/32
        with the contractions on packed FP32 pairs, 43/44 = 42/41 with vector pencils in a
        bank-conflict-free shared-memory layout (Q = 8), 46 = 43 with the i and j contractions
        on the tensor cores (TF32 in three-term split precision), 47 = 43 with the 1-D
        operators in even-odd form."""
        C.call("ithaca_gpu_op_set_variant", self.handle, int(variant))

    def set_variant64(self, variant):
        """FP64 hex Helmholtz kernel: 0 shared-memory (default), 1 / 2 persistent pipelined
        pencils with even-odd 1-D operators, one / two elements per group (Q even)."""
        C.call("ithaca_gpu_op_set_variant64", self.handle, int(variant))

    def autotune(self, reps=10):
        """Times each kernel variant on this collection and keeps the fastest."""
        chosen = ctypes.c_int()
        variants = (0, 2, 4, 21, 22, 31, 32, 41, 42, 43, 44, 46, 47)
        times = np.zeros(len(variants))
        C.call("ithaca_gpu_op_autotune", self.handle, int(reps), ctypes.byref(chosen),
               ctypes.c_void_p(times.ctypes.data))
        return chosen.value, dict(zip(variants, times.tolist()))

    def helmholtz_diag(self, lam, out=None):
        out = out if out is not None else np.zeros(self.E * self.nm)
        po, d = _ptr(out)
        C.call("ithaca_gpu_helmholtz_diag", self.handle, ctypes.c_double(lam), po, d)
        return out

    def close(self):
        if getattr(self, "handle", None):
            C.call("ithaca_gpu_op_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GlobalLinSysIterativeFullGPU:
    """C0 global Helmholtz system + Jacobi-preconditioned CG on the GPU."""

    def __init__(self, coll, amap):
        if coll.precision != "fp64":
            raise ValueError("the global system needs an FP64 collection (mixed mode derives its FP32 copy)")
        self.coll, self.amap = coll, amap
        l2g = np.ascontiguousarray(amap.l2g, dtype=np.int32)
        sign = np.ascontiguousarray(amap.sign, dtype=np.float64)
        h = ctypes.c_void_p()
        C.call("ithaca_gpu_cg_create", coll.handle, ctypes.c_void_p(l2g.ctypes.data),
               ctypes.c_void_p(sign.ctypes.data), amap.nglobal, amap.ndir, ctypes.byref(h))
        self.handle = h

    @staticmethod
    def options(tol=1e-9, max_iter=5000, mode="fp64", inner_tol=1e-2, max_outer=50, check_every=16):
        o = C.CgOpts()
        C.lib().ithaca_gpu_cg_default_opts(ctypes.byref(o))
        o.tol, o.max_iter, o.mode = tol, max_iter, SOLVE_MODES[mode]
        o.inner_tol, o.max_outer, o.check_every = inner_tol, max_outer, check_every
        return o

    def solve(self, lam, rhs, x=None, **kw):
        x = x if x is not None else _like(rhs, self.amap.nglobal)
        _same_side(rhs, x)
        res = C.CgResult()
        o = self.options(**kw)
        pr, d = _ptr(rhs, np.float64 if not _is_device(rhs) else None)
        px, _ = _ptr(x)
        C.call("ithaca_gpu_cg_solve", self.handle, ctypes.c_double(lam), pr, px, ctypes.byref(o), ctypes.byref(res), d)
        return x, res

    def apply(self, lam, x, y=None):
        y = y if y is not None else _like(x, self.amap.nglobal)
        _same_side(x, y)
        px, d = _ptr(x, np.float64 if not _is_device(x) else None)
        py, _ = _ptr(y)
        C.call("ithaca_gpu_cg_apply", self.handle, ctypes.c_double(lam), px, py, d)
        return y

    def assemble(self, loc, out=None):
        """AssemblyMapCG::Assemble on the GPU (local E*n^d -> global nglobal)."""
        out = out if out is not None else _like(loc, self.amap.nglobal)
        _same_side(loc, out)
        pl, d = _ptr(loc, np.float64 if not _is_device(loc) else None)
        po, _ = _ptr(out)
        C.call("ithaca_gpu_cg_assemble", self.handle, pl, po, d)
        return out

    def global_to_local(self, glob, out=None):
        """AssemblyMapCG::GlobalToLocal on the GPU (global -> local E*n^d)."""
        out = out if out is not None else _like(glob, self.coll.E * self.coll.nm)
        _same_side(glob, out)
        pg, d = _ptr(glob, np.float64 if not _is_device(glob) else None)
        po, _ = _ptr(out)
        C.call("ithaca_gpu_cg_global_to_local", self.handle, pg, po, d)
        return out

    def set_varcoeff(self, kappa):
        """Isotropic diffusion coefficient at the quadrature points (None restores 1)."""
        if kappa is None:
            C.call("ithaca_gpu_cg_set_varcoeff", self.handle, None, 1)
            return
        pk, d = _ptr(kappa, np.float64 if not _is_device(kappa) else None)
        C.call("ithaca_gpu_cg_set_varcoeff", self.handle, pk, d)

    def set_varcoeff_tensor(self, K):
        """Anisotropic coefficient: K has d(d+1)/2 rows (D00, D01, (D02,) D11, (D12, D22)) of
        E*Q^d values at the quadrature points."""
        K = K if _is_device(K) else np.ascontiguousarray(K, dtype=np.float64)
        pk, d = _ptr(K, np.float64 if not _is_device(K) else None)
        C.call("ithaca_gpu_cg_set_varcoeff_tensor", self.handle, pk, d)

    def misfit(self, x, u_target, J=None, dJdx=None):
        """J = sum Jw (u - u_target)^2 at the points and dJ/dx (global)."""
        dev = _is_device(x)
        if J is None:
            J = _like(x, 1)
        _same_side(x, u_target, J, dJdx)
        px, d = _ptr(x, None if dev else np.float64)
        pt, _ = _ptr(u_target)
        pj, _ = _ptr(J)
        pg = _ptr(dJdx)[0] if dJdx is not None else None
        C.call("ithaca_gpu_misfit", self.handle, px, pt, pj, pg, d)
        return J, dJdx

    def kappa_gradient(self, x, psi, grad=None):
        grad = grad if grad is not None else _like(x, self.coll.E * self.coll.nq)
        _same_side(x, psi, grad)
        px, d = _ptr(x, None if _is_device(x) else np.float64)
        pp, _ = _ptr(psi)
        pg, _ = _ptr(grad)
        C.call("ithaca_gpu_kappa_gradient", self.handle, px, pp, pg, d)
        return grad

    def set_persistent(self, mode):
        """Solver path of 2-D systems: -1 automatic (persistent up to 2^20 dofs), 0 the
        graph-captured kernels, 1 the persistent single-launch solver."""
        C.call("ithaca_gpu_cg_set_persistent", self.handle, int(mode))

    def set_fused_update(self, on):
        """1: the mixed solve's FP32 iterations fuse the assembly with the vector update (two
        launches per iteration); 0 (default): separate assembly and update."""
        C.call("ithaca_gpu_cg_set_fused_update", self.handle, int(on))

    def set_successive_rhs(self, nsuccessive):
        """SuccessiveRHS projection of later solves onto up to |nsuccessive| previous
        solutions (> 0 A-conjugate, < 0 residual-minimising, 0 off); resets the buffer."""
        C.call("ithaca_gpu_cg_set_successive_rhs", self.handle, int(nsuccessive))

    def set_wait_test(self, barrier_polls=0, drop_cta=-1, delay_ns=0):
        """Failure-path test hooks of the persistent solver: a shorter grid-barrier wait,
        a CTA that never arrives (every wait then runs out: ERR_TIMEOUT), and a pause of
        every third CTA after each barrier. The defaults restore a normal solve."""
        C.call("ithaca_gpu_cg_set_wait_test", self.handle, int(barrier_polls), int(drop_cta), int(delay_ns))

    def profile_apply(self, lam, mode="mixed", reps=20):
        """Average device time (ms) of the gather + element-apply kernel the solver
        launches for `mode`, timed with CUDA events on the context stream, and the
        algorithmic bytes of one launch."""
        ms, nbytes = ctypes.c_double(), ctypes.c_double()
        C.call("ithaca_gpu_cg_profile_apply", self.handle, SOLVE_MODES[mode], ctypes.c_double(lam), reps,
               ctypes.byref(ms), ctypes.byref(nbytes))
        return ms.value, nbytes.value

    def autotune_inner(self, lam=1.0, variants=(0, 2, 4, 21, 22, 31, 32, 41, 42, 43, 44, 46, 47), reps=10,
                       mode="mixed"):
        """Times the gathered FP32 apply of the mixed solver's inner iteration with each
        FP32 kernel variant of the collection and keeps the fastest (the solver-side
        counterpart of Collection.autotune, which times the ungathered apply). mode
        "mixed_geo16" times the applies on 16-bit geometry (variants 43 and 47 have their
        own forms at Q = 8; the others run the packed-pair kernel).
        Returns (chosen variant, {variant: ms})."""
        times = {}
        for v in variants:
            self.coll.set_variant(v)
            times[v] = self.profile_apply(lam, mode=mode, reps=reps)[0]
        best = min(times, key=times.get)
        self.coll.set_variant(best)
        return best, times

    def autotune_fp64(self, lam=1.0, variants=(0, 1, 2), reps=10):
        """Times the gathered FP64 apply (the FP64 solve's and the outer residual's) with each
        FP64 hex kernel variant and keeps the fastest. Returns (chosen variant, {variant: ms})."""
        times = {}
        for v in variants:
            self.coll.set_variant64(v)
            times[v] = self.profile_apply(lam, mode="fp64", reps=reps)[0]
        best = min(times, key=times.get)
        self.coll.set_variant64(best)
        return best, times

    def diagonal(self, lam, out=None):
        out = out if out is not None else np.zeros(self.amap.nglobal - self.amap.ndir)
        po, d = _ptr(out)
        C.call("ithaca_gpu_cg_diagonal", self.handle, ctypes.c_double(lam), po, d)
        return out

    def helmsolve(self, lam, forcing, out=None, dirichlet=None, **kw):
        """ContField::v_HelmSolve: forcing at the quadrature points -> local coefficients.
        dirichlet: the ndir Dirichlet global coefficients (None: homogeneous data)."""
        out = out if out is not None else _like(forcing, self.coll.E * self.coll.nm)
        _same_side(forcing, out, dirichlet)
        res = C.CgResult()
        o = self.options(**kw)
        pf, d = _ptr(forcing, np.float64 if not _is_device(forcing) else None)
        po, _ = _ptr(out)
        if dirichlet is None:
            C.call("ithaca_gpu_helmsolve", self.handle, ctypes.c_double(lam), pf, po, ctypes.byref(o),
                   ctypes.byref(res), d)
        else:
            if len(dirichlet) != self.amap.ndir:
                raise ValueError(f"expected {self.amap.ndir} Dirichlet values")
            pdv, _ = _ptr(dirichlet, np.float64 if not _is_device(dirichlet) else None)
            C.call("ithaca_gpu_helmsolve_dirichlet", self.handle, ctypes.c_double(lam), pf, pdv, po,
                   ctypes.byref(o), ctypes.byref(res), d)
        return out, res

    def close(self):
        if getattr(self, "handle", None):
            C.call("ithaca_gpu_cg_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GlobalLinSysIterativeStaticCondGPU:
    """Statically condensed C0 system + Jacobi-preconditioned CG on the boundary modes
    (GlobalLinSysIterativeStaticCond), on the GPU."""

    def __init__(self, coll, amap):
        if coll.precision != "fp64":
            raise ValueError("the global system needs an FP64 collection")
        self.coll, self.amap = coll, amap
        l2g = np.ascontiguousarray(amap.l2g, dtype=np.int32)
        sign = np.ascontiguousarray(amap.sign, dtype=np.float64)
        h = ctypes.c_void_p()
        C.call("ithaca_gpu_sc_create", coll.handle, ctypes.c_void_p(l2g.ctypes.data),
               ctypes.c_void_p(sign.ctypes.data), amap.nglobal, amap.ndir, ctypes.byref(h))
        self.handle = h

    def info(self):
        v = [ctypes.c_int() for _ in range(4)]
        C.call("ithaca_gpu_sc_info", self.handle, *[ctypes.byref(x) for x in v])
        return dict(nbnd_global=v[0].value, ndir_bnd=v[1].value, nbnd_local=v[2].value, nint_local=v[3].value)

    def solve_local(self, lam, loc_rhs, loc_inout=None, **kw):
        """GlobalLinSysStaticCond::v_Solve: local forcing -> local solution; loc_inout holds
        the known boundary values (Dirichlet data) and receives the solution."""
        n = self.coll.E * self.coll.nm
        if loc_inout is None:
            loc_inout = _like(loc_rhs, n)
        _same_side(loc_rhs, loc_inout)
        res = C.CgResult()
        o = GlobalLinSysIterativeFullGPU.options(**kw)
        pr, d = _ptr(loc_rhs, np.float64 if not _is_device(loc_rhs) else None)
        pio, _ = _ptr(loc_inout)
        C.call("ithaca_gpu_sc_solve", self.handle, ctypes.c_double(lam), pr, pio, ctypes.byref(o), ctypes.byref(res), d)
        return loc_inout, res

    def helmsolve(self, lam, forcing, dirichlet=None, **kw):
        """ContField::v_HelmSolve with this solve: forcing at the quadrature points ->
        local coefficients; dirichlet: the ndir Dirichlet global coefficients or None."""
        loc_rhs = self.coll.iproduct(forcing)
        loc_rhs = -loc_rhs
        n = self.coll.E * self.coll.nm
        if dirichlet is None:
            inout = _like(forcing, n)
        else:
            xg = np.zeros(self.amap.nglobal)
            xg[:self.amap.ndir] = np.asarray(dirichlet)
            inout = self.amap.sign * xg[self.amap.l2g]
            if _is_device(forcing):
                import torch
                inout = torch.from_numpy(inout).to(forcing.device)
        return self.solve_local(lam, loc_rhs, inout, **kw)

    def close(self):
        if getattr(self, "handle", None):
            C.call("ithaca_gpu_sc_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
