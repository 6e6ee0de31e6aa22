"""Batched parametric Helmholtz solves (one graph-captured batch on the GPU).

``BatchedHelmholtz(ctx, "quad", problems)`` takes a list of problem dicts with keys
nmodes, npoints, jac, df, amap (an AssemblyMap), lam, rhs; ``solve(mode=...)``
returns per-solve solutions, iteration counts and FP64 relative residuals.
``parametric_quad_problems`` builds the synthetic parametric family of the benchmark
(structured jittered quad meshes of uneven size and order, log-uniform lambda).
"""
import ctypes

import numpy as np

from . import _capi as C
from .mesh import QuadMesh
from .operators import SOLVE_MODES, SHAPES


SolveDesc = C.SolveDesc


class BatchedHelmholtz:
    def __init__(self, ctx, shape, problems):
        self.ctx = ctx
        self.problems = problems
        self._keep = []
        descs = (SolveDesc * len(problems))()
        for i, p in enumerate(problems):
            arrs = [np.ascontiguousarray(p["jac"], dtype=np.float64), np.ascontiguousarray(p["df"], dtype=np.float64),
                    np.ascontiguousarray(p["amap"].l2g, dtype=np.int32),
                    np.ascontiguousarray(p["amap"].sign, dtype=np.float64),
                    np.ascontiguousarray(p["rhs"], dtype=np.float64)]
            self._keep.append(arrs)
            E = arrs[0].size // p["npoints"] ** (2 if shape == "quad" else 3)
            descs[i] = SolveDesc(p["nmodes"], p["npoints"], E, arrs[0].ctypes.data, arrs[1].ctypes.data, 1,
                                 arrs[2].ctypes.data, arrs[3].ctypes.data, p["amap"].nglobal, p["amap"].ndir,
                                 float(p["lam"]), arrs[4].ctypes.data)
        h = ctypes.c_void_p()
        C.call("ithaca_gpu_batch_create", ctx.handle, SHAPES[shape], len(problems), descs, ctypes.byref(h))
        self.handle = h

    def solve(self, mode="fp64", tol=1e-10, max_iter=5000, inner_tol=1e-2, max_outer=50, check_every=8,
              want_x=True):
        from .operators import GlobalLinSysIterativeFullGPU
        o = GlobalLinSysIterativeFullGPU.options(tol=tol, max_iter=max_iter, mode=mode, inner_tol=inner_tol,
                                                 max_outer=max_outer, check_every=check_every)
        n = len(self.problems)
        xs = [np.zeros(p["amap"].nglobal) for p in self.problems] if want_x else None
        xp = (ctypes.c_void_p * n)(*[x.ctypes.data for x in xs]) if want_x else None
        its = np.zeros(n, dtype=np.int32)
        outer = np.zeros(n, dtype=np.int32)
        rel = np.zeros(n)
        ms = ctypes.c_double()
        C.call("ithaca_gpu_batch_solve", self.handle, ctypes.byref(o), xp, ctypes.c_void_p(its.ctypes.data),
               ctypes.c_void_p(outer.ctypes.data), ctypes.c_void_p(rel.ctypes.data), ctypes.byref(ms))
        return dict(x=xs, iterations=its, outer=outer, rel_residual=rel, elapsed_ms=ms.value)

    def autotune(self, reps=5):
        """Times the element-kernel variants (tile shapes) of every order group in FP32 and
        FP64 and keeps the fastest. Returns {nmodes: {"fp32": (variant, [ms per variant]),
        "fp64": (...)}}."""
        ng = ctypes.c_int()
        nm, v32, v64 = (np.zeros(11, dtype=np.int32) for _ in range(3))
        ms = np.zeros(11 * 2 * 3)
        C.call("ithaca_gpu_batch_autotune", self.handle, int(reps), ctypes.byref(ng),
               *[ctypes.c_void_p(a.ctypes.data) for a in (nm, v32, v64, ms)])
        out = {}
        for g in range(ng.value):
            t = ms[g * 6:(g + 1) * 6]
            out[int(nm[g])] = {"fp32": (int(v32[g]), list(t[:3])), "fp64": (int(v64[g]), list(t[3:]))}
        return out

    def set_one_launch(self, on):
        """1: each solve is one graph launch with device-side loops; 0: host-checked chunks."""
        C.call("ithaca_gpu_batch_set_one_launch", self.handle, int(on))

    def close(self):
        if getattr(self, "handle", None):
            C.call("ithaca_gpu_batch_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def parametric_quad_problems(ctx, nsolve=256, e_range=(500, 8000), p_range=(3, 9), lam_range=(1e-2, 1e2),
                             seed=4, jitter=0.1):
    """Synthetic parametric family: lambda log-uniform, E ~ U{e_range} realised as
    nx x ny structured quads of the unit square (seed-jittered), P ~ U{p_range},
    Q = P + 2 points; forcing sin(pi x) sin(pi y); rhs = -Assemble(IProductWRTBase f)."""
    from .operators import Collection, geom_factors
    rng = np.random.default_rng(seed)
    lams = 10 ** rng.uniform(np.log10(lam_range[0]), np.log10(lam_range[1]), nsolve)
    Es = rng.integers(e_range[0], e_range[1] + 1, nsolve)
    Ps = rng.integers(p_range[0], p_range[1] + 1, nsolve)
    probs = []
    for i in range(nsolve):
        nx = max(1, int(round(np.sqrt(Es[i]))))
        ny = max(1, int(round(Es[i] / nx)))
        n, Q = int(Ps[i]) + 1, int(Ps[i]) + 2
        mesh = QuadMesh(nx, ny, jitter=jitter, seed=seed * 1000 + i)
        X = mesh.coords(Q)
        jac, df = geom_factors(ctx, "quad", Q, X)
        amap = mesh.assembly(n)
        coll = Collection(ctx, "quad", n, Q, mesh.E, jac, df)
        f = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1])).reshape(-1)
        ip = coll.iproduct(f)
        rhs = -np.bincount(amap.l2g, weights=amap.sign * ip, minlength=amap.nglobal)
        coll.close()
        probs.append(dict(nmodes=n, npoints=Q, jac=jac, df=df, amap=amap, lam=float(lams[i]), rhs=rhs,
                          mesh=mesh, X=X))
    return probs
