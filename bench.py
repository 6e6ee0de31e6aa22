"""Benchmark: Helmholtz GDOF/s & CG solves/s, mixed vs FP64 on the GPU at 1e-10 relative residual.

Workload (one GPU): 3-D Helmholtz (lambda = 1) on a 32^3 hexahedral mesh of the unit
cube curved by x_a + 0.05 sin(2 pi x_b) sin(2 pi x_c) (cyclic), per-quadrature-point
Jacobians, ModifiedA P = 6 (7 modes, 8 GLL points per direction), forcing
f = sin(pi x) sin(pi y) sin(pi z), homogeneous Dirichlet boundary. A step is one
Jacobi-preconditioned CG solve of the assembled C0 system to an FP64 relative residual
||b - A x||_2 / ||b||_2 < 1e-10, FP32 inner solves inside FP64 iterative refinement (the
inner operator's geometry stored as halves with per-element scales, --mixed-mode mixed_geo16;
the FP32-geometry inner solve is measured beside it).
Inputs are synthetic and seeded; no dataset is involved.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--order P] [--mesh M] [--full 0|1]
  python bench.py --config quad2d|mixed2d|hex_orders|batched|pod|adjoint|inner_apply|peaks|all   (secondary workloads)

The default line also carries the metric's other configurations measured in the same
run (--full 1): the same hexes at P = 8, the 32 x 32 quad mesh at P = 6 and 8 with
lambda in {0.1, 1, 10} (mixed vs FP64), and the 256-solve parametric batch; and, as its
CPU baseline, one full solve of the headline workload by the compiled CPU port of the
reference path with the GPU FP64 solution's difference from it.
`--impl reference` times the reference path's CPU implementation on the host cores
(the compiled C++ port of the reference kernels and CG recurrence, oracle/cport).
Under torchrun (N > 1) every rank solves its own copy (replicas: the single solve has
no multi-GPU path); value = total solves / max time over ranks.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300")]

METRIC = "Helmholtz GDOF/s & CG solves/s: mixed vs FP64 GPU at 1e-10 rel. residual"
TOL = 1e-10
LAMBDA = 1.0


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def build_workload(mesh_n, order):
    """Mesh, quadrature coordinates, assembly map and forcing of the hex workload."""
    from ithaca_gpu.mesh import HexMesh
    n, Q = order + 1, order + 2
    mesh = HexMesh(mesh_n, mesh_n, mesh_n, curve_amp=0.05)
    X = mesh.coords(Q)
    amap = mesh.assembly(n)
    f = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1]) * np.sin(np.pi * X[2])).reshape(-1)
    return mesh, n, Q, X, amap, f


def max_over_ranks(ms, world, device="cpu"):
    """The slowest rank's time (ms): every rank's timed region is bracketed by barriers,
    and the whole job takes as long as its slowest replica."""
    if world <= 1:
        return float(ms)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(steps, ms, world):
    """Whole-job solves/s of `world` replicas that each ran `steps` solves in `ms`."""
    return world * steps / (ms / 1e3)


def fp32_kernel_name(variant, n, Q):
    """Name of the FP32 hex Helmholtz kernel an autotuner variant launches."""
    if variant == 0:
        return f"helm_kernel<float,3,{n},{Q}>"
    if variant in (2, 4):
        return f"helm3_pencil_kernel<float,{n},{Q},{variant}>"
    if variant in (43, 44, 46, 47):
        if Q != 8:  # vector pencils exist for Q = 8; elsewhere 42 / 41 run
            return fp32_kernel_name(41 if variant == 44 else 42, n, Q)
        return (f"helm3_pipe_kernel<float,{n},{Q},{1 if variant == 44 else 2},gather,1,packed,vec4"
                + {46: ",tf32x3>", 47: ",evenodd>"}.get(variant, ">"))
    return (f"helm3_pipe_kernel<float,{n},{Q},{variant % 10},gather,{2 if variant // 10 == 2 else 1}"
            + (",packed>" if variant // 10 == 4 else ">"))


def geo16_kernel_name(variant, n, Q):
    """Name of the FP32 hex Helmholtz kernel on 16-bit geometry for an autotuner variant."""
    if Q == 8 and variant in (43, 47):
        return f"helm3_pipe_kernel<float,{n},{Q},2,gather,1,half,packed,vec4" + (",evenodd>" if variant == 47 else ">")
    return f"helm3_pipe_kernel<float,{n},{Q},1,gather,1,half,packed>"


# FP32 kernel variants with a 16-bit-geometry form (any other variant runs the packed one, 42).
GEO16_VARIANTS = (42, 43, 47)


# DRAM bytes (read + write) per element of one gathered FP32 apply as the inner iteration
# launches it (scattered output: owned rows and assembly-ordered slots), from an ncu
# capture of the kernel on 28^3 hexes (variant 42: 394.1 MB read + 5.4 MB written per
# launch over 21,952 elements; variants 43 and 47: 394.1 + 5.5 MB; variant 47 on 16-bit
# geometry: 237.3 + 5.2 MB); a launch's traffic grows with the number of elements, so the
# bench scales it by E. Keys: (mixed mode, kernel variant, modes, points).
TRAFFIC_PER_ELEMENT = {("mixed", 42, 7, 8): 18200, ("mixed", 43, 7, 8): 18204, ("mixed", 47, 7, 8): 18204,
                       ("mixed_geo16", 47, 7, 8): 11044}


def inner_roofline(mode, variant, n, Q, E, ms, nbytes, peak, peak_kind):
    """Roofline entry of the inner FP32 gathered apply: algorithmic bytes per launch over its
    CUDA-event time, against the measured copy bandwidth; DRAM traffic from the ncu
    capture of the same kernel where one exists."""
    achieved = nbytes / (ms / 1e3) / 1e9
    key = (mode, variant, n, Q)
    half = mode == "mixed_geo16"
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": TRAFFIC_PER_ELEMENT[key] * E if key in TRAFFIC_PER_ELEMENT else None,
            "kernel": (geo16_kernel_name(variant, n, Q) if half else fp32_kernel_name(variant, n, Q))
                      + " gather (inner FP32 apply)",
            "kernel_ms": ms, "bytes_per_launch": nbytes, "mixed_mode": mode,
            "bytes_rule": ("per element 4 (2 n^3) + 2 (7 Q^3) + 32 + 4 n^3: FP32 coefficients in and out, J w "
                           "and the six metric terms per point as halves with 8 FP32 scales, the signed index "
                           "per local dof" if half else
                           "per element 4 (2 n^3 + 7 Q^3) + 4 n^3: FP32 coefficients in and out, J w and the "
                           "six metric terms per point, the signed index per local dof"),
            "layout_overhead_bytes_per_launch": 4.0 * E * n ** 3,
            "peak_source": peak_kind}


def workload_config(args, n, Q, E, N, ndir):
    return {"workload": f"3-D Helmholtz, {args.mesh}^3 curved hexes, P={args.order} (n={n}, Q={Q}), "
                        f"lambda={LAMBDA}, Jacobi PCG to {TOL:g} rel. residual",
            "elements": E, "modes_per_dir": n, "points_per_dir": Q, "global_dofs": N, "solve_dofs": N - ndir,
            "local_dofs": E * n ** 3, "inner": "fp32 PCG in fp64 iterative refinement",
            "l2": "inputs larger than L2 (geometry and vectors exceed 129 MB)", "parallelism": "replicas"}


def cpu_full_solve(n, Q, E, jac, df, amap, b, dinv, nthreads):
    """One full FP64 solve of the workload by the compiled CPU port of the reference
    kernels and CG recurrence (oracle/cport, pinned to the reference build by the golden
    tests): its own iteration count, solution and wall time."""
    from oracle import cportbind
    t0 = time.perf_counter()
    x, it, eps = cportbind.cg_solve(3, n, Q, E, jac, df, True, LAMBDA, amap.l2g, amap.sign, amap.nglobal, amap.ndir,
                                    dinv, b, TOL, 5000, nthreads)
    return x, it, time.perf_counter() - t0


def _solve_rate(torch, stream, fn, reps):
    """Solves/s of fn (one solve per call) over reps calls, CUDA events on `stream`."""
    a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        out = fn()
    z.record(stream)
    z.synchronize()
    return reps / (a.elapsed_time(z) / 1e3), out


def hex_order8_fields(torch, cuda):
    """32^3 curved hexes at P = 8 (n = 9, Q = 10), lambda = 1, to 1e-10: mixed and FP64
    solves/s (the largest order of the 3-D sweep)."""
    from ithaca_gpu.workload import hex_workload
    w = hex_workload(32, 8)
    ctx, sysg, b = w["ctx"], w["system"], w["b"]
    stream = torch.cuda.ExternalStream(ctx.stream, device=cuda)
    variant, _ = sysg.autotune_inner(LAMBDA, reps=5)
    variant64, _ = sysg.autotune_fp64(LAMBDA, reps=3)
    x = torch.zeros_like(b)
    sysg.solve(LAMBDA, b, x, tol=TOL, mode="mixed")
    mixed, (_, rm) = _solve_rate(torch, stream, lambda: sysg.solve(LAMBDA, b, x, tol=TOL, mode="mixed"), 2)
    xm = x.clone()
    fp64, (_, r64) = _solve_rate(torch, stream, lambda: sysg.solve(LAMBDA, b, x, tol=TOL, mode="fp64"), 1)
    out = {"workload": "32^3 curved hexes, P=8 (n=9, Q=10), lambda=1, to 1e-10",
           "solve_dofs": w["amap"].nglobal - w["amap"].ndir, "fp32_kernel_variant": variant,
           "fp64_kernel_variant": variant64,
           "mixed": {"solves_per_s": mixed, "iterations": rm.iterations, "outer": rm.outer_iterations,
                     "rel_residual": rm.rel_residual},
           "fp64": {"solves_per_s": fp64, "iterations": r64.iterations, "rel_residual": r64.rel_residual,
                    "timed": "1 solve (FP64 graph captured by the first call inside it)"},
           "speedup_mixed_vs_fp64": mixed / fp64,
           "max_rel_diff_mixed_vs_fp64": float((x - xm).abs().max() / x.abs().max())}
    del w, sysg, b, x, xm
    ctx.close()
    torch.cuda.empty_cache()
    return out


def quad_mixed_fields(torch, cuda):
    """The 32 x 32 jittered-quad mesh at P = 6 and 8, lambda in {0.1, 1, 10}, to 1e-10:
    mixed vs FP64 solves/s, one system at a time, and the difference of the mixed
    solution from the FP64 one."""
    from ithaca_gpu.workload import quad_workload
    rows = []
    for P in (6, 8):
        w = quad_workload(32, P)
        sysg, ctx = w["system"], w["ctx"]
        stream = torch.cuda.ExternalStream(ctx.stream, device=cuda)
        b = torch.from_numpy(w["b"]).to(cuda)
        x = torch.zeros_like(b)
        for lam in (0.1, 1.0, 10.0):
            row = {"P": P, "lambda": lam}
            for mode in ("fp64", "mixed"):
                for _ in range(3):
                    sysg.solve(lam, b, x, tol=TOL, mode=mode)
                rate, (_, res) = _solve_rate(torch, stream, lambda: sysg.solve(lam, b, x, tol=TOL, mode=mode), 10)
                row[mode] = {"solves_per_s": rate, "iterations": res.iterations, "outer": res.outer_iterations,
                             "rel_residual": res.rel_residual}
                if mode == "fp64":
                    x64 = x.clone()
            row["speedup"] = row["mixed"]["solves_per_s"] / row["fp64"]["solves_per_s"]
            row["max_rel_diff_mixed_vs_fp64"] = float((x - x64).abs().max() / x64.abs().max())
            rows.append(row)
        ctx.close()
    return rows


def batched_fields():
    """256 parametric 2-D solves (lambda = 10^U(-2, 2), E ~ U{500..8000}, P ~ U{3..9}) in
    one batch to 1e-10: mixed vs FP64 solves/s."""
    from ithaca_gpu.batched import BatchedHelmholtz, parametric_quad_problems
    from ithaca_gpu.operators import Context
    ctx = Context(0)
    t0 = time.perf_counter()
    probs = parametric_quad_problems(ctx, nsolve=256)
    setup_s = time.perf_counter() - t0
    bt = BatchedHelmholtz(ctx, "quad", probs)
    tiles = bt.autotune(reps=3)
    out = {"workload": "256 2-D Helmholtz solves, lambda = 10^U(-2,2), E ~ U{500..8000} jittered quads, "
                       "P ~ U{3..9}, Q = P+2, to 1e-10, one batch, each solve one graph launch",
           "host_setup_s": setup_s,
           "tile_variants": {str(n): {"fp32": c["fp32"][0], "fp64": c["fp64"][0]} for n, c in tiles.items()}}
    for mode in ("fp64", "mixed"):
        bt.solve(mode=mode, tol=TOL, want_x=False)  # warm-up (graph capture)
        t0 = time.perf_counter()
        res = bt.solve(mode=mode, tol=TOL, want_x=False)
        ms = (time.perf_counter() - t0) * 1e3
        out[mode] = {"solves_per_s": 256 / (ms / 1e3), "batch_ms": ms,
                     "max_rel_residual": float(res["rel_residual"].max()),
                     "iterations_median": float(np.median(res["iterations"]))}
    out["speedup_mixed_vs_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    bt.close()
    ctx.close()
    return out


# FP64 FMA issue rate of this machine's GB300 (2 flops per FMA), measured by
# ithaca_gpu_measure_pipe_peaks (bench.py --config peaks).
FP64_FMA_PEAK_TF = 1.254


def tri_helm_flops(n):
    """FP64 operations of one triangle Helmholtz apply in the kernel's collocation form:
    BwdTrans (2 NC Q1 + 2 N NQ), collocation derivatives and their transposes
    (4 NQ (Q0 + Q1)), 8 per point (metric products and the mass term), the inner
    product (2 N NQ + 2 NC Q1) and the top-vertex terms (4 Q1)."""
    Q0, Q1, nc = n + 1, n, n * (n + 1) // 2
    nq = Q0 * Q1
    return 4 * nc * Q1 + 4 * n * nq + 4 * nq * (Q0 + Q1) + 8 * nq + 4 * Q1


def tri_fields(torch, cuda, mesh=128, P=6):
    """Curved, jittered triangles (mesh x mesh cells, two triangles each) at order P:
    the four operators (FP64 GDOF/s), the FP64 Helmholtz apply against the FP64 pipe,
    FP32 apply, and Jacobi PCG to 1e-10 (FP64 and mixed); CPU: the compiled port of
    HelmholtzTriImpl on the host cores."""
    from ithaca_gpu.mesh import TriMesh
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU, geom_factors
    n = P + 1
    Q = n + 1
    ctx = Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream, device=cuda)
    m = TriMesh(mesh, mesh, jitter=0.15, seed=7, curve_amp=0.05)
    E = m.E
    X = m.coords(n)
    jac, df = geom_factors(ctx, "tri", Q, X)
    coll = Collection(ctx, "tri", n, Q, E, jac, df)
    coll32 = Collection(ctx, "tri", n, Q, E, jac, df, precision="fp32")
    nc, nq = coll.nm, coll.nq
    rng = np.random.default_rng(11)
    u = torch.from_numpy(rng.uniform(-1, 1, E * nc)).to(cuda)
    u32 = u.float()
    phys = torch.empty(E * nq, dtype=torch.float64, device=cuda)
    coef = torch.empty_like(u)
    coef32 = torch.empty_like(u32)
    d0, d1 = torch.empty_like(phys), torch.empty_like(phys)
    coll.bwdtrans(u, phys)
    reps = 50
    ms = {"bwdtrans": _time_device(torch, stream, lambda: coll.bwdtrans(u, phys), reps),
          "iproduct": _time_device(torch, stream, lambda: coll.iproduct(phys, coef), reps),
          "physderiv": _time_device(torch, stream, lambda: coll.physderiv(phys, [d0, d1]), reps),
          "helmholtz": _time_device(torch, stream, lambda: coll.helmholtz(1.0, u, coef), reps)}
    ms32 = _time_device(torch, stream, lambda: coll32.helmholtz(1.0, u32, coef32), reps)
    fl = tri_helm_flops(n)
    tflops = E * fl / (ms["helmholtz"] / 1e3) / 1e12
    amap = m.assembly(n)
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    f = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1])).reshape(-1) * -(1.0 + 2 * np.pi ** 2)
    loc = coll.iproduct(f)
    b_h = -amap.assemble(loc)
    b_h[:amap.ndir] = 0.0
    b = torch.from_numpy(b_h).to(cuda)
    x = torch.zeros_like(b)
    out = {"workload": f"{mesh}x{mesh} cells as {E} curved jittered triangles, P={P} (n={n}: {nc} modes, "
                       f"{Q}x{n} points), lambda=1, per-point geometry",
           "elements": E, "local_dofs": E * nc, "solve_dofs": amap.nglobal - amap.ndir,
           "fp64_gdofs": {k: E * nc / (v / 1e3) / 1e9 for k, v in ms.items()},
           "fp32_helmholtz_gdofs": E * nc / (ms32 / 1e3) / 1e9,
           "helmholtz_fp64": {"ms": ms["helmholtz"], "flop_per_element": fl, "tflops": tflops,
                              "bound": "fp64 pipe (2.8 flop per byte of per-point geometry and coefficients)",
                              "peak_tflops": FP64_FMA_PEAK_TF, "frac": tflops / FP64_FMA_PEAK_TF,
                              "peak_source": "measured FP64 FMA issue rate (bench.py --config peaks)"}}
    for mode in ("fp64", "mixed"):
        sysg.solve(1.0, b, x, tol=TOL, mode=mode)
        rate, (_, res) = _solve_rate(torch, stream, lambda: sysg.solve(1.0, b, x, tol=TOL, mode=mode), 3)
        out[mode] = {"solves_per_s": rate, "iterations": res.iterations, "outer": res.outer_iterations,
                     "rel_residual": res.rel_residual}
        if mode == "fp64":
            x64 = x.clone()
    out["speedup_mixed_vs_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    out["max_rel_diff_mixed_vs_fp64"] = float((x - x64).abs().max() / x64.abs().max())
    uh = coll.bwdtrans(sysg.global_to_local(x64.cpu().numpy()))
    out["max_error_vs_exact_sin_sin"] = float(np.max(np.abs(uh - (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1])).reshape(-1))))
    try:
        from oracle import cportbind
        from oracle import tri as otri
        if cportbind.available():
            nth = os.cpu_count() or 1
            tb = otri.TriBasis(n)
            Es = min(E, 8192)
            jh = np.asarray(jac).reshape(E, -1)[:Es].reshape(-1)
            dh = np.asarray(df).reshape(4, E, -1)[:, :Es].reshape(4, -1)
            uh_ = u.cpu().numpy()[:Es * nc]
            ms_c, _ = _time_host(lambda: cportbind.tri_helmholtz(tb, Es, jh, dh, True, 1.0, uh_, nthreads=nth), 5)
            out["cpu_baseline"] = {"value": Es * nc / (ms_c / 1e3) / 1e9, "unit": "GDOF/s (FP64 Helmholtz apply)",
                                   "cores": nth, "kind": "port",
                                   "sample": f"5 applies to the first {Es} triangles (HelmholtzTriImpl restated)"}
    except Exception as ex:
        out["cpu_baseline"] = {"value": None, "error": str(ex)[:200]}
    sysg.close()
    coll.close()
    coll32.close()
    ctx.close()
    torch.cuda.empty_cache()
    return out


def tet_helm_flops(n):
    """FP64 operations of one tetrahedron Helmholtz apply in the kernel's collocation form:
    BwdTrans and IProduct (4 NC Q + 4 NPQ Q^2 + 4 N NQ), the collapsed derivatives and
    their transposes (4 NQ (Q0 + 2 Q)) and 17 per point (metric products, mass term)."""
    Q0, Q, nc, npq = n + 1, n, n * (n + 1) * (n + 2) // 6, n * (n + 1) // 2
    nq = Q0 * Q * Q
    return 4 * nc * Q + 4 * npq * Q * Q + 4 * n * nq + 4 * nq * (Q0 + 2 * Q) + 17 * nq


def tet_fields(torch, cuda, mesh=12, P=6):
    """Curved, jittered tetrahedra (mesh^3 cubes, six Kuhn tetrahedra each) at order P: the
    four operators (FP64 GDOF/s), the FP64 Helmholtz apply against the FP64 pipe, FP32
    apply, and Jacobi PCG to 1e-10 (FP64 and mixed)."""
    from ithaca_gpu.mesh import TetMesh
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU, geom_factors
    n = P + 1
    Q = n + 1
    ctx = Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream, device=cuda)
    m = TetMesh(mesh, mesh, mesh, jitter=0.15, seed=7, curve_amp=0.03)
    E = m.E
    X = m.coords(n)
    jac, df = geom_factors(ctx, "tet", Q, X)
    coll = Collection(ctx, "tet", n, Q, E, jac, df)
    coll32 = Collection(ctx, "tet", n, Q, E, jac, df, precision="fp32")
    nc, nq = coll.nm, coll.nq
    rng = np.random.default_rng(12)
    u = torch.from_numpy(rng.uniform(-1, 1, E * nc)).to(cuda)
    u32 = u.float()
    phys = torch.empty(E * nq, dtype=torch.float64, device=cuda)
    coef, coef32 = torch.empty_like(u), torch.empty_like(u32)
    d = [torch.empty_like(phys) for _ in range(3)]
    coll.bwdtrans(u, phys)
    reps = 20
    ms = {"bwdtrans": _time_device(torch, stream, lambda: coll.bwdtrans(u, phys), reps),
          "iproduct": _time_device(torch, stream, lambda: coll.iproduct(phys, coef), reps),
          "physderiv": _time_device(torch, stream, lambda: coll.physderiv(phys, d), reps),
          "helmholtz": _time_device(torch, stream, lambda: coll.helmholtz(1.0, u, coef), reps)}
    ms32 = _time_device(torch, stream, lambda: coll32.helmholtz(1.0, u32, coef32), reps)
    fl = tet_helm_flops(n)
    tflops = E * fl / (ms["helmholtz"] / 1e3) / 1e12
    t0 = time.perf_counter()
    amap = m.assembly(n)
    asm_s = time.perf_counter() - t0
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    ex = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1]) * np.sin(np.pi * X[2])).reshape(-1)
    f = -(1.0 + 3 * np.pi ** 2) * ex
    b_h = -amap.assemble(coll.iproduct(f))
    b_h[:amap.ndir] = 0.0
    b = torch.from_numpy(b_h).to(cuda)
    x = torch.zeros_like(b)
    out = {"workload": f"{mesh}^3 cubes as {E} curved jittered tetrahedra, P={P} (n={n}: {nc} modes, "
                       f"{Q}x{n}x{n} points), lambda=1, per-point geometry",
           "elements": E, "local_dofs": E * nc, "solve_dofs": amap.nglobal - amap.ndir, "assembly_map_s": asm_s,
           "fp64_gdofs": {k: E * nc / (v / 1e3) / 1e9 for k, v in ms.items()},
           "fp32_helmholtz_gdofs": E * nc / (ms32 / 1e3) / 1e9,
           "helmholtz_fp64": {"ms": ms["helmholtz"], "flop_per_element": fl, "tflops": tflops,
                              "bound": "fp64 pipe", "peak_tflops": FP64_FMA_PEAK_TF,
                              "frac": tflops / FP64_FMA_PEAK_TF,
                              "peak_source": "measured FP64 FMA issue rate (bench.py --config peaks)"}}
    for mode in ("fp64", "mixed"):
        sysg.solve(1.0, b, x, tol=TOL, mode=mode)
        rate, (_, res) = _solve_rate(torch, stream, lambda: sysg.solve(1.0, b, x, tol=TOL, mode=mode), 2)
        out[mode] = {"solves_per_s": rate, "iterations": res.iterations, "outer": res.outer_iterations,
                     "rel_residual": res.rel_residual}
        if mode == "fp64":
            x64 = x.clone()
    out["speedup_mixed_vs_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    out["max_rel_diff_mixed_vs_fp64"] = float((x - x64).abs().max() / x64.abs().max())
    uh = coll.bwdtrans(sysg.global_to_local(x64.cpu().numpy()))
    out["max_error_vs_exact_sin_sin_sin"] = float(np.max(np.abs(uh - ex)))
    sysg.close()
    coll.close()
    coll32.close()
    ctx.close()
    torch.cuda.empty_cache()
    return out


def prism_helm_flops(n):
    """FP64 operations of one prism Helmholtz apply (collocation form): BwdTrans and
    IProduct (4 NC Q2 + 4 N^2 Q0 Q2 + 4 N NQ), the collapsed derivatives and their
    transposes (4 NQ (2 Q0 + Q2)) and 17 per point."""
    Q0, Q2, nc = n + 1, n, n * n * (n + 1) // 2
    nq = Q0 * Q0 * Q2
    return 4 * nc * Q2 + 4 * n * n * Q0 * Q2 + 4 * n * nq + 4 * nq * (2 * Q0 + Q2) + 17 * nq


def prism_fields(torch, cuda, mesh=12, P=6):
    """Curved, jittered prisms (mesh^3 cubes, two prisms each) at order P: operators,
    FP64 apply against the FP64 pipe, FP32 apply, PCG to 1e-10 (FP64 and mixed)."""
    from ithaca_gpu.mesh import PrismMesh
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU, geom_factors
    n = P + 1
    Q = n + 1
    ctx = Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream, device=cuda)
    m = PrismMesh(mesh, mesh, mesh, jitter=0.15, seed=7, curve_amp=0.03)
    E = m.E
    X = m.coords(n)
    jac, df = geom_factors(ctx, "prism", Q, X)
    coll = Collection(ctx, "prism", n, Q, E, jac, df)
    coll32 = Collection(ctx, "prism", n, Q, E, jac, df, precision="fp32")
    nc, nq = coll.nm, coll.nq
    rng = np.random.default_rng(13)
    u = torch.from_numpy(rng.uniform(-1, 1, E * nc)).to(cuda)
    u32 = u.float()
    phys = torch.empty(E * nq, dtype=torch.float64, device=cuda)
    coef, coef32 = torch.empty_like(u), torch.empty_like(u32)
    d = [torch.empty_like(phys) for _ in range(3)]
    coll.bwdtrans(u, phys)
    reps = 20
    ms = {"bwdtrans": _time_device(torch, stream, lambda: coll.bwdtrans(u, phys), reps),
          "iproduct": _time_device(torch, stream, lambda: coll.iproduct(phys, coef), reps),
          "physderiv": _time_device(torch, stream, lambda: coll.physderiv(phys, d), reps),
          "helmholtz": _time_device(torch, stream, lambda: coll.helmholtz(1.0, u, coef), reps)}
    ms32 = _time_device(torch, stream, lambda: coll32.helmholtz(1.0, u32, coef32), reps)
    fl = prism_helm_flops(n)
    tflops = E * fl / (ms["helmholtz"] / 1e3) / 1e12
    t0 = time.perf_counter()
    amap = m.assembly(n)
    asm_s = time.perf_counter() - t0
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    ex = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1]) * np.sin(np.pi * X[2])).reshape(-1)
    f = -(1.0 + 3 * np.pi ** 2) * ex
    b_h = -amap.assemble(coll.iproduct(f))
    b_h[:amap.ndir] = 0.0
    b = torch.from_numpy(b_h).to(cuda)
    x = torch.zeros_like(b)
    out = {"workload": f"{mesh}^3 cubes as {E} curved jittered prisms, P={P} (n={n}: {nc} modes, "
                       f"{Q}x{Q}x{n} points), lambda=1, per-point geometry",
           "elements": E, "local_dofs": E * nc, "solve_dofs": amap.nglobal - amap.ndir, "assembly_map_s": asm_s,
           "fp64_gdofs": {k: E * nc / (v / 1e3) / 1e9 for k, v in ms.items()},
           "fp32_helmholtz_gdofs": E * nc / (ms32 / 1e3) / 1e9,
           "helmholtz_fp64": {"ms": ms["helmholtz"], "flop_per_element": fl, "tflops": tflops,
                              "bound": "fp64 pipe", "peak_tflops": FP64_FMA_PEAK_TF,
                              "frac": tflops / FP64_FMA_PEAK_TF,
                              "peak_source": "measured FP64 FMA issue rate (bench.py --config peaks)"}}
    for mode in ("fp64", "mixed"):
        sysg.solve(1.0, b, x, tol=TOL, mode=mode)
        rate, (_, res) = _solve_rate(torch, stream, lambda: sysg.solve(1.0, b, x, tol=TOL, mode=mode), 2)
        out[mode] = {"solves_per_s": rate, "iterations": res.iterations, "outer": res.outer_iterations,
                     "rel_residual": res.rel_residual}
        if mode == "fp64":
            x64 = x.clone()
    out["speedup_mixed_vs_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    out["max_rel_diff_mixed_vs_fp64"] = float((x - x64).abs().max() / x64.abs().max())
    uh = coll.bwdtrans(sysg.global_to_local(x64.cpu().numpy()))
    out["max_error_vs_exact_sin_sin_sin"] = float(np.max(np.abs(uh - ex)))
    sysg.close()
    coll.close()
    coll32.close()
    ctx.close()
    torch.cuda.empty_cache()
    return out


def pyr_helm_flops(n):
    """FP64 operations of one pyramid Helmholtz apply (collocation form): BwdTrans and
    IProduct (4 NC Q2 + 4 N^2 Q0 Q2 + 4 N NQ), the collapsed derivatives and their
    transposes (4 NQ (2 Q0 + Q2)) and 17 per point."""
    Q0, Q2, nc = n + 1, n, n * (n + 1) * (2 * n + 1) // 6
    nq = Q0 * Q0 * Q2
    return 4 * nc * Q2 + 4 * n * n * Q0 * Q2 + 4 * n * nq + 4 * nq * (2 * Q0 + Q2) + 17 * nq


def pyr_fields(torch, cuda, mesh=10, P=6):
    """Curved, jittered pyramids (mesh^3 cubes, six pyramids each) at order P: operators,
    FP64 apply against the FP64 pipe, FP32 apply, PCG to 1e-10 (FP64 and mixed)."""
    from ithaca_gpu.mesh import PyrMesh
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU, geom_factors
    n = P + 1
    Q = n + 1
    ctx = Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream, device=cuda)
    m = PyrMesh(mesh, mesh, mesh, jitter=0.15, seed=7, curve_amp=0.03)
    E = m.E
    X = m.coords(n)
    jac, df = geom_factors(ctx, "pyr", Q, X)
    coll = Collection(ctx, "pyr", n, Q, E, jac, df)
    coll32 = Collection(ctx, "pyr", n, Q, E, jac, df, precision="fp32")
    nc, nq = coll.nm, coll.nq
    rng = np.random.default_rng(14)
    u = torch.from_numpy(rng.uniform(-1, 1, E * nc)).to(cuda)
    u32 = u.float()
    phys = torch.empty(E * nq, dtype=torch.float64, device=cuda)
    coef, coef32 = torch.empty_like(u), torch.empty_like(u32)
    d = [torch.empty_like(phys) for _ in range(3)]
    coll.bwdtrans(u, phys)
    reps = 20
    ms = {"bwdtrans": _time_device(torch, stream, lambda: coll.bwdtrans(u, phys), reps),
          "iproduct": _time_device(torch, stream, lambda: coll.iproduct(phys, coef), reps),
          "physderiv": _time_device(torch, stream, lambda: coll.physderiv(phys, d), reps),
          "helmholtz": _time_device(torch, stream, lambda: coll.helmholtz(1.0, u, coef), reps)}
    ms32 = _time_device(torch, stream, lambda: coll32.helmholtz(1.0, u32, coef32), reps)
    fl = pyr_helm_flops(n)
    tflops = E * fl / (ms["helmholtz"] / 1e3) / 1e12
    t0 = time.perf_counter()
    amap = m.assembly(n)
    asm_s = time.perf_counter() - t0
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    ex = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1]) * np.sin(np.pi * X[2])).reshape(-1)
    f = -(1.0 + 3 * np.pi ** 2) * ex
    b_h = -amap.assemble(coll.iproduct(f))
    b_h[:amap.ndir] = 0.0
    b = torch.from_numpy(b_h).to(cuda)
    x = torch.zeros_like(b)
    out = {"workload": f"{mesh}^3 cubes as {E} curved jittered pyramids, P={P} (n={n}: {nc} modes, "
                       f"{Q}x{Q}x{n} points), lambda=1, per-point geometry",
           "elements": E, "local_dofs": E * nc, "solve_dofs": amap.nglobal - amap.ndir, "assembly_map_s": asm_s,
           "fp64_gdofs": {k: E * nc / (v / 1e3) / 1e9 for k, v in ms.items()},
           "fp32_helmholtz_gdofs": E * nc / (ms32 / 1e3) / 1e9,
           "helmholtz_fp64": {"ms": ms["helmholtz"], "flop_per_element": fl, "tflops": tflops,
                              "bound": "fp64 pipe", "peak_tflops": FP64_FMA_PEAK_TF,
                              "frac": tflops / FP64_FMA_PEAK_TF,
                              "peak_source": "measured FP64 FMA issue rate (bench.py --config peaks)"}}
    for mode in ("fp64", "mixed"):
        sysg.solve(1.0, b, x, tol=TOL, mode=mode)
        rate, (_, res) = _solve_rate(torch, stream, lambda: sysg.solve(1.0, b, x, tol=TOL, mode=mode), 2)
        out[mode] = {"solves_per_s": rate, "iterations": res.iterations, "outer": res.outer_iterations,
                     "rel_residual": res.rel_residual}
        if mode == "fp64":
            x64 = x.clone()
    out["speedup_mixed_vs_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    out["max_rel_diff_mixed_vs_fp64"] = float((x - x64).abs().max() / x64.abs().max())
    uh = coll.bwdtrans(sysg.global_to_local(x64.cpu().numpy()))
    out["max_error_vs_exact_sin_sin_sin"] = float(np.max(np.abs(uh - ex)))
    sysg.close()
    coll.close()
    coll32.close()
    ctx.close()
    torch.cuda.empty_cache()
    return out


def quad_sweep_batched_fields():
    """The 32 x 32 jittered-quad mesh's lambda sweep (P = 6 and 8, lambda in {0.1, 1, 10}:
    six systems) solved as one batch to 1e-10: mixed vs FP64 solves/s, each batch solve one
    graph launch."""
    from ithaca_gpu.batched import BatchedHelmholtz
    from ithaca_gpu.operators import Context
    from ithaca_gpu.workload import quad_workload
    ctx = Context(0)
    probs = []
    for P in (6, 8):
        w = quad_workload(32, P, ctx=ctx)
        for lam in (0.1, 1.0, 10.0):
            probs.append(dict(nmodes=w["n"], npoints=w["Q"], jac=w["jac"], df=w["df"], amap=w["amap"], lam=lam,
                              rhs=w["b"]))
    bt = BatchedHelmholtz(ctx, "quad", probs)
    bt.autotune(reps=5)
    out = {"workload": "32x32 jittered quads, P in {6, 8} x lambda in {0.1, 1, 10}: 6 systems in one batch, to 1e-10"}
    xs = {}
    for mode in ("fp64", "mixed"):
        bt.solve(mode=mode, tol=TOL, want_x=False)
        reps = 10
        t0 = time.perf_counter()
        for _ in range(reps):
            res = bt.solve(mode=mode, tol=TOL, want_x=False)
        ms = (time.perf_counter() - t0) * 1e3 / reps
        xs[mode] = bt.solve(mode=mode, tol=TOL)["x"]
        out[mode] = {"solves_per_s": len(probs) / (ms / 1e3), "batch_ms": ms,
                     "max_rel_residual": float(res["rel_residual"].max()),
                     "iterations": [int(i) for i in res["iterations"]]}
    out["speedup_mixed_vs_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    out["max_rel_diff_mixed_vs_fp64"] = max(float(np.max(np.abs(a - b_)) / np.max(np.abs(b_)))
                                            for a, b_ in zip(xs["mixed"], xs["fp64"]))
    bt.close()
    ctx.close()
    return out


def run_gpu(args, rank, world):
    import torch
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU, geom_factors

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    cuda = f"cuda:{dev}"
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl")
    mesh, n, Q, X, amap, f = build_workload(args.mesh, args.order)
    E, N, ndir = mesh.E, amap.nglobal, amap.ndir
    ctx = Context(dev)
    jac, df = geom_factors(ctx, "hex", Q, torch.from_numpy(X).to(cuda))
    coll = Collection(ctx, "hex", n, Q, E, jac, df, deformed=True, precision="fp64")
    coll32 = Collection(ctx, "hex", n, Q, E, jac, df, deformed=True, precision="fp32")
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    sysg.set_fused_update(args.fused_update)
    stream = torch.cuda.ExternalStream(ctx.stream, device=cuda)
    # pick the FP32 element-kernel variant by timing the solver's own gathered inner
    # apply (CollectionOptimisation analogue), unless --variant names one (kernel captures,
    # whose serialised timings would mislead the autotuner)
    if args.variant >= 0:
        variant, variant_ms = args.variant, {}
        sysg.coll.set_variant(variant)
    else:
        variant, variant_ms = sysg.autotune_inner(
            LAMBDA, reps=10, mode=args.mixed_mode,
            **({"variants": GEO16_VARIANTS} if args.mixed_mode == "mixed_geo16" else {}))
    coll32.set_variant(variant)
    # the FP64 apply's kernel (FP64 solves, outer residuals of the mixed solve), by timing
    variant64, variant64_ms = sysg.autotune_fp64(LAMBDA, reps=5)

    # b = Assemble(-IProductWRTBase(f)) on the device (ContField::v_HelmSolve)
    fd = torch.from_numpy(f).to(cuda)
    loc = torch.empty(E * n ** 3, dtype=torch.float64, device=cuda)
    coll.iproduct(fd, loc)
    loc.neg_()
    b = torch.empty(N, dtype=torch.float64, device=cuda)
    sysg.assemble(loc, b)
    x = torch.zeros(N, dtype=torch.float64, device=cuda)
    ctx.synchronize()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- headline: mixed-precision solves, inputs resident in HBM ----
    mode = args.mixed_mode
    for _ in range(args.warmup):
        _, res = sysg.solve(LAMBDA, b, x, tol=TOL, mode=mode)
    barrier()
    l0 = ctx.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        ev0.record(stream)
        results = []
        for _ in range(args.steps):
            _, res = sysg.solve(LAMBDA, b, x, tol=TOL, mode=mode)
            results.append((res.iterations, res.outer_iterations, res.rel_residual))
        ev1.record(stream)
        ev1.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = ctx.launch_count() - l0
    ms = max_over_ranks(ms, world, cuda)
    value = replica_throughput(args.steps, ms, world)
    x_mixed = x.clone()

    # the other inner-solve variant, for comparison (not the headline)
    other = "mixed" if mode == "mixed_geo16" else "mixed_geo16"
    sysg.solve(LAMBDA, b, x, tol=TOL, mode=other)
    other_solves, (_, res_o) = _solve_rate(torch, stream, lambda: sysg.solve(LAMBDA, b, x, tol=TOL, mode=other), 2)

    # ---- dominant kernel: the FP32 gather + element Helmholtz of the inner solve ----
    k_ms, k_bytes = sysg.profile_apply(LAMBDA, mode=mode, reps=20)
    peak, peak_kind = load_peaks()
    # the other mode's inner apply (same variant), for its own roofline beside the headline's
    ko_ms, ko_bytes = sysg.profile_apply(LAMBDA, mode=other, reps=20)

    # ---- FP64 reference recurrence on the GPU ----
    sysg.solve(LAMBDA, b, x, tol=TOL, mode="fp64")
    fp64_solves, (_, res64) = _solve_rate(torch, stream, lambda: sysg.solve(LAMBDA, b, x, tol=TOL, mode="fp64"),
                                          max(1, min(2, args.steps)))
    x64_gpu = x.clone()
    sol_diff = float((x - x_mixed).abs().max() / x.abs().max())
    k64_ms, k64_bytes = sysg.profile_apply(LAMBDA, mode="fp64", reps=5)

    # ---- operator apply throughput (Ndof = E n^3 per apply) ----
    def op_rate(c, dtype, reps):
        u = torch.rand(E * n ** 3, dtype=dtype, device=cuda) * 2 - 1
        o = torch.empty_like(u)
        c.helmholtz(LAMBDA, u, o)
        torch.cuda.synchronize()
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            c.helmholtz(LAMBDA, u, o)
        z.record(stream)
        z.synchronize()
        return E * n ** 3 * reps / (a.elapsed_time(z) / 1e3) / 1e9

    gdofs64 = op_rate(coll, torch.float64, 5)
    gdofs32 = op_rate(coll32, torch.float32, 20)

    # ---- end to end through the public HelmSolve call with host buffers ----
    # host buffers in pinned memory (numpy views of pinned torch tensors): the forcing is
    # copied in and the coefficients copied out by the library inside every timed step
    f_host = torch.from_numpy(np.ascontiguousarray(f)).pin_memory().numpy()
    out_host = torch.zeros(E * n ** 3, dtype=torch.float64).pin_memory().numpy()
    sysg.helmsolve(LAMBDA, f_host, out_host, tol=TOL, mode=mode)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, rese = sysg.helmsolve(LAMBDA, f_host, out_host, tol=TOL, mode=mode)
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e = world * args.steps / e2e_s

    if rank != 0:
        return
    # host copies for the CPU reference solve below, then free the headline workload
    jac_h, df_h, b_h = jac.cpu().numpy(), df.cpu().numpy(), b.cpu().numpy()
    dinv_h = 1.0 / sysg.diagonal(LAMBDA)
    x64_h = x64_gpu.cpu().numpy()
    cfg = workload_config(args, n, Q, E, N, ndir)
    cfg["fp32_kernel_variant"] = variant
    cfg["fused_update"] = bool(args.fused_update)
    cfg["autotune_ms"] = {str(k): round(v, 4) for k, v in variant_ms.items()}
    cfg["fp64_kernel_variant"] = variant64
    cfg["autotune_fp64_ms"] = {str(k): round(v, 4) for k, v in variant64_ms.items()}
    launches_total = int(launches)
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (outer) / f32 (inner)" + (", 16-bit geometry storage" if mode == "mixed_geo16" else ""),
        "data": "synthetic (seeded mesh and forcing)",
        "config": cfg,
        "iterations": {"inner": results[-1][0], "outer": results[-1][1], "rel_residual": results[-1][2]},
        "mixed_mode": mode,
        "other_mixed_mode": {"mode": other, "solves_per_s": other_solves, "iterations": res_o.iterations,
                             "outer": res_o.outer_iterations, "rel_residual": res_o.rel_residual},
        "fp64": {"solves_per_s": fp64_solves, "iterations": res64.iterations, "rel_residual": res64.rel_residual,
                 "speedup_mixed_vs_fp64": value / world / fp64_solves, "max_rel_diff_vs_mixed": sol_diff,
                 "apply_ms": k64_ms, "apply_fp64_tflops": None},
        "helmholtz_gdofs": {"fp64": gdofs64, "fp32": gdofs32},
        "solver_gdofs": {"mixed": value / world * (N - ndir) / 1e9, "fp64": fp64_solves * (N - ndir) / 1e9},
        "roofline": dict(inner_roofline(mode, variant, n, Q, E, k_ms, k_bytes, peak, peak_kind),
                         **({"fp32_geometry_bytes_per_launch": ko_bytes,
                             "fp32_geometry_equivalent_frac": ko_bytes / (k_ms / 1e3) / 1e9 / peak}
                            if mode == "mixed_geo16" else {})),
        "roofline_other_mixed_mode": inner_roofline(other, variant, n, Q, E, ko_ms, ko_bytes, peak, peak_kind),
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": int(f_host.nbytes),
                "d2h_bytes_per_step": int(out_host.nbytes), "rel_residual": rese.rel_residual},
        "gpu_launches": launches_total,
        "clocks": clk.summary(),
    }
    # FP64 flop rate of the FP64 apply (collocation-form operation count per element; the
    # even-odd kernel, fp64_kernel_variant 1 or 2, issues fewer operations for the same
    # result, so for it this is the equivalent rate of the plain contraction)
    fl = 2 * (2 * (Q * n ** 3 + Q * Q * n * n + Q ** 3 * n) + 6 * Q ** 4 + 11 * Q ** 3)
    line["fp64"]["apply_fp64_tflops"] = E * fl / (k64_ms / 1e3) / 1e12
    line["fp64"]["apply_flop_rule"] = ("collocation-form count" if variant64 == 0 else
                                       "collocation-form count (equivalent rate: the even-odd kernel does fewer operations)")
    del coll, coll32, sysg, jac, df, b, x, x_mixed, x64_gpu, loc, fd
    ctx.close()
    torch.cuda.empty_cache()
    # the other configurations of the metric, measured in the same run
    if args.full:
        for key, fn in (("hex_p8", lambda: hex_order8_fields(torch, cuda)),
                        ("quad_32x32_mixed_sweep", lambda: quad_mixed_fields(torch, cuda)),
                        ("quad_32x32_sweep_batched", quad_sweep_batched_fields),
                        ("batched_256", batched_fields),
                        ("tri_128x128_p6", lambda: tri_fields(torch, cuda)),
                        ("tet_12x12x12_p6", lambda: tet_fields(torch, cuda)),
                        ("prism_12x12x12_p6", lambda: prism_fields(torch, cuda)),
                        ("pyr_10x10x10_p6", lambda: pyr_fields(torch, cuda))):
            try:
                line[key] = fn()
            except Exception as ex:  # one failing secondary field does not void the headline
                line[key] = {"error": str(ex)[:300]}
    # CPU baseline: one full solve of the same workload by the compiled port of the
    # reference path on the host cores, and the GPU FP64 solution's difference from it
    try:
        nth = os.cpu_count() or 1
        xc, it_c, dt_c = cpu_full_solve(n, Q, E, jac_h, df_h, amap, b_h, dinv_h, nth)
        line["cpu_baseline"] = {"value": 1.0 / dt_c, "unit": "solves/s", "cores": nth, "kind": "port",
                                "sample": f"one full FP64 Jacobi PCG solve of the workload to {TOL:g} "
                                          f"({it_c} iterations, {dt_c:.1f} s, setup included)",
                                "iterations": it_c}
        line["fp64"]["max_rel_diff_vs_cpu_reference"] = float(
            np.max(np.abs(x64_h[ndir:] - xc[ndir:])) / np.max(np.abs(xc[ndir:])))
        line["fp64"]["cpu_reference_iterations"] = it_c
    except Exception as ex:  # the GPU numbers stand even if the CPU solve fails
        line["cpu_baseline"] = {"value": None, "error": str(ex)[:200]}
    print(json.dumps(line))


def run_reference(args, rank, world):
    """CPU arm: the compiled port of the reference kernels + CG (oracle/cport), all host
    threads, on the same workload. One full solve (untimed for the steps) gives the
    recurrence's own iteration count; each timed step is a bounded sample of CG
    iterations, and solves/s = 1 / (time per iteration x that iteration count)."""
    if rank != 0:
        return
    from oracle import basis as obasis
    from oracle import cportbind
    from oracle import geom as ogeom
    from oracle import ops as oops
    from oracle import solve as osolve
    if not cportbind.available():
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "cport")], check=True)
    mesh, n, Q, X, amap, f = build_workload(args.mesh, args.order)
    E, N, ndir = mesh.E, amap.nglobal, amap.ndir
    b1 = obasis.Basis1D(n, Q)
    jac, df = ogeom.geom_factors(X, b1.D2, 3)
    jac = jac.reshape(-1)
    nth = os.cpu_count() or 1
    m = osolve.Map.of(amap)
    ip = oops.iproduct(b1, 3, jac.reshape(E, -1), f)
    rhs = -m.assemble(ip)
    dinv = osolve.jacobi_inverse(b1, 3, jac.reshape(E, -1), df, LAMBDA, m)
    _, iters_full, full_s = cpu_full_solve(n, Q, E, jac, df, amap, rhs, dinv, nth)
    if iters_full <= 0:
        raise RuntimeError(f"the CPU reference solve did not converge ({iters_full})")
    per_step = 8

    def run(k):
        t0 = time.perf_counter()
        cportbind.cg_solve(3, n, Q, E, jac, df, True, LAMBDA, amap.l2g, amap.sign, N, ndir, dinv, rhs, TOL, k, nth)
        return time.perf_counter() - t0

    def step():
        # (2k iterations) - (k iterations): the setup (CSR build, first residual) cancels
        return run(2 * per_step) - run(per_step)

    for _ in range(args.warmup):
        step()
    times = [step() for _ in range(args.steps)]
    t_iter = max(statistics.median(times), 1e-9) / per_step
    value = 1.0 / (t_iter * iters_full)
    cfg = workload_config(args, n, Q, E, N, ndir)
    cfg["parallelism"] = f"{nth} host threads"
    cfg["inner"] = "fp64 Jacobi PCG, the reference recurrence (compiled C++ port of the reference kernels)"
    print(json.dumps({
        "metric": METRIC, "impl": "reference", "value": value, "unit": "solves/s", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(times) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": cfg,
        "iterations": iters_full,
        "full_solve": {"seconds": full_s, "solves_per_s": 1.0 / full_s, "iterations": iters_full},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": nth, "kind": "port",
                         "sample": f"{per_step} CG iterations per step on the full workload, setup excluded, scaled "
                                   f"by the {iters_full} iterations of this port's own full solve to {TOL:g}"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ---------------------------------------------------------------------------------
# Secondary workloads (--config): one JSON line each, same timing rules (warm-up, CUDA
# events on the library stream, host-side timing where the call includes host copies).
# ---------------------------------------------------------------------------------
def _events(torch, stream):
    a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    return a, z


def _time_device(torch, stream, fn, reps, warmup=3):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, z = _events(torch, stream)
    a.record(stream)
    for _ in range(reps):
        fn()
    z.record(stream)
    z.synchronize()
    return a.elapsed_time(z) / reps  # ms


def _time_host(fn, reps, warmup=1):
    for _ in range(warmup):
        fn()
    t0 = time.perf_counter()
    for _ in range(reps):
        out = fn()
    return (time.perf_counter() - t0) / reps * 1e3, out  # ms


def _line(metric, value, unit, args, cfg, higher=True, **extra):
    d = {"metric": metric, "value": value, "unit": unit, "impl": "gpu", "n_gpus": 1, "steps": args.steps,
         "warmup": args.warmup, "higher_is_better": higher, "scaling": "weak", "vs_baseline": None,
         "data": "synthetic (seeded)", "config": cfg}
    d.update(extra)
    print(json.dumps(d))


def suite_quad2d(args):
    """32 x 32 jittered quads, P = 6: the four operators (GDOF/s, FP64) and Jacobi PCG
    to 1e-12 (FP64 and mixed)."""
    import torch
    from ithaca_gpu.workload import quad_workload
    w = quad_workload(32, 6)
    ctx, coll, sysg, amap = w["ctx"], w["coll"], w["system"], w["amap"]
    E, n, Q, N, ndir = w["mesh"].E, w["n"], w["Q"], amap.nglobal, amap.ndir
    stream = torch.cuda.ExternalStream(ctx.stream, device="cuda:0")
    u = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, E * n * n)).cuda()
    phys = torch.empty(E * Q * Q, dtype=torch.float64, device="cuda")
    coef = torch.empty_like(u)
    d0, d1 = torch.empty_like(phys), torch.empty_like(phys)
    coll.bwdtrans(u, phys)
    reps = 200
    ops = {"bwdtrans": lambda: coll.bwdtrans(u, phys), "iproduct": lambda: coll.iproduct(phys, coef),
           "physderiv": lambda: coll.physderiv(phys, [d0, d1]),
           "helmholtz": lambda: coll.helmholtz(1.0, u, coef)}
    gdofs = {k: E * n * n / (_time_device(torch, stream, f, reps) / 1e3) / 1e9 for k, f in ops.items()}
    b = torch.from_numpy(w["b"]).cuda()
    x = torch.zeros_like(b)
    out = {}
    for mode in ("fp64", "mixed"):
        _, res = sysg.solve(1.0, b, x, tol=1e-12, mode=mode)
        ms = _time_device(torch, stream, lambda: sysg.solve(1.0, b, x, tol=1e-12, mode=mode), args.steps, 1)
        _, res = sysg.solve(1.0, b, x, tol=1e-12, mode=mode)
        out[mode] = {"solves_per_s": 1e3 / ms, "ms": ms, "iterations": res.iterations,
                     "rel_residual": res.rel_residual}
    cfg = {"workload": "2-D Helmholtz, 32x32 jittered quads (0.1 h), P=6 (n=7, Q=8), lambda=1, Jacobi PCG to 1e-12",
           "elements": E, "global_dofs": N, "solve_dofs": N - ndir,
           "l2": "working set (~3 MB) is L2-resident: latency-bound, not an HBM roofline case"}
    cpu = None
    try:
        from oracle import cportbind
        if cportbind.available():
            diag = sysg.diagonal(1.0)
            nth = os.cpu_count() or 1
            run = lambda: cportbind.cg_solve(2, n, Q, E, w["jac"], w["df"], True, 1.0, amap.l2g, amap.sign, N, ndir,
                                             1.0 / diag, w["b"], 1e-12, 5000, nth)
            ms_c, res_c = _time_host(run, 3)
            cpu = {"value": 1e3 / ms_c, "unit": "solves/s", "cores": nth, "kind": "port",
                   "sample": f"3 full FP64 solves ({res_c[1]} iterations)"}
    except Exception as ex:
        cpu = {"value": None, "error": str(ex)[:200]}
    _line("2-D Helmholtz, 32x32 jittered quads P=6: CG solves/s (FP64, 1e-12) and operator GDOF/s", out["fp64"]["solves_per_s"],
          "solves/s", args, cfg, dtype="f64", helmholtz_gdofs_fp64=gdofs, solve=out, cpu_baseline=cpu)


def suite_mixed2d(args):
    """Config-1 mesh at P = 6 and 8, lambda in {0.1, 1, 10}: FP64 vs mixed (FP32 inner)
    solves to 1e-10."""
    import torch
    from ithaca_gpu.workload import quad_workload
    rows = []
    for P in (6, 8):
        w = quad_workload(32, P)
        sysg, ctx = w["system"], w["ctx"]
        stream = torch.cuda.ExternalStream(ctx.stream, device="cuda:0")
        b = torch.from_numpy(w["b"]).cuda()
        x = torch.zeros_like(b)
        for lam in (0.1, 1.0, 10.0):
            row = {"P": P, "lambda": lam}
            for mode in ("fp64", "mixed"):
                ms = _time_device(torch, stream, lambda: sysg.solve(lam, b, x, tol=1e-10, mode=mode), args.steps, 1)
                _, res = sysg.solve(lam, b, x, tol=1e-10, mode=mode)
                row[mode] = {"solves_per_s": 1e3 / ms, "iterations": res.iterations,
                             "outer": res.outer_iterations, "rel_residual": res.rel_residual}
            row["speedup"] = row["mixed"]["solves_per_s"] / row["fp64"]["solves_per_s"]
            rows.append(row)
    head = [r for r in rows if r["P"] == 6 and r["lambda"] == 1.0][0]
    cfg = {"workload": "2-D Helmholtz, 32x32 jittered quads, P in {6, 8}, lambda in {0.1, 1, 10}, "
                       "FP32 inner PCG in FP64 refinement to 1e-10", "l2": "L2-resident (latency-bound)"}
    _line("2-D mixed-precision solves/s, 32x32 jittered quads (P=6, lambda=1; all cases in 'cases')",
          head["mixed"]["solves_per_s"], "solves/s", args, cfg, dtype="f64 (outer) / f32 (inner)", cases=rows)


def suite_batched(args):
    """256 parametric solves (lambda log-uniform, E ~ U{500..8000}, P ~ U{3..9}) in one
    batch, FP64 and mixed: host-checked chunk launches, one graph launch per solve, and
    one launch with the per-order autotuned tile shapes."""
    from ithaca_gpu.batched import BatchedHelmholtz, parametric_quad_problems
    from ithaca_gpu.operators import Context
    ctx = Context(0)
    t0 = time.perf_counter()
    probs = parametric_quad_problems(ctx, nsolve=256)
    setup_s = time.perf_counter() - t0
    bt = BatchedHelmholtz(ctx, "quad", probs)
    out = {}
    tiles = None
    for name, one, tune in (("host_checked", 0, False), ("one_launch", 1, False), ("one_launch_tuned", 1, True)):
        bt.set_one_launch(one)
        if tune:
            tiles = bt.autotune(reps=3)
        row = {}
        for mode in ("fp64", "mixed"):
            bt.solve(mode=mode, tol=1e-10, want_x=False)  # warm-up (graph build)
            ms, res = _time_host(lambda: bt.solve(mode=mode, tol=1e-10, want_x=False), max(1, args.steps // 2), 0)
            it = res["iterations"]
            row[mode] = {"solves_per_s": 256 / (ms / 1e3), "batch_ms": ms, "device_ms": res["elapsed_ms"],
                         "iterations": {"min": int(it.min()), "median": float(np.median(it)), "max": int(it.max())},
                         "max_rel_residual": float(res["rel_residual"].max())}
        row["speedup_mixed_vs_fp64"] = row["mixed"]["solves_per_s"] / row["fp64"]["solves_per_s"]
        out[name] = row
    ndof = int(sum(p["amap"].nglobal - p["amap"].ndir for p in probs))
    cfg = {"workload": "256 2-D Helmholtz solves, lambda = 10^U(-2,2), E ~ U{500..8000} jittered quads, "
                       "P ~ U{3..9}, Q = P+2, tol 1e-10, one batch",
           "solve_dofs_total": ndof, "host_setup_s": setup_s,
           "tile_variants": {str(n): {"fp32": c["fp32"], "fp64": c["fp64"]} for n, c in tiles.items()}}
    best = out["one_launch_tuned"]
    _line("batched parametric solves/s (256 2-D solves, mixed)", best["mixed"]["solves_per_s"], "solves/s", args,
          cfg, dtype="f64 (outer) / f32 (inner)", batch=out, speedup_mixed_vs_fp64=best["speedup_mixed_vs_fp64"])


def suite_pod(args):
    """POD on the 32x32-quad, P=6 full-order model: 256 lambda snapshots (one batch), 50
    modes by the method of snapshots, reduced operators, 4096 online FP64 LU solves."""
    import torch
    from ithaca_gpu import pod
    from ithaca_gpu.batched import BatchedHelmholtz
    from ithaca_gpu.workload import quad_workload
    w = quad_workload(32, 6)
    ctx, sysg, amap = w["ctx"], w["system"], w["amap"]
    ndir = amap.ndir
    lams = 10 ** np.random.default_rng(4).uniform(-2, 2, 256)
    probs = [dict(nmodes=w["n"], npoints=w["Q"], jac=w["jac"], df=w["df"], amap=amap, lam=float(l), rhs=w["b"])
             for l in lams]
    bt = BatchedHelmholtz(ctx, "quad", probs)
    snap_ms, res = _time_host(lambda: bt.solve(mode="fp64", tol=1e-10), 1, 1)
    S = np.stack([x[ndir:] for x in res["x"]], axis=1)
    off_ms, (V, sigma, r) = _time_host(lambda: pod.offline(ctx, S, 50), args.steps)
    proj_ms, (A_L, A_M) = _time_host(lambda: pod.project(sysg, V), args.steps)
    f_r = V.T @ w["b"][ndir:]
    new = 10 ** np.random.default_rng(5).uniform(-2, 2, 4096)
    on_ms, X = _time_host(lambda: pod.online(ctx, A_L, A_M, f_r, new), args.steps)
    rec_ms, U = _time_host(lambda: pod.reconstruct(ctx, V, X[:256]), args.steps)
    errs = []
    for j in range(8):
        xf, _ = sysg.solve(float(new[j]), w["b"], tol=1e-12)
        errs.append(float(np.max(np.abs(U[j] - xf[ndir:])) / np.max(np.abs(xf))))
    cpu = None
    try:
        from oracle import pod as opod
        t0 = time.perf_counter()
        opod.pod_svd(S, nmodes=50)
        svd_ms = (time.perf_counter() - t0) * 1e3
        t0 = time.perf_counter()
        opod.online_lu(A_L, A_M, f_r, new[:512])
        lu_ms = (time.perf_counter() - t0) * 1e3 * 4096 / 512
        cpu = {"value": 4096 / (lu_ms / 1e3), "unit": "online solves/s", "cores": os.cpu_count() or 1,
               "kind": "port", "sample": f"numpy LU on 512 of the 4096 lambdas (scaled); thin SVD of S took "
                                         f"{svd_ms:.0f} ms"}
    except Exception as ex:
        cpu = {"value": None, "error": str(ex)[:200]}
    cfg = {"workload": "POD of 256 FP64 snapshots (lambda = 10^U(-2,2)) of 32x32 quads P=6, 50 modes, "
                       "4096 online lambdas, 50x50 FP64 LU", "snapshot_rows": int(S.shape[0]), "modes": r}
    _line("POD: online reduced solves/s (4096 lambdas, 50 modes)", 4096 / (on_ms / 1e3), "online solves/s", args,
          cfg, dtype="f64", ms={"snapshots_batch": snap_ms, "offline": off_ms, "project": proj_ms,
                                "online_4096": on_ms, "reconstruct_256": rec_ms},
          rom_vs_fom_max_rel_err=max(errs), sigma_ratio_50=float(sigma[49] / sigma[0]) if r >= 50 else None,
          cpu_baseline=cpu)


def suite_adjoint(args):
    """64 x 64 quads, P = 6, FP64: J(kappa) and dJ/dkappa by the adjoint (forward solve,
    adjoint solve, gradient kernel) through torch.autograd."""
    import torch
    from ithaca_gpu.adjoint import misfit
    from ithaca_gpu.workload import quad_workload, smooth_field
    w = quad_workload(64, 6)
    ctx, sysg, coll, amap = w["ctx"], w["system"], w["coll"], w["amap"]
    X = w["X"]
    kappa = torch.from_numpy((1 + 0.5 * smooth_field(X, 6)).reshape(-1)).cuda()
    kt = torch.from_numpy((1 + 0.5 * smooth_field(X, 7)).reshape(-1)).cuda()
    b = torch.from_numpy(w["b"]).cuda()
    sysg.set_varcoeff(kt)
    xt = torch.zeros_like(b)
    sysg.solve(1.0, b, xt, tol=1e-13)
    xt[:amap.ndir] = 0
    ut = coll.bwdtrans(sysg.global_to_local(xt))

    def grad():
        k = kappa.clone().requires_grad_(True)
        J = misfit(k, sysg, 1.0, b, ut, 1e-12)
        J.backward()
        return J.item(), k.grad

    ms, (J, g) = _time_host(grad, args.steps, 1)
    cfg = {"workload": "variable-coefficient Helmholtz, 64x64 jittered quads, P=6, kappa = 1 + 0.5 g (8 seeded "
                       "Fourier modes), J = sum Jw (u - u_t)^2, adjoint gradient, FP64 CG to 1e-12",
           "quadrature_points": int(kappa.numel())}
    _line("adjoint gradients/s, 64x64 quads P=6 (forward + adjoint solve + dJ/dkappa)", 1e3 / ms, "gradients/s", args, cfg,
          dtype="f64", J=J, grad_max=float(g.abs().max()))


def suite_hex_orders(args):
    """The 3-D sweep: 32^3 curved hexes at P = 4, 6, 8 (Q = P + 2): the four
    operators (GDOF/s, Ndof = E n^3; Helmholtz also in FP32 with the autotuned kernel)
    and Jacobi PCG to 1e-12, FP64 (the reference recurrence) and mixed."""
    import torch
    from ithaca_gpu.operators import Collection
    from ithaca_gpu.workload import hex_workload
    rows = []
    for P in (4, 6, 8):
        w = hex_workload(32, P)
        ctx, coll, sysg, amap = w["ctx"], w["coll"], w["system"], w["amap"]
        E, n, Q, N, ndir = w["mesh"].E, w["n"], w["Q"], amap.nglobal, amap.ndir
        stream = torch.cuda.ExternalStream(ctx.stream, device="cuda:0")
        gen = torch.Generator(device="cuda").manual_seed(P)
        u = torch.rand(E * n ** 3, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
        phys = torch.empty(E * Q ** 3, dtype=torch.float64, device="cuda")
        coef = torch.empty_like(u)
        d = [torch.empty_like(phys) for _ in range(3)]
        coll.bwdtrans(u, phys)
        ops = {"bwdtrans": lambda: coll.bwdtrans(u, phys), "iproduct": lambda: coll.iproduct(phys, coef),
               "physderiv": lambda: coll.physderiv(phys, d), "helmholtz": lambda: coll.helmholtz(1.0, u, coef)}
        gdofs = {k: E * n ** 3 / (_time_device(torch, stream, f, 10, 2) / 1e3) / 1e9 for k, f in ops.items()}
        coll32 = Collection(ctx, "hex", n, Q, E, w["jac"], w["df"], deformed=True, precision="fp32")
        v32, _ = coll32.autotune(reps=5)
        u32, o32 = u.float(), torch.empty(E * n ** 3, dtype=torch.float32, device="cuda")
        gdofs["helmholtz_fp32"] = E * n ** 3 / (
            _time_device(torch, stream, lambda: coll32.helmholtz(1.0, u32, o32), 20, 3) / 1e3) / 1e9
        sysg.autotune_inner(1.0, reps=5)
        b, x = w["b"], torch.zeros_like(w["b"])
        solves = {}
        for mode in ("fp64", "mixed"):
            reps = 1 if (mode == "fp64" and P == 8) else min(args.steps, 2)
            ms = _time_device(torch, stream, lambda: sysg.solve(1.0, b, x, tol=1e-12, mode=mode), reps, 1)
            _, res = sysg.solve(1.0, b, x, tol=1e-12, mode=mode)
            solves[mode] = {"solves_per_s": 1e3 / ms, "ms": ms, "iterations": res.iterations,
                            "outer": res.outer_iterations, "rel_residual": res.rel_residual}
        rows.append({"P": P, "n": n, "Q": Q, "global_dofs": N, "solve_dofs": N - ndir, "gdofs": gdofs,
                     "fp32_helmholtz_variant": v32, "solve_1e-12": solves})
        del w, coll, coll32, sysg, u, phys, coef, d, u32, o32, b, x
        ctx.close()
        torch.cuda.empty_cache()
    cfg = {"workload": "3-D Helmholtz, 32^3 hexes curved by x + 0.05 sin(2 pi y) sin(2 pi z), P = 4, 6, 8, "
                       "Q = P + 2, lambda = 1, Jacobi PCG to 1e-12",
           "elements": 32768, "l2": "operands exceed L2 at every order (geometry >= 200 MB)"}
    _line("3-D Helmholtz, 32^3 curved hexes at P = 4, 6, 8: operator GDOF/s and CG solves/s (1e-12)",
          rows[1]["solve_1e-12"]["mixed"]["solves_per_s"], "solves/s", args, cfg, dtype="f64 / f32 inner",
          orders=rows)


def suite_inner_apply(args):
    """The solver's gathered element applies alone, on --mesh^3 curved hexes at P =
    --order: the FP32 inner apply of the mixed solve (the --variant kernel, or the
    autotuned one) and the FP64 apply, CUDA-event time per launch against the algorithmic
    bytes. A small mesh keeps it a case the kernel captures can take."""
    from ithaca_gpu.workload import hex_workload
    args.mesh = args.mesh or 32
    w = hex_workload(args.mesh, args.order)
    sysg, E, n, Q = w["system"], w["mesh"].E, w["n"], w["Q"]
    tuned = {}
    mode = args.mixed_mode
    if args.variant < 0:
        variant, tuned = sysg.autotune_inner(LAMBDA, reps=max(3, args.steps), mode=mode,
                                             **({"variants": GEO16_VARIANTS} if mode == "mixed_geo16" else {}))
    else:
        variant = args.variant
        w["coll"].set_variant(variant)
    ms32, by32 = sysg.profile_apply(LAMBDA, mode=mode, reps=args.steps)
    ms64, by64 = sysg.profile_apply(LAMBDA, mode="fp64", reps=args.steps)
    peak, kind = load_peaks()
    cfg = {"workload": f"gathered element Helmholtz applies of the solver, {args.mesh}^3 curved hexes, P={args.order}",
           "elements": E, "fp32_kernel_variant": variant, "mixed_mode": mode,
           "autotune_ms": {str(v): round(t, 4) for v, t in tuned.items()}}
    _line("inner FP32 gathered apply: algorithmic GB/s", by32 / (ms32 / 1e3) / 1e9, "GB/s", args, cfg, dtype="f32",
          fp32={"kernel": geo16_kernel_name(variant, n, Q) if mode == "mixed_geo16" else fp32_kernel_name(variant, n, Q),
                "ms": ms32, "bytes": by32,
                "frac_of_hbm": by32 / (ms32 / 1e3) / 1e9 / peak, "peak_source": kind},
          fp64={"ms": ms64, "bytes": by64, "gbs": by64 / (ms64 / 1e3) / 1e9})


def suite_peaks(args):
    """The device's arithmetic-pipe peaks (FP64 FMA, FP64 MMA, FP32 FMA), measured by the
    library: the compute roofs of the FP64 and FP32 element operators."""
    from ithaca_gpu.operators import Context
    ctx = Context(0)
    runs = [ctx.pipe_peaks() for _ in range(max(1, args.steps))]
    best = {k: max(r[k] for r in runs) for k in runs[0]}
    _line("arithmetic pipe peaks (FP64 FMA, FP64 MMA m8n8k4, FP32 FMA)", best["fp64_fma_tflops"], "TFLOP/s", args,
          {"workload": "independent FMA / MMA chains on every SM, 8 CTAs of 256 threads per SM"}, dtype="f64/f32",
          peaks=best, runs=runs)
    ctx.close()


def suite_tri(args):
    """Triangles: 128 x 128 cells (32768 curved triangles) at P = 6."""
    import torch
    out = tri_fields(torch, "cuda:0", mesh=args.mesh or 128)
    _line("2-D Helmholtz on curved triangles, P=6: CG solves/s (FP64, 1e-10) and operator GDOF/s",
          out["fp64"]["solves_per_s"], "solves/s", args, {"workload": out["workload"]}, dtype="f64", tri=out,
          cpu_baseline=out.get("cpu_baseline"))


def suite_tet(args):
    """Tetrahedra: 12^3 cubes (10368 curved tetrahedra) at P = 6."""
    import torch
    out = tet_fields(torch, "cuda:0", mesh=args.mesh or 12)
    _line("3-D Helmholtz on curved tetrahedra, P=6: CG solves/s (FP64, 1e-10) and operator GDOF/s",
          out["fp64"]["solves_per_s"], "solves/s", args, {"workload": out["workload"]}, dtype="f64", tet=out)


def suite_prism(args):
    """Prisms: 12^3 cubes (3456 curved prisms) at P = 6."""
    import torch
    out = prism_fields(torch, "cuda:0", mesh=args.mesh or 12)
    _line("3-D Helmholtz on curved prisms, P=6: CG solves/s (FP64, 1e-10) and operator GDOF/s",
          out["fp64"]["solves_per_s"], "solves/s", args, {"workload": out["workload"]}, dtype="f64", prism=out)


def suite_pyr(args):
    """Pyramids: 10^3 cubes (6000 curved pyramids) at P = 6."""
    import torch
    out = pyr_fields(torch, "cuda:0", mesh=args.mesh or 10)
    _line("3-D Helmholtz on curved pyramids, P=6: CG solves/s (FP64, 1e-10) and operator GDOF/s",
          out["fp64"]["solves_per_s"], "solves/s", args, {"workload": out["workload"]}, dtype="f64", pyr=out)


SUITES = {"quad2d": suite_quad2d, "tri": suite_tri, "tet": suite_tet, "prism": suite_prism, "pyr": suite_pyr, "mixed2d": suite_mixed2d, "hex_orders": suite_hex_orders, "batched": suite_batched,
          "pod": suite_pod, "adjoint": suite_adjoint, "inner_apply": suite_inner_apply,
          "peaks": suite_peaks}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--order", type=int, default=6)
    ap.add_argument("--mesh", type=int, default=None,
                    help="cells per direction (default: 32 hex, 128 tri, 12 tet / prism, 10 pyr)")
    ap.add_argument("--mixed-mode", choices=["mixed", "mixed_geo16"], default="mixed_geo16",
                    help="inner solve of the headline: FP32 arithmetic on 16-bit geometry storage (default, the "
                         "faster), or on FP32 geometry (reported beside it in either case)")
    ap.add_argument("--fused-update", type=int, default=0, choices=[0, 1],
                    help="1: the inner FP32 iterations fuse the assembly with the vector update; "
                         "0: separate assembly and update kernels (default, measured faster)")
    ap.add_argument("--variant", type=int, default=-1,
                    help="FP32 hex kernel variant of the inner apply (-1: autotune; the headline and inner_apply)")
    ap.add_argument("--full", type=int, default=1,
                    help="1: add the P=8 hexes, the 2-D mixed sweep and the 256-solve batch to the line")
    ap.add_argument("--config", choices=["hex"] + list(SUITES) + ["all"], default="hex",
                    help="hex: the headline workload (default); the others: secondary workloads, one line each")
    args = ap.parse_args()
    if args.config in ("hex", "inner_apply") and args.mesh is None:
        args.mesh = 32  # the headline mesh (the other suites take their own defaults)
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.config != "hex" and args.impl == "gpu":
        sys.path.insert(0, os.path.join(ROOT, "ithaca-sem_gb300"))
        for name, fn in SUITES.items():
            if args.config in (name, "all") and rank == 0:
                fn(args)
        return None
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
