"""Benchmark: Helmholtz GDOF/s & CG solves/s, mixed vs FP64 on the GPU at 1e-10 relative residual.

Workload (one GPU): 3-D Helmholtz (lambda = 1) on a 32^3 hexahedral mesh of the unit
cube curved by x_a + 0.05 sin(2 pi x_b) sin(2 pi x_c) (cyclic), per-quadrature-point
Jacobians, ModifiedA P = 6 (7 modes, 8 GLL points per direction), forcing
f = sin(pi x) sin(pi y) sin(pi z), homogeneous Dirichlet boundary. A step is one
Jacobi-preconditioned CG solve of the assembled C0 system to an FP64 relative residual
||b - A x||_2 / ||b||_2 < 1e-10, FP32 inner solves inside FP64 iterative refinement.
Inputs are synthetic and seeded; no dataset is involved.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--order P] [--mesh M]

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


def workload_config(args, n, Q, E, N, ndir):
    return {"workload": f"3-D Helmholtz, {args.mesh}^3 curved hexes, P={args.order} (n={n}, Q={Q}), "
                        f"lambda={LAMBDA}, Jacobi PCG to {TOL:g} rel. residual",
            "elements": E, "modes_per_dir": n, "points_per_dir": Q, "global_dofs": N, "solve_dofs": N - ndir,
            "local_dofs": E * n ** 3, "inner": "fp32 PCG in fp64 iterative refinement",
            "l2": "inputs larger than L2 (geometry and vectors exceed 129 MB)", "parallelism": "replicas"}


def cpu_baseline_sample(args, n, Q, E, jac, df, amap, rhs, iters_full, nthreads, budget_s=20.0):
    """Time the compiled CPU port of the reference CG (oracle/cport) on a bounded number
    of iterations of the same workload; scale to solves/s with the iteration count of the
    full reference recurrence (iters_full)."""
    from oracle import cportbind
    from oracle import solve as osolve
    if not cportbind.available():
        return None
    dinv = np.ascontiguousarray(1.0 / rhs["diag"]) if "diag" in rhs else None
    t0 = time.perf_counter()
    cportbind.cg_solve(3, n, Q, E, jac, df, True, LAMBDA, amap.l2g, amap.sign, amap.nglobal, amap.ndir, dinv,
                       rhs["b"], TOL, 1, nthreads)
    t1 = time.perf_counter()
    base = t1 - t0  # setup + 2 operator applications
    k = 4
    while True:
        t0 = time.perf_counter()
        cportbind.cg_solve(3, n, Q, E, jac, df, True, LAMBDA, amap.l2g, amap.sign, amap.nglobal, amap.ndir, dinv,
                           rhs["b"], TOL, k + 1, nthreads)
        dt = time.perf_counter() - t0
        if dt > budget_s / 2 or k >= 64:
            break
        k *= 2
    t_iter = max(dt - base, 1e-9) / k
    return {"value": 1.0 / (t_iter * iters_full), "unit": "solves/s", "cores": nthreads, "kind": "port",
            "sample": f"{k} CG iterations of the full workload ({t_iter * 1e3:.1f} ms/iteration, setup excluded), "
                      f"scaled by the {iters_full} iterations of the FP64 reference recurrence",
            "ms_per_iteration": t_iter * 1e3}


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
    stream = torch.cuda.ExternalStream(ctx.stream, device=cuda)
    # pick the FP32 element-kernel variant by timing (CollectionOptimisation analogue)
    variant, variant_ms = coll.autotune(reps=5)
    coll32.set_variant(variant)

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
    for _ in range(args.warmup):
        _, res = sysg.solve(LAMBDA, b, x, tol=TOL, mode="mixed")
    barrier()
    l0 = ctx.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        ev0.record(stream)
        results = []
        for _ in range(args.steps):
            _, res = sysg.solve(LAMBDA, b, x, tol=TOL, mode="mixed")
            results.append((res.iterations, res.outer_iterations, res.rel_residual))
        ev1.record(stream)
        ev1.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = ctx.launch_count() - l0
    if world > 1:
        t = torch.tensor([ms], device=cuda)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * args.steps / (ms / 1e3)
    x_mixed = x.clone()

    # ---- dominant kernel: the FP32 gather + element Helmholtz of the inner solve ----
    k_ms, k_bytes = sysg.profile_apply(LAMBDA, mode="mixed", reps=20)
    peak, peak_kind = load_peaks()
    achieved = k_bytes / (k_ms / 1e3) / 1e9

    # ---- FP64 reference recurrence on the GPU ----
    _, res64 = sysg.solve(LAMBDA, b, x, tol=TOL, mode="fp64")
    torch.cuda.synchronize()
    k64 = max(1, min(2, args.steps))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(k64):
        _, res64 = sysg.solve(LAMBDA, b, x, tol=TOL, mode="fp64")
    e1.record(stream)
    e1.synchronize()
    fp64_solves = k64 / (e0.elapsed_time(e1) / 1e3)
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
    f_host = np.ascontiguousarray(f)
    out_host = np.zeros(E * n ** 3)
    sysg.helmsolve(LAMBDA, f_host, out_host, tol=TOL, mode="mixed")
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, rese = sysg.helmsolve(LAMBDA, f_host, out_host, tol=TOL, mode="mixed")
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e = world * args.steps / e2e_s

    if rank != 0:
        return
    cfg = workload_config(args, n, Q, E, N, ndir)
    cfg["fp32_kernel_variant"] = variant
    cfg["autotune_ms"] = {str(k): round(v, 4) for k, v in variant_ms.items()}
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (outer) / f32 (inner)", "data": "synthetic (seeded mesh and forcing)",
        "config": cfg,
        "iterations": {"inner": results[-1][0], "outer": results[-1][1], "rel_residual": results[-1][2]},
        "fp64": {"solves_per_s": fp64_solves, "iterations": res64.iterations, "rel_residual": res64.rel_residual,
                 "speedup_mixed_vs_fp64": value / world / fp64_solves, "max_rel_diff_vs_mixed": sol_diff,
                 "apply_ms": k64_ms, "apply_fp64_tflops": None},
        "helmholtz_gdofs": {"fp64": gdofs64, "fp32": gdofs32},
        "solver_gdofs": {"mixed": value / world * (N - ndir) / 1e9, "fp64": fp64_solves * (N - ndir) / 1e9},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "kernel": ("helm3_pencil_kernel<float,7,8>" if variant else "helm_kernel<float,3,7,8>") + " gather (inner FP32 apply)",
                     "kernel_ms": k_ms, "bytes_per_launch": k_bytes, "peak_source": peak_kind},
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": int(f_host.nbytes),
                "d2h_bytes_per_step": int(out_host.nbytes), "rel_residual": rese.rel_residual},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    # FP64 flop rate of the FP64 apply (collocation-form operation count per element)
    fl = 2 * (2 * (Q * n ** 3 + Q * Q * n * n + Q ** 3 * n) + 6 * Q ** 4 + 11 * Q ** 3)
    line["fp64"]["apply_fp64_tflops"] = E * fl / (k64_ms / 1e3) / 1e12
    # CPU baseline: compiled port of the reference path on the host cores, bounded sample
    try:
        jac_h, df_h = jac.cpu().numpy(), df.cpu().numpy()
        diag = sysg.diagonal(LAMBDA)
        full = np.zeros(N)
        full[ndir:] = diag
        rhs = {"b": b.cpu().numpy(), "diag": diag}
        line["cpu_baseline"] = cpu_baseline_sample(args, n, Q, E, jac_h, df_h, amap, rhs, res64.iterations,
                                                   os.cpu_count() or 1)
    except Exception as ex:  # the GPU numbers stand even if the CPU sample fails
        line["cpu_baseline"] = {"value": None, "error": str(ex)[:200]}
    print(json.dumps(line))


def run_reference(args, rank, world):
    """CPU arm: the compiled port of the reference kernels + CG (oracle/cport), all host
    threads, on the same workload; each step is a bounded sample of CG iterations."""
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
    iters_full = REF_ITERATIONS.get((args.mesh, args.order))
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
    if iters_full is None:
        iters_full = 1
        unit_note = "per CG iteration (no iteration count recorded for this mesh/order)"
    else:
        unit_note = f"scaled by the {iters_full} iterations of the FP64 reference recurrence"
    value = 1.0 / (t_iter * iters_full)
    cfg = workload_config(args, n, Q, E, N, ndir)
    cfg["parallelism"] = f"{nth} host threads"
    print(json.dumps({
        "metric": METRIC, "impl": "reference", "value": value, "unit": "solves/s", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(times) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": cfg,
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": nth, "kind": "port",
                         "sample": f"{per_step} CG iterations per step on the full workload, setup excluded, "
                                   + unit_note},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# Iterations of the FP64 reference recurrence (Jacobi PCG, tol 1e-10) on the bench
# workloads, as counted by the GPU FP64 path (which reproduces the recurrence).
REF_ITERATIONS = {(32, 6): 961}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--order", type=int, default=6)
    ap.add_argument("--mesh", type=int, default=32)
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
