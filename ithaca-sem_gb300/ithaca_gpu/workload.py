"""Benchmark workloads and a small command-line driver.

``hex_workload(mesh, order)`` builds the curved 32^3 (or mesh^3) hexahedral Helmholtz
problem on the GPU: geometry factors, the FP64 collection, the C0 system and the
assembled right-hand side of f = sin(pi x) sin(pi y) sin(pi z). ``quad_workload``
builds the jittered 2-D quad problems and ``smooth_field`` the seeded variable
coefficient of the adjoint benchmark.

    python ithaca-sem_gb300/ithaca_gpu/workload.py --mesh 24 --order 6 --mode mixed --solves 1

runs that many solves and prints iterations and times; it is the command the ncu
summaries under profiles/ were taken on.
"""
import argparse
import os
import sys
import time

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from ithaca_gpu.mesh import HexMesh  # noqa: E402


def hex_workload(mesh_n=32, order=6, device=0, amp=0.05):
    import torch
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU, geom_factors
    cuda = f"cuda:{device}"
    n, Q = order + 1, order + 2
    mesh = HexMesh(mesh_n, mesh_n, mesh_n, curve_amp=amp)
    X = mesh.coords(Q)
    amap = mesh.assembly(n)
    f = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1]) * np.sin(np.pi * X[2])).reshape(-1)
    ctx = Context(device)
    jac, df = geom_factors(ctx, "hex", Q, torch.from_numpy(X).to(cuda))
    coll = Collection(ctx, "hex", n, Q, mesh.E, jac, df, deformed=True, precision="fp64")
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    fd = torch.from_numpy(f).to(cuda)
    loc = torch.empty(mesh.E * n ** 3, dtype=torch.float64, device=cuda)
    coll.iproduct(fd, loc)
    loc.neg_()
    b = torch.empty(amap.nglobal, dtype=torch.float64, device=cuda)
    sysg.assemble(loc, b)
    ctx.synchronize()
    return dict(ctx=ctx, mesh=mesh, n=n, Q=Q, X=X, amap=amap, f=f, jac=jac, df=df, coll=coll, system=sysg, b=b)


def quad_workload(nx=32, order=6, device=0, jitter=0.1, seed=0, ctx=None):
    """Jittered nx x nx quads of the unit square (interior vertices moved by
    U(-jitter h, jitter h), seeded), ModifiedA with order + 1 modes on order + 2 GLL
    points, FP64 collection, C0 system and the assembled right-hand side of
    f = sin(pi x) sin(pi y) (homogeneous Dirichlet boundary)."""
    import torch
    from ithaca_gpu.mesh import QuadMesh
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU, geom_factors
    n, Q = order + 1, order + 2
    mesh = QuadMesh(nx, nx, jitter=jitter, seed=seed)
    X = mesh.coords(Q)
    amap = mesh.assembly(n)
    f = (np.sin(np.pi * X[0]) * np.sin(np.pi * X[1])).reshape(-1)
    ctx = ctx or Context(device)
    jac, df = geom_factors(ctx, "quad", Q, X)
    coll = Collection(ctx, "quad", n, Q, mesh.E, jac, df, deformed=True, precision="fp64")
    sysg = GlobalLinSysIterativeFullGPU(coll, amap)
    loc = coll.iproduct(f)
    b = -np.bincount(amap.l2g, weights=amap.sign * loc, minlength=amap.nglobal)
    return dict(ctx=ctx, mesh=mesh, n=n, Q=Q, X=X, amap=amap, f=f, jac=jac, df=df, coll=coll, system=sysg, b=b)


def smooth_field(X, seed, nmodes=8):
    """Seeded smooth 2-D field at points X (2, ...): a sum of nmodes products of shifted
    sines with integer wave numbers 1..3, normalised to max |g| = 1 (the variable
    coefficient kappa = 1 + 0.5 g of the adjoint benchmark)."""
    rng = np.random.default_rng(seed)
    g = np.zeros_like(X[0])
    for _ in range(nmodes):
        kx, ky = rng.integers(1, 4, size=2)
        a = rng.uniform(-1, 1)
        px, py = rng.uniform(0, 2 * np.pi, size=2)
        g = g + a * np.sin(np.pi * kx * X[0] + px) * np.sin(np.pi * ky * X[1] + py)
    return g / max(np.max(np.abs(g)), 1e-300)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--mesh", type=int, default=24)
    ap.add_argument("--order", type=int, default=6)
    ap.add_argument("--mode", choices=["fp64", "mixed", "mixed_geo16"], nargs="*", default=["mixed"])
    ap.add_argument("--solves", type=int, default=1)
    ap.add_argument("--variant", type=int, default=-1, help="FP32 hex kernel variant (-1: autotune)")
    ap.add_argument("--inner-tol", type=float, nargs="*", default=[1e-2],
                    help="relative reduction asked of each inner FP32 solve (mixed mode)")
    a = ap.parse_args()
    import torch
    w = hex_workload(a.mesh, a.order)
    if a.variant < 0:
        v, times = w["coll"].autotune(reps=3)
        print("autotune (ungathered apply)", v, times)
        v, times = w["system"].autotune_inner(1.0, reps=5)
        print("autotune (gathered inner apply)", v, times)
    else:
        w["coll"].set_variant(a.variant)
    x = torch.zeros_like(w["b"])
    for mode in a.mode:
        for itol in a.inner_tol if mode != "fp64" else [0.0]:
            for _ in range(a.solves):
                t0 = time.perf_counter()
                _, res = w["system"].solve(1.0, w["b"], x, tol=1e-10, mode=mode, inner_tol=itol or 1e-2)
                print(f"{mode} inner_tol {itol:g}: {res.iterations} iterations, {res.outer_iterations} outer, "
                      f"rel residual {res.rel_residual:.3e}, {time.perf_counter() - t0:.3f} s")


if __name__ == "__main__":
    main()
