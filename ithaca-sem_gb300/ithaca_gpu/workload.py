"""Benchmark workloads.

``hex_workload(mesh, order)`` builds the curved 32^3 (or mesh^3) hexahedral Helmholtz
problem on the GPU: geometry factors, the FP64 collection, the C0 system and the
assembled right-hand side of f = sin(pi x) sin(pi y) sin(pi z). ``quad_workload``
builds the jittered 2-D quad problems and ``smooth_field`` the seeded variable
coefficient of the adjoint benchmark.
"""
import numpy as np

from ithaca_gpu.mesh import HexMesh


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
