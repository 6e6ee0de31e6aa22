"""Element-partitioned CG over ranks (ithaca_gpu.distributed), world sizes 2 and 3 on
CPU processes over gloo.

Each rank applies only its own elements (here the oracle's restatement of the element
operator stands in for the rank's GPU apply), the shared dofs are completed by one
exchange per operator apply (UniversalAssemble, AssemblyMapCG.cpp:2919-2923) and the
three CG scalars are all-reduced (NekLinSysIterCG.cpp:235). The partitioned solve must
take the single-process recurrence's iteration count (within one: only the summation
order of the dot products differs) and give its solution to 1e-10 on every rank.
"""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _problem():
    from cases import quad_case
    from oracle import ops as oops
    from oracle import solve as osolve
    c = quad_case(6, 5, 6, rotate=np.random.default_rng(3).integers(0, 4, 30))
    amap = c.mesh.assembly(c.n)
    f = (np.sin(np.pi * c.X[0]) * np.sin(np.pi * c.X[1])).reshape(-1)
    m = osolve.Map.of(amap)
    rhs = -m.assemble(oops.iproduct(c.basis, 2, c.jac.reshape(c.E, -1), f))
    return c, amap, rhs


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300"), os.path.join(ROOT, "tests")]
    from ithaca_gpu.distributed import DistributedCG, partition
    from oracle import ops as oops
    from oracle import solve as osolve
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        c, amap, rhs = _problem()
        rm = partition(amap, c.nm, world)[rank]
        e0, e1 = rm.elements[0], rm.elements[-1] + 1
        jac = c.jac.reshape(c.E, -1)[e0:e1]
        df = c.df.reshape(4, c.E, -1)[:, e0:e1].reshape(4, -1)
        lm = osolve.Map.of(rm.amap)
        lam = 1.0

        def apply_local(lam_, x):
            return torch.from_numpy(osolve.global_apply(c.basis, 2, jac, df, lam_, lm, x.numpy()))

        d = np.zeros(rm.amap.nglobal)
        np.add.at(d, lm.l2g, lm.sign ** 2 * oops.helmholtz_diag(c.basis, 2, jac, df, lam).reshape(-1))
        solver = DistributedCG(rm, apply_local, torch.from_numpy(d[rm.amap.ndir:]))
        x, it = solver.solve(lam, torch.from_numpy(rhs[rm.global_ids]), tol=1e-11)
        q.put((rank, it, rm.global_ids, x.numpy(), solver.exchanges))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_partitioned_cg_matches_single_process(world):
    sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300")]
    from oracle import solve as osolve
    c, amap, rhs = _problem()
    x_ref, it_ref, _, _ = osolve.solve(c.basis, 2, c.jac.reshape(c.E, -1), c.df, 1.0, amap, rhs, tol=1e-11)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    scale = np.max(np.abs(x_ref[amap.ndir:]))
    covered = np.zeros(amap.nglobal, dtype=bool)
    for rank, it, gids, x, nex in out:
        assert abs(it - it_ref) <= 1, (rank, it, it_ref)
        assert nex == it + 1  # one exchange per operator apply, plus the diagonal's
        free = gids >= amap.ndir
        assert np.max(np.abs(x[free] - x_ref[gids[free]])) / scale < 1e-10
        covered[gids] = True
    assert covered.all()


def test_partition_bookkeeping():
    sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300")]
    from ithaca_gpu.distributed import partition
    c, amap, _ = _problem()
    maps = partition(amap, c.nm, 3)
    owners = np.zeros(amap.nglobal)
    for rm in maps:
        np.add.at(owners, rm.global_ids, rm.owner)
        assert np.all(rm.global_ids[:rm.amap.ndir] < amap.ndir) and np.all(rm.global_ids[rm.amap.ndir:] >= amap.ndir)
        for qr, ix in rm.shared.items():  # both sides list the same global dofs in the same order
            other = maps[qr]
            assert np.array_equal(rm.global_ids[ix], other.global_ids[other.shared[rm.rank]])
    assert np.all(owners == 1.0)  # every global dof is counted once in the dot products


def _gpu_rank(rank, world, port, q):
    """A rank whose element apply and diagonal are its own GPU sub-system's (CUDA
    kernels through the C ABI); the exchange and the scalar reductions go over gloo on
    the host, so the two processes' kernels never wait on one another."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300"), os.path.join(ROOT, "tests")]
    from ithaca_gpu.distributed import DistributedCG, partition
    from ithaca_gpu.operators import Collection, Context, GlobalLinSysIterativeFullGPU
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        c, amap, rhs = _problem()
        rm = partition(amap, c.nm, world)[rank]
        e0, e1 = rm.elements[0], rm.elements[-1] + 1
        jac = np.ascontiguousarray(c.jac.reshape(c.E, -1)[e0:e1]).reshape(-1)
        df = np.ascontiguousarray(c.df.reshape(4, c.E, -1)[:, e0:e1]).reshape(4, -1)
        ctx = Context(0)
        coll = Collection(ctx, "quad", c.n, c.Q, e1 - e0, jac, df)
        sysr = GlobalLinSysIterativeFullGPU(coll, rm.amap)
        lam = 1.0
        apply_local = lambda lam_, x: torch.from_numpy(sysr.apply(lam_, np.ascontiguousarray(x.numpy())))
        solver = DistributedCG(rm, apply_local, torch.from_numpy(sysr.diagonal(lam)))
        x, it = solver.solve(lam, torch.from_numpy(rhs[rm.global_ids]), tol=1e-11)
        launches = ctx.launch_count()
        q.put((rank, it, rm.global_ids, x.numpy(), launches))
        ctx.close()
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_partitioned_cg_with_gpu_element_applies():
    sys.path[:0] = [ROOT, os.path.join(ROOT, "ithaca-sem_gb300")]
    from oracle import solve as osolve
    c, amap, rhs = _problem()
    x_ref, it_ref, _, _ = osolve.solve(c.basis, 2, c.jac.reshape(c.E, -1), c.df, 1.0, amap, rhs, tol=1e-11)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gpu_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=600) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    scale = np.max(np.abs(x_ref[amap.ndir:]))
    for rank, it, gids, x, launches in out:
        assert abs(it - it_ref) <= 1, (rank, it, it_ref)
        assert launches >= it  # every operator apply ran the rank's own kernels
        free = gids >= amap.ndir
        assert np.max(np.abs(x[free] - x_ref[gids[free]])) / scale < 1e-10
