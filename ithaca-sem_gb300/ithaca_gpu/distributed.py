"""Element-partitioned C0 solve over several ranks (one GPU per rank).

The reference runs one MPI rank per partition of the mesh: each rank applies its own
elements' operator, sums the contributions of the dofs it shares with other ranks
(GsLib gather-scatter, AssemblyMapCG::UniversalAssemble,
MultiRegions/AssemblyMap/AssemblyMapCG.cpp:2919-2923), and reduces the three scalars of
each CG iteration over all ranks (NekLinSysIterCG.cpp:235, Comm::AllReduce). Dot products
count each global dof once through the "universal unique map" weights m_map
(GlobalLinSysIterative::v_UniqueMap, Vmath::Dot2 with m_map).

Here:
  * ``partition(amap, E_per_elem, nranks)`` splits the elements into contiguous blocks
    and builds each rank's ``RankMap``: its elements' local-to-global map renumbered
    into rank-local ids (Dirichlet dofs first, as the single-rank map), the rank-local
    id of every one of its global dofs, the dofs it shares with each other rank (sorted
    by global id, so both sides of a pair list them in the same order) and the owner
    weights (1 on the lowest rank touching a dof, 0 elsewhere).
  * ``DistributedCG`` runs the reference recurrence on the rank-local copy of the
    global vector: the operator is the rank's own element apply + assembly (a callable,
    e.g. ``GlobalLinSysIterativeFullGPU.apply`` of the rank's sub-collection), followed
    by one exchange step that adds the neighbours' partial sums at the shared dofs;
    the dot products are owner-weighted and all-reduced (three scalars per iteration).
Vectors are torch tensors on the rank's device; the exchange uses torch.distributed
point-to-point sends (NCCL between GPUs, gloo between CPU processes), never a
multicast. The element applies are the rank's own CUDA kernels; the vector updates of
the recurrence are small elementwise torch operations on the rank's dofs.
"""
from dataclasses import dataclass, field

import numpy as np

from .mesh import AssemblyMap


@dataclass
class RankMap:
    rank: int
    elements: np.ndarray          # global element ids of this rank (contiguous block)
    amap: AssemblyMap             # rank-local map of its elements (Dirichlet dofs first)
    global_ids: np.ndarray        # rank-local id -> global id
    owner: np.ndarray             # 1.0 where this rank owns the dof (counts it in dots)
    shared: dict = field(default_factory=dict)  # neighbour rank -> rank-local ids (by global id)


def partition(amap, nm, nranks):
    """Contiguous element blocks; nm local dofs per element. Returns [RankMap] * nranks."""
    E = amap.l2g.size // nm
    bounds = np.linspace(0, E, nranks + 1).round().astype(int)
    l2g = amap.l2g.reshape(E, nm)
    sign = amap.sign.reshape(E, nm)
    touched = [np.unique(l2g[bounds[r]:bounds[r + 1]]) for r in range(nranks)]
    # owner of a global dof: the lowest rank touching it
    owner_rank = np.full(amap.nglobal, nranks, dtype=np.int64)
    for r in range(nranks - 1, -1, -1):
        owner_rank[touched[r]] = r
    maps = []
    for r in range(nranks):
        g = touched[r]
        dirm = g < amap.ndir
        order = np.concatenate([g[dirm], g[~dirm]])  # Dirichlet first, then increasing global id
        local_of = {int(v): i for i, v in enumerate(order)}
        loc = np.vectorize(local_of.__getitem__, otypes=[np.int64])(l2g[bounds[r]:bounds[r + 1]])
        rm = RankMap(rank=r, elements=np.arange(bounds[r], bounds[r + 1]),
                     amap=AssemblyMap(loc.reshape(-1), sign[bounds[r]:bounds[r + 1]].reshape(-1), order.size,
                                      int(dirm.sum())),
                     global_ids=order, owner=(owner_rank[order] == r).astype(np.float64))
        for q in range(nranks):
            if q == r:
                continue
            common = np.intersect1d(g, touched[q], assume_unique=True)
            common = common[common >= amap.ndir]  # Dirichlet dofs are not solved for
            if common.size:
                rm.shared[q] = np.array([local_of[int(v)] for v in common], dtype=np.int64)
        maps.append(rm)
    return maps


class DistributedCG:
    """NekLinSysIterCG::DoConjugateGradient (NekLinSysIterCG.cpp:104-263) over ranks.

    apply_local(lam, x) -> y: this rank's elements' Helmholtz apply, assembled into its
    rank-local global vector (Dirichlet part of x read as zero); diag_local: the same
    rank-local assembly of its elements' diagonals (its free part). Both are partial
    sums at the shared dofs until ``exchange`` completes them."""

    def __init__(self, rmap, apply_local, diag_local, group=None):
        import torch
        import torch.distributed as dist
        self.torch, self.dist, self.group = torch, dist, group
        self.rm = rmap
        self.apply_local = apply_local
        self.nd = rmap.amap.ndir
        dev = diag_local.device
        self.owner = torch.from_numpy(rmap.owner[self.nd:]).to(dev)
        self.shared = {q: torch.from_numpy(ix).to(dev) for q, ix in sorted(rmap.shared.items())}
        d = torch.zeros(rmap.amap.nglobal, dtype=torch.float64, device=dev)
        d[self.nd:] = diag_local
        self.exchange(d)
        self.dinv = 1.0 / d[self.nd:]
        self.exchanges = 1

    def exchange(self, v):
        """Adds the neighbours' partial sums at the shared dofs (UniversalAssemble)."""
        torch, dist = self.torch, self.dist
        if not self.shared:
            return v
        sends, recvs, reqs = {}, {}, []
        for q, ix in self.shared.items():
            sends[q] = v[ix].contiguous()
            recvs[q] = torch.empty_like(sends[q])
        for q in self.shared:  # post every receive and send, then wait (no ordering deadlock)
            reqs.append(dist.irecv(recvs[q], src=q, group=self.group))
            reqs.append(dist.isend(sends[q], dst=q, group=self.group))
        for rq in reqs:
            rq.wait()
        for q, ix in self.shared.items():
            v[ix] += recvs[q]
        return v

    def _allreduce(self, vals):
        t = self.torch.stack(vals)
        self.dist.all_reduce(t, group=self.group)
        return [float(x) for x in t.cpu()]

    def _op(self, lam, x):
        y = self.apply_local(lam, x)
        self.exchange(y)
        self.exchanges += 1
        return y

    def solve(self, lam, rhs, tol=1e-9, max_iter=5000):
        """rhs: this rank's copy of the assembled global rhs (full values at shared dofs).
        Returns (x, iterations) with the same stop rule and 1e-6 magnitude floor."""
        torch = self.torch
        nd, own = self.nd, self.owner
        N = rhs.numel()
        x = torch.zeros(N, dtype=torch.float64, device=rhs.device)
        r = rhs[nd:].clone()
        w = torch.zeros(N, dtype=torch.float64, device=rhs.device)
        p = torch.zeros_like(r)
        q = torch.zeros_like(r)
        # ||b||^2 over every global entry once (Dirichlet ones owned by their lowest rank too)
        ownall = torch.from_numpy(self._owner_all()).to(rhs.device)
        eps, bb = self._allreduce([(own * r * r).sum(), (ownall * rhs * rhs).sum()])
        rhs_mag = bb if bb > 1e-6 else 1.0
        tol = max(tol, 1e-16)
        if eps < tol * tol * rhs_mag:
            return x, 0
        w[nd:] = self.dinv * r
        s = self._op(lam, w)
        rho, mu = self._allreduce([(own * r * w[nd:]).sum(), (own * s[nd:] * w[nd:]).sum()])
        beta, alpha = 0.0, rho / mu
        iters, k = 1, 0
        while True:
            if k >= max_iter:
                raise RuntimeError("Exceeded maximum number of iterations")
            p = beta * p + w[nd:]
            q = beta * q + s[nd:]
            x[nd:] += alpha * p
            r -= alpha * q
            w[nd:] = self.dinv * r
            s = self._op(lam, w)
            rho_new, mu, eps = self._allreduce([(own * r * w[nd:]).sum(), (own * s[nd:] * w[nd:]).sum(),
                                                (own * r * r).sum()])
            iters += 1
            if eps < tol * tol * rhs_mag:
                break
            beta = rho_new / rho
            alpha = rho_new / (mu - rho_new * beta / alpha)
            rho = rho_new
            k += 1
        return x, iters

    def _owner_all(self):
        """Owner weights over every rank-local dof, the Dirichlet ones included."""
        return self.rm.owner
