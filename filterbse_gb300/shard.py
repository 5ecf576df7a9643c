"""Multi-rank exchange for the filter stage (one process per GPU).

The filter shards naturally by random start: the cycles of different starts
are independent until the filtered states meet in the orthogonalisation
(filter_mpi/filter.c:102, mod_filter.c:155-159, where each MPI rank filters
its own starts).  This module is the host-side exchange of that step:

* ``start_shard``: the starts a rank filters (round robin);
* ``slab``: the grid-point range a rank owns after the redistribution;
* ``ShardedRitz``: the Rayleigh-Ritz step on states sharded by start, without
  gathering them on one rank.  The states are redistributed once from
  "my starts, all points" to "all states, my slab of points" (one
  all-to-all), the overlap and projected-H matrices are sums of per-slab
  products (one all-reduce each), the FP64 eigensolves are replicated (every
  rank gets the same matrices and solves the same small problem), and the
  rotation is local to each slab.

Every collective first checks in through the process group's store, with a
deadline: a rank that died or never arrived is reported by number
(``ShardError``) instead of hanging the others.  ``ritz`` forms the slab
products with torch on CPU tensors (gloo ranks in the tests); ``ritz_library``
forms them on the rank's GPU through the library's slab entry points
(fbse_gram, fbse_rotate), whose composition over slabs is tested on one GPU.
The exchange has not run on more than one GPU, and the benchmark runs
independent replicas.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np


class ShardError(RuntimeError):
    pass


def start_shard(nstart: int, world: int, rank: int) -> np.ndarray:
    """Round-robin starts of one rank (the reference gives rank r the starts
    r*n/size..; round robin keeps the counts within one of each other)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return np.arange(rank, nstart, world)


def slab(length: int, world: int, rank: int):
    """[lo, hi) of the grid points rank owns: contiguous, sizes within one."""
    base, extra = divmod(length, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


@dataclass
class ShardedRitz:
    """The exchange of the sharded Rayleigh-Ritz step over a torch.distributed
    process group (gloo on CPU tensors here).  ``deadline`` bounds every
    check-in (seconds)."""

    group: object = None
    deadline: float = 30.0
    tag: str = "fbse"

    def __post_init__(self):
        import torch.distributed as dist
        self.dist = dist
        self.world = dist.get_world_size(self.group)
        self.rank = dist.get_rank(self.group)
        self.store = dist.distributed_c10d._get_default_store()
        self.step = 0

    # -- liveness ---------------------------------------------------------------
    def checkin(self, what: str):
        """Every rank announces itself before a collective and waits, with a
        deadline, for all the others; raises ShardError naming the missing."""
        self.step += 1
        key = f"{self.tag}/{self.step}/{what}"
        self.store.set(f"{key}/{self.rank}", "1")
        t0 = time.monotonic()
        missing = list(range(self.world))
        while missing:
            missing = [r for r in missing if not self.store.check([f"{key}/{r}"])]
            if not missing:
                break
            if time.monotonic() - t0 > self.deadline:
                raise ShardError(f"rank(s) {missing} did not reach '{what}' within {self.deadline:.0f} s")
            time.sleep(0.01)

    # -- data movement --------------------------------------------------------------
    def _all_to_all(self, recv, send):
        """all_to_all where the backend has it (NCCL), pairwise send/receive
        otherwise (gloo has no alltoall)."""
        if self.dist.get_backend(self.group) == "nccl":
            self.dist.all_to_all(recv, send, group=self.group)
            return
        reqs = []
        for r in range(self.world):
            if r == self.rank:
                recv[r].copy_(send[r])
                continue
            reqs.append(self.dist.isend(send[r], dst=r, group=self.group))
            reqs.append(self.dist.irecv(recv[r], src=r, group=self.group))
        for q in reqs:
            q.wait()

    def counts(self, nstart_local):
        """States per rank (one small all-gather)."""
        import torch
        self.checkin("counts")
        t = torch.tensor([nstart_local], dtype=torch.int64)
        out = [torch.zeros(1, dtype=torch.int64) for _ in range(self.world)]
        self.dist.all_gather(out, t, group=self.group)
        return [int(x.item()) for x in out]

    def to_slabs(self, psi_local):
        """[n_local, L] (this rank's states, every point) -> [n_total, L_slab]
        (every state, this rank's points), states in rank order."""
        import torch
        n_local, L = psi_local.shape
        ns = self.counts(n_local)
        bounds = [slab(L, self.world, r) for r in range(self.world)]
        send = [psi_local[:, lo:hi].contiguous() for lo, hi in bounds]
        lo, hi = bounds[self.rank]
        recv = [torch.empty((ns[r], hi - lo), dtype=psi_local.dtype) for r in range(self.world)]
        self.checkin("to_slabs")
        self._all_to_all(recv, send)
        return torch.cat(recv, dim=0)

    def from_slabs(self, psi_slab, ns):
        """Inverse of to_slabs: [n_total, L_slab] -> [ns[rank], L]."""
        import torch
        offs = np.concatenate([[0], np.cumsum(ns)])
        send = [psi_slab[offs[r]:offs[r + 1]].contiguous() for r in range(self.world)]
        self.checkin("widths")
        w = torch.tensor([psi_slab.shape[1]], dtype=torch.int64)
        ws = [torch.zeros(1, dtype=torch.int64) for _ in range(self.world)]
        self.dist.all_gather(ws, w, group=self.group)
        widths = [int(x.item()) for x in ws]
        recv = [torch.empty((ns[self.rank], widths[r]), dtype=psi_slab.dtype) for r in range(self.world)]
        self.checkin("from_slabs")
        self._all_to_all(recv, send)
        return torch.cat(recv, dim=1)

    def gram(self, a_slab, b_slab, dv: float):
        """sum over slabs of dv <a_i|b_j> for states stored as rows
        (complex128), the same on every rank."""
        import torch
        g = ((a_slab.conj() @ b_slab.transpose(0, 1)) * dv).contiguous()
        self.checkin("gram")
        # reduce the (re, im) view: gloo has no complex reductions
        gr = torch.view_as_real(g) if g.is_complex() else g
        self.dist.all_reduce(gr, op=self.dist.ReduceOp.SUM, group=self.group)
        return g


def ritz(exch: ShardedRitz, psi_local, hpsi_local, dv: float, cut: float = 1e-12):
    """The sharded Rayleigh-Ritz step (mod_ortho + diag_H + calc_sigma_E on
    states sharded by start): returns (eigenvalues, sigma_E, this rank's slab
    of the normalised Ritz vectors [k, L_slab]).  The eigensolves are FP64
    and replicated."""
    import torch
    a = exch.to_slabs(psi_local)
    h = exch.to_slabs(hpsi_local)
    G = exch.gram(a, a, dv).numpy()
    M = exch.gram(a, h, dv).numpy()
    G = 0.5 * (G + G.conj().T)
    M = 0.5 * (M + M.conj().T)
    lam, V = np.linalg.eigh(G)
    keep = lam > cut * lam.max()
    X = V[:, keep] / np.sqrt(lam[keep])[None, :]
    Hp = X.conj().T @ M @ X
    e, U = np.linalg.eigh(0.5 * (Hp + Hp.conj().T))
    # new state k = sum_i C[i, k] psi_i (states are rows)
    Ct = torch.from_numpy(np.ascontiguousarray((X @ U).T))
    rot = Ct.to(a.dtype) @ a
    hrot = Ct.to(h.dtype) @ h
    r = hrot - torch.from_numpy(e).to(rot.dtype)[:, None] * rot
    # residual norms need every slab: one more all-reduce
    parts = torch.stack([(r.abs() ** 2).sum(1), (rot.abs() ** 2).sum(1)]).to(torch.float64) * dv
    exch.checkin("residuals")
    exch.dist.all_reduce(parts, op=exch.dist.ReduceOp.SUM, group=exch.group)
    nrm = parts[1].numpy()
    sigma = np.sqrt(parts[0].numpy() / nrm)
    return e, sigma, rot / torch.from_numpy(np.sqrt(nrm)).to(rot.dtype)[:, None]


def ritz_library(exch: ShardedRitz, ctx, psi_rows, hpsi_rows, off: int, length: int, cut: float = 1e-12):
    """The same step with this rank's slab products on its GPU through the
    library: psi_rows / hpsi_rows are [n_total, stlen] device rows holding
    every state's values in this rank's slab [off, off + length) (the
    redistribution writes them there); fbse_gram forms the slab Grams
    (all-reduced over the ranks as host FP64 matrices), the FP64 eigensolves
    are replicated, and fbse_rotate rotates the slab in place of a numpy
    product.  Returns (eigenvalues, sigma_E, rotated rows [k, stlen] valid in
    the slab)."""
    import torch
    G = ctx.gram(psi_rows, psi_rows, off, length)
    M = ctx.gram(psi_rows, hpsi_rows, off, length)
    both = torch.from_numpy(np.stack([G, M])).contiguous()
    exch.checkin("gram")
    br = torch.view_as_real(both)
    exch.dist.all_reduce(br, op=exch.dist.ReduceOp.SUM, group=exch.group)
    G, M = both[0].numpy(), both[1].numpy()
    G = 0.5 * (G + G.conj().T)
    M = 0.5 * (M + M.conj().T)
    lam, V = np.linalg.eigh(G)
    keep = lam > cut * lam.max()
    X = V[:, keep] / np.sqrt(lam[keep])[None, :]
    e, U = np.linalg.eigh(0.5 * (X.conj().T @ M @ X + (X.conj().T @ M @ X).conj().T))
    C = X @ U  # new state k = sum_i C[i, k] psi_i
    k = C.shape[1]
    rot = torch.zeros((k, psi_rows.shape[1]), dtype=psi_rows.dtype, device=psi_rows.device)
    hrot = torch.zeros_like(rot)
    ctx.rotate(psi_rows, C, rot, off, length)
    ctx.rotate(hpsi_rows, C, hrot, off, length)
    # residual and norm sums of the slab (the library's Gram of the rotated
    # rows gives both), then one all-reduce
    rr = ctx.gram(hrot, hrot, off, length).diagonal().real
    rh = ctx.gram(rot, hrot, off, length).diagonal().real
    pp = ctx.gram(rot, rot, off, length).diagonal().real
    parts = torch.from_numpy(np.stack([rr - 2 * e * rh + e ** 2 * pp, pp]))
    exch.checkin("residuals")
    exch.dist.all_reduce(parts, op=exch.dist.ReduceOp.SUM, group=exch.group)
    nrm = parts[1].numpy()
    return e, np.sqrt(np.abs(parts[0].numpy()) / nrm), rot
