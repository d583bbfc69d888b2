"""Work division of the BSE path over several GPUs, one process per GPU (host side).

The reference runs on one node without any distribution (its only trace is a commented-out MPI
rank test, bse.version13.cpp:3689).  Here the path is split where it shards without an exchange
step, and the results meet on the host of rank 0; no device collective is involved:

* batched models: independent problems are dealt to per-rank queues by their estimated cost
  N_BSE^3 (the dense eigensolve dominates), longest first, each to the least-loaded rank.  Every
  rank solves its queue on its own GPU (bse_solve_many) and rank 0 gathers the spectra.
* kernel build: the rows of H are split into k tiles (bse_build_kernel_rows).  Rank 0 gathers
  the row blocks and solves on one GPU (bse_set_kernel, then the eigensolve: the dense
  eigensolve does not shard, replicas only).
* eps(omega): the exciton range is split over the ranks and the partial spectra are added.

The gathers are host-side object gathers of a torch.distributed process group (gloo or NCCL
alike); with world_size 1 everything runs locally.  The per-rank compute is a parameter, so the
partition and gather logic can be exercised without a GPU.
"""
from __future__ import annotations

from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np


def plan_batch(costs: Sequence[float], n_ranks: int) -> List[List[int]]:
    """Deal problems to n_ranks queues: descending cost, each to the least-loaded queue (ties to
    the lower rank); every queue in ascending problem order.  Deterministic."""
    if n_ranks < 1:
        raise ValueError("n_ranks must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * n_ranks
    queues: List[List[int]] = [[] for _ in range(n_ranks)]
    for i in order:
        r = min(range(n_ranks), key=lambda q: (load[q], q))
        queues[r].append(i)
        load[r] += float(costs[i])
    return [sorted(q) for q in queues]


def batch_cost(prob) -> float:
    """Estimated cost of one solve: N_BSE^3 (the dense eigensolve)."""
    return float(prob.n_bse) ** 3


def ranges(n: int, n_ranks: int) -> List[Tuple[int, int]]:
    """[lo, hi) ranges splitting 0..n-1 into n_ranks contiguous, balanced pieces."""
    b = [n * r // n_ranks for r in range(n_ranks + 1)]
    return [(b[r], b[r + 1]) for r in range(n_ranks)]


def gather_to_root(obj, rank: int, world_size: int):
    """Host-side gather of a picklable object on rank 0 (None on the other ranks)."""
    if world_size == 1:
        return [obj]
    import torch.distributed as dist
    out = [None] * world_size if rank == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out


# --------------------------------------------------------------------------- batched models
def _gpu_solve_queue(probs, omega, gamma, n_workers=8, **ctx_kw) -> np.ndarray:
    from . import gpu
    ctxs = [gpu.BSEContext(p, **ctx_kw) for p in probs]
    try:
        e2, _ = gpu.solve_many(ctxs, omega, gamma, n_workers=n_workers)
    finally:
        for c in ctxs:
            c.close()
    return e2


def solve_batch(problems, omega, gamma, rank: int = 0, world_size: int = 1,
                solve_queue: Optional[Callable] = None, **ctx_kw) -> Optional[np.ndarray]:
    """eps2 (n_problems x n_omega) of every problem on rank 0 (None elsewhere).  This rank solves
    the queue plan_batch gives it; solve_queue(probs, omega, gamma, **ctx_kw) -> eps2 rows
    (default: bse_solve_many on this process's GPU)."""
    queues = plan_batch([batch_cost(p) for p in problems], world_size)
    mine = queues[rank]
    fn = solve_queue or _gpu_solve_queue
    local = np.asarray(fn([problems[i] for i in mine], omega, gamma, **ctx_kw)) if mine else \
        np.zeros((0, len(omega)))
    parts = gather_to_root((mine, local), rank, world_size)
    if rank != 0:
        return None
    eps2 = np.full((len(problems), len(omega)), np.nan)
    for idx, vals in parts:
        if idx:
            eps2[np.asarray(idx)] = vals
    return eps2


# --------------------------------------------------------------------------- kernel build
def tile_rows(n_h: int, nk: int, lo: int, hi: int) -> np.ndarray:
    """Row indices of H in the k tile [lo, hi): r = g nk + k for the n_h / nk groups g, ascending."""
    g = np.arange(n_h // nk)[:, None] * nk
    return (g + np.arange(lo, hi)[None, :]).ravel()


def assemble_rows(parts, nk: int, n_h: int) -> np.ndarray:
    """The full n_h x n_h H from (lo, hi, rows) blocks that cover every k once."""
    H = np.zeros((n_h, n_h), np.complex128)
    seen = np.zeros(nk, bool)
    for lo, hi, rows in parts:
        if seen[lo:hi].any():
            raise ValueError("overlapping k tiles")
        seen[lo:hi] = True
        H[tile_rows(n_h, nk, lo, hi)] = rows
    if not seen.all():
        raise ValueError("k tiles do not cover the k list")
    return H


def _gpu_build_rows(prob, lo, hi, **ctx_kw) -> np.ndarray:
    from . import gpu
    with gpu.BSEContext(prob, **ctx_kw) as ctx:
        return ctx.build_kernel_rows(lo, hi)


def build_sharded(prob, rank: int = 0, world_size: int = 1, build_rows: Optional[Callable] = None,
                  **ctx_kw) -> Optional[np.ndarray]:
    """H (n_h x n_h) on rank 0, every rank building the rows of its k tile;
    build_rows(prob, lo, hi, **ctx_kw) -> rows (default: bse_build_kernel_rows on this GPU)."""
    from .capi import Marshalled
    n_h = Marshalled(prob, **ctx_kw).n_h
    lo, hi = ranges(prob.nk, world_size)[rank]
    fn = build_rows or _gpu_build_rows
    rows = np.asarray(fn(prob, lo, hi, **ctx_kw)) if hi > lo else np.zeros((0, n_h), np.complex128)
    parts = gather_to_root((lo, hi, rows), rank, world_size)
    if rank != 0:
        return None
    return assemble_rows([p for p in parts if p[1] > p[0]], prob.nk, n_h)


# --------------------------------------------------------------------------- eps(omega)
def _gpu_eps_part(E, f, F, omega, gamma):
    from . import gpu
    return gpu.eps_noalloc(E, f, F, omega, gamma)


def eps_sharded(E, f, F, omega, gamma, rank: int = 0, world_size: int = 1,
                eps_part: Optional[Callable] = None) -> Optional[Tuple[np.ndarray, np.ndarray]]:
    """(eps2, eps1) on rank 0 with the excitons split over the ranks:
    eps = 1 - F sum_l |f_l|^2 / (w - E_l + i gamma) is 1 + sum over parts of (eps_part - 1)."""
    lo, hi = ranges(len(E), world_size)[rank]
    fn = eps_part or _gpu_eps_part
    om = np.asarray(omega, dtype=np.float64)
    if hi > lo:
        e2, e1 = fn(np.asarray(E[lo:hi]), np.asarray(f[lo:hi]), F, om, gamma)
    else:
        e2, e1 = np.zeros(len(om)), np.ones(len(om))
    parts = gather_to_root((np.asarray(e2), np.asarray(e1)), rank, world_size)
    if rank != 0:
        return None
    eps2 = np.sum([p[0] for p in parts], axis=0)
    eps1 = 1.0 + np.sum([p[1] - 1.0 for p in parts], axis=0)
    return eps2, eps1
