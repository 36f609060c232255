"""Multi-rank host logic: chunk sharding and the one exchange of an NR iteration.

Chunks are independent, so ranks share nothing during an iteration.  The
reference balances spectra over MPI ranks by a cost model
(``OneDQuadraticPowerEstimate::_loadBalancing``, core/quadratic_estimate.cpp:214-260:
most expensive first, each to the least-loaded rank) and sums the
Fisher matrix and the d, b, t vectors with one allreduce per iteration
(core/quadratic_estimate.cpp:469-475).  This module does the same with
``torch.distributed`` (NCCL between GPUs, gloo on CPU): every rank then holds
the global sums and runs the replicated Fisher solve.
"""
from __future__ import annotations

import heapq

import numpy as np


def chunk_cost(n_pix: int, n_stored: int) -> float:
    """Relative cost of one chunk: the C^-1 Q_s products dominate, 2 (ns + 1) n^3,
    plus the n^3 factorisation."""
    n = float(n_pix)
    return (2.0 * (n_stored + 1) + 1.0) * n ** 3


def plan_costs(bins, tables, lam, delta, ivar, offsets, r_fwhm, max_forest_length, max_mean_pixel_size=150.0,
               oversampling=0, resomat=None):
    """chunk_cost of every chunk of an add_chunks (or, with resomat,
    add_chunks_reso) call before any engine exists, from lqg_chunk_plan (the
    pre-pass lyspeq makes for its load balancing,
    OneQSOEstimate::getComputeTimeEst); 0 for a chunk the engine would reject."""
    from . import lqg
    _, info = lqg.chunk_plan(bins, tables, lam, delta, ivar, offsets, r_fwhm, max_forest_length,
                             max_mean_pixel_size, oversampling=oversampling, resomat=resomat)
    return [0.0 if i is None else chunk_cost(i["n"], i["nq"] // bins.nk * i["kbin_upp"]) for i in info]


def shard_lpt(costs, world: int) -> list[list[int]]:
    """Longest-processing-time-first assignment of items to ``world`` ranks.

    Returns, per rank, the item indices in ascending order.  Deterministic:
    ties go to the lower rank, items of equal cost in index order.
    """
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    out: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in out]


def allreduce_sums(fisher: np.ndarray, d: np.ndarray, b: np.ndarray, t: np.ndarray, device=None):
    """Sum the per-rank Fisher matrix (nkz x nkz) and d, b, t (nkz each) over the
    default process group; returns the global (fisher, d, b, t) as float64."""
    import torch
    import torch.distributed as dist

    nkz = d.shape[0]
    flat = np.concatenate([np.asarray(fisher, np.float64).ravel(), d, b, t]).astype(np.float64)
    buf = torch.from_numpy(flat)
    if device is not None:
        buf = buf.to(device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(buf, op=dist.ReduceOp.SUM)
    v = buf.cpu().numpy()
    n2 = nkz * nkz
    return v[:n2].reshape(nkz, nkz), v[n2:n2 + nkz], v[n2 + nkz:n2 + 2 * nkz], v[n2 + 2 * nkz:]
