"""Multi-GPU host logic: one process per GPU, no collective on the data path.

A single network is replicated (a sweep is tens of microseconds; exchanging cut-edge
messages every sweep would cost more than it saves).  A batch of independent networks is
sharded by network id: rank r gets a contiguous range of networks with balanced vertex
counts, solves it alone, and only the per-network log-norms are gathered at the end.
Timing takes the maximum over ranks; throughput is the sum of all ranks' work divided by
that time.  Works with the ``gloo`` (CPU tensors) and ``nccl`` (CUDA tensors) backends.
"""
from __future__ import annotations

import numpy as np


def shard_networks(sizes, rank: int, world: int):
    """Contiguous range [lo, hi) of networks for ``rank`` so that the summed ``sizes``
    (e.g. vertices or flops per network) are as even as possible across ranks."""
    sizes = np.asarray(sizes, dtype=np.float64)
    if world <= 1:
        return 0, len(sizes)
    csum = np.concatenate([[0.0], np.cumsum(sizes)])
    total = csum[-1]
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        b = int(np.searchsorted(csum, target, side="left"))
        b = min(b, len(sizes))
        if b > 0 and abs(csum[b - 1] - target) <= abs(csum[b] - target):
            b -= 1  # the split point nearest to the even share
        bounds.append(b)
    bounds.append(len(sizes))
    bounds = np.maximum.accumulate(bounds)
    return int(bounds[rank]), int(bounds[rank + 1])


def shard_batch(graphs, rank: int, world: int):
    """This rank's share of a batch of independent networks: (lo, hi, batched graph of
    graphs[lo:hi]), the split balanced by vertex count (shard_networks)."""
    from .graphs import batched
    lo, hi = shard_networks([g.nv for g in graphs], rank, world)
    return lo, hi, (batched(graphs[lo:hi]) if hi > lo else None)


def solve_shard(graphs, tensors, rank: int, world: int, *, maxiter: int, device: int = 0, dtype=None):
    """Solve this rank's networks on its GPU: ``tensors[k]`` is network k's packed site
    tensors.  Runs `maxiter` parallel sweeps from the normalised identity on the batched
    shard (one BPEngine, every network of the shard in each sweep launch) and returns
    ({network index: Bethe log-norm}, device ms of the sweeps, message updates done)."""
    from .engine import BPEngine
    lo, hi, g = shard_batch(graphs, rank, world)
    if g is None:
        return {}, 0.0, 0
    t = np.concatenate([np.asarray(tensors[k]) for k in range(lo, hi)])
    if dtype is not None:
        t = t.astype(dtype)
    with BPEngine(g, device=device) as e:
        e.set_tensors(t)
        e.init_messages()
        r = e.run(maxiter=maxiter)
        logz = e.bethe_free_energy(None)
    vals = logz if isinstance(logz, list) else [logz]
    return {lo + i: v for i, v in enumerate(vals)}, r.device_ms, maxiter * g.nslots


def _tensor(x, device):
    import torch
    return torch.tensor([float(x)], dtype=torch.float64, device=device)


def max_over_ranks(x: float, group=None, device="cpu") -> float:
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(x)
    t = _tensor(x, device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def sum_over_ranks(x: float, group=None, device="cpu") -> float:
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(x)
    t = _tensor(x, device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return float(t.item())


def gather_logz(local: dict, n_total: int, group=None, device="cpu"):
    """Per-network log-norms from every rank into one array (rank-local dict {net: value},
    real part for complex log-norms); networks no rank reports stay NaN."""
    import torch
    import torch.distributed as dist
    buf = torch.full((n_total,), float("nan"), dtype=torch.float64, device=device)
    for k, v in local.items():
        buf[k] = float(np.real(v))
    if dist.is_available() and dist.is_initialized():
        # NaN-aware merge: every entry is finite on exactly one rank
        mask = torch.isnan(buf)
        vals = torch.where(mask, torch.zeros_like(buf), buf)
        cnt = (~mask).to(torch.float64)
        dist.all_reduce(vals, group=group)
        dist.all_reduce(cnt, group=group)
        buf = torch.where(cnt > 0, vals / torch.clamp(cnt, min=1.0), torch.full_like(vals, float("nan")))
    return buf.cpu().numpy()
