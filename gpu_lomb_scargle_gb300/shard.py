"""Multi-GPU use of the engine: objects are independent, so a batch shards by object.

Each rank computes a contiguous range of objects on its own GPU with no collective in
the data path. The host then gathers the per-object results (best index and power) and
reduces the step time (max over ranks). This replaces the reference's one OpenMP thread
per GPU over contiguous object batches (source/main.cu:742-941), across processes. The
collectives here are only for results and timing, and work with any torch.distributed
backend (gloo on CPU in the tests).
"""
from __future__ import annotations

import numpy as np


def shard_range(offsets, rank: int, world: int):
    """Contiguous object range [o0, o1) of `rank`, balanced by observation count (work is
    proportional to observations x frequencies, and the frequency grid is shared)."""
    offs = np.asarray(offsets, dtype=np.int64)
    n_obj = offs.size - 1
    rows = int(offs[-1])
    cuts = [0]
    for r in range(1, world):
        o = int(np.searchsorted(offs, rows * r / world, side="left"))
        cuts.append(min(max(o, cuts[-1]), n_obj))
    cuts.append(n_obj)
    return cuts[rank], cuts[rank + 1]


def local_batch(offsets, rank: int, world: int):
    """(o0, o1, r0, r1, local_offsets) of a rank's shard: its objects, rows and offsets."""
    offs = np.asarray(offsets, dtype=np.int64)
    o0, o1 = shard_range(offs, rank, world)
    r0, r1 = int(offs[o0]), int(offs[o1])
    return o0, o1, r0, r1, (offs[o0:o1 + 1] - r0).astype(np.uint64)


def gather_best(best_idx, best_power, o0: int, n_obj: int):
    """Every rank's (index, power) per object, assembled in object order on all ranks."""
    import torch
    import torch.distributed as dist

    part = torch.tensor(np.concatenate([[o0, len(best_idx)], np.asarray(best_idx, np.int64)]),
                        dtype=torch.int64)
    pw = torch.tensor(np.asarray(best_power, np.float64), dtype=torch.float64)
    world = dist.get_world_size()
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([pw.numel()], dtype=torch.int64))
    mx = int(max(s.item() for s in sizes))
    pad_i = torch.zeros(mx + 2, dtype=torch.int64)
    pad_i[:part.numel()] = part
    pad_p = torch.zeros(max(mx, 1), dtype=torch.float64)
    pad_p[:pw.numel()] = pw
    all_i = [torch.zeros_like(pad_i) for _ in range(world)]
    all_p = [torch.zeros_like(pad_p) for _ in range(world)]
    dist.all_gather(all_i, pad_i)
    dist.all_gather(all_p, pad_p)
    idx = np.zeros(n_obj, np.int64)
    power = np.zeros(n_obj, np.float64)
    for ti, tp in zip(all_i, all_p):
        a, k = int(ti[0]), int(ti[1])
        idx[a:a + k] = ti[2:2 + k].numpy()
        power[a:a + k] = tp[:k].numpy()
    return idx, power


def max_over_ranks(value: float) -> float:
    """The largest value over all ranks (the step time of the slowest GPU)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
