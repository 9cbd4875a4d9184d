"""Multi-GPU runs of independent scenes: replicas, no collective on the data
path.

Scenes and served jobs never interact, so N GPUs share them out: each rank
simulates its own subset with the single-GPU engine, batch or server, and
only the timing and the per-job latencies are combined at the end.  The
split is by HBM footprint (the bytes a scene keeps resident), greedy
largest-first onto the least loaded rank, and every rank computes the same
split from the same list.

The reductions work with any torch.distributed backend: NCCL ranks reduce
device tensors, gloo ranks (the CPU tests) host tensors.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np


def partition_by_footprint(footprints: Sequence[int], world: int) -> List[List[int]]:
    """Indices of the items each rank takes: largest first, each onto the
    rank with the fewest bytes so far (ties: the lower rank).  Deterministic."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(footprints)), key=lambda k: (-int(footprints[k]), k))
    load = [0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for k in order:
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(k)
        load[r] += int(footprints[k])
    for p in parts:
        p.sort()
    return parts


def _device(pg):
    import torch
    if pg is None:
        return torch.device("cpu")
    backend = pg.get_backend() if hasattr(pg, "get_backend") else "gloo"
    if backend == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def reduce_scalar(pg, value: float, op: str = "max") -> float:
    """MAX or SUM of one float over all ranks (the value itself without a
    process group)."""
    if pg is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=_device(pg))
    pg.all_reduce(t, op=pg.ReduceOp.MAX if op == "max" else pg.ReduceOp.SUM)
    return float(t.item())


def gather_values(pg, values: Sequence[float]) -> np.ndarray:
    """Every rank's list of floats, concatenated in rank order, on every rank."""
    vals = np.asarray(values, np.float64)
    if pg is None:
        return vals
    import torch
    dev = _device(pg)
    world = pg.get_world_size()
    n = torch.tensor([vals.size], dtype=torch.int64, device=dev)
    sizes = [torch.zeros(1, dtype=torch.int64, device=dev) for _ in range(world)]
    pg.all_gather(sizes, n)
    m = int(max(int(s.item()) for s in sizes))
    buf = torch.zeros(max(m, 1), dtype=torch.float64, device=dev)
    buf[:vals.size] = torch.from_numpy(vals).to(dev)
    out = [torch.zeros(max(m, 1), dtype=torch.float64, device=dev) for _ in range(world)]
    pg.all_gather(out, buf)
    return np.concatenate([o[:int(s.item())].cpu().numpy() for o, s in zip(out, sizes)])


def aggregate_rate(pg, units: float, seconds: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time."""
    return reduce_scalar(pg, units, "sum") / max(reduce_scalar(pg, seconds, "max"), 1e-12)


def rank_share(items: Sequence, footprints: Sequence[int], world: int, rank: int) -> List:
    """This rank's items under partition_by_footprint."""
    return [items[k] for k in partition_by_footprint(footprints, world)[rank]]


def footprint_bytes(n: int, s: int, job_bytes: Optional[callable] = None) -> int:
    """Resident bytes of a scene of n dynamic and s static particles (the
    server's estimate when given, else the dominant arrays: state, sort and
    neighbour lists, about 710 B per particle)."""
    if job_bytes is not None:
        return int(job_bytes(n, s))
    return 712 * int(n) + 144 * int(s) + 4096
