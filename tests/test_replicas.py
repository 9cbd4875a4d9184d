"""The multi-GPU (replicas) host logic on CPU: the footprint split of scenes
and jobs across ranks, and the reductions that combine timings and latency
lists, run as two gloo ranks (no GPU)."""
import os
import socket

import numpy as np
import pytest

from sphfluidsimulation_gb300 import replicas


def test_partition_covers_every_item_once_and_balances_bytes():
    rng = np.random.default_rng(0)
    fp = (np.exp(rng.uniform(np.log(4096), np.log(131072), 96)) * 704).astype(np.int64)
    for world in (1, 2, 3, 4, 8):
        parts = replicas.partition_by_footprint(fp, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(96))
        loads = [int(fp[p].sum()) for p in parts]
        # largest-first greedy: no rank exceeds the lightest by more than the largest item
        assert max(loads) - min(loads) <= int(fp.max())
        assert parts == replicas.partition_by_footprint(list(fp), world)   # deterministic


def test_partition_edge_cases():
    assert replicas.partition_by_footprint([], 3) == [[], [], []]
    assert replicas.partition_by_footprint([5], 2) == [[0], []]
    assert replicas.partition_by_footprint([3, 3, 3, 3], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        replicas.partition_by_footprint([1], 0)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        items = list(range(10))
        fp = [10, 1, 7, 3, 3, 8, 2, 9, 4, 5]
        mine = replicas.rank_share(items, fp, world, rank)
        seconds = 1.0 + rank                     # rank 1 is the slow one
        units = 100.0 * (rank + 1)
        res = {
            "mine": mine,
            "max": replicas.reduce_scalar(dist, seconds, "max"),
            "sum": replicas.reduce_scalar(dist, units, "sum"),
            "rate": replicas.aggregate_rate(dist, units, seconds),
            "gathered": replicas.gather_values(dist, [rank + 0.5] * (rank + 2)).tolist(),
        }
        np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.array([res], dtype=object), allow_pickle=True)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_split_and_reduce(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    res = [np.load(tmp_path / f"rank{r}.npy", allow_pickle=True)[0] for r in range(2)]
    assert sorted(res[0]["mine"] + res[1]["mine"]) == list(range(10))
    assert not set(res[0]["mine"]) & set(res[1]["mine"])
    for r in res:
        assert r["max"] == 2.0
        assert r["sum"] == 300.0
        assert r["rate"] == pytest.approx(150.0)          # 300 units over the slowest rank's 2 s
        assert r["gathered"] == [0.5, 0.5, 1.5, 1.5, 1.5]  # rank order, ragged lengths
