"""Host-side checks of bench.py's bookkeeping (no GPU): the algorithmic
bytes behind roofline.achieved, the committed ncu figures it reads, and the
neighbour-count rates of the `pairs` entry."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_algorithmic_bytes(bench):
    n, s = 1_048_576, 256_002
    assert bench.alg_bytes("density", n, s) == 28 * n + 20 * s == 34_480_168
    assert bench.alg_bytes("force", n, s) == 68 * n + 20 * s
    assert bench.alg_bytes("scan", n, s) == 16 * n
    total = sum(bench.alg_bytes(k, n, s) for k in ("density", "force", "scan", "scatter")) + 24 * n + 8 * n
    assert total == 160 * n + 40 * s


def test_committed_ncu_figures_are_read(bench):
    """profiles/ncu_traffic.txt: DRAM bytes (column 2) and warp instructions
    (column 3) per launch of both neighbour passes on the 1M dam break."""
    for stage in ("density", "force"):
        dram = bench.profiled_traffic(stage, "dam_break_1m")
        inst = bench.profiled_traffic(stage, "dam_break_1m", 3)
        assert dram is not None and 1e7 < dram < 1e9
        assert inst is not None and 1e7 < inst < 1e9
    # more DRAM bytes than the algorithmic ones: the neighbour lists
    assert bench.profiled_traffic("density", "dam_break_1m") > bench.alg_bytes("density", 1_048_576, 256_002)
    assert bench.profiled_traffic("density", "dam_break_16k") is None


def test_pair_rates(bench):
    stage_ms = [0.3, 0.15, 0.015, 0.013, 0.02]
    sample = {"particles": 1000, "candidates": 150_000, "warp_slots": 220_000, "neighbours": 29_000,
              "static_neighbours": 500, "group_candidates": 200_000, "group_lane_slots": 210_000,
              "group_fallback": 10}
    r = bench.pair_rates([sample, sample], stage_ms, 6)
    assert r["group_candidates_per_particle"] == 200.0
    assert r["group_lane_slots_per_candidate"] == pytest.approx(1.05)
    assert r["group_fallback_fraction"] == pytest.approx(0.01)
    assert r["slot_walk_warp_slots_per_particle"] == 220.0
    assert r["density_candidate_tests_per_s"] == pytest.approx(200_000 / 0.3e-3)
    assert r["force_pair_evals_per_s"] == pytest.approx(29_500 / 0.15e-3)
    assert r["steps_sampled"].startswith("6..7")
    assert bench.pair_rates([], stage_ms, 6) is None
