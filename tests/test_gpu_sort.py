"""GPU counting sort (hash + count + scan + scatter) against the oracle:
keys, per-bucket counts, bucket starts and the slot order itself bit-exact.
Inside a bucket the members run by decreasing input index, the order the
reference's decrementing fill produces (SF:346-356)."""
import numpy as np
import pytest

from oracle_lib import Oracle, oracle_counting_sort, oracle_hash
from sphfluidsimulation_gb300 import scenes
from sphfluidsimulation_gb300.engine import cell_sort

pytestmark = pytest.mark.gpu


def check_sort(pos, h, buckets):
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    keys, counts, starts, order = cell_sort(pos, h, buckets)
    ref_keys = oracle_hash(pos, h, buckets)
    assert np.array_equal(keys, ref_keys), "keys"
    ref_counts, ref_starts, ref_pm = oracle_counting_sort(ref_keys, buckets)
    assert np.array_equal(counts, ref_counts), "counts"
    assert np.array_equal(starts, ref_starts), "bucket starts"
    # the reference's particleMap, slot for slot
    assert np.array_equal(order, ref_pm), "slot order"
    return keys, counts, starts, order


def test_sort_config0_initial():
    sc = scenes.config0(steps=1)
    check_sort(sc.dyn_pos, sc.params.h, 2 * sc.n)


def test_sort_oracle_positions_after_steps():
    """Stage-wise: the oracle's own positions after 40 steps (some particles
    have left the box, negative cells included)."""
    sc = scenes.dam_break((16, 12, 16), 0.02, 0.04, (0.5, 0.4, 0.5), 0, mass=0.008)
    o = Oracle(0)
    o.init(sc)
    o.update(sc.dt, 40)
    st = o.read()
    check_sort(st[:, :3].astype(np.float32), sc.params.h, 2 * sc.n)


@pytest.mark.parametrize("buckets", [1, 7, 4096, 12345, 1 << 20, 2_000_003])
def test_sort_random_positions_any_bucket_count(buckets):
    rng = np.random.default_rng(buckets)
    pos = rng.uniform(-3, 3, size=(5000, 3)).astype(np.float32)
    check_sort(pos, 0.1, buckets)


def test_sort_cell_boundaries_and_coincident():
    h = np.float32(0.04)
    k = np.arange(-20, 20, dtype=np.float32)
    on = k * h
    below = np.nextafter(on, np.float32(-np.inf))
    above = np.nextafter(on, np.float32(np.inf))
    xs = np.concatenate([on, below, above])
    pos = np.stack(np.meshgrid(xs, xs[::7], xs[::11], indexing="ij"), -1).reshape(-1, 3)
    pos = np.concatenate([pos, np.repeat(pos[:5], 50, axis=0)])   # coincident clusters
    check_sort(pos, float(h), 2 * pos.shape[0])


def test_sort_oversized_bucket_membership():
    """A bucket above the stable-rank limit (8192 members) keeps arrival
    order: membership and tables stay exact, the order inside it is not
    promised."""
    rng = np.random.default_rng(5)
    pos = rng.uniform(0.1, 0.2, size=(10000, 3)).astype(np.float32)
    keys, counts, starts, order = cell_sort(pos, 1.0, 3)
    ref_keys = oracle_hash(pos, 1.0, 3)
    assert np.array_equal(keys, ref_keys)
    ref_counts, ref_starts, _ = oracle_counting_sort(ref_keys, 3)
    assert np.array_equal(counts, ref_counts) and np.array_equal(starts, ref_starts)
    assert np.array_equal(np.sort(order), np.arange(10000, dtype=np.uint32))


def test_sort_single_and_tiny():
    check_sort(np.array([[0.5, 0.5, 0.5]], np.float32), 1.0, 2)
    check_sort(np.array([[0.5, 0.5, 0.5], [0.5, 0.5, 0.5]], np.float32), 1.0, 4)


def test_sort_ragged_tail_sizes():
    rng = np.random.default_rng(1)
    for n in (127, 128, 129, 255, 2049, 4097):
        pos = rng.uniform(0, 1, size=(n, 3)).astype(np.float32)
        check_sort(pos, 0.05, 2 * n)


def test_sort_one_million_properties():
    """Config-1 size: keys against the oracle, counts = bincount, starts
    monotone with starts[B] = N, order a permutation sorted by key."""
    sc = scenes.config1(steps=1)
    pos = sc.dyn_pos
    B = 2 * sc.n
    keys, counts, starts, order = cell_sort(pos, sc.params.h, B)
    assert np.array_equal(keys, oracle_hash(pos, sc.params.h, B))
    assert np.array_equal(counts, np.bincount(keys, minlength=B))
    assert starts[0] == 0 and starts[B] == sc.n
    assert np.array_equal(np.sort(order), np.arange(sc.n, dtype=np.uint32))
    k_sorted = keys[order]
    assert (np.diff(k_sorted.astype(np.int64)) >= 0).all()
    # inside each bucket the input indices descend, as the reference's fill leaves them
    same = np.diff(k_sorted.astype(np.int64)) == 0
    assert (np.diff(order.astype(np.int64))[same] < 0).all()


def test_sort_far_cells_and_non_finite():
    """Cells far beyond the 10-bit Morton range: the reference's float->uint
    cast wraps modulo 2^32 (through int64 on x86-64) up to 2^63 cells, on both
    sides, and NaN maps to cell 0.  Keys, counts, starts and slot order equal
    the oracle's."""
    rng = np.random.default_rng(11)
    h = 0.04
    mags = np.float32(10.0) ** rng.uniform(0, 17, size=(4000, 3)).astype(np.float32)
    signs = np.where(rng.random((4000, 3)) < 0.5, -1.0, 1.0).astype(np.float32)
    pos = (mags * signs * np.float32(h)).astype(np.float32)
    pos[::97, 1] = np.nan
    pos[::131, 0] = np.inf
    check_sort(pos, h, 8000)
