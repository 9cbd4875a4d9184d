"""sph_cell_sort_noalloc: the counting sort for callers that cannot allocate
device memory (code under a caller-owned pool or allocator, a frame loop
that must not allocate, a plugin whose host application owns all device
memory).  It takes the caller's device buffers and keeps its scratch in a
fixed array inside the library.

Checked through the C ABI against the allocating entry point sph_cell_sort
and against the oracle (the reference's hash and counting sort restated) on
the same positions: keys, bucket starts and slot order are integers and must
match exactly.  Cases: two calls in a row with different sizes (the shared
scratch left by one call must not leak into the next), the capacity edge
itself (262,144 particles, 524,288 buckets: 513 scan tiles, every one the
scratch holds), a bucket of more than 8,192 members (kept in arrival order:
membership exact, order a permutation), an empty input with null buffers, a
non-default stream, a call that leaves the device's free memory and the
torch allocator untouched, and a stream under CUDA graph capture (refused).
This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from oracle_lib import oracle_counting_sort, oracle_hash
from sphfluidsimulation_gb300 import _lib, scenes
from sphfluidsimulation_gb300.engine import cell_sort

pytestmark = pytest.mark.gpu

MAX_N = 262_144
MAX_BUCKETS = 524_288


class _Buffers:
    """Device buffers for one call, allocated by the caller (here torch)."""

    def __init__(self, pos: np.ndarray, buckets: int):
        import torch
        dev = torch.device("cuda", 0)
        p = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        self.n = p.shape[0]
        self.buckets = buckets
        self.pos = torch.from_numpy(p).to(dev) if self.n else None
        self.keys = torch.full((max(self.n, 1),), -1, dtype=torch.int32, device=dev)
        self.starts = torch.full((buckets + 1,), -1, dtype=torch.int32, device=dev)
        self.order = torch.full((max(self.n, 1),), -1, dtype=torch.int32, device=dev)

    def call(self, stream=None, null_buffers: bool = False) -> int:
        if stream is not None:
            import torch
            stream.wait_stream(torch.cuda.current_stream(0))   # the buffers' fills and copies
        ptr = lambda t: C.c_void_p(t.data_ptr()) if (t is not None and not null_buffers) else None  # noqa: E731
        return _lib.load().sph_cell_sort_noalloc(ptr(self.pos), self.n, self.h, int(self.buckets),
                                                 ptr(self.keys), C.c_void_p(self.starts.data_ptr()),
                                                 ptr(self.order),
                                                 C.c_void_p(stream.cuda_stream if stream is not None else 0))

    def results(self):
        u32 = lambda t: t.cpu().numpy().view(np.uint32)  # noqa: E731
        return u32(self.keys)[:self.n], u32(self.starts), u32(self.order)[:self.n]


def _noalloc(pos, h, buckets, stream=None):
    b = _Buffers(pos, buckets)
    b.h = float(h)
    _lib.check(b.call(stream), "sph_cell_sort_noalloc")
    if stream is not None:
        stream.synchronize()
    return b.results()


def _compare(pos, h, buckets, stream=None):
    """The no-allocation sort equals sph_cell_sort and the oracle, exactly."""
    keys, counts, starts, order = cell_sort(pos, h, buckets)
    k2, s2, o2 = _noalloc(pos, h, buckets, stream)
    assert np.array_equal(k2, keys)
    assert np.array_equal(s2, starts)
    assert np.array_equal(o2, order)
    assert np.array_equal(np.diff(s2.astype(np.int64)), counts)
    rk = oracle_hash(pos, h, buckets)
    rc, rs, rpm = oracle_counting_sort(rk, buckets)
    assert np.array_equal(k2, rk)
    assert np.array_equal(s2, rs)
    assert np.array_equal(o2, rpm)


def test_noalloc_matches_cell_sort_two_calls_in_a_row():
    sc = scenes.config0(steps=1)
    # first call: 16,384 particles, 32,768 buckets
    _compare(sc.dyn_pos, sc.params.h, 2 * sc.n)
    # second call: fewer particles and a non-power-of-two bucket count, so
    # counters and ranks left by the first call must not leak in
    rng = np.random.default_rng(7)
    pos = rng.uniform(-0.5, 0.5, size=(5000, 3)).astype(np.float32)
    _compare(pos, 0.05, 12345)


def test_noalloc_at_its_capacity():
    """n and buckets at the limits: the scan runs 513 tiles, the last one
    holding the single entry starts[524288]."""
    rng = np.random.default_rng(11)
    pos = rng.uniform(0.0, 0.64, size=(MAX_N, 3)).astype(np.float32)
    _compare(pos, 0.01, MAX_BUCKETS)
    # and a smaller call right after it
    _compare(pos[:1000], 0.02, 777)


def test_noalloc_bucket_beyond_the_stable_rank_limit():
    """10,000 particles in one cell: that bucket keeps arrival order, so only
    its membership is exact; every other bucket keeps the reference's order."""
    rng = np.random.default_rng(5)
    crowd = rng.uniform(0.3005, 0.3085, size=(10_000, 3)).astype(np.float32)   # cell (30, 30, 30)
    rest = rng.uniform(0.0, 1.0, size=(20_000, 3)).astype(np.float32)
    pos = np.concatenate([rest[:7000], crowd, rest[7000:]])
    h, buckets = 0.01, 2 * pos.shape[0]
    k2, s2, o2 = _noalloc(pos, h, buckets)
    rk = oracle_hash(pos, h, buckets)
    _, rs, rpm = oracle_counting_sort(rk, buckets)
    assert np.array_equal(k2, rk)
    assert np.array_equal(s2, rs)
    assert np.array_equal(np.sort(o2), np.arange(pos.shape[0], dtype=np.uint32))
    sizes = np.diff(rs.astype(np.int64))
    big = np.nonzero(sizes > 8192)[0]
    assert len(big) == 1
    for b in range(buckets):
        lo, hi = int(rs[b]), int(rs[b + 1])
        if hi - lo > 8192:
            assert np.array_equal(np.sort(o2[lo:hi]), np.sort(rpm[lo:hi]))
        elif hi > lo:
            assert np.array_equal(o2[lo:hi], rpm[lo:hi])


def test_noalloc_empty_input_with_null_buffers():
    b = _Buffers(np.zeros((0, 3), np.float32), 64)
    b.h = 0.01
    _lib.check(b.call(null_buffers=True), "sph_cell_sort_noalloc")
    _, starts, _ = b.results()
    assert np.array_equal(starts, np.zeros(65, np.uint32))


def test_noalloc_on_a_non_default_stream():
    import torch
    s = torch.cuda.Stream(device=0)
    rng = np.random.default_rng(3)
    _compare(rng.uniform(0.0, 0.5, size=(40_000, 3)).astype(np.float32), 0.02, 50_000, stream=s)


def test_noalloc_call_allocates_nothing():
    import torch
    rng = np.random.default_rng(9)
    b = _Buffers(rng.uniform(0.0, 0.5, size=(100_000, 3)).astype(np.float32), 200_000)
    b.h = 0.01
    _lib.check(b.call(), "sph_cell_sort_noalloc")            # warm: modules loaded
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    alloc0 = torch.cuda.memory_allocated(0)
    reserved0 = torch.cuda.memory_reserved(0)
    for _ in range(3):
        _lib.check(b.call(), "sph_cell_sort_noalloc")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0
    assert torch.cuda.memory_allocated(0) == alloc0
    assert torch.cuda.memory_reserved(0) == reserved0


def test_noalloc_refuses_a_capturing_stream():
    """The call waits for its device status word, so on a stream under CUDA
    graph capture it queues nothing and returns SPH_ERR_INVALID_ARGUMENT; the
    capture stays valid and replays, and the next plain call works."""
    import torch
    rng = np.random.default_rng(5)
    pos = rng.uniform(0.0, 0.5, size=(1_000, 3)).astype(np.float32)
    b = _Buffers(pos, 2_000)
    b.h = 0.01
    s = torch.cuda.Stream(device=0)
    x = torch.zeros(4, device="cuda:0")
    torch.cuda.synchronize()
    lib = _lib.load()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st = lib.sph_cell_sort_noalloc(C.c_void_p(b.pos.data_ptr()), b.n, b.h, b.buckets,
                                       C.c_void_p(b.keys.data_ptr()), C.c_void_p(b.starts.data_ptr()),
                                       C.c_void_p(b.order.data_ptr()), C.c_void_p(s.cuda_stream))
        x.add_(1.0)
    assert st == 1   # SPH_ERR_INVALID_ARGUMENT
    assert b"captured" in lib.sph_last_error()
    g.replay()
    torch.cuda.synchronize()
    assert x.cpu().tolist() == [1.0] * 4
    assert np.array_equal(b.results()[1], np.full(2_001, 0xFFFFFFFF, np.uint32))   # nothing queued
    _compare(pos, 0.01, 2_000)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _lib.load()
    st = lib.sph_cell_sort_noalloc(None, MAX_N + 1, 0.01, 16, None, None, None, None)
    assert st == 6   # SPH_ERR_CAPACITY
    assert b"262144" in lib.sph_last_error()
    st = lib.sph_cell_sort_noalloc(None, 16, 0.01, MAX_BUCKETS + 1, None, None, None, None)
    assert st == 6
