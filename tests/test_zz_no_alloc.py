"""sph_cell_sort_noalloc: the counting sort for callers that cannot allocate
device memory (code under a caller-owned pool or allocator, a frame loop
that must not allocate, a plugin whose host application owns all device
memory).  It takes the caller's device buffers and keeps its scratch in a
fixed array inside the library.

Checked through the C ABI against the allocating entry point sph_cell_sort
on the same positions: keys, bucket starts and slot order are integers and
must match exactly.  Two calls in a row with different sizes make sure the
shared scratch left by one call does not leak into the next.  This file is
named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from sphfluidsimulation_gb300 import _lib, scenes
from sphfluidsimulation_gb300.engine import cell_sort

pytestmark = pytest.mark.gpu


def _noalloc(pos: np.ndarray, h: float, buckets: int):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    p = torch.from_numpy(np.ascontiguousarray(pos, np.float32).reshape(-1, 3)).to(dev)
    n = p.shape[0]
    keys = torch.full((max(n, 1),), -1, dtype=torch.int32, device=dev)
    starts = torch.full((buckets + 1,), -1, dtype=torch.int32, device=dev)
    order = torch.full((max(n, 1),), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    lib = _lib.load()
    st = lib.sph_cell_sort_noalloc(C.c_void_p(p.data_ptr()), n, float(h), int(buckets),
                                   C.c_void_p(keys.data_ptr()), C.c_void_p(starts.data_ptr()),
                                   C.c_void_p(order.data_ptr()), C.c_void_p(stream.cuda_stream))
    _lib.check(st, "sph_cell_sort_noalloc")
    u32 = lambda t: t.cpu().numpy().view(np.uint32)  # noqa: E731
    return u32(keys)[:n], u32(starts), u32(order)[:n]


def _compare(pos, h, buckets):
    keys, counts, starts, order = cell_sort(pos, h, buckets)
    k2, s2, o2 = _noalloc(pos, h, buckets)
    assert np.array_equal(k2, keys)
    assert np.array_equal(s2, starts)
    assert np.array_equal(o2, order)
    assert np.array_equal(np.diff(s2.astype(np.int64)), counts)


def test_noalloc_matches_cell_sort_two_calls_in_a_row():
    sc = scenes.config0(steps=1)
    # first call: 16,384 particles, 32,768 buckets
    _compare(sc.dyn_pos, sc.params.h, 2 * sc.n)
    # second call: fewer particles and a non-power-of-two bucket count, so
    # counters and ranks left by the first call must not leak in
    rng = np.random.default_rng(7)
    pos = rng.uniform(-0.5, 0.5, size=(5000, 3)).astype(np.float32)
    _compare(pos, 0.05, 12345)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _lib.load()
    st = lib.sph_cell_sort_noalloc(None, 262145, 0.01, 16, None, None, None, None)
    assert st == 6   # SPH_ERR_CAPACITY
    assert b"262144" in lib.sph_last_error()
    st = lib.sph_cell_sort_noalloc(None, 16, 0.01, 524289, None, None, None, None)
    assert st == 6
