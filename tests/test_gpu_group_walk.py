"""The density pass's group walk against its per-slot walk.

The default density kernel walks neighbours cell by cell (density_group_tile):
a warp loads the members of a cell's 27 buckets once and tests every home of
the cell against them with one ballot per 32 candidates.  Launch shape 5 runs
the per-slot walk (density_tile) that tests each slot's candidates in its own
lane.  Both produce the same neighbour lists, counts and pressures, so whole
runs give the same bytes.  The scenes cover the three ways a home is handled
by the group walk: its group's candidates held in registers, the warp's
shared candidate store filling up (the waiting homes are finished first),
and a cell too crowded for the registers (the per-slot walk).
The exact arithmetic (the reference's bits) runs the group walk too and is
checked against the reference in test_gpu_exact.py.
"""
import numpy as np
import pytest

from sphfluidsimulation_gb300 import scenes
from sphfluidsimulation_gb300.engine import SimulationEngineCUDA

pytestmark = pytest.mark.gpu

GROUP_SLOTS = 8          # kGroupSlots: 256 candidates per group
WARP_CAND = 1280         # kWarpCand


def _expand_bits(v):
    v = np.asarray(v, np.uint64) & np.uint64(0x3FF)
    v = (v * np.uint64(0x00010001)) & np.uint64(0xFF0000FF)
    v = (v * np.uint64(0x00000101)) & np.uint64(0x0F00F00F)
    v = (v * np.uint64(0x00000011)) & np.uint64(0xC30C30C3)
    v = (v * np.uint64(0x00000005)) & np.uint64(0x49249249)
    return v


def group_walk_paths(pos_sorted, starts, h):
    """Emulates the group walk's bookkeeping on the host over warps of 32
    sorted slots: (homes held in registers, homes finished early because the
    warp's candidate store filled, homes left to the per-slot walk)."""
    n = pos_sorted.shape[0]
    b = 2 * n
    cnt = np.diff(starts.astype(np.int64))
    cell = np.floor(pos_sorted.astype(np.float32) / np.float32(h)).astype(np.int64) & 0x3FF
    e = [[_expand_bits(cell[:, ax] + d) << np.uint64(ax) for d in (-1, 0, 1)] for ax in range(3)]
    total = np.zeros(n, np.int64)
    for a in range(3):
        for bb in range(3):
            for c in range(3):
                total += cnt[((e[0][a] + e[1][bb] + e[2][c]) % np.uint64(b)).astype(np.int64)]
    code = e[0][1] + e[1][1] + e[2][1]
    held = early = slow = 0
    for w0 in range(0, n, 32):
        cursor, waiting = 0, 0
        lanes = np.arange(w0, min(w0 + 32, n))
        _, first = np.unique(code[lanes], return_index=True)
        for leader in lanes[np.sort(first)]:          # groups in order of their lowest lane
            g = int((code[lanes] == code[leader]).sum())
            if total[leader] > GROUP_SLOTS * 32:
                slow += g
                continue
            if cursor + total[leader] > WARP_CAND:
                early += waiting
                waiting, cursor = 0, 0
            waiting += g
            cursor += total[leader]
        held += waiting
    return held, early, slow


def crowded_scene():
    """About 9.4 slots per cell (spacing h / 2.12): groups of up to 256
    candidates and cells past 256 candidates."""
    h = 0.02
    sp = h / 2.12
    return scenes.dam_break((40, 24, 40), sp, h, (0.6, 0.5, 0.6), 0, name="crowded_38k")


def layered_scene():
    """Cell layers y = 0..5 of a 32 x 32 cell slab (h = 0.02, cells from 8 on
    in x and z): one slot per cell in layers 2 and 3, 26 in the others, at
    seeded uniform places inside each cell.  A layer-2 or layer-3 cell is a
    group of one home with 9 x 26 + 18 = 252 candidates, and Morton order
    runs 16 such cells back to back, so warps hold far more candidates than
    their shared store (early finishes); the crowded cells (477 candidates)
    take the per-slot walk."""
    h = 0.02
    rng = np.random.default_rng(7)
    per_layer = [26, 26, 1, 1, 26, 26]
    pts = []
    for y, k in enumerate(per_layer):
        cx, cz = np.meshgrid(np.arange(8, 40), np.arange(8, 40), indexing="ij")
        cell = np.stack([cx.ravel(), np.full(cx.size, y + 2), cz.ravel()], 1).astype(np.float64)
        cell = np.repeat(cell, k, axis=0)
        pts.append((cell + rng.uniform(0.05, 0.95, cell.shape)) * h)
    dyn = np.concatenate(pts).astype(np.float32)
    walls = scenes.box_shell((1.0, 0.3, 1.0), 0.02)
    return scenes.Scene(name="layered", dyn_pos=dyn, static_pos=walls, params=scenes.water_params(0.01, h),
                        dt=1e-5, steps=0)


def run(sc, steps, density_shape, dt=None):
    e = SimulationEngineCUDA()
    e.initialize(sc)
    e.set_launch_shapes(density_shape, 0)
    e.update(sc.dt if dt is None else dt, steps)
    return e


@pytest.mark.parametrize("which,steps", [("config0", 50), ("crowded", 20), ("layered", 3), ("config1", 3),
                                         ("config1_stable", 20)])
def test_group_walk_gives_the_per_slot_walks_bytes(which, steps):
    if which == "config0":
        sc, dt = scenes.config0(), None
    elif which == "crowded":
        sc, dt = crowded_scene(), 2.5e-5
    elif which == "layered":
        sc, dt = layered_scene(), 1e-5
    elif which == "config1":
        sc, dt = scenes.config1(), None
    else:
        sc, dt = scenes.config1(), scenes.STABLE_DT["dam_break_1m"]
    group = run(sc, steps, 0, dt)
    slot = run(sc, steps, 5, dt)
    assert group.read_dynamic_buffer().tobytes() == slot.read_dynamic_buffer().tobytes()
    st = group.neighbour_stats()
    assert st["particles"] == sc.n
    if which in ("crowded", "layered"):
        starts, ids = group.read_buckets()
        pos = group.read_dynamic()["pos"][ids]
        held, early, slow = group_walk_paths(pos, starts, sc.params.h)
        assert held > 0 and slow > 0, (held, early, slow)
        assert early > 0 or which == "crowded", (held, early, slow)
        assert st["group_fallback"] == slow
