"""The density pass's two walks, emulated on the host: same neighbour lists.

The per-slot walk (density_tile) visits the 27 neighbour buckets of a
particle's cell in the reference's order and skips the cells whose box lies
beyond h when the 27 bucket ids are distinct.  The group walk
(density_group_tile) tests every member of the 27 buckets, skipping none, and
keeps the hits in candidate order.  The kernels' exactness rests on two
facts this test checks in float32 (the reference's r^2 rounding; the cull
test with its relative margin of 1e-4 on h^2):
- a cell the per-slot walk skips holds no particle within h;
- where buckets repeat (Morton spans past the bucket count, as next to the
  10-bit wrap at cell 0) both walks visit the repeated bucket twice and skip
  the particle itself at each visit.
So both walks give every particle the same neighbour list, in the same order.
"""
import numpy as np

from sphfluidsimulation_gb300 import scenes

F = np.float32


def expand_bits(v):
    v = np.asarray(v, np.uint64) & np.uint64(0x3FF)
    v = (v * np.uint64(0x00010001)) & np.uint64(0xFF0000FF)
    v = (v * np.uint64(0x00000101)) & np.uint64(0x0F00F00F)
    v = (v * np.uint64(0x00000011)) & np.uint64(0xC30C30C3)
    v = (v * np.uint64(0x00000005)) & np.uint64(0x49249249)
    return v


def cells(p, h):
    """floor(x / h) as the x86-64 int64 conversion, low 32 bits (finite here)."""
    return np.floor((p / F(h)).astype(F)).astype(np.int64)


def sorted_state(pos, h):
    """Slots sorted by bucket (Morton code of the 10-bit cell, mod 2n), the
    bucket table, and the per-slot Morton neighbourhood codes."""
    n = pos.shape[0]
    b = 2 * n
    c = cells(pos, h)
    code = sum(expand_bits(c[:, ax]) << np.uint64(ax) for ax in range(3))
    bk = (code % np.uint64(b)).astype(np.int64)
    order = np.argsort(bk, kind="stable")
    ps = pos[order]
    starts = np.concatenate([[0], np.cumsum(np.bincount(bk, minlength=b))]).astype(np.int64)
    cs = cells(ps, h)
    e = [[expand_bits(cs[:, ax] + d) << np.uint64(ax) for d in (-1, 0, 1)] for ax in range(3)]
    return ps, starts, e, cs


def r2_ref(q, p):
    """The reference's squared distance: (dx dx + dy dy) + dz dz, each step rounded."""
    d = (q - p).astype(F)
    return ((d[..., 0] * d[..., 0]).astype(F) + (d[..., 1] * d[..., 1]).astype(F)).astype(F) + \
        (d[..., 2] * d[..., 2]).astype(F)


def neighbour_lists(pos, h):
    ps, starts, e, cs = sorted_state(pos, h)
    n = ps.shape[0]
    b = np.uint64(2 * n)
    hf = F(h)
    h2 = F(hf * hf)
    cull2 = F(h2 * F(1.0001))
    # cell_box: squared distances to the neighbour cells' faces along each axis
    cf = np.floor((ps / hf).astype(F)).astype(F)
    frac = (ps - (cf * hf).astype(F)).astype(F)
    lo = (np.maximum(frac, F(0)) ** 2).astype(F)
    hi = (np.maximum((hf - frac).astype(F), F(0)) ** 2).astype(F)
    box_ok = (np.abs(cf) < F(4194304)).all(1)
    span = sum(np.maximum(np.maximum(e[ax][0], e[ax][1]), e[ax][2]) -
               np.minimum(np.minimum(e[ax][0], e[ax][1]), e[ax][2]) for ax in range(3))
    cull = box_ok & (span < b)
    slot_lists, group_lists, culled_cells = [], [], 0
    for i in range(n):
        per_slot, group = [], []
        for a in range(3):
            for bb in range(3):
                for c in range(3):
                    bd2 = ((np.array([lo[i, 0], F(0), hi[i, 0]])[a] + np.array([lo[i, 1], F(0), hi[i, 1]])[bb]).astype(F)
                           + np.array([lo[i, 2], F(0), hi[i, 2]])[c]).astype(F)
                    code = e[0][a][i] + e[1][bb][i] + e[2][c][i]
                    k = int(code % b)
                    members = np.arange(starts[k], starts[k + 1])
                    if members.size == 0:
                        continue
                    hit = r2_ref(ps[members], ps[i]) <= h2
                    hit &= members != i
                    got = members[hit].tolist()
                    group += got                                  # every bucket, in order
                    if cull[i] and bd2 > cull2:
                        culled_cells += 1
                        assert not got, (i, a, bb, c)             # a skipped cell holds no neighbour
                        continue
                    per_slot += got
        slot_lists.append(per_slot)
        group_lists.append(group)
    return slot_lists, group_lists, culled_cells, int((~cull).sum())


def test_both_walks_list_the_same_neighbours():
    """A jittered block in the corner at the origin (cell 0: wrapped, repeating
    neighbourhoods), a block far from the origin (distinct buckets, culling),
    a scattered cloud and a few coincident pairs."""
    h = 0.04
    rng = np.random.default_rng(3)
    corner = scenes.filled_box((8, 6, 8), h / 2, (0.0, 0.0, 0.0), 0.1, scenes.SplitMix64(1))
    far = scenes.filled_box((7, 5, 7), h / 2, (1.3, 0.7, 0.9), 0.1, scenes.SplitMix64(2))
    cloud = rng.uniform(0.3, 0.9, (200, 3)).astype(F)
    twins = np.repeat(rng.uniform(1.0, 1.2, (5, 3)).astype(F), 2, axis=0)
    pos = np.concatenate([corner, far, cloud, twins]).astype(F)
    slot_lists, group_lists, culled, repeating = neighbour_lists(pos, h)
    assert culled > 500 and repeating > 50           # both situations occur
    assert sum(len(x) for x in slot_lists) > 5000
    assert slot_lists == group_lists
