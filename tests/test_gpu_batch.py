"""Batched engine: many uneven scenes per launch give, scene by scene, the
same bits as the plain engine running that scene alone (the step is
deterministic and scenes never interact), in both batch modes."""
import numpy as np
import pytest

from sphfluidsimulation_gb300 import scenes
from sphfluidsimulation_gb300.engine import Batch, SimulationEngineCUDA

pytestmark = pytest.mark.gpu


def uneven_scenes():
    out = []
    for k, (lat, s, h) in enumerate([((5, 4, 5), 0.02, 0.04), ((17, 9, 13), 0.02, 0.04), ((8, 8, 8), 0.01, 0.02),
                                     ((30, 10, 21), 0.02, 0.04), ((3, 2, 1), 0.05, 0.1), ((24, 16, 24), 0.01, 0.02)]):
        lx, ly, lz = lat[0] * s, lat[1] * s, lat[2] * s
        sc = scenes.dam_break(lat, s, h, (2 * lx + 2 * s, 1.5 * ly + 2 * s, 2 * lz + 2 * s), 0, seed=k + 1)
        sc.dyn_pos = (sc.dyn_pos + np.float32(s)).astype(np.float32)
        out.append(sc)
    return out


def alone(sc, steps):
    e = SimulationEngineCUDA()
    e.initialize(sc)
    e.update(sc.dt, steps)
    return e.read_dynamic()


@pytest.mark.parametrize("mode", [0, 1], ids=["persistent", "staged"])
def test_batch_equals_alone_bitwise(mode):
    scs = uneven_scenes()
    b = Batch()
    ids = [b.add_scene(sc) for sc in scs]
    b.finalize()
    b.set_mode(mode)
    b.step(12)
    for sid, sc in zip(ids, scs):
        got = b.read_scene(sid)
        ref = alone(sc, 12)
        assert got.tobytes() == ref.tobytes(), sc.name


def test_batch_modes_agree_over_many_steps():
    scs = uneven_scenes()[:3]
    res = []
    for mode in (0, 1):
        b = Batch()
        for sc in scs:
            b.add_scene(sc)
        b.set_mode(mode)
        b.step(40)
        res.append([b.read_scene(i).tobytes() for i in range(len(scs))])
    assert res[0] == res[1]


def test_batch_info_and_empty_scene():
    scs = uneven_scenes()[:2]
    empty = scenes.Scene(name="e", dyn_pos=np.zeros((0, 3), np.float32), static_pos=np.zeros((0, 3), np.float32),
                         params=scs[0].params, dt=1e-4, steps=0)
    b = Batch()
    b.add_scene(scs[0])
    eid = b.add_scene(empty)
    b.add_scene(scs[1])
    b.step(3)
    tot, grid, thr = b.info()
    assert tot == scs[0].n + scs[1].n
    assert grid >= 1 and thr == 128
    assert b.read_scene(eid).shape == (0,)


def test_autotune_keeps_state_and_results():
    scs = uneven_scenes()
    b = Batch()
    ids = [b.add_scene(sc) for sc in scs]
    b.finalize()
    mode, grid, ms = b.autotune(2)
    assert mode in (0, 1) and ms > 0
    assert (grid > 0) == (mode == 0)
    b.step(12)
    for sid, sc in zip(ids, scs):
        assert b.read_scene(sid).tobytes() == alone(sc, 12).tobytes(), sc.name


def test_batch_exact_arithmetic_equals_the_oracle():
    """With the reference's arithmetic every scene of a batch reproduces the
    reference CPU engine's bytes (the oracle, pinned to it), in both modes."""
    import sys, os
    sys.path.insert(0, os.path.dirname(__file__))
    from oracle_lib import Oracle
    scs = uneven_scenes()[:4]
    for mode in (0, 1):
        b = Batch()
        ids = [b.add_scene(sc) for sc in scs]
        b.finalize()
        b.set_mode(mode)
        b.set_exact(True)
        b.step(6)
        b.step(5)
        for sid, sc in zip(ids, scs):
            o = Oracle(0)
            o.init(sc)
            o.update(sc.dt, 11)
            _, _, io = o.maps()
            ref = np.empty(sc.n, o.read_raw().dtype)
            ref[io] = o.read_raw()
            assert b.read_scene(sid).tobytes() == ref.tobytes(), (mode, sc.name)


def test_batch_of_random_scenes_equals_the_oracle():
    """Six seeded random scenes (tests/oracle_lib.random_scene) of different
    smoothing radii, sizes, walls, constants and time steps in one batch:
    with the reference's arithmetic each reproduces the oracle's bytes, in
    both batch modes.  Batches do not reorder, so the oracle runs map mode."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    from oracle_lib import Oracle, differing_words, random_scene
    scs = []
    for seed in range(200, 206):
        sc, vel = random_scene(seed)
        sc.dyn_vel = vel
        sc.reorder_interval = float(np.finfo(np.float32).max)
        scs.append(sc)
    refs = []
    for sc in scs:
        o = Oracle(0)
        o.init(sc, sc.dyn_vel)
        o.update(sc.dt, 5)
        _, _, io = o.maps()
        ref = np.empty(sc.n, o.read_raw().dtype)
        ref[io] = o.read_raw()
        refs.append(ref)
    for mode in (0, 1):
        b = Batch()
        ids = [b.add_scene(sc) for sc in scs]
        b.finalize()
        b.set_mode(mode)
        b.set_exact(True)
        b.step(2)
        b.step(3)
        for sid, sc, ref in zip(ids, scs, refs):
            diff = differing_words(b.read_scene(sid), ref)
            assert not diff.any(), (mode, sc.name, int(diff.any(1).sum()))


def test_batch_triangle_scenes_equal_the_oracle():
    """Scenes with their own triangle meshes in one batch (two triangle soups
    with degenerate triangles and a particle on a vertex, and a walled dam
    break without triangles): each scene's triangle grid and offsets are its
    own, and with the reference's arithmetic every scene equals the oracle
    word for word (NaN where the oracle has NaN), in both batch modes."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    from oracle_lib import Oracle, differing_words, triangle_soup_scene
    scs = [triangle_soup_scene(1), scenes.dam_break((20, 12, 20), 0.02, 0.04, (0.6, 0.4, 0.6), 0, mass=0.008,
                                                     name="dam_4800"), triangle_soup_scene(2)]
    refs = []
    for sc in scs:
        o = Oracle(0)
        o.init(sc)
        o.update(sc.dt, 3)
        _, _, io = o.maps()
        ref = np.empty(sc.n, o.read_raw().dtype)
        ref[io] = o.read_raw()
        refs.append(ref)
    for mode in (0, 1):
        b = Batch()
        ids = [b.add_scene(sc) for sc in scs]
        b.finalize()
        b.set_mode(mode)
        b.set_exact(True)
        b.step(1)
        b.step(2)
        for sid, sc, ref in zip(ids, scs, refs):
            diff = differing_words(b.read_scene(sid), ref)
            assert not diff.any(), (mode, sc.name, int(diff.any(1).sum()))
