"""CPU oracle checks: the C restatement (oracle/sph_oracle.c) against the
golden fixtures produced by the reference itself, the reference's own debug
validators as invariants, threading and FP64 behaviour."""
import glob
import os

import numpy as np
import pytest

from oracle_lib import (REF_SO, Oracle, RefEngine, coincident_scene, differing_words, oracle_counting_sort,
                        oracle_hash, triangle_soup_scene)
from sphfluidsimulation_gb300 import scenes

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


class _FixtureScene:
    def __init__(self, z):
        p = z["params9"]
        self.dyn_pos = z["dyn_pos"]
        self.static_pos = z["static_pos"]
        self.triangles = z["triangles"]
        self.params = scenes.Params(float(p[0]), float(p[1]), float(p[2]), float(p[3]),
                                    (float(p[4]), float(p[5]), float(p[6])), float(p[7]), float(p[8]))
        self.dt = float(z["dt"])
        self.reorder_interval = float(z["reorder_interval"])
        self.dyn_vel = None


def test_golden_fixtures_present():
    names = {os.path.basename(p) for p in GOLDEN}
    assert {"debug_smallest.npz", "small_dam.npz", "small_dam_reorder.npz", "negative_cells.npz",
            "triangles.npz"} <= names


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_bit_exact_against_reference_fixtures(path):
    """Every checkpoint: raw particle buffer, hashMap, particleMap, init
    permutation and sorted statics equal the reference's, bit for bit."""
    z = np.load(path)
    sc = _FixtureScene(z)
    o = Oracle(0)
    o.init(sc)
    hm, pm, io = o.maps()
    assert np.array_equal(io, z["init_order"])
    if sc.static_pos.shape[0]:
        sp, sm = o.statics()
        assert np.array_equal(sp.astype(np.float32), z["static_sorted"])
        assert np.array_equal(sm, z["static_map"])
    done = 0
    for k, c in enumerate(z["checkpoints"]):
        o.update(sc.dt, int(c) - done)
        done = int(c)
        raw = o.read_raw().view(np.uint32).reshape(-1, 8)
        assert np.array_equal(raw, z[f"particles_{k}"]), f"checkpoint {c}"
        hm, pm, _ = o.maps()
        assert np.array_equal(hm, z[f"hash_map_{k}"])
        assert np.array_equal(pm, z[f"particle_map_{k}"])


def _validate(o: Oracle):
    """SimulationEngine.h validators: DebugParticles (hash of position, finite
    values, :115-177), DebugPrePrefixSumHashes (:178-190) and
    DebugHashAndParticleMap (:229-282)."""
    st = o.read()
    hm, pm, _ = o.maps()
    n, B = o.n, o.buckets
    assert np.isfinite(st[:, :7]).all()
    keys = oracle_hash(st[:, :3].astype(np.float32), o.h_param, B)
    assert np.array_equal(keys, st[:, 7].astype(np.uint32))
    assert hm[0] == 0 and hm[B] == n
    assert (np.diff(hm.astype(np.int64)) >= 0).all()
    counts = np.bincount(keys, minlength=B)
    assert np.array_equal(np.diff(hm.astype(np.int64)), counts)
    b_of_slot = np.repeat(np.arange(B), counts)
    assert np.array_equal(keys[pm], b_of_slot)


def test_oracle_validators_hold_over_steps():
    sc = scenes.dam_break((12, 10, 12), 0.02, 0.04, (0.5, 0.4, 0.5), 0, mass=0.008)
    o = Oracle(0)
    o.init(sc)
    o.h_param = sc.params.h
    for _ in range(5):
        o.update(sc.dt, 4)
        _validate(o)


def test_threaded_oracle_matches_serial():
    """T>0 threads: same counts and tables, particle state equal within FP32
    summation-order noise (the bucket order is non-deterministic, as in the
    reference)."""
    sc = scenes.dam_break((12, 10, 12), 0.02, 0.04, (0.5, 0.4, 0.5), 0, mass=0.008)
    a, b = Oracle(0), Oracle(4)
    a.init(sc)
    b.init(sc)
    for steps in (1, 3):
        a.update(sc.dt, steps)
        b.update(sc.dt, steps)
    sa, sb = a.by_input_order(), b.by_input_order()
    assert np.abs(sa[:, :3] - sb[:, :3]).max() < 1e-6
    assert np.abs(sa[:, 3] - sb[:, 3]).max() <= 1e-5 * 200 * 1000
    ha, _, _ = a.maps()
    hb, _, _ = b.maps()
    assert np.array_equal(ha, hb)


def test_parallel_partial_sum_matches():
    sc = scenes.dam_break((12, 10, 12), 0.02, 0.04, (0.5, 0.4, 0.5), 0, mass=0.008)
    a, b = Oracle(0), Oracle(3)
    a.init(sc)
    b.init(sc, parallel_partial_sum=True)
    a.update(sc.dt, 2)
    b.update(sc.dt, 2)
    assert np.array_equal(a.maps()[0], b.maps()[0])


def test_fp64_rerun_close_to_fp32():
    sc = scenes.dam_break((12, 10, 12), 0.02, 0.04, (0.5, 0.4, 0.5), 0, mass=0.008)
    a, b = Oracle(0), Oracle(0, double=True)
    a.init(sc)
    b.init(sc)
    a.update(sc.dt, 1)
    b.update(sc.dt, 1)
    sa, sb = a.by_input_order(), b.by_input_order()
    rho_a = sa[:, 3] / 200.0 + 1000.0
    rho_b = sb[:, 3] / 200.0 + 1000.0
    assert np.max(np.abs(rho_a - rho_b) / rho_b) < 1e-5


def test_counting_sort_semantics():
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 50, size=400).astype(np.uint32)
    counts, starts, pm = oracle_counting_sort(keys, 50)
    assert np.array_equal(counts, np.bincount(keys, minlength=50))
    assert starts[0] == 0 and starts[50] == 400
    for b in range(50):
        members = pm[starts[b]:starts[b + 1]]
        assert (keys[members] == b).all()
        # the decrementing fill lists a bucket's members in descending order
        assert (np.diff(members.astype(np.int64)) < 0).all()


def test_hash_negative_cells_wrap():
    pos = np.array([[-0.01, 0.0, 0.0], [0.0, -0.01, 0.0], [0.0, 0.0, -0.01]], np.float32)
    keys = oracle_hash(pos, 1.0, 1 << 30)
    ex = lambda v: int(''.join('00' + b for b in format(v & 1023, '010b')), 2)  # noqa: E731
    assert keys[0] == ex(1023)
    assert keys[1] == 2 * ex(1023)
    assert keys[2] == 4 * ex(1023)


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference not compiled here (no reference tree)")
def test_oracle_matches_reference_random_scene():
    sc = scenes.dam_break((11, 9, 13), 0.02, 0.04, (0.5, 0.4, 0.5), 0, mass=0.008)
    sc.dyn_pos = (sc.dyn_pos - np.float32(0.05)).astype(np.float32)
    o, r = Oracle(0), RefEngine()
    o.init(sc)
    r.init(sc)
    for steps in (1, 7):
        o.update(sc.dt, steps)
        r.update(sc.dt, steps)
        assert o.read_raw().tobytes() == r.read_raw().tobytes()
        assert all(np.array_equal(x, y) for x, y in zip(o.maps(), r.maps()))


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference not compiled here (no reference tree)")
def test_oracle_matches_reference_coincident_particles():
    """RandomDirection (SF:140-155) for coincident dynamic and static pairs:
    the oracle's restatement gives the reference's own bytes.  About half of
    the seeds make the reference's noise negative (modf keeps the sign), z
    then falls below -1 and the direction is NaN; those particles turn NaN
    in both, and NaN spreads to their neighbours in later steps."""
    sc = coincident_scene()
    o, r = Oracle(0), RefEngine()
    o.init(sc)
    r.init(sc)
    o.update(sc.dt, 1)
    r.update(sc.dt, 1)
    assert o.read_raw().tobytes() == r.read_raw().tobytes()       # same NaN bits too, at first
    assert np.isnan(o.read_raw()["pos"]).any()
    for steps in (1, 2):
        o.update(sc.dt, steps)
        r.update(sc.dt, steps)
        assert not differing_words(o.read_raw(), r.read_raw()).any()


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference not compiled here (no reference tree)")
def test_oracle_matches_reference_far_cells():
    """Cells beyond 2^31 (SF:65-76 casts floor(p/h) from float to uint): the
    reference's cast wraps modulo 2^32 through int64 on x86-64, and the
    oracle writes those two steps out; beyond 2^63 cells and for the
    infinities the conversion's "indefinite" value leaves cell 0.  Particles
    up to 2^66 cells away, on both sides, and infinite ones hash and step to
    the reference's bytes."""
    sc = scenes.dam_break((6, 5, 7), 0.02, 0.04, (0.3, 0.3, 0.3), 0, mass=0.008)
    far = np.array([[3.0e9, 0.1, 0.1], [-5.0e9, 0.2, 0.3], [1.0e12, -2.5e11, 0.1], [2.0e17, 0.3, -7.0e16],
                    [0.1, 4.1e9, 0.2], [0.2, 0.2, -2.2e9], [4.5e16, 4.5e16, 4.5e16], [1.0e20, 0.1, 0.1],
                    [0.1, -3.0e19, 0.2], [np.inf, 0.1, 0.1], [0.2, -np.inf, 0.2]], np.float32) * np.float32(0.04)
    sc.dyn_pos = np.concatenate([sc.dyn_pos, far], 0).astype(np.float32)
    o, r = Oracle(0), RefEngine()
    o.init(sc)
    r.init(sc)
    assert o.read_raw().tobytes() == r.read_raw().tobytes()
    o.update(sc.dt, 2)
    r.update(sc.dt, 2)
    assert o.read_raw().tobytes() == r.read_raw().tobytes()
    assert all(np.array_equal(x, y) for x, y in zip(o.maps(), r.maps()))


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference not compiled here (no reference tree)")
def test_oracle_matches_reference_triangle_soup():
    """Degenerate triangles and a particle on a vertex (tests/oracle_lib
    triangle_soup_scene): the oracle's CalculateTriangleForce gives the
    reference's bytes, NaN included."""
    for seed in (1, 2):
        sc = triangle_soup_scene(seed)
        o, r = Oracle(0), RefEngine()
        o.init(sc)
        r.init(sc)
        for steps in (1, 2):
            o.update(sc.dt, steps)
            r.update(sc.dt, steps)
            assert not differing_words(o.read_raw(), r.read_raw()).any(), (seed, steps)


def test_reorder_cadence_and_identity():
    """reorderTimeInterval: a negative interval reorders on every Update call,
    any interval >= 0 never does (the elapsed time is reset as soon as it
    passes the interval, SimulationEngineCPU.cpp:441,452-454).  The oracle's
    slot -> input index bookkeeping follows the reorders, so both runs agree
    particle by particle up to summation-order rounding."""
    sc = scenes.dam_break((10, 8, 12), 0.02, 0.04, (0.5, 0.4, 0.5), 0, mass=0.008)
    runs = {}
    for interval in (-1.0, 0.0, float(np.finfo(np.float32).max)):
        sc.reorder_interval = interval
        o = Oracle(0)
        o.init(sc)
        # every step of a reordering call reorders, and a reorder reverses a
        # bucket that kept its members: an odd number of steps in all
        for _ in range(3):
            o.update(sc.dt, 3)
        runs[interval] = o
    _, _, io_never = runs[0.0].maps()
    _, _, io_init = runs[float(np.finfo(np.float32).max)].maps()
    _, _, io_each = runs[-1.0].maps()
    assert np.array_equal(io_never, io_init)
    assert not np.array_equal(io_each, io_init)
    assert np.array_equal(np.sort(io_each), np.arange(sc.n, dtype=np.uint32))
    assert runs[0.0].read_raw().tobytes() == runs[float(np.finfo(np.float32).max)].read_raw().tobytes()
    a, b = runs[-1.0].by_input_order(), runs[0.0].by_input_order()
    assert np.abs(a[:, :3] - b[:, :3]).max() < 1e-6
