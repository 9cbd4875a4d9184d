"""Reference arithmetic (sph_engine_set_exact): the GPU engine reproduces the
reference's synchronous CPU engine bit for bit.

With exact arithmetic the density and force passes repeat the reference's
floating-point operations one for one (no fused multiply-adds, true
divisions), and every bucket is visited in the reference's member order,
which the sort keeps through buffer tags (the reference's buffer indices,
renumbered on reordering steps).  So the particle buffer the engine reports
in the reference's buffer order (sph_engine_read_dynamic_buffer) must equal
the reference's, all 32 bytes of every particle, at every checkpoint:

* against the golden fixtures made by the reference's own code
  (tests/golden/make_golden.py), including a scene that reorders on every
  Update call and one with triangle boundary forces;
* against the oracle (pinned to the reference) over 50 steps of a walled dam
  break in both reorder regimes, the 16,384-particle configuration, and
  scenes whose neighbour lists overflow (the bucket-walking fallback).
"""
import glob
import os

import numpy as np
import pytest

from oracle_lib import Oracle, coincident_scene, differing_words, random_scene, triangle_soup_scene
from sphfluidsimulation_gb300 import scenes
from sphfluidsimulation_gb300.engine import SimulationEngineCUDA

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
FIELDS = ["x", "y", "z", "pressure", "vx", "vy", "vz", "hash"]


def fixture_scene(z, name):
    p = z["params9"]
    params = scenes.Params(*[float(v) for v in p[:4]], (float(p[4]), float(p[5]), float(p[6])), float(p[7]),
                           float(p[8]))
    return scenes.Scene(name=name, dyn_pos=z["dyn_pos"], static_pos=z["static_pos"], params=params,
                        dt=float(z["dt"]), steps=0, triangles=z["triangles"],
                        reorder_interval=float(z["reorder_interval"]))


def assert_same_bits(got, ref, what):
    g = np.asarray(got).view(np.uint32).reshape(-1, 8)
    r = np.asarray(ref).view(np.uint32).reshape(-1, 8)
    if not np.array_equal(g, r):
        bad = (g != r).sum(0)
        rows = np.nonzero((g != r).any(1))[0]
        raise AssertionError(f"{what}: {len(rows)} of {len(r)} particles differ; words differing per field "
                             + ", ".join(f"{f}={int(b)}" for f, b in zip(FIELDS, bad)))


def exact_engine(sc):
    e = SimulationEngineCUDA()
    e.initialize(sc)
    e.set_exact(True)
    return e


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_exact_equals_reference_fixtures(path):
    z = np.load(path)
    sc = fixture_scene(z, os.path.basename(path))
    e = exact_engine(sc)
    done = 0
    for k, c in enumerate(z["checkpoints"]):
        e.update(sc.dt, int(c) - done)      # the same Update calls the fixture was recorded with
        done = int(c)
        assert_same_bits(e.read_dynamic_buffer(), z[f"particles_{k}"], f"{sc.name} after {c} steps")


def walled_dam():
    return scenes.dam_break((20, 12, 20), 0.02, 0.04, (0.6, 0.4, 0.6), 0, mass=0.008, name="dam_4800")


def run_against_oracle(sc, calls):
    o = Oracle(0)
    o.init(sc)
    e = exact_engine(sc)
    done = 0
    for steps in calls:
        o.update(sc.dt, steps)
        e.update(sc.dt, steps)
        done += steps
        assert_same_bits(e.read_dynamic_buffer(), o.read_raw(), f"{sc.name} after {done} steps")
    return o, e


@pytest.mark.parametrize("interval", [float(np.finfo(np.float32).max), -1.0], ids=["map", "reorder_each_call"])
def test_exact_equals_oracle_fifty_steps(interval):
    sc = walled_dam()
    sc.reorder_interval = interval
    o, e = run_against_oracle(sc, [1, 4, 10, 35])
    # the caller's-order readback is the same particles
    _, _, io = o.maps()
    by_input = np.empty(sc.n, o.read_raw().dtype)
    by_input[io] = o.read_raw()
    assert_same_bits(e.read_dynamic(), by_input, "input order")


def test_exact_equals_oracle_config0():
    sc = scenes.config0(steps=0)
    run_against_oracle(sc, [3, 12])


def test_exact_overflowing_neighbour_lists():
    """A lattice at h/5 has about 500 neighbours per particle (lists hold 96)
    and a wall at h/6 about 100 static ones (lists hold 48): every particle
    takes the bucket-walking path of both passes."""
    h = 0.05
    dyn = scenes.filled_box((9, 9, 9), h / 5, (0.1, 0.02, 0.1), 0.1, scenes.SplitMix64(3))
    walls = scenes.box_shell((0.4, 0.3, 0.4), h / 6)
    sc = scenes.Scene(name="dense", dyn_pos=dyn, static_pos=walls, params=scenes.water_params(h / 5, h),
                      dt=1e-4, steps=0)
    run_against_oracle(sc, [1, 2, 3])


def test_exact_switch_back_to_fast():
    """The fast arithmetic after exact steps: still within rounding of the
    oracle (the tolerance tests cover the fast form in full)."""
    sc = walled_dam()
    o = Oracle(0)
    o.init(sc)
    e = exact_engine(sc)
    o.update(sc.dt, 5)
    e.update(sc.dt, 5)
    e.set_exact(False)
    o.update(sc.dt, 5)
    e.update(sc.dt, 5)
    g = e.read_dynamic_buffer()
    r = o.read_raw()
    assert np.abs(g["pos"].astype(np.float64) - r["pos"]).max() < 1e-6


def test_exact_scene_file_with_boundary_mesh(tmp_path):
    """A scene in the reference's JSON format with an OBJ boundary mesh (a
    floor quad and a tilted panel, 3 triangles) through the loader: the exact
    engine equals the oracle, triangle forces included."""
    import json
    from sphfluidsimulation_gb300 import scene_json
    (tmp_path / "panel.obj").write_text(
        "o Floor\nv -0.1 -0.01 -0.1\nv 0.7 -0.01 -0.1\nv 0.7 -0.01 0.7\nv -0.1 -0.01 0.7\nf 1 2 3 4\n"
        "o Panel\nv 0.3 0.0 0.0\nv 0.3 0.4 0.2\nv 0.6 0.0 0.5\nf 5 6 7\n")
    doc = {
        "particleBehaviourParameters": {"particleMass": 0.008, "gasConstant": 200, "elasticity": 0,
                                        "viscosity": 0.1, "gravity": [0, -9.81, 0], "restDensity": 1000,
                                        "maxInteractionDistance": 0.04},
        "particleSetBlueprints": [
            {"layerName": "dynamic", "particleSetBlueprintType": "FilledBox",
             "properties": {"particlesPerUnit": 125000, "randomOffsetIntensity": 1, "seed": 3,
                            "spawnVolumeOffset": [0.02, 0.02, 0.02], "spawnVolumeSize": [0.24, 0.2, 0.24]}},
            {"layerName": "static", "particleSetBlueprintType": "BoxShell",
             "properties": {"particleDistance": 0.02, "randomOffsetIntensity": 0,
                            "spawnVolumeOffset": [0, 0, 0], "spawnVolumeSize": [0.6, 0.4, 0.6]}}],
        "boundaryMesh": {"path": "panel.obj"},
        "otherParameters": {"reorderTimeInterval": "-1"},
    }
    path = tmp_path / "scene.json"
    path.write_text(json.dumps(doc))
    sc = scene_json.load_scene(str(path), dt=1e-4)
    assert sc.triangles.shape == (3, 9) and sc.n == 12 * 10 * 12
    run_against_oracle(sc, [1, 4, 10])


def uv_sphere(radius, centre, rings, segments):
    """Triangles (T, 9) of a UV sphere: two per quad, one per pole quad."""
    c = np.asarray(centre, np.float64)
    th = np.linspace(0.0, np.pi, rings + 1)
    ph = np.linspace(0.0, 2.0 * np.pi, segments + 1)
    P = lambda i, j: c + radius * np.array([np.sin(th[i]) * np.cos(ph[j]), np.cos(th[i]),  # noqa: E731
                                             np.sin(th[i]) * np.sin(ph[j])])
    tris = []
    for i in range(rings):
        for j in range(segments):
            a, b, cc, d = P(i, j), P(i + 1, j), P(i + 1, j + 1), P(i, j + 1)
            if i > 0:
                tris.append(np.concatenate([a, b, d]))
            if i < rings - 1:
                tris.append(np.concatenate([b, cc, d]))
    return np.asarray(tris, np.float32)


def test_exact_triangle_cells_large_mesh():
    """A mesh much larger than the triangle reach (2.5): each particle
    evaluates only the triangles of its cell, and the result still equals
    the oracle, which evaluates all of them; particles lie at every distance
    from the sphere, many near the reach."""
    h = 2.0
    dyn = scenes.filled_box((16, 16, 16), 0.5, (-4.0, -1.0, -4.0), 0.0, None)
    params = scenes.Params(particle_mass=1.0, gas_constant=200.0, elasticity=1.0, viscosity=0.1,
                           gravity=(0.0, -9.81, 0.0), rest_density=1.0, h=h)
    sc = scenes.Scene(name="sphere_mesh", dyn_pos=dyn, static_pos=np.zeros((0, 3), np.float32), params=params,
                      dt=1e-3, steps=0, triangles=uv_sphere(7.0, (0.0, 3.0, 0.0), 18, 32))
    assert sc.triangles.shape[0] > 500
    run_against_oracle(sc, [1, 2])


def test_exact_equals_oracle_at_one_million():
    """The benchmark scene itself (1,048,576 particles, 256,002 walls): two
    exact steps equal the synchronous oracle's, all bytes of every particle."""
    sc = scenes.config1(steps=0)
    run_against_oracle(sc, [1, 1])


def test_exact_pool_drop_through_divergence():
    """A 131,072-particle pool drop at h = 0.005 with the dam-break step of
    1e-4 s, beyond the viscous limit (about h^2 / (8 mu) = 3.1e-5 s): from
    the fourth step nearly every particle changes bucket on every step, and
    by the eighth most have left the box for negative coordinates, whose cell
    indices the hash wraps.  The sort and both passes still equal the oracle
    bit for bit throughout."""
    sc = scenes.pool_drop((64, 28, 64), 131_072, (0.32, 0.96, 0.24), 0, dt=1e-4, name="pool_drop_131k_dt1e-4")
    o, e = run_against_oracle(sc, [2, 2, 2, 2])
    negative = (o.read_raw()["pos"] < 0).any(1).mean()
    assert negative > 0.25, negative        # the run did diverge


def test_pool_drop_8m_exact_and_default_arithmetic():
    """The 8,388,608-particle pool drop (1,310,722 walls, 2^24 buckets) at
    its stable step: two exact steps equal the oracle, all bytes of every
    particle; the default arithmetic stays within the density (1e-5
    relative) and position (1e-3 h RMS) tolerances; and the bucket table
    holds the reference's invariants."""
    sc = scenes.config2(steps=0, dt=scenes.STABLE_DT["pool_drop_8m"])
    o = Oracle(0)
    o.init(sc)
    o.update(sc.dt, 2)
    ref = o.read_raw()
    e = exact_engine(sc)
    e.update(sc.dt, 2)
    assert_same_bits(e.read_dynamic_buffer(), ref, "pool drop 8M after 2 steps")
    del e
    f = SimulationEngineCUDA()
    f.initialize(sc)
    f.update(sc.dt, 2)
    g = f.read_dynamic_buffer()
    k, rho0 = sc.params.gas_constant, sc.params.rest_density
    rho_ref = ref["pressure"].astype(np.float64) / k + rho0
    rho = g["pressure"].astype(np.float64) / k + rho0
    assert np.abs(rho - rho_ref).max() / rho_ref.min() <= 1e-5
    rms = np.sqrt(((g["pos"].astype(np.float64) - ref["pos"]) ** 2).sum(1).mean())
    assert rms <= 1e-3 * sc.params.h, rms / sc.params.h
    starts, ids = f.read_buckets()
    n, b = sc.n, 2 * sc.n
    assert starts[0] == 0 and starts[b] == n and (np.diff(starts.astype(np.int64)) >= 0).all()
    assert np.array_equal(np.sort(ids), np.arange(n, dtype=np.uint32))


def test_exact_coincident_particles():
    """Particles at exactly the same position as a dynamic or a static
    neighbour take the reference's RandomDirection (SF:140-155, used at
    SF:576-580 and SF:610-614): sin and cos in double, rounded to float.
    For about half of the seeds the reference's noise is negative (modf keeps
    the sign), z falls below -1 and the direction is NaN, so those particles
    turn NaN, and NaN spreads to their neighbours.  Over three steps every
    finite word equals the oracle's and the NaNs sit in the same words (their
    sign and payload are the platform's).  The device's and the host's double
    sin and cos may differ in the last bit, which reaches the float result
    only within about 1e-12 of a float rounding boundary."""
    sc = coincident_scene()
    o = Oracle(0)
    o.init(sc)
    e = exact_engine(sc)
    for step in range(1, 4):
        o.update(sc.dt, 1)
        e.update(sc.dt, 1)
        diff = differing_words(e.read_dynamic_buffer(), o.read_raw())
        assert not diff.any(), f"after {step} steps: {int(diff.any(1).sum())} particles differ, per field {diff.sum(0)}"
    assert np.isnan(o.read_raw()["pos"]).any()


@pytest.mark.parametrize("seed", range(100, 116))
def test_exact_random_scenes(seed):
    """Seeded random scenes (tests/oracle_lib.random_scene): clouds,
    clusters, sheets and face-aligned lattices, with and without walls,
    random constants, gravity, dt, reorder mode and initial velocities.
    Six exact steps equal the oracle's bytes."""
    sc, vel = random_scene(seed)
    o = Oracle(0)
    o.init(sc, vel)
    e = SimulationEngineCUDA()
    e.initialize(sc, vel)
    e.set_exact(True)
    for steps in (1, 2, 3):
        o.update(sc.dt, steps)
        e.update(sc.dt, steps)
        diff = differing_words(e.read_dynamic_buffer(), o.read_raw())
        assert not diff.any(), f"{sc.name}: {int(diff.any(1).sum())} particles differ, per field {diff.sum(0)}"


@pytest.mark.parametrize("seed", [1, 2])
def test_exact_triangle_soup(seed):
    """Degenerate triangles (two equal vertices, collinear, tiny) and a
    particle exactly on a vertex, where CalculateTriangleForce divides by a
    zero distance and the particle turns NaN: three exact steps equal the
    oracle word for word (NaN where it has NaN)."""
    sc = triangle_soup_scene(seed)
    o = Oracle(0)
    o.init(sc)
    e = exact_engine(sc)
    for step in range(1, 4):
        o.update(sc.dt, 1)
        e.update(sc.dt, 1)
        diff = differing_words(e.read_dynamic_buffer(), o.read_raw())
        assert not diff.any(), f"after {step} steps: {int(diff.any(1).sum())} particles differ, per field {diff.sum(0)}"


@pytest.mark.parametrize("interval", [float(np.finfo(np.float32).max), -1.0], ids=["map", "reorder_each_call"])
def test_exact_write_back_keeps_the_reference_state(interval):
    """Writing the engine's own state back (sph_engine_write_dynamic, caller's
    order) between Update calls re-sorts with every particle's buffer tag
    kept, so the run stays the reference's: after 3 + write + 4 + write + 5
    steps the bytes equal the oracle's 12 uninterrupted steps, in map mode
    and reordering on every call."""
    sc = walled_dam()
    sc.reorder_interval = interval
    o = Oracle(0)
    o.init(sc)
    e = exact_engine(sc)
    for steps in (3, 4, 5):
        o.update(sc.dt, steps)
        e.update(sc.dt, steps)
        e.write_dynamic(e.read_dynamic())
    assert_same_bits(e.read_dynamic_buffer(), o.read_raw(), "after writes")


def test_exact_after_reinitialising_the_engine():
    """One engine, two scenes: after a run that turned particles NaN (the
    coincident scene) the same engine initialised with a walled dam break
    that reorders on every call gives the oracle's bytes: no state of the
    first run (step graph, reorder clock, non-finite flag, tags) survives
    Initialize (SimulationEngineCPU.cpp:396-419 clears first)."""
    first = coincident_scene()
    e = exact_engine(first)
    e.update(first.dt, 3)
    assert np.isnan(e.read_dynamic_buffer()["pos"]).any()
    sc = walled_dam()
    sc.reorder_interval = -1.0
    e.initialize(sc)
    e.set_exact(True)
    o = Oracle(0)
    o.init(sc)
    for steps in (2, 3):
        o.update(sc.dt, steps)
        e.update(sc.dt, steps)
    assert_same_bits(e.read_dynamic_buffer(), o.read_raw(), "second scene")


def test_exact_one_engine_many_scenes():
    """Initialize keeps the device arrays of the previous scene when the new
    one fits and allocates afresh when it grows.  One engine taken through
    random scenes of rising and falling size, a triangle soup and a walled
    dam break (with and without statics and triangles) gives the oracle's
    bytes for every scene, so nothing of an earlier scene survives in the
    reused arrays."""
    e = SimulationEngineCUDA()
    order = [("random", 107), ("random", 100), ("soup", 1), ("random", 113), ("dam", None), ("random", 104),
             ("soup", 2), ("random", 111)]
    for kind, seed in order:
        vel = None
        if kind == "random":
            sc, vel = random_scene(seed)
        elif kind == "soup":
            sc = triangle_soup_scene(seed)
        else:
            sc = walled_dam()
            sc.reorder_interval = -1.0
        e.initialize(sc, vel)
        e.set_exact(True)
        o = Oracle(0)
        o.init(sc, vel)
        for steps in (1, 3):
            o.update(sc.dt, steps)
            e.update(sc.dt, steps)
        diff = differing_words(e.read_dynamic_buffer(), o.read_raw())
        assert not diff.any(), f"{kind} {seed}: {int(diff.any(1).sum())} particles differ, per field {diff.sum(0)}"


@pytest.mark.parametrize("interval", [float(np.finfo(np.float32).max), -1.0], ids=["map", "reorder_each_call"])
def test_exact_recorded_acceleration(interval):
    """The recorded acceleration F/rho + g of the last step
    (sph_engine_record_acceleration, SF:638-641) is the oracle's, bit for
    bit, with walls and in both reorder modes."""
    sc = walled_dam()
    sc.reorder_interval = interval
    o = Oracle(0)
    o.init(sc)
    o.record_accel(True)
    e = exact_engine(sc)
    e.record_acceleration(True)
    o.update(sc.dt, 4)
    e.update(sc.dt, 4)
    # the oracle records per slot of the step's input buffer, which a
    # reordering step then permutes: map through the order before the step
    _, _, io = o.maps()
    o.update(sc.dt, 1)
    e.update(sc.dt, 1)
    ref = np.empty((sc.n, 3), np.float32)
    ref[io] = o.accel().astype(np.float32)          # the oracle's floats, widened to double on read
    got = e.read_acceleration()
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
