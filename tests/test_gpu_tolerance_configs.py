"""The default (fused) arithmetic -- the one the benchmark times -- against
the oracle on the benchmark's own scenes, with the FP64 rerun beside it.

Scenes:
  dam_break_16k   16,384 particles, 8,602 walls, h 0.04, dt 1e-4 s (stable)
  dam_break_1m    1,048,576 particles, 256,002 walls, h 0.01: the configured
                  dt of 1e-4 s (the viscous term diverges from about step
                  15, in the reference's arithmetic too) and the stable 5e-5 s

Bars (FP32 parity):
  density   |rho_gpu - rho_ref| / rho_ref <= 1e-5 per particle, one step
  force     |a_gpu - a_ref| <= 1e-4 * max_i |a_ref|, one step (a = F / rho + g)
  position  RMS over particles of |x_gpu - x_ref| <= 1e-3 * h after 50 steps

The reference is the oracle (the CPU engine restated, pinned bit-exact to
the reference's own code).  The one-million-particle runs use its threaded
form on every host core: like the reference's multithreaded engine it fills
buckets in arrival order, so its neighbour sums round in a different order
from the synchronous engine's -- an FP32 difference of the same kind the
fused arithmetic makes.  Every error is printed against the FP32 and the
FP64 oracle, beside the FP32 oracle's own distance from FP64.

Where the configured step diverges, every rounding difference grows with
the flow, the FP32 reference's included.  That run asserts the bar while
the FP32 reference itself stays within it of FP64 (the first steps), and
from there on that the engine is no farther from FP64 than a small factor of
the FP32 reference's own distance.
"""
import os

import numpy as np
import pytest

from oracle_lib import Oracle
from sphfluidsimulation_gb300 import scenes
from sphfluidsimulation_gb300.engine import SimulationEngineCUDA

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
ACC_TOL = 1e-4
POS_TOL = 1e-3
# divergent regime: engine-vs-FP64 over FP32-reference-vs-FP64
CHAOS_FACTOR = 4.0

THREADS = os.cpu_count() or 1


def by_input(o):
    st = o.read()
    _, _, io = o.maps()
    out = np.empty_like(st)
    out[io] = st
    return out, io


def accel_by_input(o, io):
    a = np.empty((o.n, 3))
    a[io] = o.accel()
    return a


def one_step_errors(sc, threads):
    """Density and force errors of one default-arithmetic step."""
    o = Oracle(threads)
    o.init(sc)
    o.record_accel(True)
    o.update(sc.dt, 1)
    d = Oracle(threads, double=True)
    d.init(sc)
    d.record_accel(True)
    d.update(sc.dt, 1)
    e = SimulationEngineCUDA()
    e.initialize(sc)
    e.record_acceleration(True)
    e.update(sc.dt, 1)
    ref, io = by_input(o)
    ref64, io64 = by_input(d)
    g = e.read_dynamic()
    k, rho0 = sc.params.gas_constant, sc.params.rest_density
    rho_ref = ref[:, 3] / k + rho0
    rho_64 = ref64[:, 3] / k + rho0
    rho = g["pressure"].astype(np.float64) / k + rho0
    a_ref = accel_by_input(o, io)
    a_64 = accel_by_input(d, io64)
    a = e.read_acceleration().astype(np.float64)
    out = {
        "rho": float((np.abs(rho - rho_ref) / rho_ref).max()),
        "rho64": float((np.abs(rho - rho_64) / rho_64).max()),
        "rho_ref64": float((np.abs(rho_ref - rho_64) / rho_64).max()),
        "acc": float(np.abs(a - a_ref).max() / np.abs(a_ref).max()),
        "acc64": float(np.abs(a - a_64).max() / np.abs(a_64).max()),
        "acc_ref64": float(np.abs(a_ref - a_64).max() / np.abs(a_64).max()),
    }
    print(f"{sc.name} one step: density rel err vs fp32 {out['rho']:.3e}, vs fp64 {out['rho64']:.3e} "
          f"(fp32 ref vs fp64 {out['rho_ref64']:.3e}); force err / max|a| vs fp32 {out['acc']:.3e}, "
          f"vs fp64 {out['acc64']:.3e} (fp32 ref vs fp64 {out['acc_ref64']:.3e})")
    return out


def trajectory_rms(sc, checkpoints, threads):
    """Position RMS / h of the engine against the FP32 and FP64 oracles, and
    of the FP32 oracle against FP64, after each cumulative step count."""
    o = Oracle(threads)
    o.init(sc)
    d = Oracle(threads, double=True)
    d.init(sc)
    e = SimulationEngineCUDA()
    e.initialize(sc)
    h = sc.params.h
    rows, done = [], 0
    for c in checkpoints:
        o.update(sc.dt, c - done)
        d.update(sc.dt, c - done)
        e.update(sc.dt, c - done)
        done = c
        ref, _ = by_input(o)
        ref64, _ = by_input(d)
        x = np.asarray(e.read_dynamic()["pos"], np.float64)

        def rms(a, b):
            return float(np.sqrt(((a - b) ** 2).sum(1).mean()) / h)
        row = (c, rms(x, ref[:, :3]), rms(x, ref64[:, :3]), rms(ref[:, :3], ref64[:, :3]))
        rows.append(row)
        print(f"{sc.name} dt {sc.dt:g} step {c}: position RMS / h vs fp32 {row[1]:.3e}, vs fp64 {row[2]:.3e} "
              f"(fp32 ref vs fp64 {row[3]:.3e})")
    return rows


def test_fast_config0_one_step():
    err = one_step_errors(scenes.config0(steps=0), 0)
    assert err["rho"] <= RHO_TOL
    assert err["acc"] <= ACC_TOL


def test_fast_config0_trajectory():
    """50 steps (the bar) and on to the configuration's 200."""
    rows = trajectory_rms(scenes.config0(steps=0), [50, 200], 0)
    assert rows[0][1] <= POS_TOL
    assert rows[1][1] <= POS_TOL


def test_fast_config1_one_step():
    err = one_step_errors(scenes.config1(steps=0), THREADS)
    assert err["rho"] <= RHO_TOL
    assert err["acc"] <= ACC_TOL


def test_fast_config1_fifty_steps_stable_dt():
    sc = scenes.config1(steps=0, dt=scenes.STABLE_DT["dam_break_1m"])
    rows = trajectory_rms(sc, [10, 50], THREADS)
    for _, rms, _, _ in rows:
        assert rms <= POS_TOL


def test_fast_config1_fifty_steps_configured_dt():
    sc = scenes.config1(steps=0)
    rows = trajectory_rms(sc, [5, 10, 20, 50], THREADS)
    for step, rms, rms64, ref64 in rows:
        if ref64 <= POS_TOL:
            assert rms <= POS_TOL, (step, rms)
        else:
            assert rms64 <= CHAOS_FACTOR * ref64, (step, rms64, ref64)
