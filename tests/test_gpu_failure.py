"""Failure detection on the GPU without faulting it: a bounded device wait
is made to run out (the scan's look-back waits for a tile that nothing
publishes), the kernel sets its status bit and finishes, the host reports
SPH_ERR_DEVICE_TIMEOUT, and the same process keeps simulating correctly."""
import ctypes as C
import time

import pytest

from oracle_lib import Oracle
from sphfluidsimulation_gb300 import _lib, scenes
from sphfluidsimulation_gb300.engine import SimulationEngineCUDA

pytestmark = pytest.mark.gpu

SPH_ERR_DEVICE_TIMEOUT = 5


def test_expired_wait_is_reported_and_the_context_survives():
    lib = _lib.load()
    bits = C.c_uint32(0)
    t0 = time.perf_counter()
    st = lib.sph_debug_expire_wait(0, C.byref(bits))
    waited = time.perf_counter() - t0
    assert st == SPH_ERR_DEVICE_TIMEOUT, lib.sph_last_error()
    assert bits.value & 1                      # scan wait expired
    assert waited < 60
    assert b"scan wait" in lib.sph_last_error()
    # the context is intact: an exact run right after equals the oracle's bytes
    sc = scenes.dam_break((12, 8, 12), 0.02, 0.04, (0.4, 0.3, 0.4), 0, mass=0.008, name="after_timeout")
    e = SimulationEngineCUDA()
    e.initialize(sc)
    e.set_exact(True)
    e.update(sc.dt, 10)
    o = Oracle(0)
    o.init(sc)
    o.update(sc.dt, 10)
    assert e.read_dynamic_buffer().tobytes() == o.read_raw().tobytes()
