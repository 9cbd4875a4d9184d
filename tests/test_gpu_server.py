"""Served form: jobs of different sizes and horizons admitted under an HBM
budget, advanced together; each result equals the same job run alone on the
plain engine, bit for bit (and so within any tolerance)."""
import numpy as np
import pytest

from sphfluidsimulation_gb300 import scenes
from sphfluidsimulation_gb300._lib import SphError
from sphfluidsimulation_gb300.engine import Server, SimulationEngineCUDA

pytestmark = pytest.mark.gpu


def job(n, steps, seed):
    j = scenes.Job(job_id=seed, arrival_s=0.0, n=n, steps=steps, seed=seed)
    return scenes.job_scene(j)


def alone(sc):
    e = SimulationEngineCUDA()
    e.initialize(sc)
    e.update(sc.dt, sc.steps)
    return e.read_dynamic()


def test_results_alone_equal_in_the_mix():
    specs = [(3000, 17, 1), (500, 40, 2), (9000, 9, 3), (1200, 33, 4), (2500, 25, 5), (700, 3, 6)]
    scs = [job(n, st, sd) for n, st, sd in specs]
    srv = Server(budget_bytes=1 << 30, max_slots=4)
    ids = [srv.submit(sc) for sc in scs[:4]]
    # more work arrives while the first jobs are on the GPU
    a, q = srv.poll(5)
    ids += [srv.submit(sc) for sc in scs[4:]]
    done = {}
    for _ in range(200):
        a, q = srv.poll(7)
        for jid in ids:
            if jid not in done:
                r = srv.result(jid)
                if r is not None:
                    done[jid] = r
        if len(done) == len(ids) and a == 0 and q == 0:
            break
    assert len(done) == len(ids)
    for jid, sc in zip(ids, scs):
        parts, dens = done[jid]
        ref = alone(sc)
        assert parts.tobytes() == ref.tobytes(), sc.name
        rho = ref["pressure"] / np.float32(sc.params.gas_constant) + np.float32(sc.params.rest_density)
        assert np.array_equal(dens, rho.astype(np.float32))


def test_budget_admission_and_rejection():
    small = job(2000, 5, 7)
    per_job = Server.job_bytes(small.n, small.s)
    srv = Server(budget_bytes=int(per_job * 1.5), max_slots=8)
    big = job(20000, 5, 8)
    with pytest.raises(SphError) as ei:
        srv.submit(big)
    assert ei.value.status == 7
    a_id = srv.submit(small)
    b_id = srv.submit(job(2000, 5, 9))
    a, q = srv.poll(2)
    assert a == 1 and q == 1          # the second job waits for budget
    for _ in range(20):
        a, q = srv.poll(2)
        if a == 0 and q == 0:
            break
    assert srv.result(a_id) is not None and srv.result(b_id) is not None


def test_malformed_jobs_rejected():
    srv = Server(budget_bytes=1 << 28, max_slots=2)
    sc = job(100, 5, 1)
    with pytest.raises(SphError) as ei:
        srv.submit(sc, steps=0)
    assert ei.value.status == 1
    sc.params.h = -1.0
    with pytest.raises(SphError):
        srv.submit(sc)
    with pytest.raises(SphError):
        Server(budget_bytes=0)


def test_served_exact_arithmetic_equals_the_oracle():
    """Jobs served with the reference's arithmetic return the reference CPU
    engine's bytes (the oracle), whatever the mix and the poll chunks."""
    import os, sys
    sys.path.insert(0, os.path.dirname(__file__))
    from oracle_lib import Oracle
    specs = [(1500, 13, 11), (800, 21, 12), (2600, 8, 13)]
    scs = [job(n, st, sd) for n, st, sd in specs]
    srv = Server(budget_bytes=1 << 30, max_slots=4)
    srv.set_exact(True)
    ids = [srv.submit(sc) for sc in scs]
    done = {}
    for _ in range(100):
        a, q = srv.poll(6)
        for jid in ids:
            if jid not in done:
                r = srv.result(jid)
                if r is not None:
                    done[jid] = r
        if len(done) == len(ids):
            break
    assert len(done) == len(ids)
    for jid, sc in zip(ids, scs):
        o = Oracle(0)
        o.init(sc)
        o.update(sc.dt, sc.steps)
        _, _, io = o.maps()
        ref = np.empty(sc.n, o.read_raw().dtype)
        ref[io] = o.read_raw()
        assert done[jid][0].tobytes() == ref.tobytes(), sc.name


def test_served_random_scenes_equal_the_oracle():
    """Five seeded random scenes (tests/oracle_lib.random_scene: different
    smoothing radii, sizes, walls, constants and time steps) served together
    with different horizons and three slots, so admissions and finishes
    interleave: with the reference's arithmetic every job returns the
    oracle's bytes.  Jobs start at rest and do not reorder."""
    import os, sys
    sys.path.insert(0, os.path.dirname(__file__))
    from oracle_lib import Oracle, random_scene
    scs = []
    for seed, steps in zip(range(300, 305), (7, 12, 5, 9, 3)):
        sc, _ = random_scene(seed)
        sc.steps = steps
        sc.reorder_interval = float(np.finfo(np.float32).max)
        scs.append(sc)
    srv = Server(budget_bytes=1 << 30, max_slots=3)
    srv.set_exact(True)
    ids = [srv.submit(sc) for sc in scs]
    done = {}
    for _ in range(200):
        srv.poll(4)
        for jid in ids:
            if jid not in done:
                r = srv.result(jid)
                if r is not None:
                    done[jid] = r
        if len(done) == len(ids):
            break
    assert len(done) == len(ids)
    for jid, sc in zip(ids, scs):
        o = Oracle(0)
        o.init(sc)
        o.update(sc.dt, sc.steps)
        _, _, io = o.maps()
        ref = np.empty(sc.n, o.read_raw().dtype)
        ref[io] = o.read_raw()
        assert done[jid][0].tobytes() == ref.tobytes(), sc.name


def test_finished_reports_each_job_once():
    """sph_server_finished drains the ids of retired jobs: every job appears
    once, in retirement order (the shortest horizon first here), and the
    results fetched for those ids equal each job run alone."""
    scs = [job(1200, 9, 21), job(900, 3, 22), job(1500, 14, 23)]
    srv = Server(budget_bytes=1 << 30, max_slots=2)
    ids = [srv.submit(sc) for sc in scs]
    seen = []
    for _ in range(100):
        srv.poll(4)
        seen += srv.finished()
        if len(seen) == len(ids):
            break
    assert sorted(seen) == sorted(ids) and seen[0] == ids[1]
    assert srv.finished() == []
    for jid, sc in zip(ids, scs):
        assert srv.result(jid)[0].tobytes() == alone(sc).tobytes()


def test_poll_phases_are_reported():
    """sph_server_stats: every poll is counted, the steps run add up to the
    largest horizon served, and the host time of each phase is recorded."""
    scs = [job(1500, 6, 31), job(800, 11, 32)]
    srv = Server(budget_bytes=1 << 30, max_slots=4)
    ids = [srv.submit(sc) for sc in scs]
    polls = 0
    while True:
        a, q = srv.poll(4)
        polls += 1
        if a == 0 and q == 0:
            break
    st = srv.stats()
    assert st["polls"] == polls
    assert st["steps"] == 11
    assert all(st[k] >= 0.0 for k in st if k.endswith("_s"))
    assert st["steps_wait_s"] > 0.0
    for jid, sc in zip(ids, scs):
        assert srv.result(jid)[0].tobytes() == alone(sc).tobytes()
