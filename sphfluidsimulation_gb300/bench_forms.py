"""Batched and served forms of the SPH step, measured against the plain
engine on the same GPU.

batched: the 96 independent dam breaks (N log-uniform in [4096, 131072]) are
advanced together, one persistent launch per step, and compared with the
plain engine advancing the same scenes one scene at a time.

served: jobs (N log-uniform in [8192, 1048576], horizon uniform) are
(1) all submitted at once to measure aggregate throughput (total particle
steps / makespan) of the server against FIFO one-at-a-time plain runs, and
(2) submitted as a Poisson stream at 80 % of the FIFO plain engine's measured
capacity to measure job latency (p50/p95/p99) for both.  Latency runs use a
clock that advances by the measured wall time of each scheduling round and
jumps over idle gaps, so no GPU time is spent waiting for arrivals.
"""
from __future__ import annotations

import math
import time
from typing import Dict, List

import numpy as np

from . import replicas, scenes
from .engine import Batch, Server, SimulationEngineCUDA


def _percentiles(lat: List[float]) -> Dict[str, float]:
    a = np.asarray(lat, np.float64)
    return {"p50_s": float(np.percentile(a, 50)), "p95_s": float(np.percentile(a, 95)),
            "p99_s": float(np.percentile(a, 99)), "mean_s": float(a.mean())}


def _barrier(pg):
    if pg is not None:
        pg.barrier()


def run_batched(steps: int, count: int = 96, seed: int = 0, mode: int = -1, pg=None, world: int = 1,
                rank: int = 0) -> Dict:
    """With world > 1 each rank batches its share of the scenes (split by
    footprint) and the rates are whole-job aggregates."""
    all_scs = scenes.batched_scenes(count=count, seed=seed, steps=steps)
    scs = replicas.rank_share(all_scs, [replicas.footprint_bytes(sc.n, sc.s) for sc in all_scs], world, rank)
    total = sum(sc.n for sc in scs)
    b = Batch()
    for sc in scs:
        b.add_scene(sc)
    b.finalize()
    if mode < 0:
        chosen = b.autotune(3)                  # picks staged graph or persistent grid size
    else:
        b.set_mode(mode)
        chosen = None
    launch = b.launch_config()
    b.step(2)                                   # warm-up
    _barrier(pg)
    t0 = time.perf_counter()
    b.step(steps)
    tb = time.perf_counter() - t0
    _, grid, thr = b.info()
    b.close()
    # plain engine, one scene at a time (each scene advanced `steps` steps)
    engines = []
    for sc in scs:
        e = SimulationEngineCUDA()
        e.initialize(sc)
        e.update(sc.dt, 2)                      # warm-up, builds each step graph
        engines.append(e)
    _barrier(pg)
    t0 = time.perf_counter()
    for e, sc in zip(engines, scs):
        e.update(sc.dt, steps)
    tp = time.perf_counter() - t0
    for e in engines:
        e.close()
    batched_rate = replicas.aggregate_rate(pg, total * steps, tb)
    plain_rate = replicas.aggregate_rate(pg, total * steps, tp)
    tb, tp = replicas.reduce_scalar(pg, tb), replicas.reduce_scalar(pg, tp)
    total = int(replicas.reduce_scalar(pg, total, "sum"))
    return {"scenes": count, "particles": total, "steps": steps, "ranks": world,
            "batched_particle_steps_per_s": batched_rate, "plain_looped_particle_steps_per_s": plain_rate,
            "speedup": batched_rate / plain_rate, "batched_ms_per_step": 1e3 * tb / steps,
            "plain_looped_ms_per_step": 1e3 * tp / steps,
            "persistent_grid": [grid, thr],
            "mode": ("autotuned " if chosen else "") + ("persistent" if (chosen[0] if chosen else mode) == 0 else "staged"),
            "autotune_ms_per_step": chosen[2] if chosen else None, "launch": launch}


def _job_set(n_jobs: int, horizon_scale: float, seed: int):
    jobs = scenes.serving_jobs(count=n_jobs, seed=seed)
    out = []
    for j in jobs:
        j.steps = max(1, int(round(j.steps * horizon_scale)))
        out.append((j, scenes.job_scene(j)))
    return out


def _fifo(jobset, arrivals=None):
    """FIFO one-at-a-time plain engine.  Returns (makespan, latencies)."""
    clock = 0.0
    lat = []
    e = SimulationEngineCUDA()
    for k, (j, sc) in enumerate(jobset):
        arr = 0.0 if arrivals is None else arrivals[k]
        clock = max(clock, arr)
        t0 = time.perf_counter()
        e.initialize(sc)
        e.update(sc.dt, j.steps)
        e.read_dynamic()
        clock += time.perf_counter() - t0
        lat.append(clock - arr)
    e.close()
    return clock, lat


def _served(jobset, arrivals, budget: int, slots: int, chunk: int, phases=None):
    """Continuous batching.  Returns (makespan, latencies); `phases`, when
    given, receives the server's poll-phase breakdown (sph_server_stats)."""
    srv = Server(budget_bytes=budget, max_slots=slots)
    clock = 0.0
    lat = [None] * len(jobset)
    in_flight = {}
    k = 0
    n = len(jobset)
    finished = 0
    while finished < n:
        t0 = time.perf_counter()                # submission (the job's copy) is timed too
        while k < n and arrivals[k] <= clock:
            in_flight[srv.submit(jobset[k][1], steps=jobset[k][0].steps)] = k
            k += 1
        if not in_flight:
            clock = max(clock, arrivals[k])    # idle until the next arrival
            continue
        srv.poll(chunk)
        done = srv.finished()                  # only the retired jobs are fetched
        for jid in done:
            srv.result(jid)
        clock += time.perf_counter() - t0
        for jid in done:
            idx = in_flight.pop(jid)
            lat[idx] = clock - arrivals[idx]
            finished += 1
    if phases is not None:
        phases.update(srv.stats())
    srv.close()
    return clock, lat


def run_served(n_jobs: int = 200, horizon_scale: float = 0.1, seed: int = 0, budget: int = 120 << 30,
               slots: int = 128, chunk: int = 50, pg=None, world: int = 1, rank: int = 0) -> Dict:
    """With world > 1 each rank serves its share of the jobs (split by
    footprint) on its own GPU: throughput is the whole-job aggregate and the
    latency percentiles are over every rank's jobs."""
    full = _job_set(n_jobs, horizon_scale, seed)
    jobset = replicas.rank_share(full, [Server.job_bytes(sc.n, sc.s) for _, sc in full], world, rank)
    n_jobs_all, n_jobs = n_jobs, len(jobset)
    work = sum(j.n * j.steps for j, _ in jobset)
    zeros = [0.0] * n_jobs
    # warm-up both paths on the first small job
    _fifo(jobset[:1])
    _served(jobset[:1], [0.0], budget, slots, chunk)
    _barrier(pg)
    fifo_span, _ = _fifo(jobset)
    _barrier(pg)
    phases = {}
    srv_span, srv_lat_closed = _served(jobset, zeros, budget, slots, chunk, phases)
    cap_fifo = work / fifo_span
    # Poisson arrivals at 80 % of the FIFO plain capacity
    mean_work = work / n_jobs
    rate = 0.8 * cap_fifo / mean_work
    rng = scenes.SplitMix64((seed ^ 0xA77) + 7919 * rank)
    u = rng.uniform(n_jobs).astype(np.float64)
    arrivals = list(np.cumsum(-np.log(np.maximum(1e-12, 1.0 - u)) / rate))
    fifo_span2, fifo_lat = _fifo(jobset, arrivals)
    srv_span2, srv_lat = _served(jobset, arrivals, budget, slots, chunk)
    served_rate = replicas.aggregate_rate(pg, work, srv_span)
    fifo_rate = replicas.aggregate_rate(pg, work, fifo_span)
    srv_lat, fifo_lat = replicas.gather_values(pg, srv_lat), replicas.gather_values(pg, fifo_lat)
    work = replicas.reduce_scalar(pg, work, "sum")
    return {"jobs": n_jobs_all, "ranks": world, "horizon_scale": horizon_scale, "particle_steps": work,
            "served_particle_steps_per_s": served_rate, "fifo_plain_particle_steps_per_s": fifo_rate,
            "speedup": served_rate / fifo_rate, "arrival_rate_per_s": rate, "load_vs_fifo_capacity": 0.8,
            "served_latency": _percentiles(srv_lat), "fifo_latency": _percentiles(fifo_lat),
            "budget_bytes": budget, "slots": slots, "chunk_steps": chunk,
            "served_poll_phases": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in phases.items()},
            "served_makespan_s": srv_span, "fifo_makespan_s": fifo_span}


def run(args, world, rank, local, pg) -> Dict:
    """--workload batched|served: one JSON line in the bench contract."""
    if args.workload == "batched":
        r = run_batched(args.steps, pg=pg, world=world, rank=rank)
        return {"metric": "aggregate particle-steps/s, 96 batched dam breaks", "value": r["batched_particle_steps_per_s"],
                "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": r["batched_ms_per_step"], "higher_is_better": True, "scaling": "strong",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam breaks)",
                "config": {"workload": "batched_96", "particles": r["particles"]}, "batched": r,
                "gpu_launches": args.steps}
    r = run_served(n_jobs=getattr(args, "served_jobs", 2000), horizon_scale=getattr(args, "served_horizon_scale", 0.1),
                   pg=pg, world=world, rank=rank)
    return {"metric": "aggregate particle-steps/s, served jobs", "value": r["served_particle_steps_per_s"],
            "unit": "particle-steps/s", "n_gpus": world, "steps": None, "warmup": 1,
            "ms_per_step": None, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded dam-break jobs, Poisson arrivals)",
            "config": {"workload": "served", "jobs": r["jobs"], "horizon_scale": r["horizon_scale"]}, "served": r}
