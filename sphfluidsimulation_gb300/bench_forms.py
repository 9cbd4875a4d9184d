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

from . import scenes
from .engine import Batch, Server, SimulationEngineCUDA


def _percentiles(lat: List[float]) -> Dict[str, float]:
    a = np.asarray(lat, np.float64)
    return {"p50_s": float(np.percentile(a, 50)), "p95_s": float(np.percentile(a, 95)),
            "p99_s": float(np.percentile(a, 99)), "mean_s": float(a.mean())}


def run_batched(steps: int, count: int = 96, seed: int = 0, mode: int = -1) -> Dict:
    scs = scenes.batched_scenes(count=count, seed=seed, steps=steps)
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
    b.step(2)                                   # warm-up
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
    t0 = time.perf_counter()
    for e, sc in zip(engines, scs):
        e.update(sc.dt, steps)
    tp = time.perf_counter() - t0
    for e in engines:
        e.close()
    return {"scenes": count, "particles": total, "steps": steps,
            "batched_particle_steps_per_s": total * steps / tb, "plain_looped_particle_steps_per_s": total * steps / tp,
            "speedup": tp / tb, "batched_ms_per_step": 1e3 * tb / steps, "plain_looped_ms_per_step": 1e3 * tp / steps,
            "persistent_grid": [grid, thr],
            "mode": ("autotuned " if chosen else "") + ("persistent" if (chosen[0] if chosen else mode) == 0 else "staged"),
            "autotune_ms_per_step": chosen[2] if chosen else None}


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


def _served(jobset, arrivals, budget: int, slots: int, chunk: int):
    """Continuous batching.  Returns (makespan, latencies)."""
    srv = Server(budget_bytes=budget, max_slots=slots)
    clock = 0.0
    lat = [None] * len(jobset)
    in_flight = {}
    k = 0
    n = len(jobset)
    finished = 0
    while finished < n:
        while k < n and arrivals[k] <= clock:
            in_flight[srv.submit(jobset[k][1], steps=jobset[k][0].steps)] = k
            k += 1
        if not in_flight:
            clock = max(clock, arrivals[k])    # idle until the next arrival
            continue
        t0 = time.perf_counter()
        srv.poll(chunk)
        done = [jid for jid in in_flight if srv.result(jid) is not None]
        clock += time.perf_counter() - t0
        for jid in done:
            idx = in_flight.pop(jid)
            lat[idx] = clock - arrivals[idx]
            finished += 1
    srv.close()
    return clock, lat


def run_served(n_jobs: int = 200, horizon_scale: float = 0.1, seed: int = 0, budget: int = 120 << 30,
               slots: int = 128, chunk: int = 50) -> Dict:
    jobset = _job_set(n_jobs, horizon_scale, seed)
    work = sum(j.n * j.steps for j, _ in jobset)
    zeros = [0.0] * n_jobs
    # warm-up both paths on the first small job
    _fifo(jobset[:1])
    _served(jobset[:1], [0.0], budget, slots, chunk)
    fifo_span, _ = _fifo(jobset)
    srv_span, srv_lat_closed = _served(jobset, zeros, budget, slots, chunk)
    cap_fifo = work / fifo_span
    # Poisson arrivals at 80 % of the FIFO plain capacity
    mean_work = work / n_jobs
    rate = 0.8 * cap_fifo / mean_work
    rng = scenes.SplitMix64(seed ^ 0xA77)
    u = rng.uniform(n_jobs).astype(np.float64)
    arrivals = list(np.cumsum(-np.log(np.maximum(1e-12, 1.0 - u)) / rate))
    fifo_span2, fifo_lat = _fifo(jobset, arrivals)
    srv_span2, srv_lat = _served(jobset, arrivals, budget, slots, chunk)
    return {"jobs": n_jobs, "horizon_scale": horizon_scale, "particle_steps": work,
            "served_particle_steps_per_s": work / srv_span, "fifo_plain_particle_steps_per_s": cap_fifo,
            "speedup": fifo_span / srv_span, "arrival_rate_per_s": rate, "load_vs_fifo_capacity": 0.8,
            "served_latency": _percentiles(srv_lat), "fifo_latency": _percentiles(fifo_lat),
            "budget_bytes": budget, "slots": slots, "chunk_steps": chunk}


def run(args, world, rank, local, pg) -> Dict:
    """--workload batched|served: one JSON line in the bench contract."""
    if args.workload == "batched":
        r = run_batched(args.steps)
        return {"metric": "aggregate particle-steps/s, 96 batched dam breaks", "value": r["batched_particle_steps_per_s"],
                "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": r["batched_ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam breaks)",
                "config": {"workload": "batched_96", "particles": r["particles"]}, "batched": r,
                "gpu_launches": args.steps}
    r = run_served()
    return {"metric": "aggregate particle-steps/s, served jobs", "value": r["served_particle_steps_per_s"],
            "unit": "particle-steps/s", "n_gpus": world, "steps": None, "warmup": 1,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded dam-break jobs, Poisson arrivals)",
            "config": {"workload": "served", "jobs": r["jobs"], "horizon_scale": r["horizon_scale"]}, "served": r}
