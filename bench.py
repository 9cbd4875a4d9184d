"""Benchmark: particle-steps/s of the SPH step on the 1,048,576-particle dam
break (FP32), through the engine's C ABI, plus the batched and served forms.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload dam_break_1m|dam_break_16k|pool_drop_8m|batched|served]
                    [--dt SECONDS] [--exact]

One JSON line on stdout (rank 0).  A "step" is one SPH step of the whole
scene: density, force/integrate, scan, scatter, gather.  The device-resident
value is timed with CUDA events on the engine's stream, one step at a time,
with L2 flushed (256 MiB write) before each timed step; e2e repeats the step
through the C ABI with the particle state copied in from pinned host memory
and read back each step.  The scenes run at their configured step of 1e-4 s
unless --dt says otherwise; at the 1M and 8M scenes' smoothing radii that
step makes the viscosity term diverge within tens of steps (in the
reference's arithmetic too), so the timed window covers the onset of the
divergence.  With --gpus N (torchrun) every rank advances its own
replica of the scene (the path does not shard); value = all ranks' particle-
steps / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0
STAGES = ["density", "force", "scan", "scatter", "gather"]


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", HBM_FALLBACK_GBS)), "measured"
    return HBM_FALLBACK_GBS, "fallback"


def workload_scene(name: str, steps: int, dt=None):
    """The named scene; ``dt`` replaces its time step when given (the
    configured 1e-4 s diverges at the 1M and 8M scenes' h; scenes.STABLE_DT
    holds the stable steps)."""
    from sphfluidsimulation_gb300 import scenes
    if name == "dam_break_1m":
        sc = scenes.config1(steps)
    elif name == "dam_break_16k":
        sc = scenes.config0(steps)
    elif name == "pool_drop_8m":
        sc = scenes.config2(steps)
    else:
        raise ValueError(name)
    if dt is not None:
        sc.dt = float(dt)
    return sc


def alg_bytes(stage: str, n: int, s: int) -> float:
    """Algorithmic bytes per launch: each array read or written once in the
    reference data flow with 2n buckets (per particle: density 28 B, force
    68 B, scan 16 B, scatter 16 B, gather counted as the scatter's move 16 B;
    static particles 20 B each per neighbour pass)."""
    per = {"density": 28.0, "force": 68.0, "scan": 16.0, "scatter": 16.0, "gather": 16.0}[stage]
    extra = 20.0 * s if stage in ("density", "force") else 0.0
    return per * n + extra


def _nvtx(name):
    """Pushes (name) or pops (None) an NVTX range; a profiler marker only."""
    import torch
    try:
        if name is None:
            torch.cuda.nvtx.range_pop()
        else:
            torch.cuda.nvtx.range_push(name)
    except Exception:
        pass


def pair_rates(samples, stage_ms, first_step: int):
    """Candidate tests and in-range pairs per particle (means of
    sph_engine_neighbour_stats samples over the stage-timing steps) and the
    rates they imply.  The default density pass (the group walk) tests each
    particle against every member of its cell's 27 buckets,
    `group_candidates`, spending `group_lane_slots` lane-slots (32 per
    ballot round); the per-slot walk (launch shape 5) would test the
    `candidates` of the cells it does not skip, spending `warp_slots`.
    Force evaluates the in-range pairs."""
    if not samples:
        return None
    mean = {k: float(np.mean([s[k] for s in samples])) for k in samples[0]}
    n = max(mean["particles"], 1.0)
    dens_s = float(stage_ms[STAGES.index("density")]) * 1e-3
    force_s = float(stage_ms[STAGES.index("force")]) * 1e-3
    in_range = mean["neighbours"] + mean["static_neighbours"]
    gc = mean.get("group_candidates", 0.0)
    return {
        "group_candidates_per_particle": gc / n,
        "group_lane_slots_per_particle": mean.get("group_lane_slots", 0.0) / n,
        "group_lane_slots_per_candidate": mean.get("group_lane_slots", 0.0) / gc if gc else None,
        "group_fallback_fraction": mean.get("group_fallback", 0.0) / n,
        "slot_walk_candidates_per_particle": mean["candidates"] / n,
        "slot_walk_warp_slots_per_particle": mean["warp_slots"] / n,
        "neighbours_per_particle": mean["neighbours"] / n,
        "static_neighbours_per_particle": mean["static_neighbours"] / n,
        "density_candidate_tests_per_s": gc / dens_s if dens_s > 0 else None,
        "force_pair_evals_per_s": in_range / force_s if force_s > 0 else None,
        "steps_sampled": f"{first_step}..{first_step + len(samples) - 1}, every step (the timed window)",
    }


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 25 ms (the timed
    region of the default run lasts a few tens of ms)."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, value: float, local: int) -> float:
    from sphfluidsimulation_gb300 import replicas
    return replicas.reduce_scalar(pg, value, "max")


# ---------------------------------------------------------------------------
# CPU baseline (the oracle port of the reference CPU engine, threaded)
# ---------------------------------------------------------------------------

def cpu_baseline(scene, warmup: int, steps: int, threads: int, max_s: float = 60.0):
    """The oracle port of the reference CPU engine on `threads` host threads,
    over the GPU arm's window: `warmup` untimed steps, then one update() call
    over the next `steps` steps, timed.  If one step costs so much that the
    window would take more than `max_s` seconds, fewer steps are timed (the
    sample says so).  Returns (particle-steps/s, seconds, steps timed)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle
    o = Oracle(threads)
    o.init(scene)
    t0 = time.perf_counter()
    o.update(scene.dt, max(1, warmup))
    per_step = max((time.perf_counter() - t0) / max(1, warmup), 1e-6)
    timed = max(1, min(steps, int(max_s / per_step)))
    t0 = time.perf_counter()
    o.update(scene.dt, timed)
    dt = time.perf_counter() - t0
    return scene.n * timed / dt, dt, timed


def run_reference(args):
    world, rank, local, pg = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0, None
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    scene = workload_scene(args.workload if args.workload not in ("batched", "served") else "dam_break_1m", 1,
                           args.dt)
    # the GPU arm's window: W untimed warm-up steps, then K timed steps in
    # one update() call (capped at about a minute of CPU work)
    warm = args.warmup
    value, secs, steps = cpu_baseline(scene, warm, args.steps, threads)
    sample = (f"{scene.name}: {scene.n} particles, steps {warm + 1}..{warm + steps} timed after {warm} warm-up "
              f"steps, one update() call ({secs:.1f} s)")
    line = {
        "impl": "reference", "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
        "n_gpus": world, "steps": steps, "warmup": warm, "ms_per_step": 1000.0 * secs / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 dam break)",
        "config": {"workload": scene.name, "particles": scene.n, "static_particles": scene.s,
                   "h": scene.params.h, "dt": scene.dt},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm: the plain engine
# ---------------------------------------------------------------------------

def run_plain(args, world, rank, local, pg):
    import torch
    from sphfluidsimulation_gb300.engine import DYN_DTYPE, SimulationEngineCUDA

    torch.cuda.set_device(local)
    scene = workload_scene(args.workload, args.steps, args.dt)
    n, s = scene.n, scene.s
    eng = SimulationEngineCUDA(local)
    eng.initialize(scene)
    if args.exact:
        eng.set_exact(True)
    stream = torch.cuda.ExternalStream(eng.stream_handle(), device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    # warm-up (also builds the step graph), then a device checkpoint: every
    # measurement below replays the same steps W+1..W+K from it, bit for bit
    eng.update(scene.dt, args.warmup)
    if args.launch_shapes:            # fixed launch shapes (density, force), e.g. 5,0: the per-slot walk
        d_shape, f_shape = (int(x) for x in args.launch_shapes.split(","))
        eng.set_launch_shapes(d_shape, f_shape)
        launch = {"density_shape": d_shape, "force_shape": f_shape, "from": "--launch-shapes"}
    else:
        launch = eng.autotune(3)      # launch shapes of the two passes, timed on this state
    eng.save_state()
    issue_peak = fp32_issue_peak(local)

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    barrier(pg)
    torch.cuda.synchronize()
    clocks.start()
    wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()                       # L2 flush between timed steps
            starts[k].record(stream)
            eng.update_async(scene.dt, 1)
            ends[k].record(stream)
    eng.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    barrier(pg)
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_s = sum(step_ms) / 1000.0
    total_s = max_over_ranks(pg, total_s, local)
    value = world * n * args.steps / total_s

    # per-stage times over the same steps (events around each stage), and
    # the neighbour walk's counts at each of them.  The NVTX range
    # "stage_window" marks these launches for ncu (--nvtx --nvtx-include
    # "stage_window/"), so profiled counts describe the timed steps too.
    eng.restore_state()
    eng.set_timing(True)
    per_step = []
    _nvtx("stage_window")
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        eng.update(scene.dt, 1)
        per_step.append(eng.kernel_times().astype(np.float64))
    _nvtx(None)
    eng.set_timing(False)
    eng.restore_state()
    nstats = []
    for k in range(args.steps):
        nstats.append(eng.neighbour_stats())
        eng.update(scene.dt, 1)
    stage_ms = np.mean(np.asarray(per_step), axis=0)
    pairs = pair_rates(nstats, stage_ms, args.warmup + 1)
    dom = int(np.argmax(stage_ms))
    dom_name = STAGES[dom]
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes(dom_name, n, s) / (stage_ms[dom] * 1e-3) / 1e9
    traffic = profiled_traffic(dom_name, args.workload)

    # e2e through the C ABI with host buffers: upload state, one step, read back
    pinned_in = torch.empty(n * 32, dtype=torch.uint8, pin_memory=True)
    pinned_out = torch.empty(n * 32, dtype=torch.uint8, pin_memory=True)
    host_in = pinned_in.numpy().view(DYN_DTYPE)
    host_out = pinned_out.numpy().view(DYN_DTYPE)
    eng.read_dynamic(host_in)
    e2e_steps = max(1, min(args.steps, 10))
    barrier(pg)
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        eng.write_dynamic_async(host_in)     # queued: upload, re-sort,
        eng.update_async(scene.dt, 1)        # step, and the readback, which
        eng.read_dynamic(host_out)           # waits for all of it
        host_in, host_out = host_out, host_in
    e2e_s = max_over_ranks(pg, time.perf_counter() - t0, local)
    e2e_value = world * n * e2e_steps / e2e_s

    render_line = None
    if not args.no_forms and rank == 0:
        render_line = time_render(eng, scene)

    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 dam break, reference generators)",
        "config": {"workload": scene.name, "particles": n, "static_particles": s, "h": scene.params.h,
                   "dt": scene.dt, "buckets": 2 * n, "l2": "flushed (256 MiB write) before every timed step",
                   "arithmetic": "exact (the reference's operations)" if args.exact else "fast (fused)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "stage_ms": dict(zip(STAGES, [round(float(x), 5) for x in stage_ms])),
        "stage_ms_window": (f"steps {args.warmup + 1}..{args.warmup + args.steps}, replayed from a device "
                            "checkpoint: the same steps as value, mean per stage"),
        "stage_sum_ms": round(float(np.sum(stage_ms)), 5),
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                     "alg_bytes_per_launch": alg_bytes(dom_name, n, s)},
        "pairs": pairs,
        "launch": launch,
        "issue_roofline": issue_roofline(dom_name, args.workload, float(stage_ms[dom]), issue_peak,
                                         float(clk.get("sm_mhz") or 0.0) if isinstance(clk, dict) else 0.0),
        "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": 32 * n,
                "d2h_bytes_per_step": 32 * n, "steps": e2e_steps},
        # per step: density, force, overflow force (which also clears the
        # scan's look-back state), scan, scatter, gather
        "gpu_launches": 6 * args.steps,
        "clocks": clk,
        "wall_s_timed_region": wall,
    }
    if render_line is not None:
        line["render"] = render_line
    return line, scene


def time_render(eng, scene, width: int = 1920, height: int = 1080, frames: int = 5):
    """Headless splat frames of the current state at 1080p with the reference
    application's layers (dynamic 0.1, static 0.03; 120 degree field of view):
    the box scaled to 5 times its size by the model matrix and seen from 8
    units, so it fills most of the frame.  Wall time per sph_engine_render
    call, which includes copying the RGBA8 and depth images to the host."""
    import math
    from sphfluidsimulation_gb300 import render
    lo = scene.static_pos.min(0) if scene.s else scene.dyn_pos.min(0)
    hi = scene.static_pos.max(0) if scene.s else scene.dyn_pos.max(0)
    centre = 5.0 * (lo + hi) / 2.0
    eye = centre + np.array([0.0, 3.0, 7.4])
    view = render.look_at(eye, centre)
    proj = render.perspective(math.radians(120.0), width / height, 0.1, 1000.0)
    model = np.diag([5.0, 5.0, 5.0, 1.0]).astype(np.float32).reshape(16)
    rgba, _ = eng.render(proj, view, model, width, height)   # warm-up, allocates the targets
    t0 = time.perf_counter()
    for _ in range(frames):
        rgba, _ = eng.render(proj, view, model, width, height)
    ms = 1000.0 * (time.perf_counter() - t0) / frames
    return {"width": width, "height": height, "particles": scene.n + scene.s, "frames": frames,
            "ms_per_frame": ms, "covered_pixels": int((rgba[..., 3] > 0).sum()),
            "d2h_bytes_per_frame": width * height * 8,
            "camera": "box x5, eye 8 units off its centre, fov 120 deg, sizes 0.1 / 0.03"}


def profiled_traffic(stage: str, workload: str, column: int = 2):
    """A per-launch figure of the kernel from the committed ncu summary
    (profiles/ncu_traffic.txt, lines "workload stage dram_bytes
    warp_instructions"): column 2 the DRAM bytes, column 3 the warp
    instructions."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for ln in f:
            parts = ln.split()
            if len(parts) > column and parts[0] == workload and parts[1] == stage:
                try:
                    return float(parts[column])
                except ValueError:
                    return None
    return None


def fp32_issue_peak(device: int):
    """The GPU's FP32 issue rate, measured now by the library's FMA
    microbenchmark (sph_probe_fp32_issue): warp FMA instructions per second
    with every SM fully occupied."""
    import ctypes as C
    from sphfluidsimulation_gb300 import _lib
    rate, ms = C.c_double(), C.c_float()
    _lib.check(_lib.load().sph_probe_fp32_issue(int(device), C.byref(rate), C.byref(ms)), "sph_probe_fp32_issue")
    return {"warp_instructions_per_s": rate.value, "probe_ms": ms.value}


def issue_roofline(stage: str, workload: str, stage_ms: float, probe, sm_mhz: float):
    """The bound the neighbour passes actually meet: warp instructions per
    launch (ncu smsp__inst_executed.sum, mean over the same steps, committed
    in profiles/ncu_traffic.txt) over the live launch time, against the
    FP32 issue rate measured by the FMA probe in this run.  The nominal
    152 SMs x 4 schedulers x the sampled clock is given beside it."""
    inst = profiled_traffic(stage, workload, 3)
    if inst is None or not probe:
        return None
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    achieved = inst / (stage_ms * 1e-3)
    peak = probe["warp_instructions_per_s"]
    out = {"kernel": stage, "achieved": achieved, "peak": peak, "unit": "warp instructions/s",
           "frac": achieved / peak, "warp_instructions_per_launch": inst,
           "instructions_window": "ncu mean over steps 6..25 of --steps 20 --warmup 5 (profiles/ncu_traffic.txt)",
           "peak_basis": "measured: FP32 FMA microbenchmark (sph_probe_fp32_issue) in this run",
           "probe_ms": probe["probe_ms"]}
    if sm_mhz:
        out["nominal_peak"] = sms * 4 * sm_mhz * 1e6
        out["nominal_basis"] = f"{sms} SMs x 4 schedulers x {sm_mhz:.0f} MHz (sampled)"
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)     # steps 6..25: the window of profiles/ncu_traffic.txt
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="dam_break_1m",
                    choices=["dam_break_1m", "dam_break_16k", "pool_drop_8m", "batched", "served"])
    ap.add_argument("--dt", type=float, default=None,
                    help="time step in s (default: the workload's configured 1e-4)")
    ap.add_argument("--exact", action="store_true",
                    help="time the reference's arithmetic (sph_engine_set_exact) instead of the fused form")
    ap.add_argument("--served-jobs", type=int, default=2000,
                    help="served sample (default line and --workload served): jobs taken from the 2,000-job mix")
    ap.add_argument("--served-horizon-scale", type=float, default=0.1,
                    help="served sample: factor on every job's horizon")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--launch-shapes", default=None,
                    help="density,force launch shapes instead of the autotuner's (sph_engine_set_launch_shapes)")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the bounded batched/served samples in the default line")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    from sphfluidsimulation_gb300 import build
    world, rank, local, pg = dist_setup(args)
    if local == 0:
        build.build()
    barrier(pg)                      # the other ranks load what local rank 0 built
    if args.workload in ("batched", "served"):
        from sphfluidsimulation_gb300 import bench_forms
        line = bench_forms.run(args, world, rank, local, pg)
        scene = None
    else:
        line, scene = run_plain(args, world, rank, local, pg)
    if rank == 0 and scene is not None and not args.no_forms and world == 1:
        # bounded samples of the two production forms on the same GPU
        from sphfluidsimulation_gb300 import bench_forms
        b = bench_forms.run_batched(min(args.steps, 20))
        line["batched"] = {k: b[k] for k in ("scenes", "particles", "steps", "batched_particle_steps_per_s",
                                             "plain_looped_particle_steps_per_s", "speedup", "mode", "launch")}
        sv = bench_forms.run_served(n_jobs=args.served_jobs, horizon_scale=args.served_horizon_scale)
        line["served"] = {k: sv[k] for k in ("jobs", "horizon_scale", "served_particle_steps_per_s",
                                             "fifo_plain_particle_steps_per_s", "speedup", "served_latency",
                                             "fifo_latency", "load_vs_fifo_capacity", "served_poll_phases",
                                             "served_makespan_s", "fifo_makespan_s")}
        line["served"]["sample"] = (f"{args.served_jobs} jobs of the 2,000-job mix (Poisson stream), horizons "
                                    f"x{args.served_horizon_scale:g}; --served-jobs / --served-horizon-scale change it")
    if rank == 0:
        if scene is not None and not args.no_cpu_baseline and world == 1:
            threads = os.cpu_count() or 1
            v, secs, steps = cpu_baseline(scene, args.warmup, args.steps, threads)
            line["cpu_baseline"] = {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                                    "sample": f"{scene.name}: {scene.n} particles, steps {args.warmup + 1}.."
                                              f"{args.warmup + steps} after {args.warmup} warm-up steps "
                                              f"({secs:.1f} s), oracle port of the reference CPU engine"}
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
