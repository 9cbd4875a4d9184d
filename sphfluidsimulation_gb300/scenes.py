"""Seeded synthetic scenes: the dam-break, pool-plus-drop, batched and served
workloads, plus the reference's own particle-set generators.

The reference builds scenes from JSON "particle set blueprints"
(SPHFluidSimulation/source/SPH/Core/SceneBlueprint.cpp:134-183):

* ``FilledBox`` (SPHFluidSimulation/source/SPH/ParticleSetBlueprints/
  FilledBoxParticleSetBlueprint.cpp:38-66) -- a lattice, i over x outermost,
  k over z innermost, position ``(i, j, k) * d + d/2 + offset`` plus jitter;
* ``BoxShell`` (BoxShellParticleSetBlueprint.cpp:41-116) -- the six faces,
  twelve edges and eight corners of a box at spacing ``d``, in that order.

Both draw jitter from the Blaze Engine's ``Random``, which is not available and
not pinned, so every random draw here comes from SplitMix64 (Steele, Lea and
Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014) seeded
explicitly.  All position arithmetic is float32, as in the reference.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


class SplitMix64:
    """Counter-based SplitMix64 stream; ``uniform(n)`` returns float32 in [0, 1)
    built from the top 24 bits of each output."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)

    def next_u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            idx = np.arange(1, n + 1, dtype=np.uint64)
            z = self.state + idx * _GAMMA
            self.state = self.state + np.uint64(n) * _GAMMA
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            z = z ^ (z >> np.uint64(31))
        return z

    def uniform(self, n: int) -> np.ndarray:
        bits = (self.next_u64(n) >> np.uint64(40)).astype(np.float64)
        return (bits * (1.0 / (1 << 24))).astype(np.float32)

    def uniform_pm1(self, n: int) -> np.ndarray:
        """Uniform in [-1, 1) as float32 (the FilledBox ``Random::Float(-1, 1)``)."""
        u = self.uniform(n)
        return (u * np.float32(2.0) - np.float32(1.0)).astype(np.float32)


@dataclasses.dataclass
class Params:
    """The scene's ``particleBehaviourParameters`` (SceneBlueprint.cpp:15-33)."""

    particle_mass: float
    gas_constant: float
    elasticity: float
    viscosity: float
    gravity: Tuple[float, float, float]
    rest_density: float
    h: float  # maxInteractionDistance

    def as9(self) -> np.ndarray:
        g = self.gravity
        return np.array([self.particle_mass, self.gas_constant, self.elasticity, self.viscosity,
                         g[0], g[1], g[2], self.rest_density, self.h], dtype=np.float32)


@dataclasses.dataclass
class Scene:
    name: str
    dyn_pos: np.ndarray            # (N, 3) float32
    static_pos: np.ndarray         # (S, 3) float32
    params: Params
    dt: float
    steps: int
    triangles: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 9), np.float32))
    dyn_vel: Optional[np.ndarray] = None
    reorder_interval: float = float(np.finfo(np.float32).max)
    other_parameters: dict = dataclasses.field(default_factory=dict)   # the scene file's otherParameters

    @property
    def n(self) -> int:
        return int(self.dyn_pos.shape[0])

    @property
    def s(self) -> int:
        return int(self.static_pos.shape[0])


def filled_box(counts: Sequence[int], spacing: float, offset: Sequence[float], jitter: float,
               rng: Optional[SplitMix64], limit: Optional[int] = None) -> np.ndarray:
    """Lattice ``counts`` = (nx, ny, nz) at ``spacing``; x outermost, z innermost
    (FilledBoxParticleSetBlueprint.cpp:51-64).  Jitter is uniform in
    +-``jitter`` x spacing per axis.  ``limit`` truncates the lattice in that
    order (a partly filled top layer)."""
    nx, ny, nz = (int(c) for c in counts)
    d = np.float32(spacing)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    idx = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float32)
    if limit is not None:
        idx = idx[:limit]
    base = np.float32(spacing) / np.float32(2.0) + np.asarray(offset, np.float32)
    pos = (idx * d + base).astype(np.float32)
    if jitter and rng is not None:
        amp = np.float32(jitter) * d
        r = rng.uniform_pm1(pos.size).reshape(pos.shape)
        pos = (pos + r * amp).astype(np.float32)
    return pos


def box_shell(size: Sequence[float], spacing: float, offset: Sequence[float] = (0.0, 0.0, 0.0),
              intensity: float = 0.0, rng: Optional[SplitMix64] = None) -> np.ndarray:
    """Particles on the faces, edges and corners of a box, in the order of
    BoxShellParticleSetBlueprint.cpp:66-115; the count matches :27-39."""
    d = np.float32(spacing)
    g = (np.asarray(size, np.float32) / d).astype(np.uint64) + 1
    gx, gy, gz = (int(v) for v in g)
    fx, fy, fz = np.float32(gx - 1), np.float32(gy - 1), np.float32(gz - 1)
    pts: List[np.ndarray] = []

    def grid2(a, b):
        A, B = np.meshgrid(np.arange(1, a - 1), np.arange(1, b - 1), indexing="ij")
        return A.ravel().astype(np.float32), B.ravel().astype(np.float32)

    x, y = grid2(gx, gy)
    z0, z1 = np.zeros_like(x), np.full_like(x, fz)
    pts.append(np.stack([np.stack([x, y, z0], 1), np.stack([x, y, z1], 1)], 1).reshape(-1, 3))
    x, z = grid2(gx, gz)
    y0, y1 = np.zeros_like(x), np.full_like(x, fy)
    pts.append(np.stack([np.stack([x, y0, z], 1), np.stack([x, y1, z], 1)], 1).reshape(-1, 3))
    y, z = grid2(gy, gz)
    x0, x1 = np.zeros_like(y), np.full_like(y, fx)
    pts.append(np.stack([np.stack([x0, y, z], 1), np.stack([x1, y, z], 1)], 1).reshape(-1, 3))
    x = np.arange(1, gx - 1, dtype=np.float32)
    o = np.zeros_like(x)
    pts.append(np.stack([np.stack([x, o, o], 1), np.stack([x, o + fy, o], 1),
                         np.stack([x, o, o + fz], 1), np.stack([x, o + fy, o + fz], 1)], 1).reshape(-1, 3))
    y = np.arange(1, gy - 1, dtype=np.float32)
    o = np.zeros_like(y)
    pts.append(np.stack([np.stack([o, y, o], 1), np.stack([o + fx, y, o], 1),
                         np.stack([o, y, o + fz], 1), np.stack([o + fx, y, o + fz], 1)], 1).reshape(-1, 3))
    z = np.arange(1, gz - 1, dtype=np.float32)
    o = np.zeros_like(z)
    pts.append(np.stack([np.stack([o, o, z], 1), np.stack([o + fx, o, z], 1),
                         np.stack([o, o + fy, z], 1), np.stack([o + fx, o + fy, z], 1)], 1).reshape(-1, 3))
    corners = np.array([[0, 0, 0], [fx, 0, 0], [0, fy, 0], [fx, fy, 0],
                        [0, 0, fz], [fx, 0, fz], [0, fy, fz], [fx, fy, fz]], np.float32)
    pts.append(corners)
    lat = np.concatenate(pts, 0).astype(np.float32)
    pos = (lat * d).astype(np.float32)
    if intensity and rng is not None:
        r = rng.uniform(pos.size).reshape(pos.shape)
        pos = (pos + (r * np.float32(intensity)) * d).astype(np.float32)
    pos = (pos + np.asarray(offset, np.float32)).astype(np.float32)
    count = (gx * gy + gx * gz + gy * gz - 2 * gx - 2 * gy - 2 * gz + 4) * 2
    assert pos.shape[0] == count, (pos.shape, count)
    return pos


def water_params(spacing: float, h: float, mass: Optional[float] = None) -> Params:
    """Dam-break constants: rest density 1000, gas constant 200, viscosity 0.1,
    gravity -9.81 y; mass 1000 * spacing^3 unless given."""
    m = float(np.float32(1000.0) * np.float32(spacing) ** 3) if mass is None else mass
    return Params(particle_mass=m, gas_constant=200.0, elasticity=0.0, viscosity=0.1,
                  gravity=(0.0, -9.81, 0.0), rest_density=1000.0, h=h)


def dam_break(lattice: Sequence[int], spacing: float, h: float, box: Sequence[float],
              steps: int, seed: int = 0, mass: Optional[float] = None, name: str = "dam_break",
              dt: float = 1e-4, limit: Optional[int] = None) -> Scene:
    """A fluid block in the low corner of a walled box.  The walls are a
    static BoxShell at the lattice spacing."""
    rng = SplitMix64(seed)
    dyn = filled_box(lattice, spacing, (0.0, 0.0, 0.0), 0.1, rng, limit=limit)
    walls = box_shell(box, spacing)
    return Scene(name=name, dyn_pos=dyn, static_pos=walls, params=water_params(spacing, h, mass),
                 dt=dt, steps=steps)


def config0(steps: int = 200) -> Scene:
    """16,384 particles, spacing 0.02, h 0.04, mass 0.008.  The 32x32x16
    lattice is laid 32 (x) x 16 (y, vertical) x 32 (z); a 1.0 x 0.6 x 0.6 box
    cannot hold two 0.64 m sides, so the box is 1.0 x 0.6 x 0.7."""
    return dam_break((32, 16, 32), 0.02, 0.04, (1.0, 0.6, 0.7), steps, mass=0.008, name="dam_break_16k")


def config1(steps: int = 1000, dt: float = 1e-4) -> Scene:
    """1,048,576 particles: 128 (x) x 64 (y) x 128 (z) at 0.005, h 0.01, in a
    1.6 x 0.8 x 0.8 box (256,002 wall particles).  dt defaults to the
    dam-break 1e-4 s, which diverges at this h (see STABLE_DT)."""
    return dam_break((128, 64, 128), 0.005, 0.01, (1.6, 0.8, 0.8), steps, name="dam_break_1m", dt=dt)


def pool_drop(pool_lattice: Sequence[int], n_total: int, box: Sequence[float], steps: int,
              seed: int = 0, dt: float = 2.5e-5, spacing: float = 0.0025, h: float = 0.005,
              name: str = "pool_drop") -> Scene:
    """A pool lattice in the low corner of a walled box plus the lattice points
    nearest the centre of a sphere (n_total - pool particles of them, in x-y-z
    scan order) whose bottom is 0.3 m above the pool, centred over it.  Both
    carry the FilledBox jitter of +-0.1 spacing; water constants."""
    s = spacing
    rng = SplitMix64(seed)
    pool = filled_box(pool_lattice, s, (0.0, 0.0, 0.0), 0.1, rng)
    n_drop = int(n_total) - pool.shape[0]
    if n_drop < 1:
        raise ValueError("n_total must exceed the pool's particle count")
    radius = (3.0 * n_drop / (4.0 * math.pi)) ** (1.0 / 3.0)  # in lattice units
    r = int(math.ceil(radius)) + 2
    ax = np.arange(-r, r + 1)
    I, J, K = np.meshgrid(ax, ax, ax, indexing="ij")
    lat = np.stack([I.ravel(), J.ravel(), K.ravel()], 1)
    d2 = (lat.astype(np.int64) ** 2).sum(1)
    order = np.argsort(d2, kind="stable")[:n_drop]
    chosen = np.sort(order)  # back to x-y-z scan order
    lat = lat[chosen].astype(np.float32)
    px, py, pz = (float(np.float32(c * s)) for c in pool_lattice)
    centre = np.array([px / 2, py + 0.3 + radius * s, pz / 2], np.float32)
    drop = (lat * np.float32(s) + centre).astype(np.float32)
    drop = (drop + rng.uniform_pm1(drop.size).reshape(drop.shape) * np.float32(0.1 * s)).astype(np.float32)
    dyn = np.concatenate([pool, drop], 0)
    walls = box_shell(box, s)
    return Scene(name=name, dyn_pos=dyn, static_pos=walls, params=water_params(s, h), dt=dt, steps=steps)


# The explicit viscosity term bounds the step like h^2 / mu.  With mu = 0.1
# the dam-break dt of 1e-4 s is stable at h = 0.04 (configuration 0) but
# diverges at h = 0.01 (the 1M dam break: median speed 30 m/s by step 20)
# and at h = 0.005 (the 8M pool drop: every particle leaves its cell on every
# step from step 4), in the reference's arithmetic as in this engine's.
# These are the largest halvings of 1e-4 s that stay stable at those h,
# measured with the oracle (at h = 0.01, 1e-4 s with mu = 0 is stable too).
STABLE_DT = {"dam_break_1m": 5e-5, "pool_drop_8m": 2.5e-5}


def config2(steps: int = 500, seed: int = 0, dt: float = 1e-4) -> Scene:
    """8,388,608 particles: a 256 (x) x 112 (y) x 256 (z) pool at 0.0025 plus
    the 1,048,576 lattice points nearest the centre of a sphere whose bottom
    is 0.3 m above the pool; box 1.28 (x) x 1.28 (y) x 0.96 (z); h 0.005 and
    the dam-break constants.  dt defaults to the dam-break 1e-4 s, which
    diverges at this h (see STABLE_DT)."""
    return pool_drop((256, 112, 256), 8_388_608, (1.28, 1.28, 0.96), steps, seed=seed, dt=dt,
                     name="pool_drop_8m")


def debug_smallest_scene() -> Scene:
    """The reference's debugSmallestScene.json (FluidSimulationProject/assets/
    simulationScenes/debugSmallestScene.json:1-36): a 2x2x2 FilledBox at
    spacing 0.5 centred on the origin and a 2 m BoxShell at 0.2 with random
    offset intensity 1 (drawn from SplitMix64 seed 0 here)."""
    dyn = filled_box((2, 2, 2), 0.5, (-0.5, -0.5, -0.5), 0.0, None)
    walls = box_shell((2, 2, 2), 0.2, (-1, -1, -1), 1.0, SplitMix64(0))
    p = Params(particle_mass=1.0, gas_constant=200.0, elasticity=0.5, viscosity=0.5,
               gravity=(0.0, -9.81, 0.0), rest_density=7.0, h=1.0)
    return Scene(name="debug_smallest", dyn_pos=dyn, static_pos=walls, params=p, dt=0.01, steps=10,
                 reorder_interval=10000.0)


def batched_scenes(count: int = 96, seed: int = 0, steps: int = 500,
                   n_min: int = 4096, n_max: int = 131072) -> List[Scene]:
    """Independent dam breaks: N log-uniform in [n_min, n_max], block aspect
    (x:z over y) uniform in [0.5, 2], spacing 0.01, h 0.02, mass 1000 s^3; the
    box is proportional to the block (2x wide, 1.5x high, 2x deep)."""
    rng = SplitMix64(seed)
    u = rng.uniform(2 * count).astype(np.float64).reshape(count, 2)
    scenes = []
    s, h = 0.01, 0.02
    for q in range(count):
        n = int(round(math.exp(math.log(n_min) + u[q, 0] * (math.log(n_max) - math.log(n_min)))))
        aspect = 0.5 + 1.5 * u[q, 1]
        ny = max(2, int(round((n / aspect ** 2) ** (1.0 / 3.0))))
        nx = max(2, int(math.ceil(math.sqrt(n / ny))))
        nz = max(2, int(math.ceil(n / (nx * ny))))
        lx, ly, lz = nx * s, ny * s, nz * s
        box = (2.0 * lx + 2 * s, 1.5 * ly + 2 * s, 2.0 * lz + 2 * s)
        sc = dam_break((nx, ny, nz), s, h, box, steps, seed=seed * 1000 + q + 1, limit=n,
                       name=f"batched_{q}")
        sc.dyn_pos = (sc.dyn_pos + np.float32(s)).astype(np.float32)  # one spacing off the walls
        scenes.append(sc)
    return scenes


@dataclasses.dataclass
class Job:
    job_id: int
    arrival_s: float
    n: int
    steps: int
    seed: int


def serving_jobs(count: int = 2000, seed: int = 0, n_min: int = 8192, n_max: int = 1_048_576,
                 steps_min: int = 100, steps_max: int = 2000, rate_per_s: float = 1.0) -> List[Job]:
    """Poisson arrivals at ``rate_per_s``; N log-uniform, horizon uniform."""
    rng = SplitMix64(seed ^ 0x5EEDF00D)
    u = rng.uniform(3 * count).astype(np.float64).reshape(count, 3)
    t = 0.0
    jobs = []
    for q in range(count):
        t += -math.log(max(1e-12, 1.0 - u[q, 0])) / rate_per_s
        n = int(round(math.exp(math.log(n_min) + u[q, 1] * (math.log(n_max) - math.log(n_min)))))
        steps = int(steps_min + u[q, 2] * (steps_max - steps_min))
        jobs.append(Job(job_id=q, arrival_s=t, n=n, steps=steps, seed=seed * 100003 + q + 1))
    return jobs


def job_scene(job: Job) -> Scene:
    """The dam-break scene a served job simulates (config-0 constants scaled:
    spacing 0.01, h 0.02, cube-ish block)."""
    s, h = 0.01, 0.02
    ny = max(2, int(round(job.n ** (1.0 / 3.0))))
    nx = max(2, int(math.ceil(math.sqrt(job.n / ny))))
    nz = max(2, int(math.ceil(job.n / (nx * ny))))
    box = (2.0 * nx * s + 2 * s, 1.5 * ny * s + 2 * s, 2.0 * nz * s + 2 * s)
    sc = dam_break((nx, ny, nz), s, h, box, job.steps, seed=job.seed, limit=job.n, name=f"job_{job.job_id}")
    sc.dyn_pos = (sc.dyn_pos + np.float32(s)).astype(np.float32)
    return sc
