"""Python face of the C ABI: the engine, the counting-sort stage and the batch.

``SimulationEngineCUDA`` keeps the reference's engine vocabulary
(SPHFluidSimulation/include/SPH/Core/SimulationEngine.h:35-76):
``clear``, ``initialize``, ``update``, ``system_implementation_name``,
``get_simulation_time``, plus readback of the dynamic and static particle
buffers.  Every call goes through libsph_gb300.so.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import SphParams, check

# the reference's 32-byte DynamicParticle (Particles.h:9-17)
DYN_DTYPE = np.dtype([("pos", "<f4", 3), ("pressure", "<f4"), ("vel", "<f4", 3), ("hash", "<u4")])
STATIC_DTYPE = np.dtype([("pos", "<f4", 3), ("pressure", "<f4")])


def _fptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _uptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_uint32))


def make_params(p) -> SphParams:
    """From a ``scenes.Params`` (or anything with the same fields)."""
    g = p.gravity
    return SphParams(p.particle_mass, p.gas_constant, p.elasticity, p.viscosity, g[0], g[1], g[2],
                     p.rest_density, p.h)


def _f32(a, cols: int) -> Optional[np.ndarray]:
    if a is None:
        return None
    a = np.ascontiguousarray(a, np.float32)
    if a.size == 0:
        return None
    return a.reshape(-1, cols)


class SimulationEngineCUDA:
    """SPH step engine on one GPU (reference SimulationEngineCPU's interface)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        check(self.lib.sph_engine_create(C.byref(h), int(device)), "sph_engine_create")
        self.h = h
        self.n = 0
        self.s = 0

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.sph_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- SimulationEngine ----------------------------------------------------
    @staticmethod
    def system_implementation_name() -> str:
        return _lib.load().sph_engine_implementation_name().decode()

    def clear(self) -> None:
        check(self.lib.sph_engine_clear(self.h), "sph_engine_clear")
        self.n = self.s = 0

    def initialize(self, scene, vel: Optional[np.ndarray] = None) -> None:
        """``scene`` is a ``scenes.Scene`` (positions, statics, params, triangles)."""
        dyn = _f32(scene.dyn_pos, 3)
        st = _f32(scene.static_pos, 3)
        tri = _f32(scene.triangles, 9)
        v = _f32(vel if vel is not None else scene.dyn_vel, 3)
        p = make_params(scene.params)
        n = 0 if dyn is None else dyn.shape[0]
        s = 0 if st is None else st.shape[0]
        t = 0 if tri is None else tri.shape[0]
        check(self.lib.sph_engine_initialize(self.h, C.byref(p), _fptr(dyn), _fptr(v), n, _fptr(st), s,
                                             _fptr(tri), t, float(scene.reorder_interval)),
              "sph_engine_initialize")
        self.n, self.s = n, s

    def update(self, dt: float, steps: int) -> None:
        check(self.lib.sph_engine_update(self.h, float(dt), int(steps)), "sph_engine_update")

    def update_async(self, dt: float, steps: int) -> None:
        check(self.lib.sph_engine_update_async(self.h, float(dt), int(steps)), "sph_engine_update_async")

    def synchronize(self) -> None:
        check(self.lib.sph_engine_synchronize(self.h), "sph_engine_synchronize")

    def get_simulation_time(self) -> float:
        t = C.c_double()
        check(self.lib.sph_engine_simulation_time(self.h, C.byref(t)), "sph_engine_simulation_time")
        return t.value

    # -- buffers ---------------------------------------------------------------
    def read_dynamic(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.zeros(self.n, DYN_DTYPE)
        check(self.lib.sph_engine_read_dynamic(self.h, out.ctypes.data_as(C.c_void_p)), "sph_engine_read_dynamic")
        return out

    def read_dynamic_buffer(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """The particles in the reference's buffer order (its LockRead bytes)."""
        if out is None:
            out = np.zeros(self.n, DYN_DTYPE)
        check(self.lib.sph_engine_read_dynamic_buffer(self.h, out.ctypes.data_as(C.c_void_p)),
              "sph_engine_read_dynamic_buffer")
        return out

    def write_dynamic(self, particles: np.ndarray) -> None:
        p = np.ascontiguousarray(particles, DYN_DTYPE)
        check(self.lib.sph_engine_write_dynamic(self.h, p.ctypes.data_as(C.c_void_p)), "sph_engine_write_dynamic")

    def write_dynamic_async(self, particles: np.ndarray) -> None:
        """Queued upload (sph_engine_write_dynamic_async): `particles` must be
        a contiguous DYN_DTYPE array the caller keeps unchanged until the
        next waiting call (synchronize, update, a read)."""
        if particles.dtype != DYN_DTYPE or not particles.flags.c_contiguous:
            raise ValueError("write_dynamic_async needs a contiguous DYN_DTYPE array (no copy is made)")
        check(self.lib.sph_engine_write_dynamic_async(self.h, particles.ctypes.data_as(C.c_void_p)),
              "sph_engine_write_dynamic_async")

    def read_static(self):
        out = np.zeros(self.s, STATIC_DTYPE)
        starts = np.zeros(self.s + 1, np.uint32)
        check(self.lib.sph_engine_read_static(self.h, out.ctypes.data_as(C.c_void_p), _uptr(starts)),
              "sph_engine_read_static")
        return out, starts

    def read_buckets(self):
        """(bucket_starts[2n+1], slot_ids[n]) in the reference's hashMap sense."""
        starts = np.zeros(2 * self.n + 1, np.uint32)
        ids = np.zeros(self.n, np.uint32)
        check(self.lib.sph_engine_read_buckets(self.h, _uptr(starts), _uptr(ids)), "sph_engine_read_buckets")
        return starts, ids

    def set_exact(self, exact: bool = True) -> None:
        """Neighbour-pass arithmetic: the reference's own operations (exact,
        bit-identical to its synchronous CPU engine) or the fast fused form."""
        check(self.lib.sph_engine_set_exact(self.h, int(exact)), "sph_engine_set_exact")

    def render(self, proj, view, model, width: int, height: int, dynamic_layer=(0.1, (1.0, 1.0, 1.0, 1.0)),
               static_layer=(0.03, (0.0, 0.0, 1.0, 1.0))):
        """Headless particle splats (sph_engine_render): (rgba (height, width,
        4) uint8 with row 0 at the bottom, depth (height, width) float32).
        Matrices are column-major 4x4 (sphfluidsimulation_gb300.render); a
        layer is (size, rgba) or None."""
        v = _lib.SphRenderView()
        for name, m in (("proj", proj), ("view", view), ("model", model)):
            arr = np.ascontiguousarray(np.asarray(m, np.float32).reshape(16))
            getattr(v, name)[:] = arr.tolist()
        v.width, v.height = int(width), int(height)

        def layer(l):
            if l is None:
                return None
            out = _lib.SphRenderLayer()
            out.size = float(l[0])
            out.color[:] = [float(c) for c in l[1]]
            return C.byref(out)

        rgba = np.empty((height, width, 4), np.uint8)
        depth = np.empty((height, width), np.float32)
        check(self.lib.sph_engine_render(self.h, C.byref(v), layer(dynamic_layer), layer(static_layer),
                                         rgba.ctypes.data_as(C.c_void_p), _fptr(depth)), "sph_engine_render")
        return rgba, depth

    def record_acceleration(self, on: bool = True) -> None:
        check(self.lib.sph_engine_record_acceleration(self.h, int(on)), "sph_engine_record_acceleration")

    def read_acceleration(self) -> np.ndarray:
        out = np.zeros((self.n, 3), np.float32)
        check(self.lib.sph_engine_read_acceleration(self.h, _fptr(out)), "sph_engine_read_acceleration")
        return out

    def autotune(self, trial_steps: int = 3) -> dict:
        """Launch shapes of the density and force passes chosen by timing
        (sph_engine_autotune); replaces a save_state() copy."""
        cfg = _lib.SphLaunchConfig()
        check(self.lib.sph_engine_autotune(self.h, int(trial_steps), C.byref(cfg)), "sph_engine_autotune")
        return {name: getattr(cfg, name) for name, _ in cfg._fields_}

    def set_launch_shapes(self, density_shape: int, force_shape: int) -> None:
        check(self.lib.sph_engine_set_launch_shapes(self.h, int(density_shape), int(force_shape)),
              "sph_engine_set_launch_shapes")

    def save_state(self) -> None:
        """Device-side checkpoint (sph_engine_save_state)."""
        check(self.lib.sph_engine_save_state(self.h), "sph_engine_save_state")

    def restore_state(self) -> None:
        """Back to the checkpoint, bit for bit (sph_engine_restore_state)."""
        check(self.lib.sph_engine_restore_state(self.h), "sph_engine_restore_state")

    def stream_handle(self) -> int:
        """The engine's cudaStream_t as an integer."""
        st = C.c_void_p()
        check(self.lib.sph_engine_get_stream(self.h, C.byref(st)), "sph_engine_get_stream")
        return st.value or 0

    def set_timing(self, on: bool = True) -> None:
        check(self.lib.sph_engine_set_timing(self.h, int(on)), "sph_engine_set_timing")

    def kernel_times(self) -> np.ndarray:
        ms = np.zeros(5, np.float32)
        check(self.lib.sph_engine_kernel_times(self.h, _fptr(ms), 5), "sph_engine_kernel_times")
        return ms

    def neighbour_stats(self) -> dict:
        """Counts over the current state (sph_engine_neighbour_stats):
        particles, candidates, warp_slots, neighbours, static_neighbours."""
        st = _lib.SphNeighbourStats()
        check(self.lib.sph_engine_neighbour_stats(self.h, C.byref(st)), "sph_engine_neighbour_stats")
        return {name: int(getattr(st, name)) for name, _ in st._fields_}


def cell_sort(pos: np.ndarray, h: float, buckets: int, device: int = 0):
    """The counting-sort stage alone: (keys, counts, starts, order)."""
    lib = _lib.load()
    p = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    n = p.shape[0]
    keys = np.zeros(n, np.uint32)
    counts = np.zeros(buckets, np.uint32)
    starts = np.zeros(buckets + 1, np.uint32)
    order = np.zeros(n, np.uint32)
    check(lib.sph_cell_sort(int(device), _fptr(p), n, float(h), int(buckets), _uptr(keys), _uptr(counts),
                            _uptr(starts), _uptr(order)), "sph_cell_sort")
    return keys, counts, starts, order


class Batch:
    """Many independent scenes advanced together (one persistent launch per step)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        check(self.lib.sph_batch_create(C.byref(h), int(device)), "sph_batch_create")
        self.h = h
        self.sizes = []

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.sph_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, scene, dt: Optional[float] = None) -> int:
        dyn = _f32(scene.dyn_pos, 3)
        st = _f32(scene.static_pos, 3)
        tri = _f32(scene.triangles, 9)
        v = _f32(scene.dyn_vel, 3)
        p = make_params(scene.params)
        sid = C.c_uint32()
        check(self.lib.sph_batch_add_scene(self.h, C.byref(p), _fptr(dyn), _fptr(v), 0 if dyn is None else dyn.shape[0],
                                           _fptr(st), 0 if st is None else st.shape[0], _fptr(tri),
                                           0 if tri is None else tri.shape[0],
                                           float(scene.dt if dt is None else dt), C.byref(sid)),
              "sph_batch_add_scene")
        self.sizes.append(0 if dyn is None else dyn.shape[0])
        return sid.value

    def finalize(self) -> None:
        check(self.lib.sph_batch_finalize(self.h), "sph_batch_finalize")

    def set_mode(self, mode: int) -> None:
        check(self.lib.sph_batch_set_mode(self.h, int(mode)), "sph_batch_set_mode")

    def set_exact(self, exact: bool = True) -> None:
        check(self.lib.sph_batch_set_exact(self.h, int(exact)), "sph_batch_set_exact")

    def step(self, steps: int = 1) -> None:
        check(self.lib.sph_batch_step(self.h, int(steps)), "sph_batch_step")

    def autotune(self, trial_steps: int = 3):
        """(mode, grid_ctas, ms_per_step) of the configuration chosen."""
        mode = C.c_int()
        grid = C.c_uint32()
        ms = C.c_float()
        check(self.lib.sph_batch_autotune(self.h, int(trial_steps), C.byref(mode), C.byref(grid), C.byref(ms)),
              "sph_batch_autotune")
        return mode.value, grid.value, ms.value

    def launch_config(self) -> dict:
        """The step configuration in use (sph_batch_launch_config)."""
        cfg = _lib.SphLaunchConfig()
        check(self.lib.sph_batch_launch_config(self.h, C.byref(cfg)), "sph_batch_launch_config")
        return {name: getattr(cfg, name) for name, _ in cfg._fields_}

    def read_scene(self, scene_id: int) -> np.ndarray:
        out = np.zeros(self.sizes[scene_id], DYN_DTYPE)
        check(self.lib.sph_batch_read_scene(self.h, int(scene_id), out.ctypes.data_as(C.c_void_p)),
              "sph_batch_read_scene")
        return out

    def info(self):
        tot = C.c_uint64()
        grid = C.c_uint32()
        thr = C.c_uint32()
        check(self.lib.sph_batch_info(self.h, C.byref(tot), C.byref(grid), C.byref(thr)), "sph_batch_info")
        return tot.value, grid.value, thr.value


class Server:
    """Continuous-batching server: jobs admitted under an HBM budget, resident
    on the device, advanced together; results returned per job."""

    def __init__(self, budget_bytes: int, max_slots: int = 64, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        check(self.lib.sph_server_create(C.byref(h), int(device), int(budget_bytes), int(max_slots)),
              "sph_server_create")
        self.h = h
        self.sizes = {}

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.sph_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def job_bytes(n: int, s: int) -> int:
        return int(_lib.load().sph_server_job_bytes(int(n), int(s)))

    def submit(self, scene, steps: Optional[int] = None) -> int:
        dyn = _f32(scene.dyn_pos, 3)
        st = _f32(scene.static_pos, 3)
        p = make_params(scene.params)
        jid = C.c_uint64()
        n = 0 if dyn is None else dyn.shape[0]
        check(self.lib.sph_server_submit(self.h, C.byref(p), _fptr(dyn), n, _fptr(st),
                                         0 if st is None else st.shape[0], float(scene.dt),
                                         int(scene.steps if steps is None else steps), C.byref(jid)),
              "sph_server_submit")
        self.sizes[jid.value] = n
        return jid.value

    def set_exact(self, exact: bool = True) -> None:
        check(self.lib.sph_server_set_exact(self.h, int(exact)), "sph_server_set_exact")

    def poll(self, chunk_steps: int = 50):
        a = C.c_uint32()
        q = C.c_uint32()
        check(self.lib.sph_server_poll(self.h, int(chunk_steps), C.byref(a), C.byref(q)), "sph_server_poll")
        return a.value, q.value

    PHASES = ("admit", "admit_wait", "table", "enqueue", "steps_wait", "readback")

    def stats(self) -> dict:
        """Host seconds per poll phase and counts (sph_server_stats)."""
        sec = (C.c_double * 6)()
        cnt = (C.c_uint64 * 3)()
        check(self.lib.sph_server_stats(self.h, sec, cnt), "sph_server_stats")
        out = {f"{k}_s": float(v) for k, v in zip(self.PHASES, sec)}
        out.update({"polls": int(cnt[0]), "steps": int(cnt[1]), "table_builds": int(cnt[2])})
        return out

    def finished(self) -> list:
        """Ids of the jobs retired since the last call (sph_server_finished)."""
        out = []
        buf = (C.c_uint64 * 256)()
        cnt = C.c_uint32()
        while True:
            check(self.lib.sph_server_finished(self.h, buf, 256, C.byref(cnt)), "sph_server_finished")
            out.extend(buf[:cnt.value])
            if cnt.value < 256:
                return out

    def result(self, job_id: int):
        """(particles, density) of a finished job, or None while it runs."""
        n = self.sizes[job_id]
        out = np.zeros(n, DYN_DTYPE)
        dens = np.zeros(n, np.float32)
        st = self.lib.sph_server_result(self.h, C.c_uint64(job_id), out.ctypes.data_as(C.c_void_p), _fptr(dens))
        if st == 8:
            return None
        check(st, "sph_server_result")
        del self.sizes[job_id]
        return out, dens
