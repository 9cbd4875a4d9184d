"""ctypes access to the CPU oracle (test infrastructure).

``Oracle`` wraps oracle/sph_oracle.c (float or double build); ``RefEngine``
wraps oracle/_ref/libsph_ref.so, the reference's own SPHFunctions.cpp compiled
from source, when that library exists (only where the reference tree is
present).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
_F32 = os.path.join(ORACLE_DIR, "_build", "libsph_oracle_f32.so")
_F64 = os.path.join(ORACLE_DIR, "_build", "libsph_oracle_f64.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libsph_ref.so")

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint32)
_vp = C.c_void_p

# numpy dtype of the reference's 32-byte DynamicParticle (SF:12-16)
DYN_DTYPE = np.dtype([("pos", "<f4", 3), ("pressure", "<f4"), ("vel", "<f4", 3), ("hash", "<u4")])


def build_oracle() -> None:
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def _ptr(a: Optional[np.ndarray], t):
    if a is None:
        return None
    return a.ctypes.data_as(t)


def _load(path: str):
    if not os.path.exists(path):
        build_oracle()
    lib = C.CDLL(path)
    lib.sph_oracle_create.restype = _vp
    lib.sph_oracle_create.argtypes = [C.c_int]
    lib.sph_oracle_destroy.argtypes = [_vp]
    lib.sph_oracle_init.restype = C.c_int
    lib.sph_oracle_init.argtypes = [_vp, _fp, _fp, _fp, C.c_uint32, _fp, C.c_uint32, _fp, C.c_uint32,
                                    C.c_float, C.c_int]
    lib.sph_oracle_update.restype = C.c_int
    lib.sph_oracle_update.argtypes = [_vp, C.c_float, C.c_uint32]
    lib.sph_oracle_record_accel.argtypes = [_vp, C.c_int]
    lib.sph_oracle_count.restype = C.c_uint32
    lib.sph_oracle_count.argtypes = [_vp, C.c_int]
    lib.sph_oracle_sim_time.restype = C.c_double
    lib.sph_oracle_sim_time.argtypes = [_vp]
    lib.sph_oracle_read_dynamic.argtypes = [_vp, _dp]
    lib.sph_oracle_read_raw.restype = C.c_int
    lib.sph_oracle_read_raw.argtypes = [_vp, _vp]
    lib.sph_oracle_read_maps.argtypes = [_vp, _up, _up, _up]
    lib.sph_oracle_read_static.argtypes = [_vp, _dp, _up]
    lib.sph_oracle_read_accel.argtypes = [_vp, _dp]
    lib.sph_oracle_derived.argtypes = [_vp, _dp, _dp]
    lib.sph_oracle_hash.argtypes = [_fp, C.c_uint32, C.c_float, C.c_uint32, _up]
    lib.sph_oracle_counting_sort.argtypes = [_up, C.c_uint32, C.c_uint32, _up, _up, _up]
    if hasattr(lib, "sph_oracle_splat"):
        lib.sph_oracle_splat.restype = C.c_int
        lib.sph_oracle_splat.argtypes = [_fp, _fp, _fp, C.c_uint32, C.c_uint32, _fp, C.c_uint32, C.c_float, _fp,
                                         _fp, C.c_uint32, C.c_float, _fp, _vp, _vp, _fp]
    return lib


_LIBS = {}


def lib(double: bool = False):
    key = "f64" if double else "f32"
    if key not in _LIBS:
        _LIBS[key] = _load(_F64 if double else _F32)
    return _LIBS[key]


class Oracle:
    """The reference CPU engine restated: Initialize / Update / readback."""

    def __init__(self, threads: int = 0, double: bool = False):
        self.lib = lib(double)
        self.double = double
        self.h = self.lib.sph_oracle_create(int(threads))

    def __del__(self):
        try:
            self.lib.sph_oracle_destroy(self.h)
        except Exception:
            pass

    def init(self, scene, vel: Optional[np.ndarray] = None, parallel_partial_sum: bool = False) -> None:
        p9 = scene.params.as9()
        dyn = np.ascontiguousarray(scene.dyn_pos, np.float32)
        st = np.ascontiguousarray(scene.static_pos, np.float32)
        tri = np.ascontiguousarray(scene.triangles, np.float32)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32)
        rc = self.lib.sph_oracle_init(self.h, _ptr(p9, _fp), _ptr(dyn, _fp), _ptr(v, _fp), dyn.shape[0],
                                      _ptr(st, _fp), st.shape[0], _ptr(tri, _fp), tri.shape[0],
                                      float(scene.reorder_interval), int(parallel_partial_sum))
        assert rc == 0

    def update(self, dt: float, steps: int) -> None:
        assert self.lib.sph_oracle_update(self.h, float(dt), int(steps)) == 0

    def record_accel(self, on: bool = True) -> None:
        self.lib.sph_oracle_record_accel(self.h, int(on))

    @property
    def n(self) -> int:
        return self.lib.sph_oracle_count(self.h, 0)

    @property
    def s(self) -> int:
        return self.lib.sph_oracle_count(self.h, 1)

    @property
    def buckets(self) -> int:
        return self.lib.sph_oracle_count(self.h, 2)

    def sim_time(self) -> float:
        return self.lib.sph_oracle_sim_time(self.h)

    def read(self) -> np.ndarray:
        """(N, 8) float64: px, py, pz, pressure, vx, vy, vz, hash (slot order)."""
        out = np.zeros((self.n, 8), np.float64)
        self.lib.sph_oracle_read_dynamic(self.h, _ptr(out, _dp))
        return out

    def read_raw(self) -> np.ndarray:
        out = np.zeros(self.n, DYN_DTYPE)
        assert self.lib.sph_oracle_read_raw(self.h, out.ctypes.data) == 0
        return out

    def maps(self):
        """(hash_map[B+1], particle_map[N], order[N]) -- order[slot] is the
        input index of the particle in that slot of the current buffer (the
        init permutation until a reordering step permutes it)."""
        hm = np.zeros(self.buckets + 1, np.uint32)
        pm = np.zeros(self.n, np.uint32)
        io = np.zeros(self.n, np.uint32)
        self.lib.sph_oracle_read_maps(self.h, _ptr(hm, _up), _ptr(pm, _up), _ptr(io, _up))
        return hm, pm, io

    def statics(self):
        pos = np.zeros((self.s, 4), np.float64)
        sm = np.zeros(self.s + 1, np.uint32)
        self.lib.sph_oracle_read_static(self.h, _ptr(pos, _dp), _ptr(sm, _up))
        return pos, sm

    def accel(self) -> np.ndarray:
        a = np.zeros((self.n, 3), np.float64)
        self.lib.sph_oracle_read_accel(self.h, _ptr(a, _dp))
        return a

    def derived(self):
        sd, kc = C.c_double(), C.c_double()
        self.lib.sph_oracle_derived(self.h, C.byref(sd), C.byref(kc))
        return sd.value, kc.value

    def by_input_order(self) -> np.ndarray:
        """Current particle state (N, 8) re-indexed by input particle."""
        st = self.read()
        _, _, io = self.maps()
        out = np.empty_like(st)
        out[io] = st
        return out


def oracle_hash(pos: np.ndarray, h: float, buckets: int) -> np.ndarray:
    p = np.ascontiguousarray(pos, np.float32)
    keys = np.zeros(p.shape[0], np.uint32)
    lib().sph_oracle_hash(_ptr(p, _fp), p.shape[0], float(h), int(buckets), _ptr(keys, _up))
    return keys


def oracle_counting_sort(keys: np.ndarray, buckets: int):
    k = np.ascontiguousarray(keys, np.uint32)
    counts = np.zeros(buckets, np.uint32)
    starts = np.zeros(buckets + 1, np.uint32)
    pm = np.zeros(k.shape[0], np.uint32)
    lib().sph_oracle_counting_sort(_ptr(k, _up), k.shape[0], int(buckets), _ptr(counts, _up),
                                   _ptr(starts, _up), _ptr(pm, _up))
    return counts, starts, pm


class RefEngine:
    """The reference's own SPHFunctions.cpp, compiled from source (only where
    the reference tree is present)."""

    def __init__(self):
        if not os.path.exists(REF_SO):
            raise FileNotFoundError(REF_SO)
        L = C.CDLL(REF_SO)
        L.sph_ref_create.restype = _vp
        L.sph_ref_destroy.argtypes = [_vp]
        L.sph_ref_init.restype = C.c_int
        L.sph_ref_init.argtypes = [_vp, _fp, _fp, _fp, C.c_uint32, _fp, C.c_uint32, _fp, C.c_uint32, C.c_float]
        L.sph_ref_update.restype = C.c_int
        L.sph_ref_update.argtypes = [_vp, C.c_float, C.c_uint32]
        L.sph_ref_read_raw.argtypes = [_vp, _vp]
        L.sph_ref_read_maps.argtypes = [_vp, _up, _up, _up]
        L.sph_ref_read_static.argtypes = [_vp, _fp, _up]
        L.sph_ref_hash.argtypes = [_fp, C.c_uint32, C.c_float, C.c_uint32, _up]
        self.L = L
        self.h = L.sph_ref_create()
        self.n = 0
        self.s = 0

    def __del__(self):
        try:
            self.L.sph_ref_destroy(self.h)
        except Exception:
            pass

    def init(self, scene, vel: Optional[np.ndarray] = None) -> None:
        p9 = scene.params.as9()
        dyn = np.ascontiguousarray(scene.dyn_pos, np.float32)
        st = np.ascontiguousarray(scene.static_pos, np.float32)
        tri = np.ascontiguousarray(scene.triangles, np.float32)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32)
        assert self.L.sph_ref_init(self.h, _ptr(p9, _fp), _ptr(dyn, _fp), _ptr(v, _fp), dyn.shape[0],
                                   _ptr(st, _fp), st.shape[0], _ptr(tri, _fp), tri.shape[0],
                                   float(scene.reorder_interval)) == 0
        self.n, self.s = dyn.shape[0], st.shape[0]

    def update(self, dt: float, steps: int) -> None:
        assert self.L.sph_ref_update(self.h, float(dt), int(steps)) == 0
        # the reference prints warnings with C stdio (coincident particles);
        # flush them while the caller's output capture is still in place
        C.CDLL(None).fflush(None)

    def read_raw(self) -> np.ndarray:
        out = np.zeros(self.n, DYN_DTYPE)
        self.L.sph_ref_read_raw(self.h, out.ctypes.data)
        return out

    def maps(self):
        hm = np.zeros(2 * self.n + 1, np.uint32)
        pm = np.zeros(self.n, np.uint32)
        io = np.zeros(self.n, np.uint32)
        self.L.sph_ref_read_maps(self.h, _ptr(hm, _up), _ptr(pm, _up), _ptr(io, _up))
        return hm, pm, io

    def statics(self):
        pos = np.zeros((self.s, 4), np.float32)
        sm = np.zeros(self.s + 1, np.uint32)
        self.L.sph_ref_read_static(self.h, _ptr(pos, _fp), _ptr(sm, _up))
        return pos, sm

    def hash(self, pos: np.ndarray, h: float, mod: int) -> np.ndarray:
        p = np.ascontiguousarray(pos, np.float32)
        keys = np.zeros(p.shape[0], np.uint32)
        self.L.sph_ref_hash(_ptr(p, _fp), p.shape[0], float(h), int(mod), _ptr(keys, _up))
        return keys


def oracle_splat(proj, view, model, width: int, height: int, dyn4, dyn_layer, stat3, stat_layer):
    """The CPU restatement of sph_engine_render (oracle/sph_splat.c).  dyn4:
    (n, 4) x, y, z, pressure in the reference's buffer order; stat3: (s, 3)
    in its sorted static order; a layer is (size, rgba) or None.  Returns
    (rgba (height, width, 4) uint8, depth (height, width) float32)."""
    L = lib()
    m = [np.ascontiguousarray(np.asarray(x, np.float32).reshape(16)) for x in (proj, view, model)]
    d = np.ascontiguousarray(dyn4, np.float32).reshape(-1, 4)
    st = np.ascontiguousarray(stat3, np.float32).reshape(-1, 3)
    dc = None if dyn_layer is None else np.ascontiguousarray(dyn_layer[1], np.float32)
    sc = None if stat_layer is None else np.ascontiguousarray(stat_layer[1], np.float32)
    zkey = np.empty(width * height, np.uint64)
    rgba = np.empty((height, width, 4), np.uint8)
    depth = np.empty((height, width), np.float32)
    rc = L.sph_oracle_splat(_ptr(m[0], _fp), _ptr(m[1], _fp), _ptr(m[2], _fp), width, height,
                            _ptr(d, _fp), d.shape[0], 0.0 if dyn_layer is None else float(dyn_layer[0]), _ptr(dc, _fp),
                            _ptr(st, _fp), st.shape[0], 0.0 if stat_layer is None else float(stat_layer[0]),
                            _ptr(sc, _fp), zkey.ctypes.data, rgba.ctypes.data, _ptr(depth, _fp))
    assert rc == 0
    return rgba, depth



def coincident_scene():
    """A walled dam break (4,800 particles) plus 64 exact duplicates of fluid
    particles and 8 fluid particles placed exactly on floor wall particles:
    every coincident pair takes RandomDirection (SPHFunctions.cpp:140-155)
    in the force pass, against a dynamic (SF:576-580) or a static
    (SF:610-614) neighbour."""
    from sphfluidsimulation_gb300 import scenes
    base = scenes.dam_break((20, 12, 20), 0.02, 0.04, (0.6, 0.4, 0.6), 0, mass=0.008, name="dam_4800")
    rng = np.random.default_rng(7)
    dup = base.dyn_pos[rng.choice(base.n, 64, replace=False)]
    w = base.static_pos
    floor = w[(w[:, 1] == 0.0) & (w[:, 0] > 0.1) & (w[:, 0] < 0.3) & (w[:, 2] > 0.1) & (w[:, 2] < 0.3)]
    on_wall = floor[rng.choice(floor.shape[0], 8, replace=False)]
    pos = np.concatenate([base.dyn_pos, dup, on_wall], 0).astype(np.float32)
    return scenes.Scene(name="coincident", dyn_pos=pos, static_pos=w, params=base.params, dt=base.dt, steps=0)


def differing_words(a, b) -> np.ndarray:
    """(n, 8) mask of the 32-bit words in which two particle buffers (the
    reference's 32-byte DynamicParticle records) differ, where any NaN equals
    any NaN in the seven float fields: the sign and payload of a NaN depend
    on the platform that produced it.  The hash field is compared as an
    integer."""
    ua = np.asarray(a).view(np.uint32).reshape(-1, 8)
    ub = np.asarray(b).view(np.uint32).reshape(-1, 8)
    diff = ua != ub
    both_nan = np.isnan(ua[:, :7].view(np.float32)) & np.isnan(ub[:, :7].view(np.float32))
    diff[:, :7] &= ~both_nan
    return diff


def random_scene(seed: int):
    """A seeded random scene for exact-arithmetic fuzzing: h from 0.02 to 1,
    50-4000 particles as a uniform cloud, Gaussian clusters, a thin sheet or
    a lattice at h/2 placed on cell faces (+-1e-6); walls (a BoxShell at h/2
    around them) on 60 % of seeds; random mass, gas constant, viscosity,
    gravity direction, rest density, dt, reorder mode and initial
    velocities.  Returns (scene, velocities or None)."""
    from sphfluidsimulation_gb300 import scenes
    rng = np.random.default_rng(seed)
    h = float(rng.choice([0.02, 0.05, 0.1, 0.3, 1.0]))
    n = int(rng.integers(50, 4000))
    kind = rng.integers(0, 4)
    if kind == 0:
        pos = rng.uniform(-3 * h * n ** (1 / 3) / 4, 3 * h * n ** (1 / 3) / 4, size=(n, 3))
    elif kind == 1:
        c = rng.uniform(-5 * h, 5 * h, size=(5, 3))
        pos = c[rng.integers(0, 5, n)] + rng.normal(0, h * 0.7, size=(n, 3))
    elif kind == 2:
        pos = np.stack([rng.uniform(0, 20 * h, n), rng.uniform(0, 0.3 * h, n), rng.uniform(0, 20 * h, n)], 1)
    else:
        m = int(round(n ** (1 / 3))) + 1
        g = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
        pos = g * (h / 2) + rng.uniform(-1e-6, 1e-6, size=g.shape)
    pos = pos.astype(np.float32)
    walls = np.zeros((0, 3), np.float32)
    if rng.random() < 0.6:
        lo, hi = pos.min(0) - h * 0.3, pos.max(0) + h * 0.3
        walls = scenes.box_shell(hi - lo, h / 2, offset=lo).astype(np.float32)
    params = scenes.Params(particle_mass=float(rng.uniform(0.001, 2.0)),
                           gas_constant=float(rng.choice([50.0, 200.0, 2000.0])), elasticity=0.0,
                           viscosity=float(rng.choice([0.0, 0.1, 1.0])),
                           gravity=tuple(float(v) for v in rng.normal(0, 5, 3)),
                           rest_density=float(rng.choice([100.0, 1000.0])), h=h)
    interval = float(rng.choice([np.finfo(np.float32).max, -1.0]))
    vel = rng.normal(0, 0.5, size=(n, 3)).astype(np.float32) if rng.random() < 0.5 else None
    sc = scenes.Scene(name=f"random_{seed}", dyn_pos=pos, static_pos=walls, params=params,
                      dt=float(rng.choice([1e-4, 1e-3])), steps=0, reorder_interval=interval)
    return sc, vel


def triangle_soup_scene(seed: int):
    """A 600-particle block (h = 0.5) among 40 random triangles, some of them
    degenerate (two equal vertices, three collinear ones, a tiny one), and
    one particle exactly on a triangle's vertex: CalculateTriangleForce
    (SPHFunctions.cpp:207-223) at and near its divisions by zero."""
    from sphfluidsimulation_gb300 import scenes
    rng = np.random.default_rng(seed)
    h = 0.5
    dyn = scenes.filled_box((10, 6, 10), 0.25, (1.0, 1.0, 1.0), 0.1, scenes.SplitMix64(seed))
    tris = rng.uniform(0.0, 5.0, size=(40, 9)).astype(np.float32)
    tris[0, 3:6] = tris[0, 0:3]                                   # two equal vertices
    tris[1, 3:6] = tris[1, 0:3] + np.float32(0.5) * (tris[1, 6:9] - tris[1, 0:3])   # collinear
    tris[2, 3:9] = tris[2, 0:6] + np.float32(1e-6)                # tiny
    dyn = np.concatenate([dyn, tris[5:6, 0:3]], 0).astype(np.float32)   # on a vertex
    params = scenes.water_params(0.25, h, mass=1.0)
    return scenes.Scene(name=f"triangle_soup_{seed}", dyn_pos=dyn, static_pos=np.zeros((0, 3), np.float32),
                        params=params, dt=1e-3, steps=0, triangles=tris)
