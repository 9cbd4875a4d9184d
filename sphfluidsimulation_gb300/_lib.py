"""ctypes binding of libsph_gb300.so (the C ABI in include/sph_gb300.h).

The library is the product: this module only loads it and declares the
argument types.  It fails loudly if the library is missing; there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from typing import List

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", "libsph_gb300.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "sph_gb300.h")

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)
_vp = C.c_void_p
_st = C.c_int


class SphParams(C.Structure):
    _fields_ = [("particle_mass", C.c_float), ("gas_constant", C.c_float), ("elasticity", C.c_float),
                ("viscosity", C.c_float), ("gravity_x", C.c_float), ("gravity_y", C.c_float),
                ("gravity_z", C.c_float), ("rest_density", C.c_float), ("max_interaction_distance", C.c_float)]


class SphRenderView(C.Structure):
    _fields_ = [("proj", C.c_float * 16), ("view", C.c_float * 16), ("model", C.c_float * 16),
                ("width", C.c_uint32), ("height", C.c_uint32)]


class SphRenderLayer(C.Structure):
    _fields_ = [("size", C.c_float), ("color", C.c_float * 4)]


class SphLaunchConfig(C.Structure):
    _fields_ = [("mode", C.c_int), ("persistent_ctas", C.c_uint32), ("density_threads", C.c_int),
                ("density_min_ctas", C.c_int), ("force_threads", C.c_int), ("force_min_ctas", C.c_int),
                ("ms_per_step", C.c_float), ("from_cache", C.c_int), ("density_walk", C.c_int)]


class SphNeighbourStats(C.Structure):
    _fields_ = [("particles", C.c_uint64), ("candidates", C.c_uint64), ("warp_slots", C.c_uint64),
                ("neighbours", C.c_uint64), ("static_neighbours", C.c_uint64),
                ("group_candidates", C.c_uint64), ("group_lane_slots", C.c_uint64),
                ("group_fallback", C.c_uint64)]


STATUS = {0: "SPH_OK", 1: "SPH_ERR_INVALID_ARGUMENT", 2: "SPH_ERR_NOT_INITIALIZED", 3: "SPH_ERR_CUDA",
          4: "SPH_ERR_OUT_OF_MEMORY", 5: "SPH_ERR_DEVICE_TIMEOUT", 6: "SPH_ERR_CAPACITY", 7: "SPH_ERR_BUDGET",
          8: "SPH_ERR_NOT_FOUND"}


class SphError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        super().__init__(f"{what}: {STATUS.get(status, status)} {detail}".strip())


_SIGS = {
    "sph_status_string": (C.c_char_p, [_st]),
    "sph_last_error": (C.c_char_p, []),
    "sph_engine_implementation_name": (C.c_char_p, []),
    "sph_engine_create": (_st, [C.POINTER(_vp), C.c_int]),
    "sph_engine_destroy": (_st, [_vp]),
    "sph_engine_clear": (_st, [_vp]),
    "sph_engine_initialize": (_st, [_vp, C.POINTER(SphParams), _fp, _fp, C.c_uint32, _fp, C.c_uint32, _fp,
                                    C.c_uint32, C.c_float]),
    "sph_engine_update": (_st, [_vp, C.c_float, C.c_uint32]),
    "sph_engine_update_async": (_st, [_vp, C.c_float, C.c_uint32]),
    "sph_engine_synchronize": (_st, [_vp]),
    "sph_engine_read_dynamic": (_st, [_vp, _vp]),
    "sph_engine_read_dynamic_buffer": (_st, [_vp, _vp]),
    "sph_engine_write_dynamic": (_st, [_vp, _vp]),
    "sph_engine_write_dynamic_async": (_st, [_vp, _vp]),
    "sph_engine_read_static": (_st, [_vp, _vp, _up]),
    "sph_engine_read_buckets": (_st, [_vp, _up, _up]),
    "sph_engine_simulation_time": (_st, [_vp, _dp]),
    "sph_engine_count": (_st, [_vp, C.c_int, _u64p]),
    "sph_engine_record_acceleration": (_st, [_vp, C.c_int]),
    "sph_engine_set_exact": (_st, [_vp, C.c_int]),
    "sph_debug_expire_wait": (_st, [C.c_int, _up]),
    "sph_batch_set_exact": (_st, [_vp, C.c_int]),
    "sph_server_set_exact": (_st, [_vp, C.c_int]),
    "sph_engine_render": (_st, [_vp, C.POINTER(SphRenderView), C.POINTER(SphRenderLayer), C.POINTER(SphRenderLayer),
                                _vp, _fp]),
    "sph_engine_read_acceleration": (_st, [_vp, _fp]),
    "sph_engine_set_timing": (_st, [_vp, C.c_int]),
    "sph_engine_kernel_times": (_st, [_vp, _fp, C.c_int]),
    "sph_engine_neighbour_stats": (_st, [_vp, C.POINTER(SphNeighbourStats)]),
    "sph_engine_get_stream": (_st, [_vp, C.POINTER(_vp)]),
    "sph_probe_fp32_issue": (_st, [C.c_int, _dp, _fp]),
    "sph_engine_save_state": (_st, [_vp]),
    "sph_engine_restore_state": (_st, [_vp]),
    "sph_cell_sort": (_st, [C.c_int, _fp, C.c_uint32, C.c_float, C.c_uint32, _up, _up, _up, _up]),
    "sph_cell_sort_noalloc": (_st, [_vp, C.c_uint32, C.c_float, C.c_uint32, _vp, _vp, _vp, _vp]),
    "sph_batch_create": (_st, [C.POINTER(_vp), C.c_int]),
    "sph_batch_destroy": (_st, [_vp]),
    "sph_batch_add_scene": (_st, [_vp, C.POINTER(SphParams), _fp, _fp, C.c_uint32, _fp, C.c_uint32, _fp,
                                  C.c_uint32, C.c_float, _up]),
    "sph_batch_finalize": (_st, [_vp]),
    "sph_batch_step": (_st, [_vp, C.c_uint32]),
    "sph_batch_set_mode": (_st, [_vp, C.c_int]),
    "sph_batch_autotune": (_st, [_vp, C.c_uint32, C.POINTER(C.c_int), _up, _fp]),
    "sph_batch_launch_config": (_st, [_vp, C.POINTER(SphLaunchConfig)]),
    "sph_engine_autotune": (_st, [_vp, C.c_uint32, C.POINTER(SphLaunchConfig)]),
    "sph_engine_set_launch_shapes": (_st, [_vp, C.c_int, C.c_int]),
    "sph_batch_read_scene": (_st, [_vp, C.c_uint32, _vp]),
    "sph_batch_info": (_st, [_vp, _u64p, _up, _up]),
    "sph_server_create": (_st, [C.POINTER(_vp), C.c_int, C.c_uint64, C.c_uint32]),
    "sph_server_destroy": (_st, [_vp]),
    "sph_server_submit": (_st, [_vp, C.POINTER(SphParams), _fp, C.c_uint32, _fp, C.c_uint32, C.c_float,
                                C.c_uint32, _u64p]),
    "sph_server_poll": (_st, [_vp, C.c_uint32, _up, _up]),
    "sph_server_result": (_st, [_vp, C.c_uint64, _vp, _fp]),
    "sph_server_finished": (_st, [_vp, C.POINTER(C.c_uint64), C.c_uint32, _up]),
    "sph_server_job_bytes": (C.c_uint64, [C.c_uint32, C.c_uint32]),
    "sph_server_stats": (_st, [_vp, _dp, _u64p]),
}

_LIB = None


def header_symbols() -> List[str]:
    """Function names declared with SPH_API in include/sph_gb300.h."""
    text = open(HEADER).read()
    return re.findall(r"SPH_API\s+[\w\s\*]+?\b(sph_\w+)\s*\(", text)


def load() -> C.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (nvcc) first; "
                          "there is no CPU fallback")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name, None)
        if f is None:
            continue
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def check(status: int, what: str) -> None:
    if status != 0:
        detail = load().sph_last_error().decode(errors="replace")
        raise SphError(status, what, detail)
