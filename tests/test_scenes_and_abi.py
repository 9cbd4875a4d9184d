"""Host-side checks that need no GPU: scene generators, the C ABI library
exports every declared symbol and rejects work cleanly without a device."""
import ctypes as C
import subprocess

import numpy as np

from conftest import gpu_available
from sphfluidsimulation_gb300 import _lib, scenes


def test_config0_shapes():
    sc = scenes.config0(steps=1)
    assert sc.n == 16384 and sc.s == 8602
    assert sc.dyn_pos.dtype == np.float32
    assert sc.params.particle_mass == 0.008 and sc.params.h == 0.04
    # jitter is within +-0.1 spacing of the lattice
    lat = (sc.dyn_pos / np.float32(0.02)) - 0.5
    assert np.abs(lat - np.round(lat)).max() <= 0.1 + 1e-4


def test_config1_static_count():
    walls = scenes.box_shell((1.6, 0.8, 0.8), 0.005)
    assert walls.shape[0] == 256002


def test_box_shell_matches_reference_count_formula():
    for size, d in [((1.0, 0.6, 0.7), 0.02), ((2, 2, 2), 0.2), ((0.3, 0.5, 0.4), 0.05)]:
        g = (np.asarray(size, np.float32) / np.float32(d)).astype(np.uint64) + 1
        x, y, z = (int(v) for v in g)
        assert scenes.box_shell(size, d).shape[0] == (x * y + x * z + y * z - 2 * x - 2 * y - 2 * z + 4) * 2


def test_splitmix_reproducible():
    a = scenes.SplitMix64(7).uniform(10)
    b = scenes.SplitMix64(7).uniform(10)
    assert np.array_equal(a, b)
    assert (a >= 0).all() and (a < 1).all()


def test_batched_and_served_workloads():
    sc = scenes.batched_scenes(count=96, steps=1)
    ns = np.array([s.n for s in sc])
    assert len(sc) == 96 and ns.min() >= 4096 and ns.max() <= 131072
    jobs = scenes.serving_jobs(count=2000)
    assert len(jobs) == 2000
    assert min(j.n for j in jobs) >= 8192 and max(j.n for j in jobs) <= 1048576
    assert all(100 <= j.steps <= 2000 for j in jobs)
    assert all(b.arrival_s >= a.arrival_s for a, b in zip(jobs, jobs[1:]))


def test_library_exports_every_header_symbol():
    lib = _lib.load()
    names = _lib.header_symbols()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(names) <= exported


def test_host_only_entry_points():
    lib = _lib.load()
    assert lib.sph_engine_implementation_name() == b"CUDA-sm_103a"
    assert lib.sph_status_string(5) == b"bounded device wait expired"
    assert lib.sph_server_job_bytes(1000, 10) > 1000 * 32


def test_no_device_is_an_error_not_a_crash():
    if gpu_available():
        return
    lib = _lib.load()
    h = C.c_void_p()
    st = lib.sph_engine_create(C.byref(h), 0)
    assert st != 0
    assert lib.sph_last_error() != b""


def test_ctypes_structs_match_the_header(tmp_path):
    """The Python binding's ctypes structs have the C header's layout: every
    field at the offset the C compiler gives it, and the same total size
    (a C program built from include/sph_gb300.h prints them)."""
    import os
    pairs = {"sph_params": _lib.SphParams, "sph_render_view": _lib.SphRenderView,
             "sph_render_layer": _lib.SphRenderLayer, "sph_launch_config": _lib.SphLaunchConfig,
             "sph_neighbour_stats": _lib.SphNeighbourStats}
    c_names = {"sph_params": ["particle_mass", "gas_constant", "elasticity", "viscosity", "gravity_x",
                              "gravity_y", "gravity_z", "rest_density", "max_interaction_distance"]}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "sph_gb300.h"', "int main(void) {"]
    for cname, cls in pairs.items():
        fields = c_names.get(cname, [f for f, _ in cls._fields_])
        lines.append(f'printf("{cname} :sizeof %zu\\n", sizeof({cname}));')
        for f in fields:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(_lib.PKG), "include")
    subprocess.run(["gcc", "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        name, field, value = line.split()
        got[(name, field)] = int(value)
    for cname, cls in pairs.items():
        assert got[(cname, ":sizeof")] == C.sizeof(cls), cname
        fields = c_names.get(cname, [f for f, _ in cls._fields_])
        for cf, (pf, _) in zip(fields, cls._fields_):
            assert got[(cname, cf)] == getattr(cls, pf).offset, (cname, cf)
