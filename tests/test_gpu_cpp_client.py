"""The C ABI driven from C++ (tests/cpp/abi_client.cpp, compiled here with
g++ against include/sph_gb300.h and linked to the in-tree library), as the
reference's C++ application would drive the engine: create, an Update before
Initialize (reported, not run), initialize, three Update calls with the
reference's reorder cadence, read the buffer in the reference's order,
destroy.  With exact arithmetic the bytes equal the oracle's."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from oracle_lib import Oracle
from sphfluidsimulation_gb300 import build, scenes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def write_scene(path, sc, exact, calls, steps):
    with open(path, "wb") as f:
        f.write(sc.params.as9().astype("<f4").tobytes())
        f.write(struct.pack("<ff", sc.dt, sc.reorder_interval))
        f.write(struct.pack("<6I", int(exact), sc.n, sc.s, sc.triangles.shape[0], calls, steps))
        f.write(np.ascontiguousarray(sc.dyn_pos, "<f4").tobytes())
        f.write(np.ascontiguousarray(sc.static_pos, "<f4").tobytes())
        f.write(np.ascontiguousarray(sc.triangles, "<f4").tobytes())


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not present")
def test_cpp_client_exact_equals_oracle(tmp_path):
    lib_dir = os.path.dirname(build.build())
    exe = tmp_path / "abi_client"
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "abi_client.cpp"), "-L", lib_dir, "-lsph_gb300",
                    f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    sc = scenes.dam_break((20, 12, 20), 0.02, 0.04, (0.6, 0.4, 0.6), 0, mass=0.008, name="dam_4800")
    sc.reorder_interval = -1.0          # reorders on every Update call
    calls, steps = 3, 4
    write_scene(tmp_path / "scene.bin", sc, True, calls, steps)
    r = subprocess.run([str(exe), str(tmp_path / "scene.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "4800 particles" in r.stdout
    got = np.fromfile(tmp_path / "out.bin", np.uint8)
    o = Oracle(0)
    o.init(sc)
    for _ in range(calls):
        o.update(sc.dt, steps)
    assert got.tobytes() == o.read_raw().tobytes()
