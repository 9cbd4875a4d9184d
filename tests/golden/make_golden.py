"""Generates the golden fixtures in this folder from the reference itself.

Runs the reference's own SPHFunctions.cpp, compiled from source by
``make -C oracle ref`` (oracle/_ref/libsph_ref.so, only where the reference
tree is present), through the synchronous SimulationEngineCPU orchestration in
oracle/ref_harness.cpp, on small seeded scenes, and stores inputs and outputs:

    python tests/golden/make_golden.py

Each .npz holds the scene (positions, statics, triangles, 9 parameters, dt,
reorder interval), then for every checkpoint the raw 32-byte particle buffer
the reference's LockRead() would return, its hashMap and particleMap, the
init permutation, and the sorted statics with their table.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from sphfluidsimulation_gb300 import scenes  # noqa: E402
from oracle_lib import RefEngine  # noqa: E402


def golden_scenes():
    out = []
    s = scenes.debug_smallest_scene()
    out.append((s, [1, 4, 15]))
    s = scenes.dam_break((10, 8, 12), 0.02, 0.04, (0.5, 0.4, 0.5), 0, mass=0.008, name="small_dam")
    out.append((s, [1, 9, 20]))
    # reorderTimeInterval 0: the elapsed time is reset whenever it passes the
    # interval, so the reference never reorders (SimulationEngineCPU.cpp:441,452-454)
    s = scenes.dam_break((10, 8, 12), 0.02, 0.04, (0.5, 0.4, 0.5), 0, mass=0.008, name="small_dam_reorder")
    s.reorder_interval = 0.0
    out.append((s, [1, 2, 3]))
    # a negative interval reorders on every Update call
    s = scenes.dam_break((10, 8, 12), 0.02, 0.04, (0.5, 0.4, 0.5), 0, mass=0.008, name="small_dam_reorder_each_call")
    s.reorder_interval = -1.0
    out.append((s, [1, 2, 5, 9]))
    # fluid block straddling the origin: negative cells on every axis
    s = scenes.dam_break((9, 7, 9), 0.02, 0.04, (0.4, 0.3, 0.4), 0, mass=0.008, name="negative_cells")
    s.dyn_pos = (s.dyn_pos - np.float32(0.09)).astype(np.float32)
    s.static_pos = (s.static_pos - np.float32(0.1)).astype(np.float32)
    out.append((s, [1, 6]))
    # two triangles under a small block (boundary-mesh force, SF:156-223)
    s = scenes.dam_break((6, 5, 6), 0.1, 0.2, (1.0, 1.0, 1.0), 0, mass=1.0, name="triangles")
    s.static_pos = np.zeros((0, 3), np.float32)
    s.dyn_pos = (s.dyn_pos + np.float32(0.3)).astype(np.float32)
    s.triangles = np.array([[0, 0, 0, 2, 0, 0, 0, 0, 2], [2, 0, 0, 2, 0, 2, 0, 0, 2]], np.float32)
    s.dt = 1e-3
    out.append((s, [1, 5]))
    return out


def record(scene, checkpoints):
    eng = RefEngine()
    eng.init(scene)
    data = {
        "dyn_pos": scene.dyn_pos, "static_pos": scene.static_pos, "triangles": scene.triangles,
        "params9": scene.params.as9(), "dt": np.float32(scene.dt),
        "reorder_interval": np.float32(scene.reorder_interval),
        "checkpoints": np.array(checkpoints, np.int32),
    }
    hm, pm, io = eng.maps()
    data["init_order"] = io
    sp, sm = eng.statics()
    data["static_sorted"] = sp
    data["static_map"] = sm
    done = 0
    for k, c in enumerate(checkpoints):
        eng.update(scene.dt, c - done)
        done = c
        raw = eng.read_raw()
        hm, pm, _ = eng.maps()
        data[f"particles_{k}"] = raw.view(np.uint32).reshape(-1, 8)
        data[f"hash_map_{k}"] = hm
        data[f"particle_map_{k}"] = pm
    return data


def main():
    for scene, cps in golden_scenes():
        data = record(scene, cps)
        path = os.path.join(HERE, f"{scene.name}.npz")
        np.savez_compressed(path, **data)
        print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
