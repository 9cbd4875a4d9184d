"""Scenes from the reference's scene-description JSON files.

The reference loads a scene with ``SceneBlueprint::LoadScene``
(SPHFluidSimulation/source/SPH/Core/SceneBlueprint.cpp:134-183) from a JSON
object with four entries:

* ``particleBehaviourParameters`` (required, :15-33): particleMass,
  gasConstant, elasticity, viscosity, restDensity, maxInteractionDistance
  (numbers) and gravity (three numbers);
* ``particleSetBlueprints`` (:34-61): a list of ``{layerName,
  particleSetBlueprintType, properties}``; the engines take the layers named
  "dynamic" and "static" (SimulationEngineCPU.cpp:463,479), each the
  concatenation of its blueprints in file order (SceneBlueprint.h:23-51).
  Types: ``FilledBox`` and ``BoxShell``; unknown types are skipped, as the
  reference does after a warning;
* ``boundaryMesh`` (:62-90): ``{path, objectName?}``, a Wavefront OBJ file
  whose triangles become the boundary mesh;
* ``otherParameters`` (:91-104): string values; the engines read
  ``reorderTimeInterval`` (a decimal) and ``parallelPartialSum`` ("true",
  "1", "false", "0") (SimulationEngineCPU.cpp:401-402,
  ParticleSimulationEngine.cpp:6-35).

Type checks follow SPHFluidSimulation/source/SPH/Utility/JSONParsing.h:
``float`` entries accept any number, ``uint32`` entries only non-negative
integer literals, vectors exactly three numbers, strings only strings.  A
violation raises :class:`SceneError` (the reference logs and marks the scene
invalid).

The particle generators follow the reference's float arithmetic operation by
operation (FilledBoxParticleSetBlueprint.cpp:38-66,
BoxShellParticleSetBlueprint.cpp:27-116).  Their jitter comes from the Blaze
Engine's ``Random``, which is not available; it is replaced by SplitMix64
seeded with the blueprint's ``seed`` (default 0), so positions of a jittered
blueprint are reproducible but are not the reference's draws.  A blueprint
with zero jitter gives the reference's positions exactly.

The Blaze Engine's OBJ reader (``Graphics::BasicIndexedMesh::Load``) is not
available either.  :func:`load_obj` reads the standard format: ``v`` lines,
``f`` lines with ``v``, ``v/vt``, ``v//vn`` or ``v/vt/vn`` references
(1-based, negative = relative to the end), polygons split into a fan from
their first vertex, and ``o`` names selecting an object.
"""
from __future__ import annotations

import json
import os
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import scenes

F32 = np.float32


class SceneError(ValueError):
    """A scene file the reference would reject."""


# ---- JSONParsing.h ------------------------------------------------------------

def _expect(obj: dict, name: str):
    if not isinstance(obj, dict) or name not in obj:
        raise SceneError(f'expected an entry named "{name}"')
    return obj[name]


def _is_number(v) -> bool:
    return isinstance(v, (int, float)) and not isinstance(v, bool)


def expect_float(obj: dict, name: str) -> np.float32:
    v = _expect(obj, name)
    if not _is_number(v):
        raise SceneError(f'"{name}": expected a float')
    return F32(v)


def expect_uint32(obj: dict, name: str) -> int:
    v = _expect(obj, name)
    if not isinstance(v, int) or isinstance(v, bool) or v < 0 or v > 0xFFFFFFFF:
        raise SceneError(f'"{name}": expected an unsigned integer')
    return int(v)


def expect_vec3(obj: dict, name: str) -> np.ndarray:
    v = _expect(obj, name)
    if not isinstance(v, list) or len(v) != 3 or not all(_is_number(x) for x in v):
        raise SceneError(f'"{name}": expected an array of 3 floats')
    return np.array([F32(x) for x in v], np.float32)


def expect_string(obj: dict, name: str) -> str:
    v = _expect(obj, name)
    if not isinstance(v, str):
        raise SceneError(f'"{name}": expected a string')
    return v


# ---- particle set blueprints ----------------------------------------------------

def filled_box_positions(props: dict) -> np.ndarray:
    """FilledBoxParticleSetBlueprint (:23-66): a lattice of particlesPerUnit
    particles per unit volume filling spawnVolumeSize at spawnVolumeOffset,
    i over x outermost, jittered by +-randomOffsetIntensity half spacings."""
    ppu = expect_uint32(props, "particlesPerUnit")
    intensity = expect_uint32(props, "randomOffsetIntensity")   # read as uint32 (:28)
    offset = expect_vec3(props, "spawnVolumeOffset")
    size = expect_vec3(props, "spawnVolumeSize")
    seed = expect_uint32(props, "seed") if "seed" in props else 0
    lin = F32(np.power(F32(ppu), F32(1.0) / F32(3.0)))        # Math::Pow(ppu, 1.0f / 3)
    d = F32(F32(1.0) / lin)
    grid = [int(x) for x in (size * lin).astype(np.float32)]   # Vec3<uintMem>(size * lin): truncation
    grid = [max(g, 0) for g in grid]
    base = (np.full(3, d / F32(2.0), np.float32) + offset).astype(np.float32)
    amp = F32(F32(d / F32(2.0)) * F32(intensity))
    n = grid[0] * grid[1] * grid[2]
    if n == 0:
        return np.zeros((0, 3), np.float32)
    i, j, k = np.meshgrid(np.arange(grid[0]), np.arange(grid[1]), np.arange(grid[2]), indexing="ij")
    idx = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float32)
    pos = ((idx * d).astype(np.float32) + base).astype(np.float32)
    if intensity != 0:
        r = scenes.SplitMix64(seed).uniform_pm1(pos.size).reshape(pos.shape)
        pos = (pos + (r * amp).astype(np.float32)).astype(np.float32)
    return pos


def box_shell_positions(props: dict) -> np.ndarray:
    """BoxShellParticleSetBlueprint (:14-116): the faces, edges and corners of
    a box at particleDistance, offset by spawnVolumeOffset, jittered by
    randomOffsetIntensity spacings in [0, 1)."""
    d = expect_float(props, "particleDistance")
    intensity = expect_float(props, "randomOffsetIntensity")
    offset = expect_vec3(props, "spawnVolumeOffset")
    size = expect_vec3(props, "spawnVolumeSize")
    seed = expect_uint32(props, "seed") if "seed" in props else 0
    rng = scenes.SplitMix64(seed) if intensity != 0 else None
    return scenes.box_shell(size, float(d), offset, float(intensity), rng)


BLUEPRINTS = {"FilledBox": filled_box_positions, "BoxShell": box_shell_positions}


# ---- OBJ meshes ------------------------------------------------------------------

def load_obj(path: str, object_name: str = "") -> np.ndarray:
    """Triangles (T, 9) float32 of a Wavefront OBJ file: every face of the
    object ``object_name`` (all faces when empty), polygons as fans."""
    verts: List[Tuple[float, float, float]] = []
    tris: List[List[float]] = []
    current = ""
    found = not object_name
    with open(path, "r", encoding="utf-8", errors="replace") as f:
        for line_no, raw in enumerate(f, 1):
            line = raw.split("#", 1)[0].strip()
            if not line:
                continue
            parts = line.split()
            tag = parts[0]
            if tag == "v":
                if len(parts) < 4:
                    raise SceneError(f"{path}:{line_no}: vertex needs three coordinates")
                verts.append((float(parts[1]), float(parts[2]), float(parts[3])))
            elif tag == "o":
                current = " ".join(parts[1:])
                found = found or current == object_name
            elif tag == "f":
                if object_name and current != object_name:
                    continue
                ids = []
                for ref in parts[1:]:
                    s = ref.split("/")[0]
                    try:
                        k = int(s)
                    except ValueError:
                        raise SceneError(f"{path}:{line_no}: bad vertex reference {ref!r}")
                    k = k - 1 if k > 0 else len(verts) + k
                    if not 0 <= k < len(verts):
                        raise SceneError(f"{path}:{line_no}: vertex {s} out of range")
                    ids.append(k)
                if len(ids) < 3:
                    raise SceneError(f"{path}:{line_no}: a face needs three vertices")
                for m in range(1, len(ids) - 1):
                    a, b, c = verts[ids[0]], verts[ids[m]], verts[ids[m + 1]]
                    tris.append([*a, *b, *c])
    if not found:
        raise SceneError(f'{path}: no object named "{object_name}"')
    return np.asarray(tris, np.float32).reshape(-1, 9)


# ---- the scene ------------------------------------------------------------------

def _params(obj: dict) -> scenes.Params:
    g = expect_vec3(obj, "gravity")
    return scenes.Params(particle_mass=float(expect_float(obj, "particleMass")),
                         gas_constant=float(expect_float(obj, "gasConstant")),
                         elasticity=float(expect_float(obj, "elasticity")),
                         viscosity=float(expect_float(obj, "viscosity")),
                         gravity=(float(g[0]), float(g[1]), float(g[2])),
                         rest_density=float(expect_float(obj, "restDensity")),
                         h=float(expect_float(obj, "maxInteractionDistance")))


def _parse_decimal(s: str) -> Optional[float]:
    try:
        return float(s)
    except ValueError:
        return None


def _find_mesh(path: str, base_dir: str) -> Optional[str]:
    """The mesh file: absolute, else under the scene's directory or one of its
    ancestors (the reference resolves against the application's working
    directory, usually an ancestor of the scene folder), else the working
    directory."""
    if os.path.isabs(path):
        return path if os.path.isfile(path) else None
    d = os.path.abspath(base_dir)
    while True:
        c = os.path.join(d, path)
        if os.path.isfile(c):
            return c
        parent = os.path.dirname(d)
        if parent == d:
            break
        d = parent
    return path if os.path.isfile(path) else None


def parse_scene(doc: dict, base_dir: str = ".", name: str = "scene", dt: float = 1e-4,
                steps: int = 0) -> scenes.Scene:
    """A scene from a parsed scene JSON object (relative mesh paths resolve
    as in :func:`_find_mesh`)."""
    if not isinstance(doc, dict):
        raise SceneError("a scene is a JSON object")
    params = _params(_expect(doc, "particleBehaviourParameters"))
    layers: Dict[str, List[np.ndarray]] = {}
    if "particleSetBlueprints" in doc:
        bps = doc["particleSetBlueprints"]
        if not isinstance(bps, list):
            raise SceneError('"particleSetBlueprints": expected an array')
        for bp in bps:
            layer = expect_string(bp, "layerName")
            kind = expect_string(bp, "particleSetBlueprintType")
            props = _expect(bp, "properties")
            gen = BLUEPRINTS.get(kind)
            if gen is None:
                continue
            layers.setdefault(layer, []).append(gen(props))
    tris = np.zeros((0, 9), np.float32)
    if "boundaryMesh" in doc:
        mesh = doc["boundaryMesh"]
        path = expect_string(mesh, "path")
        obj_name = expect_string(mesh, "objectName") if "objectName" in mesh else ""
        found = _find_mesh(path, base_dir)
        if found is None:
            raise SceneError(f'boundary mesh "{path}" is not a file')
        tris = load_obj(found, obj_name)
    other: Dict[str, str] = {}
    if "otherParameters" in doc:
        op = doc["otherParameters"]
        if not isinstance(op, dict):
            raise SceneError('"otherParameters": expected an object')
        for k in op:
            other[k] = expect_string(op, k)
    reorder = float(np.finfo(np.float32).max)
    if "reorderTimeInterval" in other:
        v = _parse_decimal(other["reorderTimeInterval"])
        if v is not None:
            reorder = float(F32(v))
    empty = np.zeros((0, 3), np.float32)
    dyn = np.concatenate(layers.get("dynamic", [empty]), 0).astype(np.float32)
    stat = np.concatenate(layers.get("static", [empty]), 0).astype(np.float32)
    return scenes.Scene(name=name, dyn_pos=dyn, static_pos=stat, params=params, dt=dt, steps=steps,
                        triangles=tris, reorder_interval=reorder, other_parameters=other)


def load_scene(path: str, dt: float = 1e-4, steps: int = 0) -> scenes.Scene:
    """``SceneBlueprint::LoadScene(path)`` flattened to a :class:`scenes.Scene`."""
    with open(path, "r", encoding="utf-8") as f:
        try:
            doc = json.load(f)
        except json.JSONDecodeError as e:
            raise SceneError(f"{path}: {e}") from None
    name = os.path.splitext(os.path.basename(path))[0]
    return parse_scene(doc, os.path.dirname(os.path.abspath(path)), name, dt, steps)
