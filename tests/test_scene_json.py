"""Scene files in the reference's JSON format (host side, no GPU): parameter
and type checks, the FilledBox and BoxShell generators, OBJ boundary meshes
and otherParameters, on scene files written here; plus the reference's own
scene assets when its tree is present."""
import json
import os

import numpy as np
import pytest

from sphfluidsimulation_gb300 import scene_json, scenes
from sphfluidsimulation_gb300.scene_json import SceneError

PARAMS = {"particleMass": 0.008, "gasConstant": 200, "elasticity": 0, "viscosity": 0.1,
          "gravity": [0, -9.81, 0], "restDensity": 1000, "maxInteractionDistance": 0.04}

QUAD_OBJ = """# a unit quad in y = 0 and a triangle in another object
o Floor
v 0 0 0
v 1 0 0
v 1 0 1
v 0 0 1
vn 0 1 0
f 1//1 2//1 3//1 4//1
o Ramp
v 0 0.5 0
v 1 0.2 0
v 0 0.2 1
f -3/1/1 -2/2/1 -1/3/1
"""


def write_scene(tmp_path, doc, obj=None, obj_name="mesh.obj"):
    if obj is not None:
        (tmp_path / obj_name).write_text(obj)
    p = tmp_path / "scene.json"
    p.write_text(json.dumps(doc))
    return str(p)


def base_doc():
    return {
        "particleBehaviourParameters": dict(PARAMS),
        "particleSetBlueprints": [
            {"layerName": "dynamic", "particleSetBlueprintType": "FilledBox",
             "properties": {"particlesPerUnit": 125000, "randomOffsetIntensity": 0,
                            "spawnVolumeOffset": [0.02, 0.02, 0.02], "spawnVolumeSize": [0.2, 0.1, 0.2]}},
            {"layerName": "static", "particleSetBlueprintType": "BoxShell",
             "properties": {"particleDistance": 0.02, "randomOffsetIntensity": 0,
                            "spawnVolumeOffset": [0, 0, 0], "spawnVolumeSize": [0.5, 0.3, 0.5]}},
        ],
        "otherParameters": {"reorderTimeInterval": "-1", "parallelPartialSum": "true"},
    }


def test_filled_box_and_box_shell_match_the_reference_generators(tmp_path):
    sc = scene_json.load_scene(write_scene(tmp_path, base_doc()))
    # FilledBox: 125000 per unit volume = 50 per unit length, spacing 0.02
    lin = np.float32(np.power(np.float32(125000), np.float32(1) / np.float32(3)))
    d = np.float32(1) / lin
    grid = (np.array([0.2, 0.1, 0.2], np.float32) * lin).astype(np.int64)
    assert sc.n == int(np.prod(grid))
    first = np.float32(d / np.float32(2)) + np.float32(0.02)
    assert sc.dyn_pos[0].tolist() == [first, first, first]
    # i over x outermost, k over z innermost
    assert sc.dyn_pos[1, 2] == np.float32(np.float32(1) * d + np.float32(np.float32(d / np.float32(2)) + np.float32(0.02)))
    # BoxShell: count formula of BoxShellParticleSetBlueprint.cpp:27-39
    g = (np.array([0.5, 0.3, 0.5], np.float32) / np.float32(0.02)).astype(np.int64) + 1
    gx, gy, gz = (int(v) for v in g)
    assert sc.s == (gx * gy + gx * gz + gy * gz - 2 * gx - 2 * gy - 2 * gz + 4) * 2
    assert np.array_equal(sc.static_pos, scenes.box_shell((0.5, 0.3, 0.5), 0.02))
    p = sc.params
    assert (p.particle_mass, p.h, p.gravity[1]) == (float(np.float32(0.008)), float(np.float32(0.04)),
                                                    float(np.float32(-9.81)))
    assert sc.reorder_interval == -1.0
    assert sc.other_parameters["parallelPartialSum"] == "true"
    assert sc.triangles.shape == (0, 9)


def test_jitter_is_seeded_and_bounded(tmp_path):
    doc = base_doc()
    doc["particleSetBlueprints"][0]["properties"]["randomOffsetIntensity"] = 1
    doc["particleSetBlueprints"][0]["properties"]["seed"] = 7
    a = scene_json.load_scene(write_scene(tmp_path, doc))
    b = scene_json.load_scene(write_scene(tmp_path, doc))
    plain = scene_json.load_scene(write_scene(tmp_path, base_doc()))
    assert np.array_equal(a.dyn_pos, b.dyn_pos)
    off = np.abs(a.dyn_pos.astype(np.float64) - plain.dyn_pos)
    assert 0 < off.max() <= 0.01 + 1e-6          # at most half a spacing
    doc["particleSetBlueprints"][0]["properties"]["seed"] = 8
    c = scene_json.load_scene(write_scene(tmp_path, doc))
    assert not np.array_equal(a.dyn_pos, c.dyn_pos)


def test_layers_concatenate_in_file_order_and_unknown_types_are_skipped(tmp_path):
    doc = base_doc()
    second = json.loads(json.dumps(doc["particleSetBlueprints"][0]))
    second["properties"]["spawnVolumeOffset"] = [0.3, 0.02, 0.3]
    doc["particleSetBlueprints"].insert(1, second)
    doc["particleSetBlueprints"].append({"layerName": "dynamic", "particleSetBlueprintType": "Sphere",
                                         "properties": {}})
    doc["particleSetBlueprints"].append({"layerName": "decor", "particleSetBlueprintType": "FilledBox",
                                         "properties": doc["particleSetBlueprints"][0]["properties"]})
    sc = scene_json.load_scene(write_scene(tmp_path, doc))
    one = scene_json.filled_box_positions(doc["particleSetBlueprints"][0]["properties"])
    assert sc.n == 2 * one.shape[0]
    assert np.array_equal(sc.dyn_pos[:one.shape[0]], one)
    assert np.array_equal(sc.dyn_pos[one.shape[0]:], scene_json.filled_box_positions(second["properties"]))


def test_obj_mesh_fans_objects_and_relative_indices(tmp_path):
    doc = base_doc()
    doc["boundaryMesh"] = {"path": "mesh.obj"}
    sc = scene_json.load_scene(write_scene(tmp_path, doc, QUAD_OBJ))
    assert sc.triangles.shape == (3, 9)
    assert sc.triangles[0].tolist() == [0, 0, 0, 1, 0, 0, 1, 0, 1]
    assert sc.triangles[1].tolist() == [0, 0, 0, 1, 0, 1, 0, 0, 1]
    assert np.allclose(sc.triangles[2], [0, 0.5, 0, 1, 0.2, 0, 0, 0.2, 1])
    doc["boundaryMesh"] = {"path": "mesh.obj", "objectName": "Ramp"}
    ramp = scene_json.load_scene(write_scene(tmp_path, doc, QUAD_OBJ))
    assert ramp.triangles.shape == (1, 9)
    doc["boundaryMesh"] = {"path": "mesh.obj", "objectName": "Nothing"}
    with pytest.raises(SceneError):
        scene_json.load_scene(write_scene(tmp_path, doc, QUAD_OBJ))
    doc["boundaryMesh"] = {"path": "missing.obj"}
    with pytest.raises(SceneError):
        scene_json.load_scene(write_scene(tmp_path, doc))


@pytest.mark.parametrize("where, key, value", [
    ("params", "particleMass", "1.0"),            # a float entry must be a number
    ("params", "gravity", [0, -9.81]),            # three numbers
    ("params", "maxInteractionDistance", None),   # missing
    ("box", "particlesPerUnit", 20.0),            # uint32 entries: integer literals only
    ("box", "randomOffsetIntensity", -1),
    ("box", "spawnVolumeSize", "big"),
    ("other", "reorderTimeInterval", 5),          # otherParameters are strings
])
def test_type_errors_are_rejected(tmp_path, where, key, value):
    doc = base_doc()
    target = {"params": doc["particleBehaviourParameters"],
              "box": doc["particleSetBlueprints"][0]["properties"],
              "other": doc["otherParameters"]}[where]
    if value is None:
        del target[key]
    else:
        target[key] = value
    with pytest.raises(SceneError):
        scene_json.load_scene(write_scene(tmp_path, doc))


def test_malformed_json_is_rejected(tmp_path):
    p = tmp_path / "bad.json"
    p.write_text("{ not json")
    with pytest.raises(SceneError):
        scene_json.load_scene(str(p))


ASSETS = os.path.join(os.environ.get("SPH_REFERENCE_ROOT", "/root/reference"),
                      "FluidSimulationProject", "assets", "simulationScenes")


@pytest.mark.skipif(not os.path.isdir(ASSETS), reason="reference tree not present")
def test_reference_scene_assets_load():
    """The reference's own scene files: counts from the generators' count
    formulas, the boundary mesh of the triangle test scene, and the debug
    scene equal to the restated debug_smallest_scene()."""
    small = scene_json.load_scene(os.path.join(ASSETS, "debugSmallestScene.json"), dt=0.01)
    ref = scenes.debug_smallest_scene()
    assert np.array_equal(small.dyn_pos, ref.dyn_pos)
    assert small.s == ref.s
    assert np.array_equal(small.params.as9(), ref.params.as9())
    assert small.reorder_interval == ref.reorder_interval
    tri = scene_json.load_scene(os.path.join(ASSETS, "triangleTestScene.json"))
    assert tri.triangles.shape == (1096, 9)
    assert tri.n == 21 ** 3
    big = scene_json.load_scene(os.path.join(ASSETS, "scene.json"))
    assert big.n > 0 and big.s > 0
