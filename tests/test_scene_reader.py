"""The host scene reader (io/SceneReader.cpp semantics) on the CPU.

Checks the flattened description against independent numpy restatements: transforms
(translate * eulerXYZ * scale, Math.h:848-859) and their inverses, the rectangle and
volume layouts (SceneReader.cpp:385-645), the camera basis (Camera.cpp:7-26), light and
material fields, the .vol loader (ResourceManager.cpp:222-288) and the error codes that
replace the reference's LOG(FATAL).
"""
import copy
import json
import math
import os

import numpy as np
import pytest

from conftest import scene_path

pytestmark = pytest.mark.usefixtures("built")


def ne():
    import narvalengine_gb300 as m
    return m


def mat(a):
    return np.array(list(a), np.float64).reshape(4, 4).T  # column-major storage


def transform(pos, rot_deg, scale):
    rx, ry, rz = (math.radians(v) for v in rot_deg)
    Rx = np.array([[1, 0, 0], [0, math.cos(rx), -math.sin(rx)], [0, math.sin(rx), math.cos(rx)]])
    Ry = np.array([[math.cos(ry), 0, math.sin(ry)], [0, 1, 0], [-math.sin(ry), 0, math.cos(ry)]])
    Rz = np.array([[math.cos(rz), -math.sin(rz), 0], [math.sin(rz), math.cos(rz), 0], [0, 0, 1]])
    M = np.eye(4)
    M[:3, :3] = Rx @ Ry @ Rz @ np.diag(scale)
    M[:3, 3] = pos
    return M


def load(d):
    return ne().SceneHost.from_string(json.dumps(d))


def test_cornell_structure_and_transforms():
    d = json.load(open(scene_path("cornell_c1")))
    h = ne().SceneHost.from_json(scene_path("cornell_c1"))
    D = h.desc
    assert D.n_instances == 7 and D.n_light_instances == 1  # 5 walls + 2 spheres, then the lamp
    prims = [p for p in d["primitives"]]
    nonlight = [p for p in prims if p["materialName"] != "lamp"]
    for i, p in enumerate(nonlight + [p for p in prims if p["materialName"] == "lamp"]):
        inst = D.instances[i]
        tr = p["transform"]
        if p["type"] == "sphere":  # rotation and scale ignored (SceneReader.cpp:378)
            want = transform(tr["position"], [0, 0, 0], [1, 1, 1])
        else:
            want = transform(tr["position"], tr["rotation"], tr["scale"])
        got = mat(inst.to_wcs)
        assert np.allclose(got, want, atol=2e-6), p["name"]
        assert np.allclose(mat(inst.to_ocs) @ got, np.eye(4), atol=2e-6)
    # rectangles: OCS unit square z = 0 with normal (0, 0, -1)
    rect = D.prims[D.models[D.instances[0].model].prim_begin]
    assert list(rect.p0) == [-0.5, -0.5, 0.0] and list(rect.p1) == [0.5, 0.5, 0.0] and list(rect.p2) == [0, 0, -1]
    # the floor normal faces up, the ceiling normal down
    n_floor = mat(D.instances[0].to_wcs)[:3, :3] @ np.array([0, 0, -1.0])
    n_ceil = mat(D.instances[1].to_wcs)[:3, :3] @ np.array([0, 0, -1.0])
    assert n_floor[1] > 0.999 and n_ceil[1] < -0.999
    # the lamp: a DiffuseLight in the light list, with its primitive registered
    lamp_model = D.models[D.instances[7].model]
    assert lamp_model.light_count == 1 and lamp_model.prim_count == 0
    lp = D.prims[lamp_model.light_begin]
    L = D.lights[D.materials[lp.material].light]
    assert L.type == 0 and list(L.li) == [17.0, 12.0, 4.0] and L.primitive == lamp_model.light_begin
    # glossy materials: roughness used as-is, textures present, textureTypes = last added
    white = D.materials[D.prims[D.models[D.instances[0].model].prim_begin].material]
    assert white.bsdf == 1 and abs(white.roughness - 0.9) < 1e-7 and white.tex_types == 1 << 2
    assert h.spp == 16 and h.bounces == 8 and D.settings.rr_enabled == 1 and D.settings.rr_after == 3


def test_camera_basis():
    h = ne().SceneHost.from_json(scene_path("cornell_c1"))
    c = h.camera_dict()
    pos, look = np.array([0, 1, -2.6]), np.array([0, 1, 0])
    front = (pos - look) / np.linalg.norm(pos - look)
    side = np.cross([0, 1, 0], front)
    side /= np.linalg.norm(side)
    hh = math.tan(math.radians(60) / 2)
    hw = hh * 1.0
    f = 3.0  # autoFocus: glm's vec3::length() is the component count
    ll = pos - f * hw * -side - f * hh * np.array([0, 1, 0]) - f * -front
    assert np.allclose(c["lower_left"], ll, atol=1e-5)
    assert np.allclose(c["horizontal"], 2 * f * hw * -side, atol=1e-5)
    assert np.allclose(c["vertical"], 2 * f * hh * np.array([0, 1, 0]), atol=1e-5)
    assert c["lens_radius"] == np.float32(np.float32(0.0001) / np.float32(2))


def test_medium_scene():
    h = ne().SceneHost.from_json(scene_path("medium_c2"))
    D = h.desc
    assert D.n_media == 1 and D.n_light_instances == 2
    m = D.media[0]
    assert m.type == 0 and list(m.res) == [128, 128, 128] and abs(m.density - 20) < 1e-6
    g = np.ctypeslib.as_array(m.grid, shape=(128 * 128 * 128,))
    assert g.min() == 0.0 and 0.1 < g.max() < 2.0
    assert (g > 0).mean() > 0.05
    # outside the falloff sphere the density is 0
    vol = g.reshape(128, 128, 128)
    assert vol[0, 0, 0] == 0 and vol[64, 64, 0] == 0
    sun = D.lights[0]
    assert sun.type == 1 and list(sun.le) == [3.0, 3.0, 3.0] and list(sun.li) == [0, 0, 0]
    assert abs(math.degrees(math.asin(-sun.direction[1])) - 30.0) < 1e-3
    sky = D.lights[1]
    assert sky.type == 2 and abs(sky.env_radiance[0] - 0.2) < 1e-7 and sky.env_map_pdf == 1.0


def test_fbm_grid_is_deterministic():
    a = ne().SceneHost.from_json(scene_path("medium_c2"))
    b = ne().SceneHost.from_json(scene_path("medium_c2"))
    ga = np.ctypeslib.as_array(a.desc.media[0].grid, shape=(128 ** 3,)).copy()
    gb = np.ctypeslib.as_array(b.desc.media[0].grid, shape=(128 ** 3,))
    assert np.array_equal(ga, gb)
    assert abs(float(ga.astype(np.float64).sum()) - json.load(open(os.path.join(
        os.path.dirname(__file__), "golden", "fbm_checksum.json")))["sum"]) < 1e-3


def test_vol_file_loader(tmp_path):
    # ResourceManager::loadVolasTexture: "X Y Z " line, a skipped line, space-separated values
    (tmp_path / "g.vol").write_text("2 2 1 \nignored\n0.5 1.5 0.25 2 ")
    d = {"version": "1", "materials": [
        {"name": "v", "type": "volume", "scattering": [1, 1, 1], "absorption": [0, 0, 0], "phaseFunction": "isotropic",
         "path": "g.vol", "density": 3}],
         "primitives": [{"name": "b", "type": "volume", "transform": {"position": [0, 0, 0], "scale": [1, 1, 1],
                                                                       "rotation": [0, 0, 0]}, "materialName": "v"}],
         "camera": {"position": [0, 0, -3], "lookAt": [0, 0, 0], "up": [0, 1, 0], "vfov": 45, "aperture": 0.1,
                    "focus": 2}, "renderer": {"resolution": [8, 8], "spp": 1, "bounces": 4, "HDR": False}}
    h = ne().SceneHost.from_string(json.dumps(d), str(tmp_path))
    m = h.desc.media[0]
    assert list(m.res) == [2, 2, 1]
    assert list(np.ctypeslib.as_array(m.grid, shape=(4,))) == [0.5, 1.5, 0.25, 2.0]
    # focus from the descriptor when autoFocus is absent
    assert np.allclose(h.camera_dict()["vertical"], [0, 2 * 2 * math.tan(math.radians(22.5)), 0], atol=1e-5)


def base_scene():
    return json.load(open(scene_path("cornell_c1")))


def fbm_material(**grid):
    g = {"generator": "fbm", "resolution": [8, 8, 8]}
    g.update(grid)
    return {"name": "v", "type": "volume", "scattering": [1, 1, 1], "absorption": [0, 0, 0],
            "phaseFunction": "hg", "g": 0.1, "density": 1, "grid": g}


@pytest.mark.parametrize("mutate,status", [
    (lambda d: d.pop("version"), -2),
    (lambda d: d["materials"].append({"name": "x", "type": "plastic"}), -2),
    (lambda d: d["primitives"][0].update(materialName="nope"), -2),
    (lambda d: d["primitives"][0].update(type="torus"), -2),
    (lambda d: d["materials"][0].pop("roughness"), -2),
    (lambda d: d["primitives"].append({"name": "m", "type": "obj", "path": "a.obj",
                                       "transform": {"position": [0, 0, 0], "scale": [1, 1, 1],
                                                     "rotation": [0, 0, 0]}}), -6),
    (lambda d: d["materials"][0].update(albedo="missing_tex.png"), -3),  # albedo texture file absent
    (lambda d: d["materials"].append({"name": "v", "type": "volume", "scattering": [1, 1, 1],
                                      "absorption": [0, 0, 0], "phaseFunction": "hg", "g": 0.1,
                                      "path": "missing.vol", "density": 1}), -3),
    (lambda d: d["materials"].append({"name": "v", "type": "volume", "scattering": [1, 1, 1],
                                      "absorption": [0, 0, 0], "phaseFunction": "hg", "g": 0.1,
                                      "path": "cloud.vdb", "density": 1}), -3),
    # the grid generator's inputs (an extension): whole voxels per axis, bounded octaves and seed
    (lambda d: d["materials"].append(fbm_material(resolution=[-5, 8, 8])), -2),
    (lambda d: d["materials"].append(fbm_material(resolution=[1e30, 8, 8])), -2),
    (lambda d: d["materials"].append(fbm_material(resolution=[100000, 8, 8])), -2),
    (lambda d: d["materials"].append(fbm_material(octaves=1000000)), -2),
    (lambda d: d["materials"].append(fbm_material(seed=-1)), -2),
])
def test_errors_are_status_codes(mutate, status):
    d = copy.deepcopy(base_scene())
    mutate(d)
    with pytest.raises(ne().NarvalError) as e:
        load(d)
    assert e.value.status == status


def test_malformed_json():
    with pytest.raises(ne().NarvalError) as e:
        ne().SceneHost.from_string('{"version": "1", "materials": [')
    assert e.value.status == -2
    with pytest.raises(ne().NarvalError) as e:
        ne().SceneHost.from_json("/nonexistent/scene.json")
    assert e.value.status == -3


def test_mesh_primitive_and_groups():
    d = base_scene()
    d["primitives"].append({"name": "blob", "type": "mesh", "generator": "icosphere", "subdivisions": 2,
                            "displacement": {"amplitude": 0.1, "frequency": 3, "seed": 7},
                            "groups": {"count": 4, "roughness": [0.05, 0.9], "albedo": [0.2, 0.9], "seed": 3},
                            "transform": {"position": [0, 0.5, 0], "scale": [0.3, 0.3, 0.3], "rotation": [0, 30, 0]}})
    h = load(d)
    D = h.desc
    mesh = D.models[D.instances[D.n_instances - 1].model]
    assert mesh.use_bvh == 1 and mesh.has_bbox == 1 and mesh.prim_count == 20 * 4 ** 2 and mesh.mat_count == 4
    tri = D.prims[mesh.prim_begin]
    assert tri.type == 3 and tri.area > 0
    mats = {D.prims[mesh.prim_begin + k].material for k in range(mesh.prim_count)}
    assert len(mats) == 4
    for m in mats:
        assert 0.05 <= D.materials[m].roughness <= 0.9
