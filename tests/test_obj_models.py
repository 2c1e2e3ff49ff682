"""OBJ models ("type": "obj" primitives, SceneReader.cpp:245-266): the file reader, shared
models for instances of the same file and material, and the reference's BVH test on a cube
model (unitTests/tests.cpp:866-889, whose cube.obj is not in the reference tree; the cube
here spans [-1, 1] as that test states)."""
import json

import numpy as np
import pytest

CUBE = """# unit cube [-1, 1]
v -1 -1 -1
v 1 -1 -1
v 1 1 -1
v -1 1 -1
v -1 -1 1
v 1 -1 1
v 1 1 1
v -1 1 1
f 1 2 3 4
f 5/1 8/2 7/3 6/4
f 1//1 5//1 6//1 2//1
f 4/1/1 3/2/1 7/3/1 8/4/1
f -8 -4 -1 -5
f 2 6 7 3
"""


def scene(tmp_path, prims):
    (tmp_path / "cube.obj").write_text(CUBE)
    d = {"version": "0.0.1a",
         "materials": [{"name": "grey", "type": "microfacet", "roughness": 0.5, "metallic": 0.0,
                        "albedo": [0.7, 0.7, 0.7]},
                       {"name": "red", "type": "microfacet", "roughness": 0.3, "metallic": 0.0,
                        "albedo": [0.8, 0.1, 0.1]},
                       {"name": "lamp", "type": "emitter", "albedo": [8.0, 8.0, 8.0]}],
         "primitives": prims + [{"name": "light", "type": "rectangle", "materialName": "lamp",
                                 "transform": {"position": [0, 4, 0], "scale": [1, 1, 1], "rotation": [-90, 0, 0]}}],
         "camera": {"position": [0, 1, -6], "lookAt": [0, 0, 0], "up": [0, 1, 0], "vfov": 50, "aperture": 0.0001,
                    "autoFocus": True, "focus": 1},
         "renderer": {"resolution": [48, 32], "spp": 2, "bounces": 6, "mode": "offline", "HDR": True}}
    return json.dumps(d)


def obj(name, mat, pos, scale=1.0, rot=0.0):
    return {"name": name, "type": "obj", "path": "cube.obj", "materialName": mat,
            "transform": {"position": pos, "scale": [scale] * 3, "rotation": [0, rot, 0]}}


def test_obj_reader_and_shared_models(built, tmp_path):
    import narvalengine_gb300 as ne
    host = ne.SceneHost.from_string(scene(tmp_path, [obj("a", "grey", [-1.5, 0, 0]), obj("b", "grey", [1.5, 0, 0], 0.5, 30),
                                                     obj("c", "red", [0, 0, 2])]), str(tmp_path))
    d = host.desc
    inst_models = [d.instances[i].model for i in range(d.n_instances)]
    assert inst_models[0] == inst_models[1] != inst_models[2]  # same file + material: one model
    m = d.models[inst_models[0]]
    assert m.prim_count == 12 and m.use_bvh
    tris = np.array([[list(d.prims[m.prim_begin + t].p0), list(d.prims[m.prim_begin + t].p1),
                      list(d.prims[m.prim_begin + t].p2)] for t in range(12)], np.float32)
    assert np.all(np.abs(tris) == 1.0)
    # fan triangulation of the first quad "f 1 2 3 4": (1,2,3), (1,3,4)
    assert np.array_equal(tris[0], [[-1, -1, -1], [1, -1, -1], [1, 1, -1]])
    assert np.array_equal(tris[1], [[-1, -1, -1], [1, 1, -1], [-1, 1, -1]])
    # the negative-index face "f -8 -4 -1 -5" = vertices 1 5 8 4
    assert np.array_equal(tris[8], [[-1, -1, -1], [-1, -1, 1], [-1, 1, 1]])


@pytest.mark.parametrize("prims,status", [
    ([{"name": "a", "type": "obj", "path": "missing.obj", "materialName": "grey",
       "transform": {"position": [0, 0, 0], "scale": [1, 1, 1], "rotation": [0, 0, 0]}}], -3),
    ([{"name": "a", "type": "obj", "path": "cube.obj",
       "transform": {"position": [0, 0, 0], "scale": [1, 1, 1], "rotation": [0, 0, 0]}}], -6),
    ([{"name": "a", "type": "gltf", "path": "cube.gltf", "materialName": "grey",
       "transform": {"position": [0, 0, 0], "scale": [1, 1, 1], "rotation": [0, 0, 0]}}], -6),
])
def test_obj_errors(built, tmp_path, prims, status):
    import narvalengine_gb300 as ne
    with pytest.raises(ne.NarvalError) as e:
        ne.SceneHost.from_string(scene(tmp_path, prims), str(tmp_path))
    assert e.value.status == status


def test_reference_bvh_cube_intersections(built, oracle_lib, tmp_path):
    """tests.cpp:866-889: a ray from (0,0,-2) along +z and one from the centre along +z both hit
    the cube at t = 1 (the faces behind the origin are rejected by the triangle test)."""
    import narvalengine_gb300 as ne
    text = scene(tmp_path, [obj("cube", "grey", [0, 0, 0])])
    orc = oracle_lib.OracleScene.from_json(text=text, resources_dir=str(tmp_path))
    try:
        rays = np.array([[0, 0, -2, 0, 0, 1], [0, 0, 0, 0, 0, 1]], np.float32)
        h = orc.trace_closest(rays, 1e-11, float("inf"))
    finally:
        orc.close()
    assert np.all(h["hit"] == 1)
    assert np.allclose(h["t_near"], 1.0, atol=1e-3)


@pytest.mark.gpu
def test_obj_scene_parity(built, oracle_lib, tmp_path):
    import narvalengine_gb300 as ne
    text = scene(tmp_path, [obj("a", "grey", [-1.5, 0, 0]), obj("b", "grey", [1.5, 0, 0], 0.5, 30),
                            obj("c", "red", [0, 0, 2])])
    host = ne.SceneHost.from_string(text, str(tmp_path))
    ctx = ne.Context(0)
    orc = oracle_lib.OracleScene.from_json(text=text, resources_dir=str(tmp_path))
    try:
        gpu_scene = ctx.upload(host)
        for kernel in (0, 3):
            gpu_scene.set_tuning(kernel=kernel)
            img, _ = gpu_scene.render(seed=4, spp=2)
            ref, _ = orc.render(ne.render_params(seed=4, spp=2))
            assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), kernel
    finally:
        orc.close()
        ctx.close()
