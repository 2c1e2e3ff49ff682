"""The library's (parallel) BVH build against the oracle's sequential BVH::init: the node
arrays (bounds bits, ranges, right offsets) and the primitive order must be identical."""
import ctypes as C
import json
import time

import numpy as np
import pytest

from conftest import scene_path


@pytest.mark.parametrize("subdiv", [3, 6, 8])
def test_parallel_build_equals_reference_build(built, oracle_lib, subdiv):
    import narvalengine_gb300 as ne
    d = json.load(open(scene_path("mesh_c3")))
    d["primitives"][0]["subdivisions"] = subdiv
    text = json.dumps(d)
    host = ne.SceneHost.from_string(text)
    desc = host.desc
    m = next(i for i in range(desc.n_models) if desc.models[i].use_bvh and desc.models[i].prim_count > 4)
    model = desc.models[m]
    n = model.prim_count
    nodes = np.empty((2 * n + 1, 9), np.float32)
    order = np.empty(n, np.uint32)
    count = C.c_size_t()
    t0 = time.perf_counter()
    st = ne.library().ne_debug_bvh(C.cast(desc.prims, C.c_void_p), model.prim_begin, n, nodes.ctypes.data, len(nodes),
                                   order.ctypes.data, C.byref(count))
    t_lib = time.perf_counter() - t0
    assert st == 0
    nodes = nodes[:count.value]
    orc = oracle_lib.OracleScene.from_json(text=text)
    try:
        ref_nodes, ref_order = orc.model_bvh(m, n)
    finally:
        orc.close()
    assert len(nodes) == len(ref_nodes)
    assert np.array_equal(nodes.view(np.uint32), ref_nodes.view(np.uint32))
    assert np.array_equal(order, ref_order)
    print(f"{n} triangles, {len(nodes)} nodes, library build {t_lib * 1e3:.1f} ms")


@pytest.mark.parametrize("kind", ["coincident", "exponential", "thin"])
def test_degenerate_meshes_build_alike(built, oracle_lib, kind):
    """Meshes the midpoint split cannot separate (every centroid equal: the range is halved),
    that it separates one triangle at a time (exponentially spaced), or that are flat along
    two axes: the library's build and the oracle's BVH::init give the same nodes and order."""
    import narvalengine_gb300 as ne
    rng = np.random.default_rng(3)
    n = 3000
    if kind == "coincident":
        c = np.full((n, 3), 0.5)
    elif kind == "exponential":
        c = np.zeros((n, 3))
        c[:, 0] = 2.0 ** (np.arange(n) % 40 - 20)
    else:
        c = np.zeros((n, 3))
        c[:, 2] = rng.random(n)
    pos = (c[:, None, :] + 0.01 * rng.standard_normal((n, 3, 3))).astype(np.float32).reshape(-1)
    d = json.load(open(scene_path("cornell_c1")))
    d["primitives"].append({"name": "blob", "type": "mesh", "positions": [float(x) for x in pos],
                            "indices": list(range(3 * n)), "materialName": d["materials"][0]["name"],
                            "transform": {"position": [0, 0, 0], "rotation": [0, 0, 0], "scale": [1, 1, 1]}})
    text = json.dumps(d)
    host = ne.SceneHost.from_string(text)
    desc = host.desc
    m = next(i for i in range(desc.n_models) if desc.models[i].use_bvh and desc.models[i].prim_count == n)
    model = desc.models[m]
    nodes = np.empty((2 * n + 1, 9), np.float32)
    order = np.empty(n, np.uint32)
    count = C.c_size_t()
    assert ne.library().ne_debug_bvh(C.cast(desc.prims, C.c_void_p), model.prim_begin, n, nodes.ctypes.data,
                                     len(nodes), order.ctypes.data, C.byref(count)) == 0
    nodes = nodes[:count.value]
    orc = oracle_lib.OracleScene.from_json(text=text)
    try:
        ref_nodes, ref_order = orc.model_bvh(m, n)
    finally:
        orc.close()
    assert np.array_equal(nodes.view(np.uint32), ref_nodes.view(np.uint32))
    assert np.array_equal(order, ref_order)
    assert sorted(order.tolist()) == list(range(model.prim_begin, model.prim_begin + n))
