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
