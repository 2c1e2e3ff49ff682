"""The GPU binned-SAH BVH ("bvh": "sah" in a scene's renderer block; bvh_build.cu).

The tree is checked for validity on the host (every triangle once, leaves of at most four,
bounds that contain their contents, depth within the traversal stack), the device traversal
over it against the oracle traversing the same tree (bit-exact hits, paths and images), and
its closest hits against the reference's own midpoint tree (equal except for ties at exactly
the same distance).
"""
import json

import numpy as np
import pytest

from conftest import scene_path

pytestmark = pytest.mark.gpu


def mesh_json(subdivisions, bvh="sah", res=(160, 120)):
    d = json.load(open(scene_path("mesh_c3")))
    d["primitives"][0]["subdivisions"] = subdivisions
    d["renderer"]["resolution"] = list(res)
    d["renderer"]["bvh"] = bvh
    return json.dumps(d)


def camera_rays(host, n, seed):
    import test_gpu_parity as t
    return t.camera_rays(host, n, seed)


def tri_bounds(host, model):
    import ctypes as C
    from narvalengine_gb300 import _abi
    d = C.cast(host.desc_ptr, C.POINTER(_abi.NeSceneDesc)).contents
    m = d.models[model]
    prims = np.ctypeslib.as_array(d.prims, shape=(d.n_prims,))[m.prim_begin:m.prim_begin + m.prim_count]
    pts = np.stack([prims["p0"], prims["p1"], prims["p2"]], axis=1).astype(np.float32)
    return m.prim_begin, pts.min(axis=1), pts.max(axis=1)


def check_tree(nodes, order, first, lo, hi):
    n = len(order)
    bits = nodes[:, 6:9].view(np.uint32)
    assert np.array_equal(np.sort(order), np.arange(first, first + n, dtype=np.uint32))
    depth_max = 0
    stack = [(0, 0)]
    seen = 0
    while stack:
        i, depth = stack.pop()
        depth_max = max(depth_max, depth)
        start, count, ro = bits[i]
        mn, mx = nodes[i, 0:3], nodes[i, 3:6]
        if ro == 0:  # leaf
            assert 1 <= count <= 4
            idx = order[start:start + count] - first
            assert np.all(lo[idx] >= mn) and np.all(hi[idx] <= mx)
            seen += count
        else:
            for c in (i + 1, i + ro):
                assert np.all(nodes[c, 0:3] >= mn) and np.all(nodes[c, 3:6] <= mx)
                stack.append((c, depth + 1))
    assert seen == n
    assert depth_max <= 62
    return depth_max


@pytest.mark.parametrize("subdivisions", [4, 8])
def test_sah_tree_valid_and_parity(built, oracle_lib, subdivisions):
    import narvalengine_gb300 as ne
    text = mesh_json(subdivisions)
    host = ne.SceneHost.from_string(text)
    ctx = ne.Context(0)
    orc = oracle_lib.OracleScene.from_json(text=text)
    try:
        scene = ctx.upload(host)
        models = [m for m in range(host.n_models) if host.model_uses_bvh(m)]
        assert models
        rays = camera_rays(host, 20000, 11)
        ref_hits = orc.trace_closest(rays, 1e-11, float("inf"))  # the oracle's own (reference) tree
        for m in models:
            nodes, order = scene.bvh(m)
            first, lo, hi = tri_bounds(host, m)
            if len(order) <= 100000:  # the host walk of the tree is slow beyond that
                check_tree(nodes, order, first, lo, hi)
            else:
                assert np.array_equal(np.sort(order), np.arange(first, first + len(order), dtype=np.uint32))
            orc.set_model_bvh(m, nodes, order)
        g = scene.trace_closest(rays, 1e-11, float("inf"))
        c = orc.trace_closest(rays, 1e-11, float("inf"))
        for f in ("hit", "instance", "primitive"):
            assert np.array_equal(g[f], c[f]), f
        for f in ("t_near", "point", "normal"):
            assert np.array_equal(g[f].view(np.uint32), c[f].view(np.uint32)), f
        # against the reference's midpoint tree: the same closest hits but for exact ties
        same = (g["primitive"] == ref_hits["primitive"]) & (g["t_near"] == ref_hits["t_near"])
        assert same.mean() >= 0.999, same.mean()
        hit = g["hit"].astype(bool)
        assert np.array_equal(hit, ref_hits["hit"].astype(bool))
        assert np.array_equal(g["t_near"][hit], ref_hits["t_near"][hit])
        keys = np.array([[p, s] for p in range(0, host.width * host.height, 7) for s in range(2)], np.uint32)
        for kernel in (0, 3):
            scene.set_tuning(kernel=kernel)
            gp = scene.trace_paths(keys, ne.render_params(seed=8))
            cp = orc.trace_paths(keys, ne.render_params(seed=8))
            assert np.array_equal(gp.view(np.uint32), cp.view(np.uint32)), kernel
        img, _ = scene.render(ne.render_params(seed=2, spp=1))
        ref, _ = orc.render(ne.render_params(seed=2, spp=1))
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    finally:
        orc.close()
        ctx.close()


def test_sah_tree_is_deterministic_and_cheaper(built):
    """Two uploads build the same tree; its traversal visits fewer nodes than the midpoint
    tree's on the same camera paths."""
    import narvalengine_gb300 as ne
    ctx = ne.Context(0)
    try:
        hs = ne.SceneHost.from_string(mesh_json(7))
        a, b = ctx.upload(hs), ctx.upload(hs)
        m = [k for k in range(hs.n_models) if hs.model_uses_bvh(k)][0]
        na, oa = a.bvh(m)
        nb, ob = b.bvh(m)
        assert np.array_equal(na.view(np.uint32), nb.view(np.uint32)) and np.array_equal(oa, ob)
        hr = ne.SceneHost.from_string(mesh_json(7, bvh="reference"))
        r = ctx.upload(hr)
        p = ne.render_params(seed=1, spp=1, flags=ne.NE_RENDER_COUNT_WORK)
        _, ss = a.render(p)
        _, sr = r.render(p)
        assert ss["bvh_nodes"] < sr["bvh_nodes"], (ss["bvh_nodes"], sr["bvh_nodes"])
    finally:
        ctx.close()
