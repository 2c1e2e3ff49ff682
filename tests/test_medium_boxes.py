"""World-space medium boxes against the oracle's closest hits (CPU only).

The kernels for meshes with media skip intersectTr's walk (VolumetricPathIntegrator.cpp:10-32)
for an MIS ray whose forward line misses every box that ne_scene_upload bounds the media with;
the walk can report a hit and draw random numbers only at a medium. Here every ray whose closest
hit in the oracle (Scene::intersectScene, Scene.cpp:30-56) is a medium primitive must pass the
box test: rays aimed at the medium's corners, edges and faces (grazing ones included), rays
leaving points on its surface, and rays in random directions. Rays aimed away must be rejected,
or the skip would save nothing.
"""
import ctypes as C
import json

import numpy as np

from conftest import scene_path


def mixed_json():
    d = json.load(open(scene_path("views_c5")))
    for p in d["primitives"]:
        if p.get("type") == "mesh":
            p["subdivisions"] = 3
    d["renderer"]["resolution"] = [64, 48]
    d["renderer"]["bvh"] = "reference"
    return json.dumps(d)


def mixed_host(ne):
    return ne.SceneHost.from_string(mixed_json())


def medium_boxes(ne, host):
    n = C.c_int32()
    buf = np.zeros((64, 6), np.float32)
    st = ne.library().ne_debug_medium_boxes(host.desc_ptr, buf.ctypes.data, 64, C.byref(n))
    assert st == 0
    return buf[:max(n.value, 0)], n.value


def may_reach(boxes, o, d):
    """The kernels' test (mayReachMedium), vectorised: the forward line meets a box."""
    ok = np.zeros(len(o), bool)
    with np.errstate(divide="ignore", invalid="ignore"):
        for b in boxes:
            lo, hi = b[:3], b[3:]
            t_near = np.zeros(len(o), np.float32)
            t_far = np.full(len(o), np.inf, np.float32)
            miss = np.zeros(len(o), bool)
            for a in range(3):
                zero = d[:, a] == 0
                miss |= zero & ((o[:, a] < lo[a]) | (o[:, a] > hi[a]))
                t0 = (lo[a] - o[:, a]) / d[:, a]
                t1 = (hi[a] - o[:, a]) / d[:, a]
                tn = np.where(zero, -np.inf, np.minimum(t0, t1))
                tf = np.where(zero, np.inf, np.maximum(t0, t1))
                t_near = np.maximum(t_near, tn)
                t_far = np.minimum(t_far, tf)
            ok |= ~miss & ~(t_near > t_far)
    return ok


def medium_prims(host):
    """(primitive index, world-space corners) of every primitive with a medium material."""
    D = host.desc
    out = []
    for i in range(D.n_instances + D.n_light_instances):
        inst = D.instances[i]
        m = D.models[inst.model]
        W = np.array(inst.to_wcs[:16], np.float64).reshape(4, 4).T  # column-major
        for k in range(m.prim_begin, m.prim_begin + m.prim_count):
            p = D.prims[k]
            if p.material >= 0 and D.materials[p.material].medium >= 0:
                lo = np.array(p.p0[:3], np.float64)
                hi = np.array(p.p1[:3], np.float64)
                c = np.array([[(hi if j & 1 else lo)[0], (hi if j & 2 else lo)[1], (hi if j & 4 else lo)[2], 1.0]
                              for j in range(8)])
                out.append((k, (W @ c.T).T[:, :3]))
    return out


def test_medium_boxes_cover_oracle_hits(built, oracle_lib):
    import narvalengine_gb300 as ne
    host = mixed_host(ne)
    boxes, n = medium_boxes(ne, host)
    assert n == 1
    (prim, corners), = medium_prims(host)
    lo, hi = corners.min(0), corners.max(0)
    assert np.all(boxes[0, :3] < lo) and np.all(boxes[0, 3:] > hi)
    assert np.all(boxes[0, 3:] - boxes[0, :3] < (hi - lo) * 1.01 + 0.05)

    rng = np.random.default_rng(7)
    n_rays = 60000
    origins = rng.uniform([-6, 0.0, -6], [6, 5, 6], (n_rays, 3))
    # targets on the medium's surface: a random face point, an edge point, or a corner
    face = rng.integers(0, 3, n_rays)
    t = rng.uniform(lo, hi, (n_rays, 3))
    side = rng.integers(0, 2, n_rays)
    t[np.arange(n_rays), face] = np.where(side == 1, hi[face], lo[face])
    edge = rng.random(n_rays) < 0.3
    face2 = (face + 1) % 3
    t[edge, face2[edge]] = np.where(rng.integers(0, 2, edge.sum()) == 1, hi[face2[edge]], lo[face2[edge]])
    corner = rng.random(n_rays) < 0.1
    t[corner] = corners[rng.integers(0, 8, corner.sum())]
    t += rng.normal(0, 1e-5, t.shape) * (rng.random((n_rays, 1)) < 0.5)
    aimed_d = t - origins
    # rays leaving points on the surface, and rays in random directions
    leave_o = t[: n_rays // 3]
    leave_d = rng.normal(size=(len(leave_o), 3))
    rand_d = rng.normal(size=(n_rays, 3))
    o = np.concatenate([origins, leave_o, origins]).astype(np.float32)
    d = np.concatenate([aimed_d, leave_d, rand_d]).astype(np.float32)

    orc = oracle_lib.OracleScene.from_json(text=mixed_json())
    try:
        hits = orc.trace_closest(np.concatenate([o, d], 1), 1e-3, float("inf"))
    finally:
        orc.close()
    reaches = hits["primitive"] == prim
    passes = may_reach(boxes, o, d)
    assert reaches[:n_rays].sum() > n_rays // 2
    assert not np.any(reaches & ~passes), f"{np.sum(reaches & ~passes)} medium hits outside the boxes"
    rand = slice(n_rays + len(leave_o), None)
    assert (~passes[rand]).mean() > 0.5


def test_scene_without_media_has_no_boxes(built):
    import narvalengine_gb300 as ne
    host = ne.SceneHost.from_json(scene_path("cornell_c1"))
    boxes, n = medium_boxes(ne, host)
    assert n == 0 and len(boxes) == 0
    assert ne.library().ne_debug_medium_boxes(None, None, 0, C.byref(C.c_int32())) != 0


def test_rectangle_media_are_bounded_only_when_their_hits_are(built):
    """Rectangle::intersect (Rectangle.cpp:50-76) checks containment only on the axes where the
    corners differ, so a rectangle's corners bound its hits only when they agree on exactly one
    axis and the plane normal lies along it; otherwise no boxes are given (every ray walks)."""
    import narvalengine_gb300 as ne
    host = mixed_host(ne)
    (prim, _), = medium_prims(host)
    p = host.desc.prims[prim]
    p.type = 1  # NE_PRIM_RECTANGLE
    p.p0[0], p.p0[1], p.p0[2] = -0.5, -0.5, 0.0
    p.p1[0], p.p1[1], p.p1[2] = 0.5, 0.5, 0.0
    p.p2[0], p.p2[1], p.p2[2] = 0.0, 0.0, -1.0
    assert medium_boxes(ne, host)[1] == 1
    p.p2[0] = 0.5  # tilted plane: z is free within the x extent
    assert medium_boxes(ne, host)[1] == -1
    p.p2[0] = 0.0
    p.p1[1] = -0.5  # corners agree on y and z: a hit's y is free on the plane
    assert medium_boxes(ne, host)[1] == -1
