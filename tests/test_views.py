"""Many views in one launch (ne_views) against the oracle, view by view.

Each view's image must equal the oracle's per-pixel mean of the same camera paths (the
view's camera and size, random stream = view index + 1), summed in sample order, bit for
bit; the launch order, the fetch size, the resident blocks and the CUDA-graph replay must
not change any image."""
import numpy as np
import pytest

from conftest import scene_path

pytestmark = pytest.mark.gpu


def oracle_mean(L, w, h, spp):
    acc = np.zeros((w * h, 3), np.float32)
    L = L.reshape(w * h, spp, 3)
    for k in range(spp):
        acc = (acc + L[:, k]).astype(np.float32)
    return (acc / np.float32(spp)).reshape(h, w, 3)


@pytest.fixture(scope="module", params=["cornell_c1", "medium_c2"])
def batch(request, built, oracle_lib):
    import narvalengine_gb300 as ne
    ctx = ne.Context(0)
    host = ne.SceneHost.from_json(scene_path(request.param))
    scene = ctx.upload(host)
    cam0 = host.desc.camera
    look = [0, 1, 0] if request.param == "cornell_c1" else [0, 0, 0]
    eye = list(cam0.position)
    sizes = [(32, 32, 3), (48, 24, 2), (16, 16, 4), (40, 56, 1), (64, 40, 2)]
    views = []
    for i, (w, h, spp) in enumerate(sizes):
        pos = [eye[0] + 0.15 * i, eye[1] + 0.05 * i, eye[2]]
        views.append((ne.camera_look_at(pos, look, 50.0 + 3 * i, w, h), w, h, spp))
    vb = ne.Views(scene, views, seed=11)
    orc = oracle_lib.OracleScene.from_json(scene_path(request.param))
    yield ne, scene, vb, views, orc
    orc.close()
    vb.close()
    ctx.close()


def oracle_images(ne, orc, views):
    out = []
    p = ne.render_params(seed=11)
    for v, (cam, w, h, spp) in enumerate(views):
        keys = np.array([[px, s] for px in range(w * h) for s in range(spp)], np.uint32)
        L = orc.trace_view_paths(cam, w, h, v + 1, keys, p)
        out.append(oracle_mean(L, w, h, spp))
    return out


def test_views_match_oracle(batch):
    ne, scene, vb, views, orc = batch
    st = vb.render()
    assert st["paths"] == sum(w * h * s for _, w, h, s in views)
    want = oracle_images(ne, orc, views)
    for v in range(len(views)):
        got = vb.image(v)
        assert np.array_equal(got.view(np.uint32), want[v].view(np.uint32)), f"view {v}"


def test_tunings_do_not_change_images(batch):
    ne, scene, vb, views, orc = batch
    vb.set_tuning(fetch=32, order=0, graph=False, split_passes=1)
    vb.render()
    ref = [vb.image(v) for v in range(len(views))]
    for fetch, bps, order, graph, sp, groups, pre in [(128, 0, 1, True, 0, 1, 0), (64, 2, 2, True, 1, 1, 0),
                                                      (32, 1, 1, False, 4, 1, 0), (32, 0, 2, True, 8, 1, 0),
                                                      (128, 0, 0, False, 2, 1, 0), (32, 0, 1, True, -12, 1, 0),
                                                      (64, 0, 2, False, -5, 1, 0), (32, 0, 2, True, -12, 2, 0),
                                                      (32, 0, 2, False, 4, 3, 0), (128, 0, 1, True, -8, 5, 0),
                                                      (32, 0, 0, True, 1, 16, 0), (32, 0, 2, True, -12, 2, 1),
                                                      (64, 0, 1, False, 6, 1, 1), (32, 0, 2, True, 1, 1, 1),
                                                      (32, 0, 2, True, -12, 2, 2), (64, 0, 1, False, 6, 1, 2),
                                                      (32, 0, 2, True, 1, 1, 2)]:
        # negative: that many passes with deferral points every half bounce; pre: the bounce
        # rays (1), and the camera rays too (2), traced ahead of each pass
        vb.set_tuning(fetch=fetch, blocks_per_sm=bps, order=order, graph=graph, split_passes=abs(sp),
                      split_half=int(sp < 0), groups=groups, pretrace=pre)
        st = vb.render()
        for v in range(len(views)):
            assert np.array_equal(vb.image(v), ref[v]), (fetch, bps, order, graph, sp, groups, pre, v)
        lat = vb.latency()
        assert np.all(lat > 0) and lat.max() <= st["ms"] * 1.5 + 1.0, (lat, st)
        assert st["latency_p50_ms"] <= st["latency_p99_ms"] <= st["latency_max_ms"]
        passes = abs(sp) or 6
        passes += 1 if pre == 2 and passes > 1 else 0  # the pass that only queues the paths
        per_group = passes + (passes - 1 if pre and passes > 1 else 0)
        launches = st["kernel_launches"] - 1  # the pixel means
        assert launches % per_group == 0 and 1 <= launches // per_group <= min(groups, len(views)), st


def test_groups_complete_views_early(batch):
    """Views of the first group (smallest first) complete before the batch's last group
    starts: their latency is well below the last view's."""
    ne, scene, vb, views, orc = batch
    vb.set_tuning(fetch=32, order=2, graph=True, split_passes=8, split_half=0, groups=len(views))
    vb.render()
    st = vb.render()
    lat = vb.latency()
    sizes = np.array([w * h * s for _, w, h, s in views])
    first = np.argmin(sizes)
    assert lat[first] < 0.8 * lat.max(), (lat, sizes)
    assert st["latency_p50_ms"] < st["latency_max_ms"]


def test_autotune(batch):
    ne, scene, vb, views, orc = batch
    vb.render()
    ref = [vb.image(v) for v in range(len(views))]
    best, ms = vb.autotune(repeats=1)
    assert ms > 0 and best["fetch"] in (32, 128) and best["order"] in (1, 2) and best["graph"] == 1
    assert (best["split_passes"], best["split_half"]) in ((8, 0), (12, 1), (16, 1)) and best["groups"] in (1, 2, 4)
    assert best["pretrace"] in (0, 1, 2)
    assert vb.tuning() == best
    vb.render()
    for v in range(len(views)):
        assert np.array_equal(vb.image(v), ref[v])
