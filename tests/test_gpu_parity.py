"""GPU parity: the CUDA integrator against the CPU oracle, through the C ABI.

Bar: bit-exact for hit/miss decisions, hit indices, t values, random numbers and the
shared elementary functions; per-path radiance within 1e-4 relative (per channel,
denominator max(|oracle|, 1e-6)) on identical (seed, pixel, sample) keys. In practice the
two sides perform the same IEEE operations, so the radiance is expected to match exactly
and the tests also report the exact-match fraction.
"""
import numpy as np
import pytest

from conftest import scene_path

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4


@pytest.fixture(scope="module")
def ne(built):
    import narvalengine_gb300 as ne
    return ne


@pytest.fixture(scope="module")
def ctx(ne):
    c = ne.Context(0)
    yield c
    c.close()


KERNELS = {0: "straight", 1: "regrouped", 2: "lanes", 3: "split"}


@pytest.fixture(scope="module", params=[(s, k) for s in ("cornell_c1", "medium_c2") for k in KERNELS],
                ids=lambda p: f"{p[0]}-{KERNELS[p[1]]}")
def scenes(request, ne, ctx, oracle_lib):
    name, kernel = request.param
    host = ne.SceneHost.from_json(scene_path(name))
    scene = ctx.upload(host)
    scene.set_tuning(kernel=kernel)
    orc = oracle_lib.OracleScene.from_json(scene_path(name))
    yield name, host, scene, orc
    scene.close()
    orc.close()


def rel_err(gpu, cpu):
    return np.abs(gpu - cpu) / np.maximum(np.abs(cpu), 1e-6)


def spread_keys(host, n_pixels, spp, seed=0):
    rng = np.random.default_rng(seed)
    pix = rng.choice(host.width * host.height, size=n_pixels, replace=False)
    return np.array([[p, s] for p in pix for s in range(spp)], dtype=np.uint32)


@pytest.mark.parametrize("fn,lo,hi", [(0, 1e-30, 1e30), (1, -100.0, 88.0), (2, -60.0, 60.0), (3, -60.0, 60.0),
                                      (4, -1.0, 1.0), (5, -3.0, 3.0), (6, -50.0, 50.0), (7, 0.0, 1.0 - 2 ** -24)])
def test_fmath_bit_exact(ctx, oracle_lib, fn, lo, hi):
    rng = np.random.default_rng(fn)
    if fn == 0:
        x = np.exp(rng.uniform(np.log(lo), np.log(hi), 200000)).astype(np.float32)
        x = np.concatenate([x, np.array([1.0, 2.0, 0.5, 1e-45, 3.4e38, 1 - 2 ** -24, 2 ** -24], np.float32)])
    else:
        x = rng.uniform(lo, hi, 200000).astype(np.float32)
        x = np.concatenate([x, np.array([0.0, -0.0, lo, hi], np.float32)])
    g = ctx.fmath(fn, x)
    c = oracle_lib.fmath(fn, x)
    assert np.array_equal(g.view(np.uint32), c.view(np.uint32)), f"fn {fn}: {np.sum(g != c)} mismatches"


def test_rng_bit_exact(ctx, oracle_lib):
    rng = np.random.default_rng(3)
    n = 100000
    keys = rng.integers(0, 2 ** 32, size=(n, 2), dtype=np.uint64).astype(np.uint32)
    dims = rng.integers(0, 5000, size=n, dtype=np.uint64).astype(np.uint32)
    for seed in (0, 0x4E415256, 2 ** 63 + 12345):
        g = ctx.rng(seed, keys, dims)
        c = oracle_lib.rng(seed, keys, dims)
        assert np.array_equal(g.view(np.uint32), c.view(np.uint32))
        assert g.min() >= 0.0 and g.max() < 1.0


def camera_rays(host, n, seed):
    """Rays from the camera through random pixels, plus rays from random interior points."""
    rng = np.random.default_rng(seed)
    cam = host.camera_dict()
    u = rng.random(n, dtype=np.float32)
    v = rng.random(n, dtype=np.float32)
    ll = np.array(cam["lower_left"], np.float32)
    pos = np.array(cam["position"], np.float32)
    pt = ll + u[:, None] * np.array(cam["horizontal"], np.float32) + v[:, None] * np.array(cam["vertical"], np.float32)
    d = -(pt - pos)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.broadcast_to(pos, d.shape)
    o2 = rng.uniform(-0.9, 0.9, size=(n, 3)).astype(np.float32) + np.array([0, 1.0, 0], np.float32)
    d2 = rng.normal(size=(n, 3)).astype(np.float32)
    d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
    rays = np.concatenate([np.concatenate([o, d], 1), np.concatenate([o2, d2], 1)]).astype(np.float32)
    return rays


@pytest.mark.parametrize("tmin", [1e-11, 1e-3])
def test_closest_hit_bit_exact(scenes, tmin):
    name, host, scene, orc = scenes
    rays = camera_rays(host, 20000, 5)
    g = scene.trace_closest(rays, tmin, float("inf"))
    c = orc.trace_closest(rays, tmin, float("inf"))
    assert np.array_equal(g["hit"], c["hit"])
    assert np.array_equal(g["instance"], c["instance"])
    assert np.array_equal(g["primitive"], c["primitive"])
    for f in ("t_near", "t_far", "point", "normal"):
        assert np.array_equal(g[f].view(np.uint32), c[f].view(np.uint32)), f"{name}: field {f} differs"
    assert g["hit"].sum() > 0


def test_camera_paths_parity(scenes, ne):
    name, host, scene, orc = scenes
    keys = spread_keys(host, 1024, 4, seed=1)
    for seed in (0, 77):
        p = ne.render_params(seed=seed)
        g = scene.trace_paths(keys, p)
        c = orc.trace_paths(keys, p)
        assert np.isfinite(g).all()
        err = rel_err(g, c)
        exact = np.mean(np.all(g == c, axis=1))
        assert err.max() <= REL_TOL, f"{name} seed {seed}: max rel {err.max():.3e}, exact {exact:.4f}"
        assert exact == 1.0, f"{name}: only {exact:.4f} of paths bit-identical"


def test_li_batch_parity(scenes, ne):
    name, host, scene, orc = scenes
    rays = camera_rays(host, 2048, 9)
    rng = np.random.default_rng(2)
    keys = rng.integers(0, 1 << 20, size=(len(rays), 2), dtype=np.uint64).astype(np.uint32)
    p = ne.render_params(seed=5)
    for first_dim in (0, 4, 1001):
        g = scene.li_batch(rays, keys, first_dim, p)
        c = orc.li_batch(rays, keys, first_dim, p)
        assert rel_err(g, c).max() <= REL_TOL, f"{name} first_dim {first_dim}"


def test_render_matches_oracle(scenes, ne):
    name, host, scene, orc = scenes
    p = ne.render_params(seed=3, spp=2)
    g, stats = scene.render(p)
    c, _ = orc.render(p)
    assert stats["paths"] == host.width * host.height * 2
    assert rel_err(g, c).max() <= REL_TOL, f"{name}: image differs"
    assert np.array_equal(g, c), f"{name}: image not bit-identical"


def test_render_ref_tiles(ne, ctx, oracle_lib):
    # 250 x 130: the reference's 40 x 10 tiles of (6, 13) cover 240 x 130 pixels only
    host = ne.SceneHost.from_json(scene_path("cornell_c1"))
    import json
    d = json.load(open(scene_path("cornell_c1")))
    d["renderer"]["resolution"] = [250, 130]
    text = json.dumps(d)
    host = ne.SceneHost.from_string(text)
    scene = ctx.upload(host)
    p = ne.render_params(seed=1, spp=1, flags=ne.NE_RENDER_REF_TILES)
    g, stats = scene.render(p)
    c, _ = oracle_lib.OracleScene.from_json(text=text).render(p)
    assert stats["paths"] == 240 * 130
    assert np.all(g[:, 240:] == 0)
    assert np.array_equal(g, c)


def test_progressive_and_deterministic(ne, ctx):
    host = ne.SceneHost.from_json(scene_path("cornell_c1"))
    scene = ctx.upload(host)
    a, _ = scene.render(ne.render_params(seed=9, spp=4))
    b, _ = scene.render(ne.render_params(seed=9, spp=4))
    assert np.array_equal(a, b)
    # samples [0, 2) and [2, 4) rendered separately: their means average to the 4-sample mean
    lo, _ = scene.render(ne.render_params(seed=9, spp=2, sample_offset=0))
    hi, _ = scene.render(ne.render_params(seed=9, spp=2, sample_offset=2))
    assert np.allclose((lo + hi) / 2, a, rtol=1e-5, atol=1e-6)


def test_invalid_arguments(ne, ctx):
    host = ne.SceneHost.from_json(scene_path("cornell_c1"))
    scene = ctx.upload(host)
    with pytest.raises(ne.NarvalError) as e:
        scene.trace_paths(np.array([[host.width * host.height, 0]], np.uint32))
    assert e.value.status == -1
    out = scene.trace_paths(np.zeros((0, 2), np.uint32))
    assert out.shape == (0, 3)
    assert scene.trace_closest(np.zeros((0, 6), np.float32)).shape == (0,)


def test_kernels_and_tunings_agree(ne, ctx):
    """Every path kernel and launch configuration renders the same bits."""
    host = ne.SceneHost.from_json(scene_path("medium_c2"))
    scene = ctx.upload(host)
    p = ne.render_params(seed=21, spp=2)
    ref = None
    for kernel, share, bps, passes in [(0, 16, 0, 0), (0, 16, 1, 0), (1, 16, 0, 0), (1, 1, 0, 0), (1, 32, 0, 0),
                                       (1, 8, 1, 0), (2, 16, 0, 0), (2, 16, 1, 0), (3, 16, 0, 2), (3, 16, 1, 3),
                                       (3, 16, 0, 5), (3, 16, 0, 16), (3, 16, 0, -8), (3, 16, 0, -3),
                                       (3, 16, 0, -64), (3, 16, 1, -12), (3, 16, 0, 6)]:
        for quarters in ((3,) if kernel != 3 else (3, 1, 8)):
            scene.set_tuning(kernel=kernel, track_share=share, blocks_per_sm=bps, split_passes=abs(passes),
                             split_half=int(passes < 0), queue_quarters=quarters)
            img, stats = scene.render(p)
            if ref is None:
                ref = img
            assert np.array_equal(img, ref), (kernel, share, bps, passes, quarters)
    with pytest.raises(ne.NarvalError):
        scene.set_tuning(kernel=4)
    with pytest.raises(ne.NarvalError):
        scene.set_tuning(kernel=3, split_passes=1)

    with pytest.raises(ne.NarvalError):
        scene.set_tuning(kernel=1, track_share=0)
    with pytest.raises(ne.NarvalError):
        scene.set_tuning(kernel=3, queue_quarters=9)


def test_counting_kernels_agree(ne, ctx):
    """The instrumented variants count the same work on both kernels and render the same image."""
    host = ne.SceneHost.from_json(scene_path("medium_c2"))
    scene = ctx.upload(host)
    out = {}
    for kernel in (0, 1, 2):
        scene.set_tuning(kernel=kernel)
        img, st = scene.render(ne.render_params(seed=2, spp=1, flags=ne.NE_RENDER_COUNT_WORK))
        out[kernel] = (img, st["density_lookups"], st["scene_queries"])
    for k in (1, 2):
        assert np.array_equal(out[0][0], out[k][0])
        assert out[0][1] == out[k][1] and out[0][2] == out[k][2] and out[0][1] > 0


def mesh_scene_json(subdivisions):
    import json
    d = json.load(open(scene_path("mesh_c3")))
    d["primitives"][0]["subdivisions"] = subdivisions
    d["renderer"]["resolution"] = [160, 120]
    d["renderer"]["bvh"] = "reference"  # the oracle builds the reference's tree itself
    return json.dumps(d)


@pytest.mark.parametrize("subdivisions", [3, 8])
def test_mesh_bvh_parity(ne, ctx, oracle_lib, subdivisions):
    """Triangle meshes through the reference's midpoint BVH (BVH.cpp:6-193): hits bit-exact,
    camera paths bit-identical, on a small mesh and on the 1.3 M-triangle icosphere."""
    text = mesh_scene_json(subdivisions)
    host = ne.SceneHost.from_string(text)
    scene = ctx.upload(host)
    orc = oracle_lib.OracleScene.from_json(text=text)
    rays = camera_rays(host, 20000, 11)
    g = scene.trace_closest(rays, 1e-11, float("inf"))
    c = orc.trace_closest(rays, 1e-11, float("inf"))
    assert np.array_equal(g["primitive"], c["primitive"]) and np.array_equal(g["instance"], c["instance"])
    assert np.array_equal(g["t_near"].view(np.uint32), c["t_near"].view(np.uint32))
    assert (g["primitive"] >= 0).sum() > 1000
    keys = spread_keys(host, 512, 4, seed=3)
    cp = orc.trace_paths(keys, ne.render_params(seed=8))
    for kernel in (0, 1, 2, 3):
        scene.set_tuning(kernel=kernel)
        gp = scene.trace_paths(keys, ne.render_params(seed=8))
        assert np.array_equal(gp, cp), f"kernel {kernel}: max rel {rel_err(gp, cp).max():.3e}"
    # the bounce rays (and the camera rays) traced ahead of each pass by their own kernel
    for passes, pre in ((2, 1), (3, 1), (6, 1), (2, 2), (3, 2), (5, 2), (2, 3), (5, 3), (12, 3), (30, 3)):
        scene.set_tuning(kernel=3, split_passes=passes, split_half=0, pretrace=pre)
        gp = scene.trace_paths(keys, ne.render_params(seed=8))
        assert np.array_equal(gp, cp), f"pretrace {pre}, {passes} passes: max rel {rel_err(gp, cp).max():.3e}"


def test_pretrace_surface_scene(ne, ctx):
    """Cornell box split by bounce with the bounce rays traced ahead of each pass: the same
    image as the one-pass kernel, one k_trace launch before every resume pass."""
    host = ne.SceneHost.from_json(scene_path("cornell_c1"))
    scene = ctx.upload(host)
    try:
        p = ne.render_params(seed=4, spp=4)
        scene.set_tuning(kernel=0)
        ref, _ = scene.render(p)
        for passes in (2, 4, 8):
            scene.set_tuning(kernel=3, split_passes=passes, split_half=0, pretrace=1)
            assert scene.tuning()["pretrace"] == 1
            img, st = scene.render(p)
            assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), passes
            assert st["kernel_launches"] == 2 * passes - 1 + 1, st["kernel_launches"]
            # camera rays too: one more pass that only queues the new paths; then the shadow rays
            for pre in (2, 3):
                scene.set_tuning(kernel=3, split_passes=passes, split_half=0, pretrace=pre)
                img, st = scene.render(p)
                assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), (passes, pre)
                assert st["kernel_launches"] == 2 * (passes + 1) - 1 + 1, st["kernel_launches"]
        # by half bounce the knob has no effect
        scene.set_tuning(kernel=3, split_passes=8, split_half=1, pretrace=1)
        img, st = scene.render(p)
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)) and st["kernel_launches"] == 9
        with pytest.raises(ne.NarvalError):
            scene.set_tuning(kernel=3, pretrace=4)
    finally:
        scene.close()


def test_mesh_and_medium_parity(ne, ctx, oracle_lib):
    """A displaced mesh beside a grid medium (the many-views scene at 96x72 with a 5120-triangle
    blob, the reference's midpoint BVH): MIS rays from the surfaces that miss the medium's box
    skip intersectTr's walk, the others walk it. Camera paths are bit-identical to the oracle on
    every kernel."""
    import json
    d = json.load(open(scene_path("views_c5")))
    for p in d["primitives"]:
        if p.get("type") == "mesh":
            p["subdivisions"] = 4
    d["renderer"]["resolution"] = [96, 72]
    d["renderer"]["bvh"] = "reference"
    text = json.dumps(d)
    host = ne.SceneHost.from_string(text)
    scene = ctx.upload(host)
    orc = oracle_lib.OracleScene.from_json(text=text)
    try:
        keys = spread_keys(host, 1024, 4, seed=5)
        cp = orc.trace_paths(keys, ne.render_params(seed=12))
        assert (cp.sum(1) > 0).sum() > 1000
        for kernel in (0, 1, 2, 3):
            scene.set_tuning(kernel=kernel)
            gp = scene.trace_paths(keys, ne.render_params(seed=12))
            assert np.array_equal(gp.view(np.uint32), cp.view(np.uint32)), f"kernel {kernel}"
    finally:
        scene.close()
        orc.close()


def test_destroy_order(ne):
    """Destroying a context first destroys its scenes; closing them afterwards is harmless."""
    c = ne.Context(0)
    host = ne.SceneHost.from_json(scene_path("cornell_c1"))
    s1 = c.upload(host)
    s2 = c.upload(host)
    s1.close()
    c.close()
    s2.close()
    s1.close()
    c.close()


def test_fp64_accumulation(ne, ctx):
    """ne_render_accumulate sums the same per-path radiance as ne_render, in FP64."""
    host = ne.SceneHost.from_json(scene_path("cornell_c1"))
    scene = ctx.upload(host)
    acc = np.zeros((host.height, host.width, 3), np.float64)
    for off in (0, 3):
        scene.accumulate(acc, seed=6, spp=3, sample_offset=off)
    img, _ = scene.render(seed=6, spp=6)
    assert np.allclose(acc / 6, img, rtol=1e-5, atol=1e-6)
    keys = np.array([[1000, s] for s in range(6)], np.uint32)
    L = scene.trace_paths(keys, seed=6).astype(np.float64)
    assert np.allclose(acc.reshape(-1, 3)[1000], L.sum(0), rtol=1e-12, atol=1e-12)


def test_dense_cloud_parity(ne, ctx, oracle_lib):
    """512^3 fBm cloud (density 80, albedo 0.99, g 0.85, depth 256) at a 96x96 image: camera
    paths and a 2-spp render against the oracle. The density-cell array is 4.3 GB, well
    beyond L2, so this also covers the HBM-resident lookup path."""
    import json
    d = json.load(open(scene_path("cloud_c4")))
    d["renderer"]["resolution"] = [96, 96]
    text = json.dumps(d)
    host = ne.SceneHost.from_string(text)
    scene = ctx.upload(host)
    orc = oracle_lib.OracleScene.from_json(text=text)
    try:
        keys = spread_keys(host, 2048, 2, seed=4)
        p = ne.render_params(seed=21)
        g = scene.trace_paths(keys, p)
        c = orc.trace_paths(keys, p)
        assert np.array_equal(g.view(np.uint32), c.view(np.uint32)), f"max rel {rel_err(g, c).max():.3e}"
        assert np.mean(np.abs(c.sum(1) - 9.6) > 1e-3) > 0.2  # a good share of the paths enter the cloud
        img, _ = scene.render(seed=2, spp=2)
        ref, _ = orc.render(ne.render_params(seed=2, spp=2))
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    finally:
        scene.close()
        orc.close()


def test_split_queue_overflow(ne, ctx, oracle_lib):
    """The split kernel's queue classes (by the light the next draw picks) hold half and a
    quarter of the paths (at least 2048 and 1024). All paths here start through the dense
    centre of the medium, so far more than that scatter towards each light; those beyond the
    queue finish in the first pass, and every path still matches the oracle bit for bit."""
    host = ne.SceneHost.from_json(scene_path("medium_c2"))
    scene = ctx.upload(host)
    orc = oracle_lib.OracleScene.from_json(scene_path("medium_c2"))
    try:
        centre = (host.height // 2) * host.width + host.width // 2
        keys = np.array([[centre, s] for s in range(8192)], np.uint32)
        p = ne.render_params(seed=5)
        c = orc.trace_paths(keys, p)
        for quarters in (1, 3, 8):  # a quarter, three quarters and twice the paths
            scene.set_tuning(kernel=3, queue_quarters=quarters)
            g = scene.trace_paths(keys, p)
            assert np.array_equal(g.view(np.uint32), c.view(np.uint32)), quarters
    finally:
        scene.close()
        orc.close()


def test_autotune_keeps_the_image(ne, ctx):
    """The scene autotuner only changes how the paths are scheduled."""
    host = ne.SceneHost.from_json(scene_path("cornell_c1"))
    scene = ctx.upload(host)
    ref, _ = scene.render(seed=13, spp=2)
    best, ms = scene.autotune(repeats=1, seed=1, spp=1)
    assert ms > 0 and best["kernel"] in (0, 1, 2, 3) and 1 <= best["queue_quarters"] <= 4
    img, st = scene.render(seed=13, spp=2)
    assert np.array_equal(img, ref)
    if best["kernel"] == 3:
        assert st["kernel_launches"] == best["split_passes"] + 1
    scene.close()
