"""Status codes of the newer entry points on invalid input (no kernel runs for these)."""
import ctypes as C

import numpy as np
import pytest

from conftest import scene_path

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built):
    import narvalengine_gb300 as ne
    ctx = ne.Context(0)
    scene = ctx.upload(ne.SceneHost.from_json(scene_path("cornell_c1")))
    yield ne, ctx, scene
    ctx.close()


def test_views_errors(env):
    ne, ctx, scene = env
    from narvalengine_gb300 import _abi
    lib = ne.library()
    h = C.c_void_p()
    cam = ne.camera_look_at([0, 1, -3], [0, 1, 0], 50, 16, 16)
    bad = (_abi.NeView * 1)()
    bad[0].camera = cam
    bad[0].width, bad[0].height, bad[0].spp = 16, 0, 1
    p = ne.render_params(seed=1)
    assert lib.ne_views_create(scene._h, bad, 1, C.byref(p), C.byref(h)) == _abi.NE_ERR_INVALID_ARG
    assert lib.ne_views_create(scene._h, bad, 0, C.byref(p), C.byref(h)) == _abi.NE_ERR_INVALID_ARG
    vb = ne.Views(scene, [(cam, 16, 16, 1)], seed=1)
    for t in [dict(fetch=16), dict(fetch=48), dict(order=3), dict(split_passes=65), dict(blocks_per_sm=65),
              dict(split_half=2)]:
        with pytest.raises(ne.NarvalError):
            vb.set_tuning(**t)
    with pytest.raises(ne.NarvalError):
        vb.image(1)
    out = np.empty((16, 16, 3), np.float32)
    ptr = out.ctypes.data_as(C.POINTER(C.c_float))
    assert lib.ne_views_image(vb._h, 1, ptr) == _abi.NE_ERR_INVALID_ARG
    assert lib.ne_views_image(vb._h, -1, ptr) == _abi.NE_ERR_INVALID_ARG
    vb.close()


def test_cache_errors(env):
    ne, ctx, scene = env
    from narvalengine_gb300 import _abi
    lib = ne.library()
    cache = ne.RadianceCache(ctx, seed=1)
    assert lib.ne_cache_train(cache._h, None, None, None, None, 0, 1, None, None, 0) == _abi.NE_ERR_INVALID_ARG
    with pytest.raises(ValueError):
        cache.set_params(np.zeros(10, np.float32))
    # the Cornell box has no grid medium: the cached render is refused
    with pytest.raises(ne.NarvalError) as e:
        scene.render_cached(cache, bounce=1, seed=1, spp=1)
    assert e.value.status == _abi.NE_ERR_UNSUPPORTED
    cache.close()


def test_tuning_errors(env):
    ne, ctx, scene = env
    for t in [dict(kernel=-1), dict(kernel=4), dict(kernel=3, split_passes=1), dict(kernel=3, split_passes=65),
              dict(blocks_per_sm=-1), dict(kernel=1, track_share=33), dict(kernel=3, split_half=2),
              dict(kernel=3, split_half=-1)]:
        with pytest.raises(ne.NarvalError):
            scene.set_tuning(**t)
    assert ne.library().ne_scene_autotune(scene._h, None, 0, None, None) != 0


def test_cache_limit(env):
    """Released device memory is cached up to the context's limit; any limit, including none,
    gives the same images."""
    ne, ctx, scene = env
    from narvalengine_gb300 import _abi
    lib = ne.library()
    assert lib.ne_context_set_cache_limit(None, 0) == _abi.NE_ERR_INVALID_ARG
    host = ne.SceneHost.from_json(scene_path("cornell_c1"))
    p = ne.render_params(seed=3, spp=2)
    first, _ = scene.render(p)
    try:
        for limit in (0, 1 << 20, 64 << 30):
            ctx.set_cache_limit(limit)
            for _ in range(2):
                s = ctx.upload(host)
                s.set_tuning(**scene.tuning())
                img, _ = s.render(p)
                s.close()
                assert np.array_equal(img, first)
    finally:
        import torch
        ctx.set_cache_limit(max(16 << 30, torch.cuda.get_device_properties(0).total_memory // 4))
