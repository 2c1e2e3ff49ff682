"""Rendering with the learned radiance cache (ne_render_cached) on the medium scene.

* With no path reaching the termination bounce, and with every path a training path, the
  cached render is the plain render, bit for bit (the cache changes nothing else).
* With a zero network every terminated path keeps only the radiance gathered before its
  termination vertex, so the image is at most the plain image in every pixel.
* The gain of the trained network: against an FP64 plain reference, cloud paths truncated
  at their second scattering event without the network are strongly biased; after online
  training on the integrator's own path suffixes the cached image's relMSE is several times
  lower.
"""
import json

import numpy as np
import pytest

from conftest import scene_path

pytestmark = pytest.mark.gpu


def medium(ne, w=96, h=64):
    d = json.load(open(scene_path("medium_c2")))
    d["renderer"]["resolution"] = [w, h]
    return ne.SceneHost.from_string(json.dumps(d))


@pytest.fixture(scope="module")
def env(built):
    import narvalengine_gb300 as ne
    ctx = ne.Context(0)
    scene = ctx.upload(medium(ne))
    cache = ne.RadianceCache(ctx, seed=5)
    yield ne, ctx, scene, cache
    cache.close()
    ctx.close()


def test_no_termination_is_plain(env):
    ne, ctx, scene, cache = env
    plain, _ = scene.render(seed=3, spp=4)
    img, st, cst = scene.render_cached(cache, bounce=100000, seed=3, spp=4)
    assert cst["queries"] == 0 and cst["train_samples"] == 0
    assert np.array_equal(img.view(np.uint32), plain.view(np.uint32))
    img, st, cst = scene.render_cached(cache, bounce=2, train_stride=1, seed=3, spp=4)
    assert cst["queries"] == 0 and cst["train_samples"] > 100
    assert np.array_equal(img.view(np.uint32), plain.view(np.uint32))


def test_zero_network_only_truncates(env):
    ne, ctx, scene, cache = env
    cache.set_params(np.zeros(ne.RadianceCache.N_PARAMS, np.float32))
    plain, _ = scene.render(seed=9, spp=4)
    img, st, cst = scene.render_cached(cache, bounce=2, seed=9, spp=4)
    assert cst["queries"] > 100
    assert np.all(img <= plain)
    assert img.sum() < plain.sum()


def test_training_suffix_ends_training_paths_in_the_cache(env):
    """With train_suffix n, a training path recorded at its first scattering vertex at or after
    `bounce` ends in the cache n bounces later. With a zero network and every path a training
    path, bounce 2 and n = 1 therefore render the image of bounce 3 without training, bit for
    bit (the medium scene scatters only in the medium, so the recorded vertex is bounce 2's),
    while each training path still records a sample."""
    ne, ctx, scene, cache = env
    cache.set_params(np.zeros(ne.RadianceCache.N_PARAMS, np.float32))
    want, _, cw = scene.render_cached(cache, bounce=3, seed=4, spp=4)
    img, _, ci = scene.render_cached(cache, bounce=2, train_stride=1, train_suffix=1, seed=4, spp=4)
    assert cw["queries"] > 100 and ci["train_samples"] > 100
    assert ci["queries"] == cw["queries"]
    assert np.array_equal(img.view(np.uint32), want.view(np.uint32))
    # a trained network: the end vertices' answers go into the targets, the loss stays finite
    cache.set_params(np.random.default_rng(2).normal(0, 0.05, ne.RadianceCache.N_PARAMS).astype(np.float32))
    img, _, ci = scene.render_cached(cache, bounce=2, train_stride=4, train_suffix=2, train_steps=2, seed=5, spp=4)
    assert np.isfinite(img).all() and np.isfinite(ci["loss"]) and ci["train_samples"] > 0
    with pytest.raises(ne.NarvalError):
        scene.render_cached(cache, bounce=2, train_stride=4, train_suffix=-1, seed=5, spp=1)


def test_trained_cache_reduces_bias(env):
    """On the dense cloud (albedo 0.99) paths ended at their second scattering event lose a
    visible share of the light; the trained network restores most of it. relMSE against an
    FP64 plain reference = bias^2 + noise; the plain image at the same sample count gives the
    noise, so bias is measured as the excess over it."""
    ne, ctx, _, _ = env
    from narvalengine_gb300.convergence import reference_image, relmse
    d = json.load(open(scene_path("cloud_c4")))
    d["renderer"]["resolution"] = [64, 64]
    scene = ctx.upload(ne.SceneHost.from_string(json.dumps(d)))
    zero = ne.RadianceCache(ctx, seed=5)
    fresh = ne.RadianceCache(ctx, seed=5)
    try:
        ref, _ = reference_image(scene, 32768, chunk=4096)
        zero.set_params(np.zeros(ne.RadianceCache.N_PARAMS, np.float32))
        trunc, _, cst0 = scene.render_cached(zero, bounce=1, seed=1, spp=8192)
        for frame in range(60):
            scene.render_cached(fresh, bounce=1, train_stride=4, train_steps=4, train_batch=8192, seed=100 + frame,
                                spp=16)
        img, _, cst = scene.render_cached(fresh, bounce=1, seed=1, spp=8192)
        plain, _ = scene.render(seed=1, spp=8192)
        e_trunc, e_cache, e_plain = relmse(trunc, ref), relmse(img, ref), relmse(plain, ref)
        assert cst0["queries"] > 0.05 * 64 * 64 * 8192
        assert e_trunc - e_plain > 1e-4, (e_trunc, e_plain)
        assert e_cache - e_plain < (e_trunc - e_plain) / 3, (e_cache, e_trunc, e_plain)
        # what the network adds is light that truncation removed
        assert img.sum() > trunc.sum()
    finally:
        zero.close()
        fresh.close()
        scene.close()
