"""relMSE against an FP64-accumulated reference image (plain integrator)."""
import json

import numpy as np
import pytest

from conftest import scene_path


def small_scene(name, w, h):
    d = json.load(open(scene_path(name)))
    d["renderer"]["resolution"] = [w, h]
    return json.dumps(d)


def test_relmse_definition():
    from narvalengine_gb300.convergence import relmse
    ref = np.array([[0.0, 1.0, 2.0]])
    x = np.array([[0.1, 1.0, 1.0]])
    want = np.mean([0.01 / 0.01, 0.0, 1.0 / 4.01])
    assert relmse(x, ref) == pytest.approx(want, rel=1e-12)
    assert relmse(ref, ref) == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["medium_c2"])
def test_relmse_falls_as_one_over_spp(built, name):
    """Monte Carlo error: relMSE ~ 1/spp, so on the medium scene 4x the samples gives about
    1/4 the relMSE. (The Cornell box is left out: its GGX paths produce rare radiance values
    of order 1e3-1e4, so its relMSE falls irregularly even at 64k samples per pixel.)"""
    import narvalengine_gb300 as ne
    from narvalengine_gb300.convergence import reference_image, time_to_relmse
    ctx = ne.Context(0)
    try:
        scene = ctx.upload(ne.SceneHost.from_string(small_scene(name, 96, 64)))
        ref, ms = reference_image(scene, 8192, chunk=2048)
        assert ms > 0 and np.all(np.isfinite(ref)) and ref.min() >= 0
        res = time_to_relmse(scene, ref, target=1e-9, max_spp=1024)
        curve = {c["spp"]: c["relmse"] for c in res["curve"]}
        assert not res["reached"] and sorted(curve)[0] == 16 and 896 in curve
        for s in (16, 32, 64, 224):
            ratio = curve[s] / curve[4 * s]
            assert 2.5 < ratio < 6.5, (s, ratio, curve)
        times = [c["ms"] for c in res["curve"]]
        assert all(b >= a for a, b in zip(times, times[1:]))
        # the accumulated mean of a render equals ne_render's image
        img, _ = scene.render(seed=7, spp=8)
        acc = np.zeros_like(ref)
        scene.accumulate(acc, seed=7, spp=8)
        assert np.allclose(acc / 8, img, rtol=1e-5, atol=1e-6)
    finally:
        ctx.close()
