"""ne_render_noalloc against ne_render, through the C ABI.

ne_render_noalloc renders into a caller-owned device image and takes its per-path scratch
from a fixed array in the library, for callers that cannot allocate device memory while
rendering. Each case makes two calls in a row with different parameters, so a second
call that saw the first call's counters, error flag or paths would show. Tolerance: the
per-channel relative bound of the parity suite (1e-4); both entry points run the same
kernels on the same keys, so the images are expected to match exactly.

Collected last (file name) so it also runs after every other GPU test in one process.
"""
import ctypes as C

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


def noalloc(ne, scene, params, out_dev):
    from narvalengine_gb300 import _abi
    stats = _abi.NeRenderStats()
    st = ne.library().ne_render_noalloc(scene._h, C.byref(params), C.c_void_p(out_dev.data_ptr()), C.byref(stats))
    return st, {f: getattr(stats, f) for f, _ in _abi.NeRenderStats._fields_ if f != "pad"}


def check_close(got, want):
    # a pixel whose samples include one of the reference's NaN paths (HG sampling at the ends
    # of [0, 1), materials/Medium.h:96-114) is NaN on both sides
    nan = np.isnan(want)
    assert np.array_equal(nan, np.isnan(got)), "NaN pixels differ"
    den = np.maximum(np.abs(want[~nan]), 1e-6)
    err = np.max(np.abs(got[~nan] - want[~nan]) / den)
    assert err <= REL_TOL, f"max relative error {err}"


@pytest.mark.parametrize("name,calls", [
    # cornell 256x256: 16 spp fills the scratch (2^20 paths) exactly
    ("cornell_c1", [dict(seed=11, spp=16), dict(seed=12, spp=5, sample_offset=16, flags=2)]),
    # medium 512x512: 4 spp fills it exactly; the second call renders fewer paths
    ("medium_c2", [dict(seed=3, spp=4), dict(seed=3, spp=1, sample_offset=9)]),
])
def test_noalloc_matches_render(ne, ctx, name, calls):
    import torch
    from narvalengine_gb300 import _abi
    host = ne.SceneHost.from_json(scene_path(name))
    scene = ctx.upload(host)
    try:
        out = torch.empty((host.height, host.width, 3), dtype=torch.float32, device="cuda:0")
        for kw in calls:
            kw = dict(kw)
            kw["flags"] = kw.get("flags", 0) | _abi.NE_RENDER_COUNT_WORK
            want, want_stats = scene.render(ne.render_params(**kw))
            out.fill_(float("nan"))
            st, stats = noalloc(ne, scene, ne.render_params(**kw), out)
            assert st == 0, ctx.error()
            got = out.cpu().numpy()
            check_close(got, want)
            # counters start at zero on every call
            for key in ("paths", "density_lookups", "scene_queries", "bvh_nodes", "prim_tests"):
                assert stats[key] == want_stats[key], key
    finally:
        scene.close()


@pytest.mark.parametrize("name", ["cornell_c1", "medium_c2"])
def test_noalloc_production_kernels(ne, ctx, name):
    """Without the counting flag, on every tuning the scene can have (kernels 0-2 as tuned; a
    scene tuned to the split kernel 3 renders with kernel 0) and after the autotuner: two
    calls in a row, each image against ne_render's at the same tuning."""
    import torch
    host = ne.SceneHost.from_json(scene_path(name))
    scene = ctx.upload(host)
    spp = 16 if name == "cornell_c1" else 4
    try:
        out = torch.empty((host.height, host.width, 3), dtype=torch.float32, device="cuda:0")
        tunings = [dict(kernel=k) for k in (0, 1, 2, 3)] + [dict(kernel=3, split_passes=12, split_half=1), None]
        for t in tunings:
            if t is None:
                scene.autotune(repeats=1, seed=7, spp=2)
            else:
                scene.set_tuning(**t)
            for kw in (dict(seed=21, spp=spp), dict(seed=22, spp=max(1, spp // 2), sample_offset=3)):
                want, _ = scene.render(ne.render_params(**kw))
                out.fill_(float("nan"))
                st, stats = noalloc(ne, scene, ne.render_params(**kw), out)
                assert st == 0, ctx.error()
                got = out.cpu().numpy()
                check_close(got, want)
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (t, kw)
                assert stats["paths"] == host.width * host.height * kw["spp"]
    finally:
        scene.close()


def test_noalloc_rejects_oversize(ne, ctx):
    import torch
    from narvalengine_gb300 import _abi
    host = ne.SceneHost.from_json(scene_path("cornell_c1"))
    scene = ctx.upload(host)
    try:
        out = torch.zeros((host.height, host.width, 3), dtype=torch.float32, device="cuda:0")
        st, _ = noalloc(ne, scene, ne.render_params(seed=1, spp=17), out)
        assert st == _abi.NE_ERR_INVALID_ARG
        assert "exceed" in ctx.error()
        assert float(out.abs().sum()) == 0.0
        st, _ = noalloc(ne, scene, ne.render_params(seed=1, spp=1), out)
        assert st == 0, ctx.error()
        want, _ = scene.render(ne.render_params(seed=1, spp=1))
        check_close(out.cpu().numpy(), want)
    finally:
        scene.close()
