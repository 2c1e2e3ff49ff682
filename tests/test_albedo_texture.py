"""Microfacet albedo from an image file (io/SceneReader.cpp:80-103, Texture::sample with the
mirror wrap and nearest texel, materials/Texture.cpp:88-129): the rectangle's texture
coordinates from its object-space hit point (primitives/Rectangle.cpp:71, 91-157), (0, 0) on
every other primitive. GPU against the oracle on every path kernel, bit for bit; the texture
changes the image (on the oracle, CPU)."""
import json

import numpy as np
import pytest

from test_image_load import encode_png

T = lambda p, r=(0, 0, 0), s=(1, 1, 1): {"position": list(p), "rotation": list(r), "scale": list(s)}


def write_textures(tmp_path, seed=9):
    rng = np.random.default_rng(seed)
    checker = np.zeros((8, 12, 3), np.uint8)
    checker[(np.add.outer(np.arange(8), np.arange(12)) % 2) == 0] = (230, 40, 30)
    checker[(np.add.outer(np.arange(8), np.arange(12)) % 2) == 1] = (20, 60, 220)
    (tmp_path / "checker.png").write_bytes(encode_png(checker, 2, 8))
    noise = rng.integers(0, 256, size=(16, 16, 4), dtype=np.uint8)
    (tmp_path / "noise.png").write_bytes(encode_png(noise, 6, 8))


def scene_text(wall_tex="checker.png", ball_tex="noise.png"):
    mats = [
        {"name": "white", "type": "microfacet", "roughness": 0.9, "metallic": 0.0, "albedo": [0.73, 0.73, 0.73]},
        {"name": "wallpaper", "type": "microfacet", "roughness": 0.8, "metallic": 0.0, "albedo": wall_tex},
        {"name": "floorpaper", "type": "microfacet", "roughness": 0.5, "metallic": 0.2, "albedo": ball_tex},
        {"name": "ballpaper", "type": "microfacet", "roughness": 0.4, "metallic": 0.0, "albedo": ball_tex},
        {"name": "lamp", "type": "emitter", "albedo": [17.0, 12.0, 4.0]},
    ]
    prims = [
        {"name": "floor", "type": "rectangle", "transform": T((0, 0, 0), (90, 0, 0), (2, 2, 1)),
         "materialName": "floorpaper"},
        {"name": "ceiling", "type": "rectangle", "transform": T((0, 2, 0), (-90, 0, 0), (2, 2, 1)),
         "materialName": "white"},
        {"name": "back", "type": "rectangle", "transform": T((0, 1, 1), (0, 0, 0), (2, 2, 1)),
         "materialName": "wallpaper"},
        {"name": "left", "type": "rectangle", "transform": T((-1, 1, 0), (0, -90, 0), (2, 2, 1)),
         "materialName": "wallpaper"},
        {"name": "right", "type": "rectangle", "transform": T((1, 1, 0), (10, 80, 5), (2, 2.5, 1)),
         "materialName": "white"},
        {"name": "ball", "type": "sphere", "radius": 0.35, "transform": T((0.3, 0.35, 0.1)),
         "materialName": "ballpaper"},
        {"name": "light", "type": "rectangle", "transform": T((0, 1.99, 0), (-90, 0, 0), (0.5, 0.5, 1)),
         "materialName": "lamp"},
    ]
    cam = {"position": [0, 1, -2.6], "lookAt": [0, 1, 0], "up": [0, 1, 0], "speed": 5, "vfov": 60,
           "aperture": 0.0001, "autoFocus": True, "focus": 1}
    return json.dumps({"version": "0.0.1a", "materials": mats, "primitives": prims, "camera": cam,
                       "renderer": {"resolution": [64, 48], "spp": 2, "bounces": 6, "mode": "offline",
                                    "HDR": True}})


def test_texture_changes_the_image(built, oracle_lib, tmp_path):
    write_textures(tmp_path)
    p_args = dict(seed=3, spp=4)
    import narvalengine_gb300 as ne
    a, _ = oracle_lib.OracleScene.from_json(text=scene_text(), resources_dir=str(tmp_path)).render(
        ne.render_params(**p_args))
    b, _ = oracle_lib.OracleScene.from_json(text=scene_text("noise.png", "checker.png"),
                                            resources_dir=str(tmp_path)).render(ne.render_params(**p_args))
    assert np.isfinite(a).all() and np.abs(a - b).mean() > 1e-3
    # the back wall seen straight on shows the checker: neighbouring texel columns alternate red
    # and blue in the directly lit first-bounce colour of its pixels
    red = a[:, :, 0] > a[:, :, 2]
    assert 0.1 < red.mean() < 0.9


@pytest.mark.gpu
def test_textured_albedo_parity(built, oracle_lib, tmp_path):
    import narvalengine_gb300 as ne
    write_textures(tmp_path)
    text = scene_text()
    host = ne.SceneHost.from_string(text, str(tmp_path))
    ctx = ne.Context(0)
    scene = ctx.upload(host)
    orc = oracle_lib.OracleScene.from_json(text=text, resources_dir=str(tmp_path))
    try:
        rng = np.random.default_rng(1)
        pix = rng.choice(host.width * host.height, size=800, replace=False)
        keys = np.array([[p, s] for p in pix for s in range(3)], np.uint32)
        c = orc.trace_paths(keys, ne.render_params(seed=17))
        ref, _ = orc.render(ne.render_params(seed=8, spp=2))
        for kernel in (0, 1, 2, 3):
            scene.set_tuning(kernel=kernel)
            g = scene.trace_paths(keys, ne.render_params(seed=17))
            err = np.abs(g - c) / np.maximum(np.abs(c), 1e-6)
            assert err.max() <= 1e-4, (kernel, err.max())
            assert np.array_equal(g.view(np.uint32), c.view(np.uint32)), kernel
            img, _ = scene.render(ne.render_params(seed=8, spp=2))
            assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), kernel
        assert (c.sum(1) > 0).mean() > 0.5
    finally:
        scene.close()
        orc.close()
        ctx.close()
