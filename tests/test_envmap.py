"""InfiniteAreaLight with a texture (lights/InfiniteAreaLight.h:20-129, utils/Sampling.h:5-112).

The texture is decoded as the reference's loader gives it (RGBA8), Le looks it up by the
direction's spherical angles in the frame of (0, 0, 1), and sampleLi draws directions from the
Distribution2D the constructor builds (green channel x sin(theta); every conditional row takes
`height` values, Sampling.h:87). CPU: loading rules and an independent float64 restatement of
the Le lookup for rays that escape. GPU: per-path radiance and images bit-identical to the
oracle on a surface scene and a medium scene lit by a rotated environment map.
"""
import json

import numpy as np
import pytest

from test_image_load import encode_png

REL_TOL = 1e-4


def sky_texels(w=64, h=32, seed=3):
    """A sky: vertical gradient, noise and a bright sun disc (some texels black)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    img = np.zeros((h, w, 3))
    img[..., 0] = 40 + 150 * y / h
    img[..., 1] = 80 + 120 * y / h
    img[..., 2] = 200 - 60 * y / h
    img += rng.integers(0, 30, size=img.shape)
    sun = (x - 0.3 * w) ** 2 + (y - 0.35 * h) ** 2 < (0.06 * w) ** 2
    img[sun] = 255
    img[h - 3:, : w // 4] = 0  # a black corner: the sky sphere is then hit, not skipped
    return np.clip(img, 0, 255).astype(np.int64)


def write_sky(tmp_path, w=64, h=32):
    texels = sky_texels(w, h)
    (tmp_path / "sky.png").write_bytes(encode_png(texels, 2, 8))
    return texels


def scene_json(prims, sky_rot=(20, 35, 0), medium=False, sky_path="sky.png"):
    mats = [{"name": "grey", "type": "microfacet", "roughness": 0.6, "metallic": 0.0, "albedo": [0.7, 0.7, 0.7]},
            {"name": "gold", "type": "microfacet", "roughness": 0.2, "metallic": 0.8, "albedo": [0.9, 0.7, 0.3]},
            {"name": "sky", "type": "infiniteAreaLight", "path": sky_path}]
    if medium:
        mats.append({"name": "fog", "type": "volume", "scattering": [0.8, 0.8, 0.8], "absorption": [0.2, 0.2, 0.2],
                     "phaseFunction": "hg", "g": 0.5, "density": 6,
                     "grid": {"generator": "fbm", "resolution": [32, 32, 32], "octaves": 3, "frequency": 0.125,
                              "falloff_radius": 16, "seed": 7}})
    d = {"version": "0.0.1a", "materials": mats,
         "primitives": prims + [{"name": "skySphere", "type": "sphere", "radius": 100, "materialName": "sky",
                                 "transform": {"position": [0, 0, 0], "scale": [1, 1, 1], "rotation": list(sky_rot)}}],
         "camera": {"position": [0, 1.2, -4], "lookAt": [0, 0.3, 0], "up": [0, 1, 0], "vfov": 55, "aperture": 0.0001,
                    "autoFocus": True, "focus": 1},
         "renderer": {"resolution": [48, 32], "spp": 2, "bounces": 8, "mode": "offline", "HDR": True}}
    return json.dumps(d)


SURFACE = [{"name": "ball", "type": "sphere", "radius": 0.6, "materialName": "gold",
            "transform": {"position": [0.4, 0.6, 0.5]}},
           {"name": "ball2", "type": "sphere", "radius": 0.4, "materialName": "grey",
            "transform": {"position": [-0.8, 0.4, -0.2]}},
           {"name": "ground", "type": "rectangle", "materialName": "grey",
            "transform": {"position": [0, 0, 0], "scale": [6, 6, 1], "rotation": [90, 0, 0]}}]
MEDIUM = [{"name": "fogBox", "type": "volume", "materialName": "fog",
           "transform": {"position": [0, 0.5, 0], "scale": [1.5, 1.5, 1.5], "rotation": [0, 20, 0]}},
          {"name": "ground", "type": "rectangle", "materialName": "grey",
           "transform": {"position": [0, -0.3, 0], "scale": [6, 6, 1], "rotation": [90, 0, 0]}}]


def test_envmap_load_errors(built, tmp_path):
    import narvalengine_gb300 as ne
    write_sky(tmp_path)
    ne.SceneHost.from_string(scene_json(SURFACE), str(tmp_path))  # loads
    (tmp_path / "tall.png").write_bytes(encode_png(sky_texels(16, 32), 2, 8))
    with pytest.raises(ne.NarvalError) as e:
        ne.SceneHost.from_string(scene_json(SURFACE, sky_path="tall.png"), str(tmp_path))
    assert e.value.status == -6  # the reference's Distribution2D reads past a taller-than-wide image
    with pytest.raises(ne.NarvalError) as e:
        ne.SceneHost.from_string(scene_json(SURFACE, sky_path="missing.png"), str(tmp_path))
    assert e.value.status == -3


def sky_to_ocs(host):
    """The sky sphere's invTransformToWCS (column-major 4x4) as a 3x3 numpy matrix."""
    import ctypes as C
    from narvalengine_gb300 import _abi
    d = C.cast(host.desc_ptr, C.POINTER(_abi.NeSceneDesc)).contents
    m = np.array(d.instances[d.n_instances].to_ocs[:], np.float64).reshape(4, 4).T
    return m[:3, :3]


def test_envmap_le_of_escaping_rays(built, oracle_lib, tmp_path):
    """Rays that leave the scene at bounce 0 carry Le: the direction in the sky sphere's object
    frame, expressed in generateOrthonormalCS((0, 0, 1)) = (s, t, n) = ((0, 1, 0), (-1, 0, 0),
    (0, 0, 1)), indexes the texel at (phi / 2pi, theta / pi)."""
    import narvalengine_gb300 as ne
    texels = write_sky(tmp_path)
    rot = (20, 35, 0)
    text = scene_json([], sky_rot=rot)
    host = ne.SceneHost.from_string(text, str(tmp_path))
    orc = oracle_lib.OracleScene.from_json(text=text, resources_dir=str(tmp_path))
    try:
        rng = np.random.default_rng(5)
        d = rng.normal(size=(20000, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        rays = np.concatenate([np.zeros_like(d), d], 1).astype(np.float32)
        keys = np.zeros((len(rays), 2), np.uint32)
        L = orc.li_batch(rays, keys, 0, ne.render_params(seed=1, bounces=1))
    finally:
        orc.close()
    w = d @ sky_to_ocs(host).T
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    lx, ly, lz = w[:, 1], -w[:, 0], w[:, 2]  # toLCS
    phi = np.mod(np.arctan2(ly, lx), 2 * np.pi)
    theta = np.arccos(np.clip(lz, -1, 1))
    H, W = texels.shape[:2]
    x = np.minimum((phi / (2 * np.pi) * W).astype(int), W - 1)
    y = np.minimum((theta / np.pi * H).astype(int), H - 1)
    want = texels[y, x] / 255.0
    same = np.all(np.abs(L - want) < 1e-6, axis=1)
    # texel-boundary directions may round to the neighbour in float32
    assert same.mean() > 0.995, same.mean()
    assert (L.max(axis=1) > 0).mean() > 0.9


@pytest.fixture(scope="module")
def env_scenes(built, oracle_lib, tmp_path_factory):
    import narvalengine_gb300 as ne
    tmp = tmp_path_factory.mktemp("env")
    write_sky(tmp)
    ctx = ne.Context(0)
    out = []
    for name, prims, medium in (("surface", SURFACE, False), ("medium", MEDIUM, True)):
        text = scene_json(prims, medium=medium)
        host = ne.SceneHost.from_string(text, str(tmp))
        out.append((name, host, ctx.upload(host), oracle_lib.OracleScene.from_json(text=text, resources_dir=str(tmp))))
    yield ne, out
    for _, _, _, orc in out:
        orc.close()
    ctx.close()


@pytest.mark.gpu
def test_envmap_paths_bit_exact(env_scenes):
    ne, scenes = env_scenes
    for name, host, scene, orc in scenes:
        keys = np.array([[p, s] for p in range(host.width * host.height) for s in range(2)], np.uint32)
        for kernel in (0, 3):
            scene.set_tuning(kernel=kernel)
            p = ne.render_params(seed=11)
            g = scene.trace_paths(keys, p)
            c = orc.trace_paths(keys, p)
            err = np.abs(g - c) / np.maximum(np.abs(c), 1e-6)
            assert err.max() <= REL_TOL, f"{name} kernel {kernel}: max rel {err.max():.3e}"
            assert np.array_equal(g.view(np.uint32), c.view(np.uint32)), f"{name} kernel {kernel}"
            assert (g.max(axis=1) > 0).mean() > 0.5


@pytest.mark.gpu
def test_envmap_render_bit_exact(env_scenes):
    ne, scenes = env_scenes
    for name, host, scene, orc in scenes:
        p = ne.render_params(seed=3, spp=4)
        g, _ = scene.render(p)
        c, _ = orc.render(p)
        assert np.array_equal(g.view(np.uint32), c.view(np.uint32)), name
