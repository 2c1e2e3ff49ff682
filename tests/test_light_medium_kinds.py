"""GPU parity for the integrator's less common branches, on every path kernel.

* HomogeneousMedia::sample / Tr (materials/HomogeneousMedia.cpp:15-51, with the distance
  normalisation `t = t / distInsideVolume` of :27);
* the isotropic phase function (materials/Medium.h:43-63) in a homogeneous and in a grid medium;
* a sphere emitter: the deterministic nearest point and the pdf constant of
  primitives/Sphere.cpp:46-68;
* a point emitter (primitives/Point.cpp, a DiffuseLight on a Point);
* a triangle-mesh emitter: Triangle::samplePointOnSurface samples in object space, untransformed
  (primitives/Triangle.cpp:114-119), pdf 1/area (:159-161). SceneReader never puts a mesh among
  the scene's lights (only points, spheres and rectangles, io/SceneReader.cpp:306-510), so this
  scene is assembled as a description: the oracle's reading of a mesh scene with the mesh's
  model turned into a light model.

Each scene: camera paths on several seeds and a small render, GPU against the oracle, bit for
bit (the bar of the other parity tests; the per-path tolerance of 1e-4 relative is checked
first so a failure reports its size).
"""
import ctypes as C
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
REL_TOL = 1e-4
KERNELS = (0, 1, 2, 3)

T = lambda p, r=(0, 0, 0), s=(1, 1, 1): {"position": list(p), "rotation": list(r), "scale": list(s)}
BOX = [
    {"name": "floor", "type": "rectangle", "transform": T((0, 0, 0), (90, 0, 0), (2, 2, 1)), "materialName": "white"},
    {"name": "ceiling", "type": "rectangle", "transform": T((0, 2, 0), (-90, 0, 0), (2, 2, 1)), "materialName": "white"},
    {"name": "back", "type": "rectangle", "transform": T((0, 1, 1), (0, 0, 0), (2, 2, 1)), "materialName": "white"},
    {"name": "left", "type": "rectangle", "transform": T((-1, 1, 0), (0, -90, 0), (2, 2, 1)), "materialName": "red"},
    {"name": "right", "type": "rectangle", "transform": T((1, 1, 0), (0, 90, 0), (2, 2, 1)), "materialName": "green"},
]
MATS = [
    {"name": "white", "type": "microfacet", "roughness": 0.9, "metallic": 0.0, "albedo": [0.73, 0.73, 0.73]},
    {"name": "red", "type": "microfacet", "roughness": 0.9, "metallic": 0.0, "albedo": [0.63, 0.065, 0.05]},
    {"name": "green", "type": "microfacet", "roughness": 0.9, "metallic": 0.0, "albedo": [0.14, 0.45, 0.09]},
    {"name": "glossy", "type": "microfacet", "roughness": 0.3, "metallic": 0.5, "albedo": [0.8, 0.8, 0.8]},
    {"name": "lamp", "type": "emitter", "albedo": [17.0, 12.0, 4.0]},
    {"name": "bulb", "type": "emitter", "albedo": [6.0, 6.0, 5.0]},
    {"name": "spot", "type": "emitter", "albedo": [3.0, 2.0, 2.0]},
    {"name": "fog", "type": "volume", "scattering": [0.6, 0.5, 0.4], "absorption": [0.05, 0.05, 0.05],
     "phaseFunction": "isotropic", "density": 1.3},
    {"name": "haze", "type": "volume", "scattering": [0.3, 0.3, 0.3], "absorption": [0.1, 0.1, 0.1],
     "phaseFunction": "hg", "g": 0.5, "density": 2.0},
    {"name": "cloud_iso", "type": "volume", "scattering": [0.9, 0.9, 0.9], "absorption": [0.1, 0.1, 0.1],
     "phaseFunction": "isotropic", "density": 20,
     "grid": {"generator": "fbm", "resolution": [32, 32, 32], "octaves": 3, "frequency": 0.125,
              "falloff_radius": 16, "seed": 7}},
]
CAMERA = {"position": [0, 1, -2.6], "lookAt": [0, 1, 0], "up": [0, 1, 0], "speed": 5, "vfov": 60,
          "aperture": 0.0001, "autoFocus": True, "focus": 1}


def scene_text(prims, bounces=8, res=(48, 40), spp=2):
    return json.dumps({"version": "0.0.1a", "materials": MATS, "primitives": BOX + prims, "camera": CAMERA,
                       "renderer": {"resolution": list(res), "spp": spp, "bounces": bounces, "mode": "offline",
                                    "HDR": True}})


SCENES = {
    # homogeneous isotropic fog box and a homogeneous HG box, lit by the ceiling lamp
    "homogeneous": [
        {"name": "light", "type": "rectangle", "transform": T((0, 1.99, 0), (-90, 0, 0), (0.5, 0.5, 1)),
         "materialName": "lamp"},
        {"name": "fogBox", "type": "volume", "transform": T((-0.35, 0.5, 0.1), (0, 20, 0), (0.7, 1.0, 0.7)),
         "materialName": "fog"},
        {"name": "hazeBox", "type": "volume", "transform": T((0.45, 0.4, -0.2), (0, -10, 0), (0.6, 0.8, 0.6)),
         "materialName": "haze"},
    ],
    # a grid medium with the isotropic phase function
    "grid_isotropic": [
        {"name": "light", "type": "rectangle", "transform": T((0, 1.99, 0), (-90, 0, 0), (0.5, 0.5, 1)),
         "materialName": "lamp"},
        {"name": "cloudBox", "type": "volume", "transform": T((0, 0.8, 0), (0, 0, 0), (1.2, 1.2, 1.2)),
         "materialName": "cloud_iso"},
    ],
    # a sphere emitter and a point emitter, with a glossy sphere to reflect them
    "sphere_point_lights": [
        {"name": "bulbSphere", "type": "sphere", "radius": 0.15, "transform": T((0.3, 1.6, 0.2)),
         "materialName": "bulb"},
        {"name": "spotPoint", "type": "point", "transform": T((-0.5, 1.5, -0.3)), "materialName": "spot"},
        {"name": "ball", "type": "sphere", "radius": 0.35, "transform": T((-0.2, 0.35, 0.1)), "materialName": "glossy"},
    ],
}


@pytest.fixture(scope="module")
def ne(built):
    import narvalengine_gb300 as ne
    return ne


@pytest.fixture(scope="module")
def ctx(ne):
    c = ne.Context(0)
    yield c
    c.close()


def spread_keys(w, h, n_pixels, spp, seed):
    rng = np.random.default_rng(seed)
    pix = rng.choice(w * h, size=min(n_pixels, w * h), replace=False)
    return np.array([[p, s] for p in pix for s in range(spp)], dtype=np.uint32)


def check_parity(ne, scene, orc, w, h, what):
    for kernel in KERNELS:
        scene.set_tuning(kernel=kernel)
        keys = spread_keys(w, h, 600, 4, seed=kernel)
        for seed in (1, 99):
            p = ne.render_params(seed=seed)
            g = scene.trace_paths(keys, p)
            c = orc.trace_paths(keys, p)
            err = np.abs(g - c) / np.maximum(np.abs(c), 1e-6)
            assert err.max() <= REL_TOL, f"{what} kernel {kernel} seed {seed}: max rel {err.max():.3e}"
            assert np.array_equal(g.view(np.uint32), c.view(np.uint32)), f"{what} kernel {kernel}: not bit-identical"
        img, _ = scene.render(ne.render_params(seed=5, spp=2))
        ref, _ = orc.render(ne.render_params(seed=5, spp=2))
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), f"{what} kernel {kernel}: image differs"
    return c


@pytest.mark.parametrize("name", sorted(SCENES))
def test_scene_parity(ne, ctx, oracle_lib, name):
    text = scene_text(SCENES[name])
    host = ne.SceneHost.from_string(text)
    scene = ctx.upload(host)
    orc = oracle_lib.OracleScene.from_json(text=text)
    try:
        c = check_parity(ne, scene, orc, host.width, host.height, name)
        assert (c.sum(1) > 0).mean() > 0.3, "the scene's paths should mostly carry light"
    finally:
        scene.close()
        orc.close()


def test_homogeneous_medium_changes_light(ne, oracle_lib):
    """The homogeneous boxes are really traversed: the same scene without them renders
    differently (on the oracle), and the medium branch draws random numbers."""
    with_media = oracle_lib.OracleScene.from_json(text=scene_text(SCENES["homogeneous"]))
    without = oracle_lib.OracleScene.from_json(text=scene_text(SCENES["homogeneous"][:1]))
    p = ne.render_params(seed=3, spp=4)
    a, _ = with_media.render(p)
    b, _ = without.render(p)
    assert np.abs(a - b).mean() > 1e-3


def mesh_light_desc(oracle_lib):
    """The oracle's reading of a box with an emissive tetrahedron mesh, turned into a light
    model: its triangles move from Model::primitives to Model::lights, its instance to the
    scene's lights, and the emitter's Light::primitive is the mesh's second triangle."""
    from oracle.scene_reader import OracleSceneDesc
    tet = {"name": "tet", "type": "mesh",
           "positions": [0, 0, 0, 0.4, 0, 0, 0, 0.4, 0, 0, 0, 0.4], "indices": [0, 2, 1, 0, 1, 3, 0, 3, 2, 1, 2, 3],
           "materialName": "bulb", "transform": T((-0.2, 1.3, 0.1), (15, 30, 0), (1, 1, 1))}
    ball = {"name": "ball", "type": "sphere", "radius": 0.35, "transform": T((0.2, 0.35, 0.1)),
            "materialName": "glossy"}
    sd = OracleSceneDesc(text=scene_text([ball, tet]))
    d = sd.desc
    ni = d.n_instances
    mesh_inst = next(i for i in range(ni) if d.models[d.instances[i].model].use_bvh)
    m = d.models[d.instances[mesh_inst].model]
    m.light_begin, m.light_count, m.prim_count = m.prim_begin, 4, 0
    m.has_bbox, m.use_bvh = 0, 0  # a light model is scanned linearly (Model.cpp:432-443)
    mat = d.materials[d.prims[m.light_begin].material]
    d.lights[mat.light].primitive = m.light_begin + 1
    # instances: the others in order, then the scene's lights with the mesh first
    order = [i for i in range(ni) if i != mesh_inst] + [mesh_inst] + list(range(ni, ni + d.n_light_instances))
    src = [bytes(d.instances[i]) for i in range(ni + d.n_light_instances)]
    for k, i in enumerate(order):
        C.memmove(C.addressof(d.instances[k]), src[i], len(src[i]))
    d.n_instances, d.n_light_instances = ni - 1, d.n_light_instances + 1
    return sd


def test_triangle_emitter_parity(ne, ctx, oracle_lib):
    sd = mesh_light_desc(oracle_lib)
    scene = ctx.upload(sd)
    orc = oracle_lib.OracleScene(sd.desc_ptr)
    try:
        c = check_parity(ne, scene, orc, sd.width, sd.height, "triangle emitter")
        # the light samples land at the mesh's object-space triangle (near the floor corner),
        # not where the mesh is, so few paths see light; enough do to exercise the branch
        assert (c.sum(1) > 0).mean() > 0.02
    finally:
        scene.close()
        orc.close()
