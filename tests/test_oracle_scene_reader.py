"""The oracle's own scene reader against the library's, field by field (CPU).

Both read the reference's JSON descriptor (io/SceneReader.cpp) on their own: the library in
C++ (scene_host.cpp), the oracle in Python from the reference's files and glm's published
algorithms (oracle/scene_reader.py). The parity tests give the GPU the library's scene and the
oracle its own, so any difference in reading would also fail them; this test names the field.
Every float is compared bit for bit, signs of zero included.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

from conftest import scene_path
from test_image_load import encode_png


@pytest.fixture(scope="module")
def ne(built):
    import narvalengine_gb300 as ne
    return ne


def _bytes(ptr, i, typ):
    return bytes((C.c_char * C.sizeof(typ)).from_address(C.addressof(ptr.contents) + i * C.sizeof(typ)))


def assert_same_desc(a, b):
    from narvalengine_gb300 import _abi
    assert (a.n_instances, a.n_light_instances) == (b.n_instances, b.n_light_instances)
    tables = [("instances", _abi.NeInstance, a.n_instances + a.n_light_instances),
              ("models", _abi.NeModel, a.n_models), ("prims", _abi.NePrimitive, a.n_prims),
              ("materials", _abi.NeMaterial, a.n_materials), ("model_materials", C.c_uint32, a.n_model_materials),
              ("media", None, a.n_media), ("lights", None, a.n_lights)]
    for name, typ, n in tables:
        nb = {"instances": b.n_instances + b.n_light_instances}.get(name, getattr(b, "n_" + name, None))
        assert n == nb, f"{name}: {n} vs {nb}"
        if typ is None or n == 0:
            continue
        if name == "prims":
            x = np.frombuffer((C.c_char * (n * C.sizeof(typ))).from_address(C.addressof(a.prims.contents)), np.uint32)
            y = np.frombuffer((C.c_char * (n * C.sizeof(typ))).from_address(C.addressof(b.prims.contents)), np.uint32)
            bad = np.nonzero(x != y)[0]
            assert bad.size == 0, f"prims differ at primitive {bad[0] * 4 // C.sizeof(typ)}"
            continue
        for i in range(n):
            if name == "materials":  # every field but the texel pointer, then the texels
                ma, mb = a.materials[i], b.materials[i]
                k = _abi.NeMaterial.albedo_texels.offset
                assert _bytes(a.materials, i, typ)[:k] == _bytes(b.materials, i, typ)[:k], f"materials[{i}] differs"
                if ma.albedo_width:
                    nt = ma.albedo_width * ma.albedo_height * 4
                    assert C.string_at(ma.albedo_texels, nt) == C.string_at(mb.albedo_texels, nt), f"materials[{i}] texels"
                continue
            assert _bytes(getattr(a, name), i, typ) == _bytes(getattr(b, name), i, typ), f"{name}[{i}] differs"
    for i in range(a.n_lights):
        la, lb = a.lights[i], b.lights[i]
        for f in ("type", "primitive", "env_width", "env_height"):
            assert getattr(la, f) == getattr(lb, f), f"lights[{i}].{f}"
        for f in ("li", "le", "direction", "env_radiance"):
            assert bytes(getattr(la, f)) == bytes(getattr(lb, f)), f"lights[{i}].{f}"
        assert np.float32(la.env_map_pdf).tobytes() == np.float32(lb.env_map_pdf).tobytes()
        if la.env_width:
            n = la.env_width * la.env_height * 4
            assert C.string_at(la.env_texels, n) == C.string_at(lb.env_texels, n), f"lights[{i}] texels"
    for i in range(a.n_media):
        ma, mb = a.media[i], b.media[i]
        for f in ("type", "density"):
            assert getattr(ma, f) == getattr(mb, f), f"media[{i}].{f}"
        for f in ("sigma_s", "sigma_a", "res"):
            assert bytes(getattr(ma, f)) == bytes(getattr(mb, f)), f"media[{i}].{f}"
        if ma.type == 0:
            n = ma.res[0] * ma.res[1] * ma.res[2]
            assert C.string_at(ma.grid, 4 * n) == C.string_at(mb.grid, 4 * n), f"media[{i}] grid"
    assert bytes(a.camera) == bytes(b.camera), "camera"
    assert bytes(a.settings) == bytes(b.settings), "settings"


@pytest.mark.parametrize("name", ["cornell_c1", "medium_c2", "mesh_c3", "views_c5"])
def test_shipped_scenes(ne, oracle_lib, name):
    from oracle.scene_reader import OracleSceneDesc
    host = ne.SceneHost.from_json(scene_path(name))
    o = OracleSceneDesc(scene_path(name))
    assert_same_desc(host.desc, o.desc)


def test_cloud_scene_small_grid(ne, oracle_lib):
    """The dense-cloud descriptor with its grid at 64^3 (the full 512^3 takes a minute per side)."""
    from oracle.scene_reader import OracleSceneDesc
    d = json.load(open(scene_path("cloud_c4")))
    d["materials"][0]["grid"]["resolution"] = [64, 64, 64]
    d["materials"][0]["grid"]["falloff_radius"] = 32
    text = json.dumps(d)
    host = ne.SceneHost.from_string(text)  # each reader owns the memory its description points into
    o = OracleSceneDesc(text=text)
    assert_same_desc(host.desc, o.desc)


def varied_scene(tmp_path):
    """Every descriptor feature the readers share: rotations about several axes, non-uniform
    scales, negative and fractional positions, every material and primitive type, .vol / raw
    grids, a homogeneous medium, an isotropic phase function, emitting spheres and points, OBJ
    models shared between instances, inline and generated meshes, a textured environment map."""
    res = 5
    g = np.random.default_rng(2).random(res ** 3).astype(np.float32)
    with open(tmp_path / "d.vol", "w") as f:
        f.write(f"{res} {res} {res} \n")
        f.write("skipped line\n")
        f.write(" ".join(repr(float(x)) for x in g) + " \n")
    g.tofile(tmp_path / "d.f32")
    (tmp_path / "quad.obj").write_text("# quad\nv -1 0 -1\nv 1 0 -1\nv 1 0.25 1\nv -1 0 1\nf 1 2/5 3//1 4/1/2\n"
                                       "f -4 -3 -1\n")
    sky = np.random.default_rng(3).integers(0, 256, size=(8, 16, 3), dtype=np.uint8)
    (tmp_path / "sky.png").write_bytes(encode_png(sky, 2, 8))
    wall = np.random.default_rng(4).integers(0, 256, size=(6, 10, 4), dtype=np.uint8)
    (tmp_path / "wall.png").write_bytes(encode_png(wall, 6, 8))
    T = lambda p, r=(0, 0, 0), s=(1, 1, 1): {"position": list(p), "rotation": list(r), "scale": list(s)}
    mats = [
        {"name": "white", "type": "microfacet", "roughness": 0.37, "metallic": 0.2, "albedo": [0.7, 0.61, 0.05]},
        {"name": "bumpy", "type": "microfacet", "roughness": 0.8, "metallic": 0.0, "albedo": [0.3, 0.3, 0.3],
         "normalMap": [0.5, 0.5, 1.0]},
        {"name": "painted", "type": "microfacet", "roughness": 0.6, "metallic": 0.1, "albedo": "wall.png"},
        {"name": "lamp", "type": "emitter", "albedo": [5.0, 4.5, 3.1]},
        {"name": "ball_lamp", "type": "emitter", "albedo": [2.0, 2.5, 1.0]},
        {"name": "point_lamp", "type": "emitter", "albedo": [1.0, 1.0, 1.0]},
        {"name": "sun", "type": "directionalLight", "albedo": [2.0, 2.0, 2.0], "position": [0.3, 0.8, -0.41]},
        {"name": "sky", "type": "infiniteAreaLight", "path": "sky.png"},
        {"name": "fog", "type": "volume", "scattering": [0.5, 0.4, 0.3], "absorption": [0.01, 0.02, 0.03],
         "phaseFunction": "isotropic", "density": 0.7},
        {"name": "vol", "type": "volume", "scattering": [0.9, 0.9, 0.9], "absorption": [0.1, 0.1, 0.1],
         "phaseFunction": "henyey-greenstein", "g": -0.3, "density": 3.5, "path": "d.vol"},
        {"name": "raw", "type": "volume", "scattering": [0.8, 0.8, 0.8], "absorption": [0.2, 0.2, 0.2],
         "phaseFunction": "hg", "g": 0.6, "density": 12,
         "grid": {"path": "d.f32", "resolution": [res, res, res]}},
        {"name": "gen", "type": "volume", "scattering": [0.8, 0.8, 0.8], "absorption": [0.2, 0.2, 0.2],
         "phaseFunction": "hg", "g": 0.6, "density": 12,
         "grid": {"generator": "fbm", "resolution": [24, 20, 16], "octaves": 3, "seed": 99}},
    ]
    prims = [
        {"name": "wall", "type": "rectangle", "transform": T((0.3, -1.25, 2), (12.5, -33, 71), (2, 3.5, 1)),
         "materialName": "white"},
        {"name": "wall2", "type": "rectangle", "transform": T((-0.7, 0.1, 0), (90, 0, 0), (1, 1, 1)),
         "materialName": "bumpy"},
        {"name": "mural", "type": "rectangle", "transform": T((0, 1, 0.9), (0, 0, 0), (1.5, 1, 1)),
         "materialName": "painted"},
        {"name": "light", "type": "rectangle", "transform": T((0, 1.99, 0.2), (-90, 5, 0), (0.5, 0.25, 1)),
         "materialName": "lamp"},
        {"name": "ball", "type": "sphere", "radius": 0.35, "transform": T((-0.4, 0.35, 0.3), (10, 20, 30)),
         "materialName": "white"},
        {"name": "ghost", "type": "sphere", "radius": 0.2, "collision": False, "transform": T((0.5, 0.5, 0.5)),
         "materialName": "white"},
        {"name": "ball_light", "type": "sphere", "radius": 0.1, "transform": T((0.1, 1.5, -0.3)),
         "materialName": "ball_lamp"},
        {"name": "pt", "type": "point", "transform": T((0.2, 1.8, 0.1), (0, 0, 0), (1, 1, 1)),
         "materialName": "point_lamp"},
        {"name": "sunPoint", "type": "point", "transform": T((0, 10, 0)), "materialName": "sun"},
        {"name": "skySphere", "type": "sphere", "radius": 100, "transform": T((0, 0, 0), (20, 35, 0)),
         "materialName": "sky"},
        {"name": "fogBox", "type": "volume", "transform": T((1.5, 0.5, -1), (0, 45, 0), (0.5, 1, 0.75)),
         "materialName": "fog"},
        {"name": "volBox", "type": "volume", "transform": T((-1.5, 0.5, 1), (30, 60, 90), (1, 1, 1)),
         "materialName": "vol"},
        {"name": "rawBox", "type": "volume", "transform": T((0, -0.5, 1)), "materialName": "raw"},
        {"name": "genBox", "type": "volume", "transform": T((0, 2.5, 1), (-15, 0, 5), (1.2, 0.8, 1)),
         "materialName": "gen"},
        {"name": "quad1", "type": "obj", "path": "quad.obj", "materialName": "white",
         "transform": T((0, 0.01, 0), (0, 30, 0), (1, 1, 1))},
        {"name": "quad2", "type": "obj", "path": "quad.obj", "materialName": "white", "collision": False,
         "transform": T((0, 0.5, 0), (0, -30, 0), (0.5, 0.5, 0.5))},
        {"name": "tri", "type": "mesh", "positions": [0, 0, 0, 1, 0, 0, 0, 1, 0.5, -0.25, 0.125, 1],
         "indices": [0, 1, 2, 0, 2, 3], "materialName": "bumpy", "transform": T((0.1, 0.2, 0.3), (5, 6, 7))},
        {"name": "blob", "type": "mesh", "generator": "icosphere", "subdivisions": 2,
         "displacement": {"amplitude": 0.1, "frequency": 3, "seed": 5},
         "groups": {"count": 7, "roughness": [0.05, 0.9], "albedo": [0.2, 0.9], "seed": 11},
         "transform": T((-1.3, 1.1, 0), (0, 0, 0), (0.4, 0.4, 0.4))},
    ]
    doc = {"version": "0.0.1a", "materials": mats, "primitives": prims,
           "camera": {"position": [0.25, 1.1, -2.6], "lookAt": [0.1, 0.9, 0], "up": [0, 1, 0], "speed": 5,
                      "vfov": 52.5, "aperture": 0.0001, "autoFocus": False, "focus": 2.25},
           "renderer": {"resolution": [96, 64], "spp": 3, "bounces": 7, "mode": "offline", "HDR": True,
                        "rr": {"after": 2}, "bvh": "sah"}}
    return json.dumps(doc)


def test_varied_scene(ne, oracle_lib, tmp_path):
    from oracle.scene_reader import OracleSceneDesc
    text = varied_scene(tmp_path)
    host = ne.SceneHost.from_string(text, str(tmp_path))
    o = OracleSceneDesc(text=text, resources_dir=str(tmp_path))
    assert_same_desc(host.desc, o.desc)
    # the obj instances share one model and keep collision on, as SceneReader.cpp:245-266 does
    d = o.desc
    obj_inst = [d.instances[i] for i in range(d.n_instances)
                if d.models[d.instances[i].model].use_bvh and d.models[d.instances[i].model].prim_count == 3]
    assert len(obj_inst) == 2 and obj_inst[0].model == obj_inst[1].model
    assert all(i.collision == 1 for i in obj_inst)


def test_glm_inverse_and_euler(oracle_lib):
    """The oracle's glm::inverse and eulerAngleXYZ restatements are the mathematical inverse and
    X(t1) Y(t2) Z(t3) rotation (float64 reference, float32 tolerance)."""
    from oracle import scene_reader as sr
    rng = np.random.default_rng(0)
    for _ in range(20):
        t, r, s = rng.uniform(-3, 3, 3), rng.uniform(-180, 180, 3), rng.uniform(0.2, 3, 3)
        M = sr.get_transform([np.float32(x) for x in t], [np.float32(x) for x in r], [np.float32(x) for x in s])
        A = np.array([[M[c][k] for c in range(4)] for k in range(4)], np.float64)
        a, b, c = np.radians(r.astype(np.float32).astype(np.float64))
        Rx = np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])
        Ry = np.array([[np.cos(b), 0, np.sin(b)], [0, 1, 0], [-np.sin(b), 0, np.cos(b)]])
        Rz = np.array([[np.cos(c), -np.sin(c), 0], [np.sin(c), np.cos(c), 0], [0, 0, 1]])
        ref = np.eye(4)
        ref[:3, :3] = Rx @ Ry @ Rz @ np.diag(s.astype(np.float32))
        ref[:3, 3] = t.astype(np.float32)
        assert np.abs(A - ref).max() < 1e-5
        inv = sr.inverse(M)
        I = np.array([[inv[c][k] for c in range(4)] for k in range(4)], np.float64)
        assert np.abs(I @ A - np.eye(4)).max() < 1e-5


@pytest.mark.parametrize("grid", [{"resolution": [-5, 8, 8]}, {"resolution": [1e30, 8, 8]},
                                  {"resolution": [100000, 8, 8]}, {"octaves": 1000000}, {"seed": -1}])
def test_both_readers_reject_bad_grid_inputs(ne, oracle_lib, grid):
    from oracle.scene_reader import OracleSceneDesc, SceneError
    d = json.load(open(scene_path("cornell_c1")))
    g = {"generator": "fbm", "resolution": [8, 8, 8]}
    g.update(grid)
    d["materials"].append({"name": "v", "type": "volume", "scattering": [1, 1, 1], "absorption": [0, 0, 0],
                           "phaseFunction": "hg", "g": 0.1, "density": 1, "grid": g})
    text = json.dumps(d)
    with pytest.raises(ne.NarvalError):
        ne.SceneHost.from_string(text)
    with pytest.raises(SceneError):
        OracleSceneDesc(text=text)


@pytest.mark.parametrize("mesh", [
    {"generator": "icosphere", "subdivisions": -1}, {"generator": "icosphere", "subdivisions": 20},
    {"generator": "icosphere", "displacement": {"amplitude": 0.1, "seed": -3}},
    {"positions": [0, 0, 0, 1, 0, 0, 0, 1, 0], "indices": [0, 1, -1]},
    {"positions": [0, 0, 0, 1, 0, 0, 0, 1, 0], "indices": [0, 1, 4294967296]},
])
def test_both_readers_reject_bad_mesh_inputs(ne, oracle_lib, mesh):
    from oracle.scene_reader import OracleSceneDesc, SceneError
    d = json.load(open(scene_path("cornell_c1")))
    prim = {"name": "m", "type": "mesh", "materialName": d["materials"][0]["name"],
            "transform": {"position": [0, 0, 0], "rotation": [0, 0, 0], "scale": [1, 1, 1]}}
    prim.update(mesh)
    d["primitives"].append(prim)
    text = json.dumps(d)
    with pytest.raises(ne.NarvalError):
        ne.SceneHost.from_string(text)
    with pytest.raises(SceneError):
        OracleSceneDesc(text=text)


@pytest.mark.parametrize("change", ["spp", "bounces", "rr", "width", "groups", "groups_seed", "vol"])
def test_both_readers_reject_out_of_range_counts(ne, oracle_lib, tmp_path, change):
    from oracle.scene_reader import OracleSceneDesc, SceneError
    d = json.load(open(scene_path("cornell_c1")))
    ren = d["renderer"]
    if change == "spp":
        ren["spp"] = 1e12
    elif change == "bounces":
        ren["bounces"] = -1e12
    elif change == "rr":
        ren["rr"] = {"after": 1e20}
    elif change == "width":
        ren["resolution"] = [1e12, 8]
    elif change in ("groups", "groups_seed"):
        groups = {"count": 1e9} if change == "groups" else {"count": 2, "seed": -1}
        d["primitives"].append({"name": "blob", "type": "mesh", "generator": "icosphere", "subdivisions": 1,
                                "groups": groups, "transform": {"position": [0, 0, 0], "rotation": [0, 0, 0],
                                                                "scale": [1, 1, 1]}})
    else:
        (tmp_path / "g.vol").write_text("-3 2 2 \nskipped\n0.5 ")
        d["materials"].append({"name": "v", "type": "volume", "scattering": [1, 1, 1], "absorption": [0, 0, 0],
                               "phaseFunction": "hg", "g": 0.1, "density": 1, "path": "g.vol"})
    text = json.dumps(d)
    with pytest.raises(ne.NarvalError) as e:
        ne.SceneHost.from_string(text, str(tmp_path))
    assert e.value.status == -2
    with pytest.raises(SceneError):
        OracleSceneDesc(text=text, resources_dir=str(tmp_path))


OBJ_BASE = ("# quad\nv -1 0 -1\nv 1 0 -1\nv 1 0.25 1\nv -1 0 1\nvt 0 0\nvn 0 1 0\nf 1 2/1 3//1 4/1/1\n"
            "f -4 -3 -1\nf 1 2 3 4 1 2\n")


def _obj_scene(tmp_path, obj_text):
    (tmp_path / "q.obj").write_bytes(obj_text)
    d = json.load(open(scene_path("cornell_c1")))
    d["primitives"].append({"name": "q", "type": "obj", "path": "q.obj", "materialName": d["materials"][0]["name"],
                            "transform": {"position": [0, 0, 0], "rotation": [0, 0, 0], "scale": [1, 1, 1]}})
    return json.dumps(d)


def _both(ne, tmp_path, obj_text):
    """(library description or None, oracle description or None) of a scene holding the OBJ."""
    from oracle.scene_reader import OracleSceneDesc, SceneError
    text = _obj_scene(tmp_path, obj_text)
    try:
        lib = ne.SceneHost.from_string(text, str(tmp_path))
    except ne.NarvalError:
        lib = None
    try:
        orc = OracleSceneDesc(text=text, resources_dir=str(tmp_path))
    except SceneError:
        orc = None
    return lib, orc


@pytest.mark.parametrize("line", ["v 1 2", "v 1 0.25.1 3", "v 1e 2 3", "v 1 2 nan", "f 1 2x 3", "f", "f 1 2",
                                  "f 0 1 2", "f 1 2 99", "v 1 2 3_0"])
def test_both_obj_readers_reject(ne, oracle_lib, tmp_path, line):
    lib, orc = _both(ne, tmp_path, (OBJ_BASE + line + "\n").encode())
    assert lib is None and orc is None


def test_obj_readers_agree_on_mutated_files(ne, oracle_lib, tmp_path):
    """Random edits of a small OBJ: both readers reject it, or both read the same description."""
    rng = np.random.default_rng(5)
    alphabet = list(b"0123456789-/ \nfvte.+#\t")
    accepted = 0
    for _ in range(250):
        b = bytearray(OBJ_BASE.encode())
        for _ in range(rng.integers(1, 6)):
            k = int(rng.integers(0, len(b)))
            op = rng.integers(0, 3)
            if op == 0:
                b[k] = alphabet[rng.integers(0, len(alphabet))]
            elif op == 1:
                b[k:k] = bytes(alphabet[j] for j in rng.integers(0, len(alphabet), rng.integers(1, 12)))
            else:
                del b[k:k + int(rng.integers(1, 10))]
        lib, orc = _both(ne, tmp_path, bytes(b))
        assert (lib is None) == (orc is None), bytes(b)
        if lib is not None:
            assert_same_desc(lib.desc, orc.desc)
            accepted += 1
    assert accepted > 20


def test_oracle_stof_matches_the_c_library():
    """The oracle's std::stof (used for .vol files) against the C library's strtof on random
    strings: the same float bits, and no number / out of range where strtof reads nothing or
    overflows."""
    import ctypes
    import random
    from oracle.scene_reader import SceneError, _stof_prefix
    strtof = ctypes.CDLL(None).strtof
    strtof.restype = ctypes.c_float
    strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]
    rnd = random.Random(8)
    alphabet = "0123456789.eE+-xXpPabcdefinINFAty \t\n"
    for i in range(20000):
        if i % 3 == 0:
            t = "%.*e" % (rnd.randint(0, 12), rnd.uniform(-1, 1) * 10 ** rnd.randint(-50, 40))
        elif i % 3 == 1:
            t = "".join(rnd.choice("0123456789") for _ in range(rnd.randint(1, 25))) + \
                rnd.choice(["e-", "e", "."]) + str(rnd.randint(0, 50))
        else:
            t = "".join(rnd.choice(alphabet) for _ in range(rnd.randint(1, 14)))
        buf = ctypes.create_string_buffer(t.encode())
        end = ctypes.c_void_p()
        want = np.float32(strtof(buf, ctypes.byref(end)))
        read = end.value - ctypes.addressof(buf)
        if read == 0 or (np.isinf(want) and "inf" not in t.lower()):
            with pytest.raises(SceneError):
                _stof_prefix(t)
        else:
            assert np.float32(_stof_prefix(t)).view(np.uint32) == want.view(np.uint32), t


def test_vol_readers_agree_on_edited_files(ne, oracle_lib, tmp_path):
    """Random edits of a small .vol file: both readers reject it, or both read the same grid."""
    rng = np.random.default_rng(6)
    g = np.random.default_rng(2).random(27).astype(np.float32)
    base = ("3 3 3 \nskipped line\n" + " ".join(repr(float(x)) for x in g) + " \n").encode()
    d = json.load(open(scene_path("cornell_c1")))
    d["materials"].append({"name": "v", "type": "volume", "scattering": [1, 1, 1], "absorption": [0, 0, 0],
                           "phaseFunction": "hg", "g": 0.1, "density": 1, "path": "g.vol"})
    d["primitives"].append({"name": "vb", "type": "volume", "materialName": "v",
                            "transform": {"position": [0, 1, 0], "rotation": [0, 0, 0], "scale": [0.5, 0.5, 0.5]}})
    text = json.dumps(d)
    from oracle.scene_reader import OracleSceneDesc, SceneError
    alphabet = list(b"0123456789-+. \neE\tx")
    accepted = 0
    for _ in range(200):
        b = bytearray(base)
        for _ in range(rng.integers(1, 5)):
            k = int(rng.integers(0, len(b)))
            op = rng.integers(0, 3)
            if op == 0:
                b[k] = alphabet[rng.integers(0, len(alphabet))]
            elif op == 1:
                b[k:k] = bytes(alphabet[j] for j in rng.integers(0, len(alphabet), rng.integers(1, 6)))
            else:
                del b[k:k + int(rng.integers(1, 6))]
        (tmp_path / "g.vol").write_bytes(bytes(b))
        try:
            lib = ne.SceneHost.from_string(text, str(tmp_path))
        except ne.NarvalError:
            lib = None
        try:
            orc = OracleSceneDesc(text=text, resources_dir=str(tmp_path))
        except SceneError:
            orc = None
        assert (lib is None) == (orc is None), bytes(b)
        if lib is not None:
            assert_same_desc(lib.desc, orc.desc)
            accepted += 1
    assert accepted > 20


@pytest.mark.parametrize("number,ok", [
    ("+1", False), (".5", False), ("1.", False), ("0x10", False), ("NaN", False), ("Infinity", False),
    ("-Infinity", False), ("nan", False), ("inf", False), ("01", False), ("1e", False), ("-", False),
    ("1.5e3", True), ("-0.0", True), ("-0", True), ("1E2", True), ("-0e0", True)])
def test_json_numbers(ne, oracle_lib, number, ok):
    """JSON's number grammar in both readers (no NaN, infinity, hex, leading '+' or '.'); "-0"
    is the integer 0 (+0.0), "-0.0" the double -0.0, as a JSON reader gives them."""
    from oracle.scene_reader import OracleSceneDesc, SceneError
    d = json.load(open(scene_path("cornell_c1")))
    d["camera"]["position"][0] = 12345.0
    text = json.dumps(d).replace("12345.0", number)
    if not ok:
        with pytest.raises(ne.NarvalError):
            ne.SceneHost.from_string(text)
        with pytest.raises(SceneError):
            OracleSceneDesc(text=text)
        return
    lib = ne.SceneHost.from_string(text)
    assert_same_desc(lib.desc, OracleSceneDesc(text=text).desc)
    if number in ("-0", "-0.0"):
        zero = json.dumps(d).replace("12345.0", "0")
        same = ne.SceneHost.from_string(zero).desc.camera
        assert (bytes(lib.desc.camera) == bytes(same)) == (number == "-0")


@pytest.mark.parametrize("name,ok", [
    ("wh\\u0069te", True), ("w\\/hite", True), ("\\u00e9t\\u00e9", True), ("\\ud83d\\ude00 glyph", True),
    ("tab\\there", True), ("bad\\xescape", False), ("raw\x01control", False), ("quote\\\"d", True),
    ("\\ud83d lone", True)])
def test_json_strings(ne, oracle_lib, name, ok):
    """JSON string escapes in both readers: a material named through escapes is found by a
    primitive naming it through others; control characters and unknown escapes are errors."""
    from oracle.scene_reader import OracleSceneDesc, SceneError
    d = json.load(open(scene_path("cornell_c1")))
    old = d["materials"][0]["name"]
    text = json.dumps(d).replace('"' + old + '"', '"@@NAME@@"').replace("@@NAME@@", name)
    try:
        lib = ne.SceneHost.from_string(text)
    except ne.NarvalError:
        lib = None
    try:
        orc = OracleSceneDesc(text=text)
    except SceneError:
        orc = None
    assert (lib is not None) == ok and (orc is not None) == ok
    if ok:
        assert_same_desc(lib.desc, orc.desc)


def test_json_repeated_keys_keep_the_first(ne, oracle_lib):
    """A key given twice in one object: both readers take the first value (rapidjson's member
    lookup searches from the start)."""
    from oracle.scene_reader import OracleSceneDesc
    d = json.load(open(scene_path("cornell_c1")))
    text = json.dumps(d).replace('"spp": 16', '"spp": 16, "spp": 3', 1)
    assert '"spp": 3' in text
    lib = ne.SceneHost.from_string(text)
    orc = OracleSceneDesc(text=text)
    assert lib.desc.settings.spp == orc.desc.settings.spp == 16
    assert_same_desc(lib.desc, orc.desc)


@pytest.mark.parametrize("text", ['{"materials": ' + "[" * 100000 + "]" * 100000 + "}", "TRAILING x", "TRAILING {}"])
def test_json_nesting_and_trailing_data(ne, oracle_lib, text):
    """Arrays nested 100 000 deep (the library stops at 256 levels instead of running out of
    stack) and data after the document: errors in both readers."""
    from oracle.scene_reader import OracleSceneDesc, SceneError
    if text.startswith("TRAILING"):
        text = open(scene_path("cornell_c1")).read() + text[len("TRAILING"):]
    with pytest.raises(ne.NarvalError):
        ne.SceneHost.from_string(text)
    with pytest.raises(SceneError):
        OracleSceneDesc(text=text)


@pytest.mark.parametrize("scattering,density", [([1e38, 1, 1], 20), ([2, 1, 1], 3e38), ([-3e38, 1, 1], 20)])
def test_both_readers_reject_overflowing_media(ne, oracle_lib, scattering, density):
    """A medium whose (scattering + absorption) x density overflows float (the tracking steps
    divide by it and would make no progress): rejected by both readers."""
    from oracle.scene_reader import OracleSceneDesc, SceneError
    d = json.load(open(scene_path("medium_c2")))
    d["materials"][0]["scattering"] = scattering
    d["materials"][0]["density"] = density
    d["materials"][0]["grid"]["resolution"] = [8, 8, 8]
    text = json.dumps(d)
    with pytest.raises(ne.NarvalError):
        ne.SceneHost.from_string(text)
    with pytest.raises(SceneError):
        OracleSceneDesc(text=text)
