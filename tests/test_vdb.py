"""OpenVDB density grids (.vdb) in grid media: the library's reader (vdb_read.cpp), the oracle's
(oracle/vdb.py) and the dense array of core/ResourceManager.cpp:165-218 (loadVDBasTexture)
computed from the sparse description the file was written from (tests/vdb_writer.py), on files
in OpenVDB 6.2's layout: every compression the library reads (none, zip, zip chunks stored raw,
active-mask compression with each node metadata case, Blosc frames stored, LZ4 in one or
several blocks and in split streams), half-float grids, every transform type, several grids,
files with and without grid offsets, the reference's dense box rule on both sides of 0, and the
errors. CPU, plus one GPU render against the oracle."""
import copy
import json

import numpy as np
import pytest

from conftest import scene_path
from test_oracle_scene_reader import assert_same_desc
from vdb_writer import Grid, vdb_file


@pytest.fixture(scope="module")
def ne(built):
    import narvalengine_gb300 as ne
    return ne


def sample_grid(half=False, shift=(0, 0, 0), background=0.0):
    """Leaves with mixed active voxels (inactive ones at the background, minus the background,
    one other value, two other values, several values), active and inactive 8^3 and (for shifts
    that are multiples of 128) inactive 128^3 tiles, spanning negative and positive coordinates;
    `shift` is a multiple of 8."""
    rng = np.random.default_rng(7)
    g = Grid(background=background, half=half)
    bg = np.float32(background)
    sx, sy, sz = shift
    cases = [
        lambda a: np.where(a, rng.random(512), bg),                           # meta 0
        lambda a: np.where(a, rng.random(512), -bg),                          # meta 1 (0 when bg = 0)
        lambda a: np.where(a, rng.random(512), 0.5),                          # one other value
        lambda a: np.where(a, rng.random(512), np.where(rng.random(512) < 0.5, bg, 0.25)),   # bg and one
        lambda a: np.where(a, rng.random(512), np.where(rng.random(512) < 0.5, 0.75, 0.25)),  # two others
        lambda a: np.where(a, rng.random(512), rng.choice([0.125, 0.375, 0.625], 512)),     # three: all
        lambda a: rng.random(512),                                            # every voxel active
    ]
    origins = [(-16, -8, 0), (-8, -8, 0), (0, 0, 0), (8, 0, -8), (16, 8, 8), (0, 16, -16), (-24, 0, 8)]
    for k, (o, make) in enumerate(zip(origins, cases)):
        act = rng.random(512) < (1.0 if k == 6 else 0.3)
        g.leaf((o[0] + sx, o[1] + sy, o[2] + sz), make(act), act)
    g.tiles8[(8 + sx, 8 + sy, 8 + sz)] = (0.5, True)
    g.tiles8[(-8 + sx, 0 + sy, 8 + sz)] = (0.25, False)
    if sx % 128 == 0 and sy % 128 == 0 and sz % 128 == 0:
        g.tiles128[(128 + sx, 0 + sy, 0 + sz)] = (0.0625, False)
        g.tiles128[(-128 + sx, -128 + sy, 128 + sz)] = (0.875, False)
    return g


def scene_with_vdb(tmp_path, data: bytes):
    (tmp_path / "cloud.vdb").write_bytes(data)
    d = json.load(open(scene_path("medium_c2")))
    mat = d["materials"][0]
    mat.pop("grid")
    mat["path"] = "cloud.vdb"
    return json.dumps(d)


def both_readers(ne, tmp_path, data):
    from oracle.scene_reader import OracleSceneDesc
    text = scene_with_vdb(tmp_path, data)
    host = ne.SceneHost.from_string(text, str(tmp_path))
    o = OracleSceneDesc(text=text, resources_dir=str(tmp_path))
    assert_same_desc(host.desc, o.desc)
    m = host.desc.media[0]
    res = [m.res[0], m.res[1], m.res[2]]
    n = res[0] * res[1] * res[2]
    grid = np.ctypeslib.as_array(m.grid, shape=(n,)).copy()
    return res, grid


def check(ne, tmp_path, g, **kw):
    res, grid = both_readers(ne, tmp_path, vdb_file([g], **kw))
    want_res, want = g.expected()
    assert res == want_res
    assert grid.tobytes() == want.tobytes()


@pytest.mark.parametrize("comp,opts", [
    (0, {}), (1, {}), (2, {}), (3, {}), (3, {"zip_raw": True}), (3, {"all_values": True}),
    (4 | 2, {"blosc": "stored"}), (4 | 2, {"blosc": "lz4"}), (4 | 2, {"blosc": "lz4split"}),
    (4 | 2, {"blosc": "raw"}), (4, {"blosc": "blocks"}), (4 | 2, {"blosc": "blocks"}),
])
def test_compressions(ne, oracle_lib, tmp_path, comp, opts):
    check(ne, tmp_path, sample_grid(), comp=comp, opts=opts)


@pytest.mark.parametrize("half", [False, True])
@pytest.mark.parametrize("background", [0.0, 0.25])
def test_half_floats_and_background(ne, oracle_lib, tmp_path, half, background):
    check(ne, tmp_path, sample_grid(half=half, background=background), comp=3)


def test_half_float_edge_values(ne, oracle_lib, tmp_path):
    """Half floats of every kind: zeros of both signs, subnormals, the largest normal, infinities,
    a NaN, converted exactly."""
    g = Grid(background=0.0, half=True)
    special = np.array([0.0, -0.0, 2.0 ** -24, 3 * 2.0 ** -24, 2.0 ** -14 - 2.0 ** -24, 2.0 ** -14, 65504.0,
                        -65504.0, np.inf, -np.inf, np.nan, 1.0 / 3.0], np.float32)
    vals = np.resize(special, 512)
    g.leaf((0, 0, 0), vals, np.ones(512, bool))
    g.leaf((8, 8, 8), np.resize(special[::-1], 512), np.ones(512, bool))
    res, grid = both_readers(ne, tmp_path, vdb_file([g], comp=3))
    want_res, want = g.expected()
    assert res == want_res and grid.tobytes() == want.tobytes()


@pytest.mark.parametrize("transform", ["UniformScaleMap", "AffineMap", "ScaleTranslateMap", "TranslationMap",
                                       "UnitaryMap", "NonlinearFrustumMap"])
def test_transforms(ne, oracle_lib, tmp_path, transform):
    check(ne, tmp_path, sample_grid(), comp=3, transform=transform)


def test_dense_box_rule(ne, oracle_lib, tmp_path):
    """Active box entirely at positive coordinates: loadVDBasTexture's box starts at -|min| and
    spans |min| + |max| voxels, so it covers background below the grid and drops its last
    plane; entirely negative: the box from min spans |min| + |max|."""
    for shift in [(40, 24, 64), (-64, -200, -48), (136, -8, 16)]:
        g = sample_grid(shift=shift)
        (lo, hi) = g.active_box()
        res, grid = both_readers(ne, tmp_path, vdb_file([g], comp=3))
        want_res, want = g.expected()
        assert res == want_res and grid.tobytes() == want.tobytes()
        dims = [abs(int(lo[a])) + abs(int(hi[a])) + (1 if lo[a] < 0 <= hi[a] else 0) for a in range(3)]
        assert res == [dims[2], dims[1], dims[0]]


def test_root_tiles(ne, oracle_lib, tmp_path):
    """A root tile inside the dense box: one leaf at z in [-4096, -4089] makes the box run from
    z = -4096 over 4096 + 4089 voxels, through the inactive root tile at (0, 0, 0)."""
    g = Grid(background=0.0)
    g.leaf((0, 0, -4096), np.full(512, 0.5), np.ones(512, bool))
    g.root_tiles[(0, 0, 0)] = (0.75, False)
    res, grid = both_readers(ne, tmp_path, vdb_file([g], comp=3))
    want_res, want = g.expected()
    assert res == want_res == [8185, 7, 7] and grid.tobytes() == want.tobytes()
    assert (grid.reshape(7, 7, 8185)[:, :, 4096:] == np.float32(0.75)).all()


def test_several_grids(ne, oracle_lib, tmp_path):
    other = sample_grid(shift=(8, 8, 8))
    other.name = "temperature"
    dens = sample_grid()
    dens2 = sample_grid(shift=(16, 0, 0))
    # with offsets: the first grid named density, after a float grid and a grid of another type
    data = vdb_file([other, other, dens, dens2], comp=3, extra_types={1: "Tree_vec3s_5_4_3"})
    res, grid = both_readers(ne, tmp_path, data)
    want_res, want = dens.expected()
    assert res == want_res and grid.tobytes() == want.tobytes()
    # without offsets: grids before it are read through
    data = vdb_file([other, dens], comp=3, offsets=False)
    res, grid = both_readers(ne, tmp_path, data)
    assert res == want_res and grid.tobytes() == want.tobytes()


def load_status(ne, tmp_path, data):
    from oracle.scene_reader import OracleSceneDesc, SceneError
    text = scene_with_vdb(tmp_path, data)
    with pytest.raises(ne.NarvalError) as e:
        ne.SceneHost.from_string(text, str(tmp_path))
    with pytest.raises(SceneError):
        OracleSceneDesc(text=text, resources_dir=str(tmp_path))
    return e.value.status


def test_errors(ne, oracle_lib, tmp_path):
    from narvalengine_gb300 import _abi
    g = sample_grid()
    good = vdb_file([g], comp=3)
    assert load_status(ne, tmp_path, b"not a vdb file at all") == _abi.NE_ERR_PARSE
    assert load_status(ne, tmp_path, good[:len(good) // 2]) == _abi.NE_ERR_PARSE
    assert load_status(ne, tmp_path, vdb_file([g], comp=3, version=221)) == _abi.NE_ERR_UNSUPPORTED
    other = copy.deepcopy(g)
    other.name = "temperature"
    assert load_status(ne, tmp_path, vdb_file([other], comp=3)) == _abi.NE_ERR_PARSE  # no density grid
    assert load_status(ne, tmp_path, vdb_file([g], comp=3, extra_types={0: "Tree_double_5_4_3"})) == \
        _abi.NE_ERR_UNSUPPORTED
    assert load_status(ne, tmp_path, vdb_file([other, g], comp=3, offsets=False,
                                              extra_types={0: "Tree_vec3s_5_4_3"})) == _abi.NE_ERR_UNSUPPORTED
    empty = Grid()
    empty.leaf((0, 0, 0), np.zeros(512), np.zeros(512, bool))
    assert load_status(ne, tmp_path, vdb_file([empty], comp=3)) == _abi.NE_ERR_PARSE  # no active voxel
    flat = Grid()
    flat.leaf((0, 0, 0), np.zeros(512), np.arange(512) == 0)  # one active voxel at 0: an empty box
    assert load_status(ne, tmp_path, vdb_file([flat], comp=3)) == _abi.NE_ERR_PARSE
    # a Blosc frame with another codec (BloscLZ, codec 0)
    data = bytearray(vdb_file([g], comp=4 | 2, opts={"blosc": "lz4"}))
    k = bytes(data).find(bytes([2, 1, (1 << 5) | 0x11, 4]))
    data[k + 2] = 0x11
    assert load_status(ne, tmp_path, bytes(data)) == _abi.NE_ERR_UNSUPPORTED


def test_corrupt_files_give_status_codes(ne, oracle_lib, tmp_path):
    """Truncated files and flipped or replaced bytes, under every compression: the library's
    reader returns a status (or reads the file when the change only hits values), never crashes,
    and the oracle's reader rejects the same files and reads the others alike."""
    from oracle.scene_reader import OracleSceneDesc, SceneError
    rng = np.random.default_rng(11)
    bases = [vdb_file([sample_grid()], comp=c, opts=o) for c, o in
             [(3, {}), (6, {"blosc": "lz4"}), (6, {"blosc": "lz4split"}), (0, {}), (4, {"blosc": "blocks"})]]
    seen = set()
    for it in range(150):
        b = bytearray(bases[it % len(bases)])
        kind = it % 3
        if kind == 0:
            b = b[:rng.integers(0, len(b))]
        else:
            for _ in range(rng.integers(1, 8)):
                k = rng.integers(0, len(b))
                b[k] = rng.integers(0, 256) if kind == 1 else b[k] ^ (1 << rng.integers(0, 8))
        text = scene_with_vdb(tmp_path, bytes(b))
        try:
            lib = ne.SceneHost.from_string(text, str(tmp_path))
            seen.add(0)
        except ne.NarvalError as e:
            assert e.status in (-2, -6), e
            seen.add(e.status)
            lib = None
        try:
            orc = OracleSceneDesc(text=text, resources_dir=str(tmp_path))
        except SceneError:
            orc = None
        assert (lib is None) == (orc is None), it
        if lib is not None:
            assert_same_desc(lib.desc, orc.desc)
    assert {-2, 0} <= seen


@pytest.mark.gpu
def test_vdb_scene_parity(ne, oracle_lib, tmp_path):
    """A medium whose density comes from a .vdb file: camera paths and a render on every path
    kernel, bit-identical to the oracle (which reads the file with its own reader)."""
    from test_light_medium_kinds import check_parity
    d = json.loads(scene_with_vdb(tmp_path, vdb_file([sample_grid()], comp=3)))
    d["renderer"]["resolution"] = [48, 32]
    d["renderer"]["spp"] = 2
    text = json.dumps(d)
    host = ne.SceneHost.from_string(text, str(tmp_path))
    orc = oracle_lib.OracleScene.from_json(text=text, resources_dir=str(tmp_path))
    ctx = ne.Context(0)
    try:
        scene = ctx.upload(host)
        c = check_parity(ne, scene, orc, host.width, host.height, "vdb")
        assert (c.sum(1) > 0).mean() > 0.1, "the paths should carry light"
        scene.close()
    finally:
        orc.close()
        ctx.close()
