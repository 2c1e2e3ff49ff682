"""The C++ host layer (include/narval_engine.hpp) compiles against the C ABI and works."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, scene_path


@pytest.fixture(scope="module")
def demo(built, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("cpp") / "engine_demo")
    lib_dir = os.path.join(ROOT, "narvalengine_gb300")
    cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp",
           "engine_demo.cpp"), "-L" + lib_dir, "-lnarval_gb300", "-Wl,-rpath," + lib_dir, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def test_cpp_scene_reader(demo):
    out = subprocess.run([demo, scene_path("medium_c2")], capture_output=True, text=True, check=True).stdout
    assert "settings 512 512 64 64" in out
    bad = subprocess.run([demo, "/nonexistent.json"], capture_output=True, text=True)
    assert bad.returncode == 1 and "status -3" in bad.stderr


@pytest.mark.gpu
def test_cpp_offline_engine(demo, tmp_path):
    import json
    d = json.load(open(scene_path("cornell_c1")))
    d["renderer"]["resolution"] = [64, 48]
    d["renderer"]["spp"] = 2
    sp = tmp_path / "s.json"
    sp.write_text(json.dumps(d))
    ppm = tmp_path / "out.ppm"
    out = subprocess.run([demo, str(sp), "--render", str(ppm)], capture_output=True, text=True, check=True).stdout
    assert "rendered 6144 paths" in out
    data = ppm.read_bytes()
    header = b"P6\n64 48\n65535\n"
    assert data.startswith(header) and len(data) == len(header) + 64 * 48 * 3 * 2
    import narvalengine_gb300 as ne
    scene = ne.Context(0).upload(ne.SceneHost.from_string(json.dumps(d)))
    hdr, _ = scene.render(seed=1)
    want = (ne.tone_map(hdr).reshape(-1, 3)[::-1] * np.float32(65535)).astype(np.uint16)
    got = np.frombuffer(data[len(header):], dtype=">u2").reshape(-1, 3)
    assert np.abs(got.astype(np.int64) - want.astype(np.int64)).max() <= 1
