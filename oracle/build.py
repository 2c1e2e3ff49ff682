"""Builds the CPU oracle (liboracle.so) from oracle.cpp.

Test infrastructure: the oracle checks the GPU library and times the CPU baseline; the
product never loads it. inputs.cpp adds the seeded generators of the synthetic grids and
meshes (a separate copy of the library's scene_gen.cpp, compiled in here) for the oracle's
own scene reader, so that a process using the oracle never loads the GPU library. Compiled like the reference's Release build (-O2, no fast-math,
no -march=native) with -ffp-contract=off so that no multiply-add is fused, which keeps
every float operation identical to the GPU code compiled with -fmad=false.

The reference itself cannot be compiled here: its headers need glm, rapidjson, glog,
gtest, magic_enum and assimp, whose submodule directories are empty, and its CMake build
targets MSVC, vcpkg and Vulkan. So there is no oracle/_ref build.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "inputs.cpp"),
           os.path.join(ROOT, "narvalengine_gb300", "csrc", "scene_gen.cpp")]
DEPS = SOURCES + [
    os.path.join(ROOT, "narvalengine_gb300", "csrc", "scene_gen.h"),
    os.path.join(HERE, "oracle.h"),
    os.path.join(ROOT, "narvalengine_gb300", "csrc", "ne_fmath.h"),
    os.path.join(ROOT, "narvalengine_gb300", "csrc", "ne_rng.h"),
    os.path.join(ROOT, "include", "narval_scene.h"),
    os.path.join(ROOT, "include", "narval_gb300.h"),
]
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
         "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "narvalengine_gb300", "csrc")]


def build(verbose: bool = False) -> str:
    if os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in DEPS):
        return LIB
    tmp = LIB + ".tmp"
    cmd = [os.environ.get("CXX", "g++")] + FLAGS + SOURCES + ["-o", tmp, "-lpthread"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
