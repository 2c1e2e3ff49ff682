"""Builds libnarval_gb300.so in-tree for sm_103a.

CUDA sources compile with nvcc for sm_103a only, host sources with g++; every
translation unit compiles in parallel and is skipped when its object is newer than
its sources. Floating-point flags are part of the product's contract: no contracted
multiply-adds (-fmad=false on the device, -ffp-contract=off on the host) and IEEE
division and square root, so that the device rounds every operation as the host does.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libnarval_gb300.so")

CUDA_SOURCES = ["api.cu", "k_query.cu", "mlp.cu", "k_views.cu", "bvh_build.cu"] + sorted(
    f for f in os.listdir(os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc")) if f.startswith("k_path_"))
HOST_SOURCES = ["scene_host.cpp", "scene_gen.cpp", "image_io.cpp", "image_load.cpp", "vdb_read.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off",
    "-I" + INCLUDE, "-I" + CSRC,
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I" + INCLUDE, "-I" + CSRC]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnarval_gb300.so")


def _headers() -> list[str]:
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    out += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) >= t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compiles every translation unit that changed and links the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    steps = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            steps.append([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            steps.append([os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-c", s, "-o", o])
    n = jobs or min(len(steps), os.cpu_count() or 4) or 1
    if steps:
        with ThreadPoolExecutor(max_workers=n) as ex:
            for f in [ex.submit(_run, c) for c in steps]:
                f.result()
    if steps or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB} ({len(steps)} translation units recompiled)")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
