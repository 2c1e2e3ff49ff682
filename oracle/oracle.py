"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg, as the checker or the timed CPU restatement of the reference; the
product (narvalengine_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from narvalengine_gb300 import _abi  # noqa: E402  (struct layouts only)
from narvalengine_gb300._abi import NeHit, NeRenderParams  # noqa: E402

LIB_PATH = os.path.join(HERE, "liboracle.so")
_lib = None

_F = C.POINTER(C.c_float)
SIGNATURES = {
    "orc_scene_create": (C.c_void_p, [C.POINTER(_abi.NeSceneDesc)]),
    "orc_scene_destroy": (None, [C.c_void_p]),
    "orc_trace_paths": (None, [C.c_void_p, C.POINTER(NeRenderParams), C.c_void_p, C.c_size_t, C.c_void_p, C.c_int]),
    "orc_trace_view_paths": (None, [C.c_void_p, C.POINTER(NeRenderParams), C.c_void_p, C.c_int, C.c_int, C.c_uint32,
                                     C.c_void_p, C.c_size_t, C.c_void_p, C.c_int]),
    "orc_model_bvh": (C.c_size_t, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_size_t, C.c_void_p]),
    "orc_model_set_bvh": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]),
    "orc_li_batch": (None, [C.c_void_p, C.POINTER(NeRenderParams), C.c_void_p, C.c_void_p, C.c_size_t, C.c_uint32,
                            C.c_void_p, C.c_int]),
    "orc_render": (C.c_double, [C.c_void_p, C.POINTER(NeRenderParams), C.c_void_p, C.c_int]),
    "orc_render_pixels": (C.c_double, [C.c_void_p, C.POINTER(NeRenderParams), C.c_uint32, C.c_uint32, C.c_void_p,
                                       C.c_int, C.POINTER(C.c_uint64)]),
    "orc_render_pixel_list": (C.c_double, [C.c_void_p, C.POINTER(NeRenderParams), C.c_void_p, C.c_uint32,
                                           C.c_void_p, C.c_int, C.POINTER(C.c_uint64)]),
    "orc_trace_closest": (None, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_float, C.c_float, C.c_void_p]),
    "orc_triangle_intersect": (C.c_int, [_F, _F, _F, C.c_void_p, _F, _F, _F, _F]),
    "orc_aabb_intersect": (C.c_int, [_F, _F, C.c_void_p, _F, _F, _F, _F]),
    "orc_orthonormal": (None, [_F, _F, _F]),
    "orc_to_lcs": (None, [_F, _F, _F, _F, _F]),
    "orc_to_world": (None, [_F, _F, _F, _F, _F]),
    "orc_sample_unit_sphere": (None, [C.c_float, C.c_float, _F]),
    "orc_hg_eval": (C.c_float, [C.c_float, _F, _F]),
    "orc_hg_sample": (None, [C.c_float, C.c_float, C.c_float, _F]),
    "orc_iso_pdf": (C.c_float, []),
    "orc_barycentric": (None, [_F, _F, _F, _F, _F]),
    "orc_triangle_area": (C.c_float, [_F, _F, _F]),
    "orc_triangle_contains": (C.c_int, [_F, _F, _F, _F]),
    "orc_point_in_triangle_range": (C.c_int, [_F, _F, _F, _F]),
    "orc_triangle_model_intersect": (C.c_int, [_F, C.c_uint32, C.POINTER(C.c_uint32), C.c_uint32, C.c_void_p,
                                               C.c_float, C.c_float, _F]),
    "orc_bvh_build_count": (C.c_uint32, [_F, C.POINTER(C.c_uint32), C.c_uint32]),
    "orc_fmath": (None, [C.c_int, C.c_void_p, C.c_size_t, C.c_void_p]),
    "orc_rng": (None, [C.c_uint64, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "orc_philox": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "orc_gen_fbm": (None, [C.POINTER(C.c_uint32), C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                           C.c_uint64, C.c_void_p]),
    "orc_gen_icosphere": (None, [C.c_int, C.c_double, C.c_double, C.c_uint64, C.c_void_p, C.c_void_p]),
    "orc_gen_hash_u01": (C.c_double, [C.c_uint64, C.c_uint64]),
}


def library() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            import importlib.util
            spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build()
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def fv(*vals) -> C.Array:
    return (C.c_float * len(vals))(*vals)


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class OracleScene:
    """CPU restatement of the reference integrator over a scene description."""

    def __init__(self, desc_ptr):
        self._lib = library()
        self._h = self._lib.orc_scene_create(desc_ptr)
        if not self._h:
            raise RuntimeError("orc_scene_create failed")
        self.width = desc_ptr.contents.settings.width
        self.height = desc_ptr.contents.settings.height
        self.spp = desc_ptr.contents.settings.spp
        self.bounces = desc_ptr.contents.settings.bounces

    @classmethod
    def from_json(cls, path: str | None = None, text: str | None = None,
                  resources_dir: str | None = None) -> "OracleScene":
        """The oracle's scene read from the reference's JSON descriptor by the oracle's own
        reader (scene_reader.py), independently of the library's reader."""
        from oracle.scene_reader import OracleSceneDesc
        sd = OracleSceneDesc(path, text, resources_dir)
        o = cls(sd.desc_ptr)
        o.reader = sd
        return o

    def trace_paths(self, keys: np.ndarray, params: NeRenderParams, threads: int = 0) -> np.ndarray:
        keys = np.ascontiguousarray(keys, dtype=np.uint32).reshape(-1, 2)
        out = np.empty((len(keys), 3), dtype=np.float32)
        self._lib.orc_trace_paths(self._h, C.byref(params), _p(keys), len(keys), _p(out), threads or os.cpu_count())
        return out

    def trace_view_paths(self, camera, width: int, height: int, stream: int, keys: np.ndarray,
                         params: NeRenderParams, threads: int = 0) -> np.ndarray:
        """Camera paths of one view: `camera` is an ne_camera structure (ctypes)."""
        keys = np.ascontiguousarray(keys, dtype=np.uint32).reshape(-1, 2)
        out = np.empty((len(keys), 3), dtype=np.float32)
        self._lib.orc_trace_view_paths(self._h, C.byref(params), C.byref(camera), width, height, stream, _p(keys),
                                       len(keys), _p(out), threads or os.cpu_count())
        return out

    def model_bvh(self, m: int, n_prims: int):
        """(nodes (n, 9) float32 with the last three words as uint32 bits, primitive order)."""
        nodes = np.empty((2 * n_prims + 1, 9), np.float32)
        order = np.empty(n_prims, np.uint32)
        n = self._lib.orc_model_bvh(self._h, m, _p(nodes), len(nodes), _p(order))
        return nodes[:n], order

    def set_model_bvh(self, m: int, nodes: np.ndarray, order: np.ndarray):
        """Traverse model m through the given tree (orc_model_bvh's format) from now on."""
        nodes = np.ascontiguousarray(nodes, dtype=np.float32).reshape(-1, 9)
        order = np.ascontiguousarray(order, dtype=np.uint32)
        if self._lib.orc_model_set_bvh(self._h, m, _p(nodes), len(nodes), _p(order), len(order)) != 0:
            raise ValueError("invalid BVH for model %d" % m)

    def li_batch(self, rays: np.ndarray, keys: np.ndarray, first_dim: int, params: NeRenderParams,
                 threads: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        keys = np.ascontiguousarray(keys, dtype=np.uint32).reshape(-1, 2)
        out = np.empty((len(rays), 3), dtype=np.float32)
        self._lib.orc_li_batch(self._h, C.byref(params), _p(rays), _p(keys), len(rays), first_dim, _p(out),
                               threads or os.cpu_count())
        return out

    def render(self, params: NeRenderParams, threads: int = 0):
        out = np.zeros((self.height, self.width, 3), dtype=np.float32)
        secs = self._lib.orc_render(self._h, C.byref(params), _p(out), threads or os.cpu_count())
        return out, secs

    def render_pixels(self, params: NeRenderParams, first: int, count: int, threads: int = 0):
        out = np.zeros((count, 3), dtype=np.float32)
        lookups = C.c_uint64(0)
        secs = self._lib.orc_render_pixels(self._h, C.byref(params), first, count, _p(out),
                                           threads or os.cpu_count(), C.byref(lookups))
        return out, secs, lookups.value

    def render_pixel_list(self, params: NeRenderParams, pixels: np.ndarray, threads: int = 0):
        """Mean radiance of the listed pixels (all spp each): (out, seconds, density lookups)."""
        pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
        out = np.zeros((len(pixels), 3), dtype=np.float32)
        lookups = C.c_uint64(0)
        secs = self._lib.orc_render_pixel_list(self._h, C.byref(params), _p(pixels), len(pixels), _p(out),
                                               threads or os.cpu_count(), C.byref(lookups))
        return out, secs, lookups.value

    def trace_closest(self, rays: np.ndarray, t_min: float, t_max: float) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        out = (NeHit * len(rays))()
        self._lib.orc_trace_closest(self._h, _p(rays), len(rays), t_min, t_max, C.addressof(out))
        buf = (C.c_char * C.sizeof(out)).from_address(C.addressof(out))
        from narvalengine_gb300 import HIT_DTYPE
        return np.frombuffer(bytes(buf), dtype=HIT_DTYPE).copy()

    def close(self):
        if self._h:
            self._lib.orc_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fmath(fn: int, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    library().orc_fmath(fn, _p(x), x.size, _p(out))
    return out


def rng(seed: int, keys: np.ndarray, dims: np.ndarray) -> np.ndarray:
    keys = np.ascontiguousarray(keys, dtype=np.uint32)
    dims = np.ascontiguousarray(dims, dtype=np.uint32)
    out = np.empty(len(dims), dtype=np.float32)
    library().orc_rng(seed, _p(keys), _p(dims), len(dims), _p(out))
    return out


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    library().orc_philox(c, k, o)
    return list(o)
