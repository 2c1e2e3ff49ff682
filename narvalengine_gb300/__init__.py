"""GB300 path integrator for NarvalEngine scenes.

Python face of libnarval_gb300.so (include/narval_gb300.h). The classes mirror the
reference's render interface:

  SceneReader(path)                  io/SceneReader.cpp:10-54   -> scene, camera, settings
  VolumetricPathIntegrator.Li(...)   integrators/Integrator.h:13-25 (batched: li_batch)
  OfflineEngine(scene).coreLoop()    core/OfflineEngine.cpp:78-146 (tone map + PPM out)

All path tracing runs in the CUDA library; there is no CPU fallback. Importing this
package needs no GPU; creating a Context does, and fails loudly without one.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

import numpy as np

from . import _abi
from ._abi import (NE_RENDER_COUNT_WORK, NE_RENDER_DROP_NONFINITE, NE_RENDER_NO_SYNC, NE_RENDER_OUT_DEVICE,
                   NE_RENDER_REF_TILES,
                   NeHit, NePathKey, NeRay, NeRenderParams, NeRenderStats)

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libnarval_gb300.so")
SCENES_DIR = os.path.join(PKG_DIR, "scenes")

_lib = None


class NarvalError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"status {status}: {message}")
        self.status = status


def library() -> C.CDLL:
    """Loads libnarval_gb300.so (built in-tree by __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA library first (__graft_entry__.build())")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in _abi.SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class SceneHost:
    """A parsed scene descriptor (host memory), the reference's SceneReader result."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        self.desc = library().ne_scene_host_desc(self._h).contents

    @classmethod
    def from_json(cls, path: str, resources_dir: str | None = None) -> "SceneHost":
        lib = library()
        h = C.c_void_p()
        err = C.create_string_buffer(1024)
        rd = resources_dir if resources_dir is not None else os.path.dirname(os.path.abspath(path))
        st = lib.ne_scene_host_load_json(path.encode(), rd.encode(), C.byref(h), err, len(err))
        if st != 0:
            raise NarvalError(st, err.value.decode(errors="replace"))
        return cls(h)

    @classmethod
    def from_string(cls, text: str, resources_dir: str = "") -> "SceneHost":
        lib = library()
        h = C.c_void_p()
        err = C.create_string_buffer(1024)
        st = lib.ne_scene_host_load_json_string(text.encode(), resources_dir.encode(), C.byref(h), err, len(err))
        if st != 0:
            raise NarvalError(st, err.value.decode(errors="replace"))
        return cls(h)

    def model_prim_count(self, model: int) -> int:
        d = C.cast(self.desc_ptr, C.POINTER(_abi.NeSceneDesc)).contents
        return int(d.models[model].prim_count)

    @property
    def n_models(self) -> int:
        return int(C.cast(self.desc_ptr, C.POINTER(_abi.NeSceneDesc)).contents.n_models)

    def model_uses_bvh(self, model: int) -> bool:
        d = C.cast(self.desc_ptr, C.POINTER(_abi.NeSceneDesc)).contents
        return bool(d.models[model].use_bvh)

    @property
    def desc_ptr(self):
        return library().ne_scene_host_desc(self._h)

    @property
    def width(self) -> int:
        return self.desc.settings.width

    @property
    def height(self) -> int:
        return self.desc.settings.height

    @property
    def spp(self) -> int:
        return self.desc.settings.spp

    @property
    def bounces(self) -> int:
        return self.desc.settings.bounces

    def camera_dict(self) -> dict:
        c = self.desc.camera
        return {k: list(getattr(c, k)) for k in ("position", "lower_left", "horizontal", "vertical", "side", "up")} | {
            "lens_radius": c.lens_radius}

    def close(self):
        if self._h:
            library().ne_scene_host_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_params(seed: int = 0, spp: int | None = None, bounces: int | None = None, rr: int | None = None,
                  rr_after: int = 3, sample_offset: int = 0, flags: int = 0) -> NeRenderParams:
    p = NeRenderParams()
    p.seed = seed
    p.spp = spp if spp is not None else 0
    p.bounces = bounces if bounces is not None else -1
    p.rr = rr if rr is not None else -1
    p.rr_after = rr_after
    p.sample_offset = sample_offset
    p.flags = flags
    return p


class Context:
    """One CUDA device and stream (ne_context)."""

    def __init__(self, device: int = 0):
        lib = library()
        h = C.c_void_p()
        st = lib.ne_context_create(device, C.byref(h))
        if st != 0:
            raise NarvalError(st, "ne_context_create failed (no CUDA device?)")
        self._h = h
        self.device = device
        self._scenes = weakref.WeakSet()

    def error(self) -> str:
        return library().ne_last_error(self._h).decode(errors="replace")

    def check(self, st: int):
        if st != 0:
            raise NarvalError(st, self.error())

    def upload(self, host: SceneHost) -> "Scene":
        h = C.c_void_p()
        self.check(library().ne_scene_upload(self._h, host.desc_ptr, C.byref(h)))
        s = Scene(self, h, host)
        self._scenes.add(s)
        return s

    def record(self, slot: int):
        self.check(library().ne_context_event_record(self._h, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        self.check(library().ne_context_event_elapsed(self._h, a, b, C.byref(ms)))
        return ms.value

    def synchronize(self):
        self.check(library().ne_context_synchronize(self._h))

    def flush_l2(self, nbytes: int = 256 << 20):
        self.check(library().ne_context_flush_l2(self._h, nbytes))

    def set_cache_limit(self, nbytes: int):
        """Bytes of released device memory the context keeps cached (ne_context_set_cache_limit)."""
        self.check(library().ne_context_set_cache_limit(self._h, nbytes))

    def read_bandwidth(self, nbytes: int, iters: int = 50) -> float:
        """GB/s of a read-only kernel over an `nbytes` buffer (ne_measure_read_bandwidth)."""
        gbs = C.c_double()
        self.check(library().ne_measure_read_bandwidth(self._h, nbytes, iters, C.byref(gbs)))
        return gbs.value

    def random_read_rate(self, nbytes: int, iters: int = 10) -> float:
        """Random 32-byte reads per second from an `nbytes` buffer (ne_measure_random_read)."""
        r = C.c_double()
        self.check(library().ne_measure_random_read(self._h, nbytes, iters, C.byref(r)))
        return r.value

    def fmath(self, fn: int, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.empty_like(x)
        self.check(library().ne_debug_fmath(self._h, fn, _ptr(x), x.size, _ptr(out)))
        return out

    def rng(self, seed: int, keys: np.ndarray, dims: np.ndarray) -> np.ndarray:
        keys = np.ascontiguousarray(keys, dtype=np.uint32)
        dims = np.ascontiguousarray(dims, dtype=np.uint32)
        out = np.empty(len(dims), dtype=np.float32)
        self.check(library().ne_debug_rng(self._h, seed, _ptr(keys), _ptr(dims), len(dims), _ptr(out)))
        return out

    def close(self):
        if self._h:
            # scenes first: the library destroys them with the context, so their handles die here
            for s in list(self._scenes):
                s._h = None
            library().ne_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    """A scene resident on the device (ne_scene)."""

    def __init__(self, ctx: Context, handle: C.c_void_p, host: SceneHost):
        self.ctx = ctx
        self._h = handle
        self.host = host

    def render(self, params: NeRenderParams | None = None, out: np.ndarray | None = None, **kw):
        """Per-pixel mean radiance (H, W, 3) float32 before tone mapping, and the stats."""
        p = params if params is not None else render_params(**kw)
        W, H = self.host.width, self.host.height
        if p.flags & NE_RENDER_OUT_DEVICE:
            if out is None:
                raise ValueError("NE_RENDER_OUT_DEVICE needs a device pointer in out")
            ptr = C.c_void_p(int(out))
            img = None
        else:
            img = out if out is not None else np.empty((H, W, 3), dtype=np.float32)
            ptr = _ptr(img)
        stats = NeRenderStats()
        self.ctx.check(library().ne_render(self._h, C.byref(p), ptr, C.byref(stats)))
        return img, {f: getattr(stats, f) for f, _ in NeRenderStats._fields_ }

    def accumulate(self, accum, params: NeRenderParams | None = None, **kw) -> dict:
        """Adds samples to an FP64 (H, W, 3) accumulator (ne_render_accumulate): a host
        float64 array, or with NE_RENDER_OUT_DEVICE in the flags a device pointer (int)."""
        p = params if params is not None else render_params(**kw)
        if p.flags & NE_RENDER_OUT_DEVICE:
            ptr = C.c_void_p(int(accum))
        else:
            if (not isinstance(accum, np.ndarray) or accum.dtype != np.float64 or not accum.flags.c_contiguous
                    or accum.size != self.host.width * self.host.height * 3):
                raise ValueError("accum must be a C-contiguous float64 array of width*height*3 values")
            ptr = _ptr(accum)
        stats = NeRenderStats()
        self.ctx.check(library().ne_render_accumulate(self._h, C.byref(p), ptr, C.byref(stats)))
        return {f: getattr(stats, f) for f, _ in NeRenderStats._fields_ }

    def render_cached(self, cache: "RadianceCache", bounce: int = 2, train_stride: int = 0, train_steps: int = 0,
                      train_batch: int = 0, params: NeRenderParams | None = None, out=None, train_suffix: int = 0,
                      **kw):
        """ne_render_cached: (image or None, render stats, cache stats)."""
        p = params if params is not None else render_params(**kw)
        W, H = self.host.width, self.host.height
        if p.flags & NE_RENDER_OUT_DEVICE:
            if out is None:
                raise ValueError("NE_RENDER_OUT_DEVICE needs a device pointer in out")
            ptr = C.c_void_p(int(out))
            img = None
        else:
            img = out if out is not None else np.empty((H, W, 3), dtype=np.float32)
            ptr = _ptr(img)
        cp = _abi.NeCacheRenderParams(bounce, train_stride, train_steps, train_batch, train_suffix)
        stats = NeRenderStats()
        cst = _abi.NeCacheRenderStats()
        self.ctx.check(library().ne_render_cached(self._h, cache._h, C.byref(p), C.byref(cp), ptr, C.byref(stats),
                                                  C.byref(cst)))
        return (img, {f: getattr(stats, f) for f, _ in NeRenderStats._fields_},
                {f: getattr(cst, f) for f, _ in _abi.NeCacheRenderStats._fields_})

    def bvh(self, model: int):
        """ne_scene_bvh: (nodes (n, 9) float32 as ne_debug_bvh writes them, primitive order) of
        one model's device BVH, or None for a model without one."""
        n = C.c_size_t()
        self.ctx.check(library().ne_scene_bvh(self._h, model, None, 0, None, C.byref(n)))
        if n.value == 0:
            return None
        prim_count = self.host.model_prim_count(model)
        nodes = np.empty((n.value, 9), np.float32)
        order = np.empty(prim_count, np.uint32)
        self.ctx.check(library().ne_scene_bvh(self._h, model, _ptr(nodes), n.value, _ptr(order), C.byref(n)))
        return nodes, order

    def set_tuning(self, kernel: int = 0, track_share: int = 16, blocks_per_sm: int = 0, split_passes: int = 0,
                   split_half: int = 1, queue_quarters: int = 3, pretrace: int = 0):
        """Launch configuration of the path kernels (see ne_tuning in include/narval_gb300.h)."""
        t = _abi.NeTuning(kernel, track_share, blocks_per_sm, split_passes, split_half, queue_quarters, pretrace)
        self.ctx.check(library().ne_scene_set_tuning(self._h, C.byref(t)))

    def autotune(self, repeats: int = 2, params: NeRenderParams | None = None, **kw):
        """ne_scene_autotune: keeps the fastest kernel configuration; returns (tuning, ms)."""
        p = params if params is not None else render_params(**kw)
        t = _abi.NeTuning()
        ms = C.c_double()
        self.ctx.check(library().ne_scene_autotune(self._h, C.byref(p), repeats, C.byref(t), C.byref(ms)))
        return self.tuning(), ms.value

    def tuning(self) -> dict:
        t = _abi.NeTuning()
        self.ctx.check(library().ne_scene_get_tuning(self._h, C.byref(t)))
        return {"kernel": t.kernel, "track_share": t.track_share, "blocks_per_sm": t.blocks_per_sm,
                "split_passes": t.split_passes, "split_half": t.split_half, "queue_quarters": t.queue_quarters,
                "pretrace": t.pretrace}

    def trace_paths(self, keys: np.ndarray, params: NeRenderParams | None = None, **kw) -> np.ndarray:
        """Camera path radiance for (pixel, sample) keys, shape (n, 3)."""
        p = params if params is not None else render_params(**kw)
        keys = np.ascontiguousarray(keys, dtype=np.uint32).reshape(-1, 2)
        out = np.empty((len(keys), 3), dtype=np.float32)
        self.ctx.check(library().ne_trace_paths(self._h, C.byref(p), _ptr(keys), len(keys), _ptr(out)))
        return out

    def li_batch(self, rays: np.ndarray, keys: np.ndarray, first_dim: int = 0,
                 params: NeRenderParams | None = None, **kw) -> np.ndarray:
        """Integrator::Li for rays (n, 6) = origin, direction."""
        p = params if params is not None else render_params(**kw)
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        keys = np.ascontiguousarray(keys, dtype=np.uint32).reshape(-1, 2)
        out = np.empty((len(rays), 3), dtype=np.float32)
        self.ctx.check(library().ne_li_batch(self._h, C.byref(p), _ptr(rays), _ptr(keys), len(rays), first_dim,
                                             _ptr(out)))
        return out

    def trace_closest(self, rays: np.ndarray, t_min: float = 1e-11, t_max: float = float("inf")) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        out = (NeHit * len(rays))()
        self.ctx.check(library().ne_trace_closest(self._h, _ptr(rays), len(rays), t_min, t_max, C.addressof(out)))
        return hits_to_numpy(out)

    def close(self):
        if self._h and self.ctx._h:
            library().ne_scene_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


HIT_DTYPE = np.dtype([("t_near", np.float32), ("t_far", np.float32), ("point", np.float32, 3),
                      ("normal", np.float32, 3), ("instance", np.int32), ("primitive", np.int32),
                      ("hit", np.int32), ("pad", np.int32)])


def hits_to_numpy(arr) -> np.ndarray:
    buf = (C.c_char * C.sizeof(arr)).from_address(C.addressof(arr))
    return np.frombuffer(bytes(buf), dtype=HIT_DTYPE).copy()


# ---------------------------------------------------------------- output stage
def camera_look_at(position, look_at, vfov: float, width: int, height: int, focus: float = 3.0) -> "_abi.NeCamera":
    """Camera::Camera as SceneReader sets it up (focus 3 = the reference's autoFocus)."""
    pos = np.ascontiguousarray(position, np.float32)
    la = np.ascontiguousarray(look_at, np.float32)
    cam = _abi.NeCamera()
    st = library().ne_camera_look_at(_ptr(pos), _ptr(la), vfov, width, height, focus, C.byref(cam))
    if st != 0:
        raise NarvalError(st, "ne_camera_look_at: invalid arguments")
    return cam


class Views:
    """A batch of views rendered by one persistent launch (ne_views)."""

    def __init__(self, scene: "Scene", views: list, params: NeRenderParams | None = None, **kw):
        """views: list of (camera, width, height, spp)."""
        self.scene = scene
        self.ctx = scene.ctx
        arr = (_abi.NeView * len(views))()
        for i, (cam, w, h, spp) in enumerate(views):
            arr[i].camera = cam
            arr[i].width, arr[i].height, arr[i].spp = w, h, spp
        self.sizes = [(w, h, spp) for _, w, h, spp in views]
        p = params if params is not None else render_params(**kw)
        hnd = C.c_void_p()
        self.ctx.check(library().ne_views_create(scene._h, arr, len(views), C.byref(p), C.byref(hnd)))
        self._h = hnd

    def set_tuning(self, fetch: int = 32, blocks_per_sm: int = 0, order: int = 0, graph: bool = True,
                   split_passes: int = 0, split_half: int = 0, groups: int = 1, pretrace: int = 0):
        t = _abi.NeViewsTuning(fetch, blocks_per_sm, order, int(graph), split_passes, split_half, groups, pretrace)
        self.ctx.check(library().ne_views_set_tuning(self._h, C.byref(t)))

    def tuning(self) -> dict:
        t = _abi.NeViewsTuning()
        self.ctx.check(library().ne_views_get_tuning(self._h, C.byref(t)))
        return {f: getattr(t, f) for f, _ in t._fields_}

    def autotune(self, repeats: int = 1):
        t = _abi.NeViewsTuning()
        ms = C.c_double()
        self.ctx.check(library().ne_views_autotune(self._h, repeats, C.byref(t), C.byref(ms)))
        return {f: getattr(t, f) for f, _ in t._fields_}, ms.value

    def render(self) -> dict:
        s = _abi.NeViewsStats()
        self.ctx.check(library().ne_views_render(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def latency(self) -> np.ndarray:
        out = np.empty(len(self.sizes), np.float32)
        self.ctx.check(library().ne_views_latency(self._h, _ptr(out)))
        return out

    def image(self, v: int) -> np.ndarray:
        if not 0 <= v < len(self.sizes):
            raise NarvalError(_abi.NE_ERR_INVALID_ARG, f"view {v} out of range (0..{len(self.sizes) - 1})")
        w, h, _ = self.sizes[v]
        out = np.empty((h, w, 3), np.float32)
        self.ctx.check(library().ne_views_image(self._h, v, _ptr(out)))
        return out

    def close(self):
        if self._h and self.scene._h:
            library().ne_views_destroy(self._h)
        self._h = None


class RadianceCache:
    """The learned radiance cache (ne_cache): a 96 -> 4x64 -> RGB network on the tensor cores."""

    N_PARAMS = 19728

    def __init__(self, ctx: Context, seed: int = 0):
        self.ctx = ctx
        h = C.c_void_p()
        ctx.check(library().ne_cache_create(ctx._h, seed, C.byref(h)))
        self._h = h

    def set_params(self, params: np.ndarray):
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != self.N_PARAMS:
            raise ValueError(f"expected {self.N_PARAMS} parameters")
        self.ctx.check(library().ne_cache_set_params(self._h, _ptr(p)))

    def params(self) -> np.ndarray:
        p = np.empty(self.N_PARAMS, np.float32)
        self.ctx.check(library().ne_cache_get_params(self._h, _ptr(p)))
        return p

    def encode(self, pos: np.ndarray, dirs: np.ndarray) -> np.ndarray:
        pos = np.ascontiguousarray(pos, np.float32)
        dirs = np.ascontiguousarray(dirs, np.float32)
        f = np.empty((len(pos), 96), np.float32)
        self.ctx.check(library().ne_cache_encode(self._h, _ptr(pos), _ptr(dirs), len(pos), _ptr(f)))
        return f

    def infer(self, pos=None, dirs=None, feats=None) -> np.ndarray:
        args, n = self._inputs(pos, dirs, feats)
        out = np.empty((n, 3), np.float32)
        self.ctx.check(library().ne_cache_infer(self._h, *args, n, _ptr(out), 0))
        return out

    def train(self, targets, pos=None, dirs=None, feats=None, apply: bool = True, want_grads: bool = False):
        """One training step; returns (mean loss, summed gradient or None)."""
        args, n = self._inputs(pos, dirs, feats)
        t = np.ascontiguousarray(targets, np.float32)
        loss = C.c_float()
        g = np.empty(self.N_PARAMS, np.float32) if want_grads else None
        self.ctx.check(library().ne_cache_train(self._h, *args, _ptr(t), n, int(apply), C.byref(loss),
                                                _ptr(g) if g is not None else None, 0))
        return loss.value, g

    def _inputs(self, pos, dirs, feats):
        if feats is not None:
            self._keep = np.ascontiguousarray(feats, np.float32)
            return (None, None, _ptr(self._keep)), len(self._keep)
        self._keep = (np.ascontiguousarray(pos, np.float32), np.ascontiguousarray(dirs, np.float32))
        return (_ptr(self._keep[0]), _ptr(self._keep[1]), None), len(self._keep[0])

    def close(self):
        if self._h and self.ctx._h:
            library().ne_cache_destroy(self._h)
        self._h = None


def save_image(path: str, rgb: np.ndarray) -> None:
    """saveImage (materials/Texture.h:44-75): PNG (clamped to [0, 1], 8 bits) or EXR (FP32) by
    the file extension; rgb is an (H, W, 3) float image."""
    img = np.ascontiguousarray(rgb, dtype=np.float32)
    h, w = img.shape[:2]
    if path.lower().endswith(".png"):
        st = library().ne_save_png(path.encode(), _ptr(img), w, h)
    elif path.lower().endswith(".exr"):
        st = library().ne_save_exr(path.encode(), _ptr(img), w, h)
    else:
        raise ValueError("save_image writes .png or .exr")
    if st != 0:
        raise NarvalError(st, f"cannot write {path}")


def load_image(path: str) -> np.ndarray:
    """ne_image_load_rgba8: the (H, W, 4) uint8 texels a texture file gives the reference's
    loader (stbi_load with four channels; PNG and binary PNM)."""
    w, h = C.c_int32(), C.c_int32()
    st = library().ne_image_load_rgba8(path.encode(), C.byref(w), C.byref(h), None, 0)
    if st != 0:
        raise NarvalError(st, f"cannot decode {path}")
    out = np.empty((h.value, w.value, 4), np.uint8)
    st = library().ne_image_load_rgba8(path.encode(), C.byref(w), C.byref(h), out.ctypes.data, out.nbytes)
    if st != 0:
        raise NarvalError(st, f"cannot decode {path}")
    return out


def tone_map(hdr: np.ndarray) -> np.ndarray:
    """OfflineEngine::postProcessing (core/OfflineEngine.cpp:39-52): exposure 0.5, gamma 2.2, clamp."""
    mapped = np.float32(1.0) - np.exp(-hdr.astype(np.float32) * np.float32(0.5))
    mapped = np.power(mapped, np.float32(1.0 / 2.2))
    return np.clip(mapped, 0.0, 1.0).astype(np.float32)


def write_ppm(path: str, ldr: np.ndarray) -> None:
    """16-bit P6 in the reference's order: pixels written from the last to the first
    (core/OfflineEngine.cpp:80-138), each channel truncated to uint16 big-endian."""
    H, W, _ = ldr.shape
    flat = ldr.reshape(-1, 3)[::-1]
    vals = (np.nan_to_num(flat, nan=0.0) * np.float32(65535)).astype(np.uint16)  # a NaN pixel as 0
    with open(path, "wb") as f:
        f.write(f"P6\n{W} {H}\n65535\n".encode())
        f.write(vals.astype(">u2").tobytes())


# ---------------------------------------------------------------- reference-shaped interface
class SceneReader:
    """io/SceneReader.h:51-54: loadScene(path) then getScene/getMainCamera/getSettings."""

    def __init__(self, path: str | None = None, resources_dir: str | None = None):
        self.host = None
        if path:
            self.loadScene(path, resources_dir)

    def loadScene(self, path: str, resources_dir: str | None = None):
        self.host = SceneHost.from_json(path, resources_dir)

    def getScene(self) -> SceneHost:
        return self.host

    def getMainCamera(self) -> dict:
        return self.host.camera_dict()

    def getSettings(self) -> dict:
        s = self.host.desc.settings
        return {"resolution": (s.width, s.height), "spp": s.spp, "bounces": s.bounces, "hdr": bool(s.hdr)}


class VolumetricPathIntegrator:
    """integrators/VolumetricPathIntegrator.h: Li(ray, scene) on the GPU, batched."""

    def __init__(self, scene: Scene, seed: int = 0):
        self.scene = scene
        self.seed = seed

    def Li(self, rays: np.ndarray, keys: np.ndarray, first_dim: int = 0) -> np.ndarray:
        return self.scene.li_batch(rays, keys, first_dim, seed=self.seed)

    def clone(self) -> "VolumetricPathIntegrator":
        return VolumetricPathIntegrator(self.scene, self.seed)


class OfflineEngine:
    """core/OfflineEngine.h:23-47: renders the scene's settings and writes output.ppm."""

    def __init__(self, scene: Scene, seed: int = 0, ref_tiles: bool = True):
        self.scene = scene
        self.seed = seed
        self.ref_tiles = ref_tiles
        self.pixels = None

    def coreLoop(self, path: str = "output.ppm") -> dict:
        flags = NE_RENDER_REF_TILES if self.ref_tiles else 0
        hdr, stats = self.scene.render(seed=self.seed, flags=flags)
        self.pixels = tone_map(hdr)
        write_ppm(path, self.pixels)
        return stats


__all__ = ["Context", "Scene", "SceneHost", "SceneReader", "VolumetricPathIntegrator", "OfflineEngine",
           "NarvalError", "render_params", "tone_map", "write_ppm", "load_image", "library", "SCENES_DIR",
           "NE_RENDER_OUT_DEVICE", "NE_RENDER_REF_TILES", "NE_RENDER_COUNT_WORK", "NE_RENDER_NO_SYNC",
           "NeRay", "NePathKey"]
