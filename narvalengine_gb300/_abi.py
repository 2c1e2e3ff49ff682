"""ctypes mirror of include/narval_scene.h and include/narval_gb300.h."""
from __future__ import annotations

import ctypes as C

f3 = C.c_float * 3


class NePrimitive(C.Structure):
    _fields_ = [("type", C.c_int32), ("material", C.c_int32), ("p0", f3), ("p1", f3), ("p2", f3),
                ("radius", C.c_float), ("area", C.c_float)]


class NeModel(C.Structure):
    _fields_ = [("prim_begin", C.c_uint32), ("prim_count", C.c_uint32), ("light_begin", C.c_uint32),
                ("light_count", C.c_uint32), ("mat_begin", C.c_uint32), ("mat_count", C.c_uint32),
                ("has_bbox", C.c_int32), ("bbox_min", f3), ("bbox_max", f3), ("use_bvh", C.c_int32)]


class NeInstance(C.Structure):
    _fields_ = [("to_wcs", C.c_float * 16), ("to_ocs", C.c_float * 16), ("model", C.c_uint32),
                ("collision", C.c_int32)]


class NeMaterial(C.Structure):
    _fields_ = [("bsdf", C.c_int32), ("light", C.c_int32), ("medium", C.c_int32), ("phase", C.c_int32),
                ("g", C.c_float), ("albedo", f3), ("roughness", C.c_float), ("metallic", C.c_float),
                ("normal_map", f3), ("tex_present", C.c_int32), ("tex_types", C.c_int32),
                ("albedo_width", C.c_int32), ("albedo_height", C.c_int32), ("albedo_texels", C.POINTER(C.c_uint8))]


class NeLight(C.Structure):
    _fields_ = [("type", C.c_int32), ("primitive", C.c_int32), ("li", f3), ("le", f3), ("direction", f3),
                ("env_radiance", f3), ("env_map_pdf", C.c_float), ("env_width", C.c_int32),
                ("env_height", C.c_int32), ("env_texels", C.POINTER(C.c_uint8))]


class NeMedium(C.Structure):
    _fields_ = [("type", C.c_int32), ("sigma_s", f3), ("sigma_a", f3), ("density", C.c_float),
                ("res", C.c_uint32 * 3), ("grid", C.POINTER(C.c_float))]


class NeCamera(C.Structure):
    _fields_ = [("position", f3), ("lower_left", f3), ("horizontal", f3), ("vertical", f3), ("side", f3),
                ("up", f3), ("lens_radius", C.c_float)]


class NeSettings(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("bounces", C.c_int32),
                ("hdr", C.c_int32), ("rr_enabled", C.c_int32), ("rr_after", C.c_int32), ("bvh_build", C.c_int32)]


class NeSceneDesc(C.Structure):
    _fields_ = [("n_instances", C.c_uint32), ("n_light_instances", C.c_uint32),
                ("instances", C.POINTER(NeInstance)),
                ("n_models", C.c_uint32), ("models", C.POINTER(NeModel)),
                ("n_prims", C.c_uint32), ("prims", C.POINTER(NePrimitive)),
                ("n_materials", C.c_uint32), ("materials", C.POINTER(NeMaterial)),
                ("n_model_materials", C.c_uint32), ("model_materials", C.POINTER(C.c_uint32)),
                ("n_lights", C.c_uint32), ("lights", C.POINTER(NeLight)),
                ("n_media", C.c_uint32), ("media", C.POINTER(NeMedium)),
                ("camera", NeCamera), ("settings", NeSettings)]


class NeRay(C.Structure):
    _fields_ = [("o", f3), ("d", f3)]


class NePathKey(C.Structure):
    _fields_ = [("pixel", C.c_uint32), ("sample", C.c_uint32)]


class NeHit(C.Structure):
    _fields_ = [("t_near", C.c_float), ("t_far", C.c_float), ("point", f3), ("normal", f3),
                ("instance", C.c_int32), ("primitive", C.c_int32), ("hit", C.c_int32), ("pad", C.c_int32)]


class NeRenderParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("spp", C.c_int32), ("bounces", C.c_int32), ("rr", C.c_int32),
                ("rr_after", C.c_int32), ("sample_offset", C.c_uint32), ("flags", C.c_uint32)]


class NeTuning(C.Structure):
    _fields_ = [("kernel", C.c_int32), ("track_share", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("split_passes", C.c_int32), ("split_half", C.c_int32), ("queue_quarters", C.c_int32),
                ("pretrace", C.c_int32)]


class NeRenderStats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("total_ms", C.c_double), ("paths", C.c_uint64),
                ("density_lookups", C.c_uint64), ("scene_queries", C.c_uint64), ("bvh_nodes", C.c_uint64),
                ("prim_tests", C.c_uint64), ("kernel_launches", C.c_uint32), ("dropped_paths", C.c_uint32)]


class NeView(C.Structure):
    _fields_ = [("camera", NeCamera), ("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32),
                ("pad", C.c_int32)]


class NeViewsTuning(C.Structure):
    _fields_ = [("fetch", C.c_uint32), ("blocks_per_sm", C.c_int32), ("order", C.c_int32), ("graph", C.c_int32),
                ("split_passes", C.c_int32), ("split_half", C.c_int32), ("groups", C.c_int32),
                ("pretrace", C.c_int32)]


class NeViewsStats(C.Structure):
    _fields_ = [("ms", C.c_double), ("paths", C.c_uint64), ("latency_p50_ms", C.c_float),
                ("latency_p99_ms", C.c_float), ("latency_max_ms", C.c_float), ("kernel_launches", C.c_uint32)]


class NeCacheRenderParams(C.Structure):
    _fields_ = [("bounce", C.c_int32), ("train_stride", C.c_uint32), ("train_steps", C.c_int32),
                ("train_batch", C.c_uint32), ("train_suffix", C.c_int32)]


class NeCacheRenderStats(C.Structure):
    _fields_ = [("queries", C.c_uint64), ("train_samples", C.c_uint64), ("loss", C.c_float), ("path_ms", C.c_float),
                ("infer_ms", C.c_float), ("train_ms", C.c_float)]


# status codes
NE_OK = 0
NE_ERR_INVALID_ARG = -1
NE_ERR_PARSE = -2
NE_ERR_MISSING_ASSET = -3
NE_ERR_CUDA = -4
NE_ERR_TIMEOUT = -5
NE_ERR_UNSUPPORTED = -6
NE_ERR_NO_DEVICE = -7
NE_ERR_OUT_OF_MEMORY = -8

# render flags
NE_RENDER_OUT_DEVICE = 1 << 0
NE_RENDER_REF_TILES = 1 << 1
NE_RENDER_COUNT_WORK = 1 << 2
NE_RENDER_NO_SYNC = 1 << 3
NE_RENDER_DROP_NONFINITE = 1 << 4

# radiance cache
NE_CACHE_PARAMS = 19728
NE_CACHE_DEVICE_PTRS = 1 << 0

# every symbol include/narval_gb300.h declares, with its ctypes signature
SIGNATURES = {
    "ne_scene_host_load_json": (C.c_int32, [C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]),
    "ne_scene_host_load_json_string": (C.c_int32, [C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p), C.c_char_p,
                                                   C.c_size_t]),
    "ne_scene_host_desc": (C.POINTER(NeSceneDesc), [C.c_void_p]),
    "ne_scene_host_destroy": (None, [C.c_void_p]),
    "ne_context_create": (C.c_int32, [C.c_int, C.POINTER(C.c_void_p)]),
    "ne_context_destroy": (None, [C.c_void_p]),
    "ne_last_error": (C.c_char_p, [C.c_void_p]),
    "ne_scene_upload": (C.c_int32, [C.c_void_p, C.POINTER(NeSceneDesc), C.POINTER(C.c_void_p)]),
    "ne_scene_destroy": (None, [C.c_void_p]),
    "ne_render": (C.c_int32, [C.c_void_p, C.POINTER(NeRenderParams), C.c_void_p, C.POINTER(NeRenderStats)]),
    "ne_render_noalloc": (C.c_int32, [C.c_void_p, C.POINTER(NeRenderParams), C.c_void_p, C.POINTER(NeRenderStats)]),
    "ne_render_accumulate": (C.c_int32, [C.c_void_p, C.POINTER(NeRenderParams), C.c_void_p,
                                         C.POINTER(NeRenderStats)]),
    "ne_trace_paths": (C.c_int32, [C.c_void_p, C.POINTER(NeRenderParams), C.c_void_p, C.c_size_t, C.c_void_p]),
    "ne_li_batch": (C.c_int32, [C.c_void_p, C.POINTER(NeRenderParams), C.c_void_p, C.c_void_p, C.c_size_t,
                                C.c_uint32, C.c_void_p]),
    "ne_trace_closest": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_float, C.c_float, C.c_void_p]),
    "ne_scene_set_tuning": (C.c_int32, [C.c_void_p, C.POINTER(NeTuning)]),
    "ne_scene_get_tuning": (C.c_int32, [C.c_void_p, C.POINTER(NeTuning)]),
    "ne_context_event_record": (C.c_int32, [C.c_void_p, C.c_int]),
    "ne_context_event_elapsed": (C.c_int32, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "ne_context_synchronize": (C.c_int32, [C.c_void_p]),
    "ne_context_flush_l2": (C.c_int32, [C.c_void_p, C.c_size_t]),
    "ne_context_set_cache_limit": (C.c_int32, [C.c_void_p, C.c_size_t]),
    "ne_measure_read_bandwidth": (C.c_int32, [C.c_void_p, C.c_size_t, C.c_int, C.POINTER(C.c_double)]),
    "ne_measure_random_read": (C.c_int32, [C.c_void_p, C.c_size_t, C.c_int, C.POINTER(C.c_double)]),
    "ne_debug_fmath": (C.c_int32, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p]),
    "ne_debug_rng": (C.c_int32, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "ne_cache_create": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "ne_cache_destroy": (None, [C.c_void_p]),
    "ne_cache_set_params": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "ne_cache_get_params": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "ne_cache_encode": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "ne_cache_infer": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p,
                                   C.c_uint32]),
    "ne_cache_train": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_int,
                                   C.c_void_p, C.c_void_p, C.c_uint32]),
    "ne_render_cached": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(NeRenderParams),
                                     C.POINTER(NeCacheRenderParams), C.c_void_p, C.POINTER(NeRenderStats),
                                     C.POINTER(NeCacheRenderStats)]),
    "ne_scene_autotune": (C.c_int32, [C.c_void_p, C.POINTER(NeRenderParams), C.c_int, C.POINTER(NeTuning),
                                      C.POINTER(C.c_double)]),
    "ne_camera_look_at": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_float, C.c_int, C.c_int, C.c_float,
                                      C.POINTER(NeCamera)]),
    "ne_views_create": (C.c_int32, [C.c_void_p, C.POINTER(NeView), C.c_uint32, C.POINTER(NeRenderParams),
                                    C.POINTER(C.c_void_p)]),
    "ne_views_destroy": (None, [C.c_void_p]),
    "ne_views_set_tuning": (C.c_int32, [C.c_void_p, C.POINTER(NeViewsTuning)]),
    "ne_views_get_tuning": (C.c_int32, [C.c_void_p, C.POINTER(NeViewsTuning)]),
    "ne_views_autotune": (C.c_int32, [C.c_void_p, C.c_int, C.POINTER(NeViewsTuning), C.POINTER(C.c_double)]),
    "ne_views_render": (C.c_int32, [C.c_void_p, C.POINTER(NeViewsStats)]),
    "ne_views_latency": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "ne_views_image": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "ne_debug_bvh": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_size_t, C.c_void_p,
                                 C.POINTER(C.c_size_t)]),
    "ne_debug_medium_boxes": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_int32)]),
    "ne_scene_bvh": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_size_t, C.c_void_p, C.POINTER(C.c_size_t)]),
    "ne_save_png": (C.c_int32, [C.c_char_p, C.c_void_p, C.c_int, C.c_int]),
    "ne_save_exr": (C.c_int32, [C.c_char_p, C.c_void_p, C.c_int, C.c_int]),
    "ne_image_load_rgba8": (C.c_int32, [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p,
                                        C.c_size_t]),
    "ne_debug_mma": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "ne_debug_mma_layout": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_uint32,
                                        C.c_void_p]),
    "ne_debug_wait_timeout": (C.c_int32, [C.c_void_p, C.c_uint32]),
}
