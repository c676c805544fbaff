"""ctypes mirror of include/crg.h (plain structs and the entry-point signatures).

Only plumbing: every byte of work happens in libcrg.so.  The struct layouts are
checked against the C header sizes by tests/test_abi.py.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

c_stream = C.c_void_p


class Ray(C.Structure):
    _fields_ = [("org", C.c_float * 3), ("tmin", C.c_float), ("dir", C.c_float * 3), ("tmax", C.c_float)]


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("prim", C.c_uint32), ("u", C.c_float), ("v", C.c_float)]


class Material(C.Structure):
    _fields_ = [
        ("shade_type", C.c_uint32),
        ("ior", C.c_float),
        ("roughness", C.c_float),
        ("reflectiveness", C.c_float),
        ("emission", C.c_float),
        ("colour", C.c_float * 4),
        ("tex", C.c_int32),
        ("pad_", C.c_uint32 * 2),
    ]


class Sun(C.Structure):
    _fields_ = [("size", C.c_float), ("intensity", C.c_float), ("direction", C.c_float * 3), ("colour", C.c_float * 3)]


class Camera(C.Structure):
    _fields_ = [
        ("position", C.c_float * 3),
        ("rotation", C.c_float * 3),
        ("fov", C.c_float),
        ("mode", C.c_uint32),
        ("scale", C.c_float),
        ("pad_", C.c_uint32),
    ]


class Settings(C.Structure):
    _fields_ = [
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("spp", C.c_uint32),
        ("max_bounces", C.c_uint32),
        ("rr_depth", C.c_uint32),
        ("mode", C.c_uint32),
        ("seed", C.c_uint32),
        ("aspect", C.c_float),
    ]


class BuildOpts(C.Structure):
    _fields_ = [("width", C.c_uint32), ("treelet", C.c_uint32), ("leaf_max", C.c_uint32), ("treelet_rounds", C.c_uint32)]


class BvhInfo(C.Structure):
    _fields_ = [
        ("ntri", C.c_uint32),
        ("width", C.c_uint32),
        ("n_bvh2_nodes", C.c_uint32),
        ("n_wide_nodes", C.c_uint32),
        ("node_bytes", C.c_uint32),
        ("n_tri_slots", C.c_uint32),
        ("depth", C.c_uint32),
        ("sah_cost", C.c_float),
        ("leaf_max", C.c_uint32),
        ("treelet", C.c_uint32),
    ]


class StageTimes(C.Structure):
    _fields_ = [("extend_ms", C.c_double), ("shade_ms", C.c_double), ("shadow_ms", C.c_double), ("other_ms", C.c_double),
                ("iterations", C.c_uint64), ("shadow_nodes", C.c_uint64), ("shadow_tris", C.c_uint64)]


class ModelInfo(C.Structure):
    _fields_ = [
        ("first_prim", C.c_uint32),
        ("ntri", C.c_uint32),
        ("node_base", C.c_uint32),
        ("n_wide_nodes", C.c_uint32),
        ("depth", C.c_uint32),
        ("ninst", C.c_uint32),
        ("built", C.c_uint32),
        ("sah_cost", C.c_float),
    ]


class View(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("pad_", C.c_uint32), ("camera", Camera), ("settings", Settings)]


class WavefrontOpts(C.Structure):
    _fields_ = [("path_pool", C.c_uint32), ("chunk_samples", C.c_uint32), ("block_size", C.c_uint32),
                ("fetch", C.c_uint32), ("max_iterations", C.c_uint32), ("count_work", C.c_uint32),
                ("host_loop", C.c_uint32), ("fuse", C.c_uint32), ("refill", C.c_uint32)]


class AutotuneOpts(C.Structure):
    _fields_ = [("sample_budget", C.c_uint64), ("widths", C.c_uint32), ("reuse", C.c_uint32), ("leaves", C.c_uint32),
                ("pad_", C.c_uint32)]


class AutotuneTrial(C.Structure):
    _fields_ = [("opts", WavefrontOpts), ("width", C.c_uint32), ("ms", C.c_float), ("msamples_per_s", C.c_float),
                ("pad_", C.c_uint32)]


class RenderStats(C.Structure):
    _fields_ = [("samples", C.c_uint64), ("segments", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("nodes_visited", C.c_uint64), ("tris_tested", C.c_uint64), ("iterations", C.c_uint64)]


class PostSettings(C.Structure):
    _fields_ = [("bloom", C.c_uint32), ("bloom_threshold", C.c_float), ("bloom_strength", C.c_float),
                ("gray_scale", C.c_uint32), ("tonemapping", C.c_uint32), ("tonemap_type", C.c_int32),
                ("exposure", C.c_float), ("gamma", C.c_float), ("mode", C.c_uint32), ("pad_", C.c_uint32)]


# numpy views of the same layouts
RAY_DTYPE = np.dtype([("org", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("prim", "<u4"), ("u", "<f4"), ("v", "<f4")])
MATERIAL_DTYPE = np.dtype(
    [
        ("shade_type", "<u4"),
        ("ior", "<f4"),
        ("roughness", "<f4"),
        ("reflectiveness", "<f4"),
        ("emission", "<f4"),
        ("colour", "<f4", 4),
        ("tex", "<i4"),
        ("pad_", "<u4", 2),
    ]
)
assert RAY_DTYPE.itemsize == 32 and HIT_DTYPE.itemsize == 16 and MATERIAL_DTYPE.itemsize == 48

SHADE_METAL, SHADE_SMOOTH, SHADE_GLASS = 0, 1, 2
MODE_FAITHFUL, MODE_EXTENDED = 0, 1
CAMERA_PERSPECTIVE, CAMERA_ORTHOGRAPHIC = 0, 1
FILM_F64, FILM_AOV = 1, 2
TONEMAP_LINEAR, TONEMAP_REINHARD, TONEMAP_JIM_RICHARD, TONEMAP_UNCHARTED = 0, 1, 2, 3
POST_FAITHFUL, POST_FULL = 0, 1
INVALID_PRIM = 0xFFFFFFFF
TRAVERSAL_THREAD, TRAVERSAL_WARP = 0, 1  # crg_traversal
NOALLOC_MAX_TRIS = 16384

STATUS = {
    0: "OK",
    1: "INVALID_ARG",
    2: "OOM",
    3: "CUDA",
    4: "TIMEOUT",
    5: "NOT_BUILT",
    6: "UNSUPPORTED",
    7: "DEVICE",
}

P = C.POINTER
vp = C.c_void_p

# (name, restype, argtypes) of every exported entry point in include/crg.h
CRG_SIGNATURES = [
    ("crg_context_create", C.c_int, [C.c_int, P(vp)]),
    ("crg_context_destroy", C.c_int, [vp]),
    ("crg_last_error_string", C.c_char_p, [vp]),
    ("crg_status_string", C.c_char_p, [C.c_int]),
    ("crg_abi_version", C.c_uint32, []),
    ("crg_debug_fail_allocation", C.c_int, [C.c_int64]),
    ("crg_debug_allocation_stats", C.c_int, [P(C.c_uint64), P(C.c_uint32), P(C.c_int64)]),
    ("crg_device_alloc", C.c_int, [vp, C.c_size_t, P(vp)]),
    ("crg_device_free", C.c_int, [vp, vp]),
    ("crg_memcpy_h2d", C.c_int, [vp, vp, vp, C.c_size_t, c_stream]),
    ("crg_memcpy_d2h", C.c_int, [vp, vp, vp, C.c_size_t, c_stream]),
    ("crg_stream_sync", C.c_int, [vp, c_stream]),
    ("crg_host_alloc", C.c_int, [vp, C.c_size_t, P(vp)]),
    ("crg_host_free", C.c_int, [vp, vp]),
    ("crg_scene_create", C.c_int, [vp, vp, C.c_uint32, vp, vp, vp, C.c_uint32, P(vp)]),
    ("crg_scene_create_device", C.c_int, [vp, vp, C.c_uint32, vp, vp, C.c_uint32, P(vp)]),
    ("crg_scene_create_indexed", C.c_int, [vp, vp, C.c_uint32, vp, C.c_uint32, vp, C.c_uint32, vp, vp, vp, C.c_uint32,
                                           P(vp)]),
    ("crg_scene_destroy", C.c_int, [vp]),
    ("crg_scene_build", C.c_int, [vp, P(BuildOpts), c_stream]),
    ("crg_scene_set_skybox", C.c_int, [vp, vp, C.c_uint32, C.c_uint32, C.c_float, C.c_float]),
    ("crg_scene_set_sun", C.c_int, [vp, C.c_int, P(Sun)]),
    ("crg_scene_set_textures", C.c_int, [vp, C.c_uint32, P(vp), vp, vp]),
    ("crg_scene_set_instances", C.c_int, [vp, vp, C.c_uint32]),
    ("crg_scene_add_model", C.c_int, [vp, vp, C.c_uint32, vp, vp, vp, C.c_uint32, P(C.c_uint32)]),
    ("crg_scene_add_model_indexed", C.c_int, [vp, vp, C.c_uint32, vp, C.c_uint32, vp, C.c_uint32, vp, vp, vp,
                                              C.c_uint32, P(C.c_uint32)]),
    ("crg_scene_set_model_instances", C.c_int, [vp, C.c_uint32, vp, C.c_uint32]),
    ("crg_scene_model_count", C.c_int, [vp, P(C.c_uint32)]),
    ("crg_scene_model_info", C.c_int, [vp, C.c_uint32, P(ModelInfo)]),
    ("crg_scene_bvh_info", C.c_int, [vp, P(BvhInfo)]),
    ("crg_scene_bvh_download", C.c_int, [vp, vp, vp, vp, vp]),
    ("crg_build_bvh_noalloc", C.c_int, [vp, C.c_uint32, P(BuildOpts), vp, C.c_size_t, vp, vp, P(BvhInfo), c_stream]),
    ("crg_noalloc_last_error", C.c_char_p, []),
    ("crg_intersect_closest", C.c_int, [vp, vp, vp, C.c_uint64, c_stream]),
    ("crg_intersect_any", C.c_int, [vp, vp, vp, C.c_uint64, c_stream]),
    ("crg_intersect_closest_counted", C.c_int, [vp, vp, vp, vp, vp, C.c_uint64, c_stream]),
    ("crg_intersect_closest_with", C.c_int, [vp, vp, vp, C.c_uint64, C.c_int, c_stream]),
    ("crg_intersect_any_with", C.c_int, [vp, vp, vp, C.c_uint64, C.c_int, c_stream]),
    ("crg_scene_poll_error", C.c_int, [vp]),
    ("crg_film_create", C.c_int, [vp, C.c_uint32, C.c_uint32, C.c_uint32, P(vp)]),
    ("crg_film_destroy", C.c_int, [vp]),
    ("crg_film_reset", C.c_int, [vp, c_stream]),
    ("crg_film_spp", C.c_int, [vp, P(C.c_uint64)]),
    ("crg_film_download", C.c_int, [vp, vp, vp, vp, vp, vp, vp, c_stream]),
    ("crg_film_download_async", C.c_int, [vp, vp, vp, vp, vp, vp, vp, c_stream]),
    ("crg_film_device_ptrs", C.c_int, [vp, P(vp), P(vp), P(vp)]),
    ("crg_film_display", C.c_int, [vp, vp, c_stream]),
    ("crg_post_settings_default", C.c_int, [P(PostSettings)]),
    ("crg_post_process", C.c_int, [vp, vp, vp, C.c_uint32, C.c_uint32, P(PostSettings), c_stream]),
    ("crg_draft_render", C.c_int, [vp, P(Camera), C.c_uint32, C.c_uint32, C.c_float, vp, c_stream]),
    ("crg_render", C.c_int, [vp, P(Camera), P(Settings), vp, c_stream]),
    ("crg_scene_set_materials", C.c_int, [vp, vp, C.c_uint32]),
    ("crg_backward", C.c_int, [vp, P(Camera), P(Settings), vp, vp, vp, c_stream]),
    ("crg_film_loss_l2", C.c_int, [vp, vp, vp, vp, c_stream]),
    ("crg_render_batch", C.c_int, [P(vp), C.c_uint32, P(View), P(vp), C.c_uint32, P(WavefrontOpts), c_stream]),
    ("crg_render_batch_async", C.c_int, [P(vp), C.c_uint32, P(View), P(vp), C.c_uint32, P(WavefrontOpts), c_stream]),
    ("crg_batch_wait", C.c_int, [vp]),
    ("crg_batch_stats_get", C.c_int, [vp, P(RenderStats)]),
    ("crg_batch_stage_times_get", C.c_int, [vp, P(StageTimes)]),
    ("crg_autotune_batch", C.c_int, [P(vp), C.c_uint32, P(View), C.c_uint32, P(AutotuneOpts), P(WavefrontOpts),
                                     P(C.c_uint32), P(AutotuneTrial), C.c_uint32, P(C.c_uint32), c_stream]),
    ("crg_autotune_cache_save", C.c_int, [vp, C.c_char_p]),
    ("crg_autotune_cache_load", C.c_int, [vp, C.c_char_p, P(C.c_uint32)]),
    ("crg_render_stats_get", C.c_int, [vp, P(RenderStats)]),
    ("crg_scene_set_counting", C.c_int, [vp, C.c_int]),
]


class OrcSceneDesc(C.Structure):
    _fields_ = [
        ("verts", vp),
        ("ntri", C.c_uint32),
        ("mat_idx", vp),
        ("mats", vp),
        ("nmat", C.c_uint32),
        ("skybox", vp),
        ("sky_w", C.c_uint32),
        ("sky_h", C.c_uint32),
        ("sky_rot_u", C.c_float),
        ("sky_rot_v", C.c_float),
        ("sun_enabled", C.c_int),
        ("sun", Sun),
        ("build", P(BuildOpts)),
        ("uvs", vp),
        ("ntex", C.c_uint32),
        ("tex_rgba", P(vp)),
        ("tex_w", vp),
        ("tex_h", vp),
        ("xforms", vp),
        ("ninst", C.c_uint32),
        ("nmodels", C.c_uint32),
        ("model_ntri", vp),
        ("model_ninst", vp),
    ]


class OrcFilm(C.Structure):
    _fields_ = [
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("sum_rgb", vp),
        ("sum64", vp),
        ("sumsq64", vp),
        ("aov_albedo", vp),
        ("aov_normal", vp),
        ("aov_depth", vp),
        ("spp", C.c_uint64),
        ("segments", C.c_uint64),
        ("shadow_rays", C.c_uint64),
        ("render_seconds", C.c_double),
    ]


ORC_SIGNATURES = [
    ("orc_bvh_build", C.c_int, [vp, C.c_uint32, P(BuildOpts), P(vp)]),
    ("orc_bvh_free", None, [vp]),
    ("orc_bvh_info", None, [vp, P(BvhInfo)]),
    ("orc_bvh_download", None, [vp, vp, vp, vp, vp]),
    ("orc_intersect_closest", None, [vp, vp, vp, C.c_uint64, C.c_int]),
    ("orc_intersect_any", None, [vp, vp, vp, C.c_uint64, C.c_int]),
    ("orc_intersect_closest_brute", None, [vp, C.c_uint32, vp, vp, C.c_uint64]),
    ("orc_intersect_closest_f64", None, [vp, C.c_uint32, vp, vp, vp, vp, C.c_uint64]),
    ("orc_render", C.c_int, [P(OrcSceneDesc), P(Camera), P(Settings), P(OrcFilm), C.c_int]),
    ("orc_render_rows", C.c_int, [P(OrcSceneDesc), P(Camera), P(Settings), P(OrcFilm), C.c_uint32, C.c_uint32, C.c_int]),
    ("orc_adjoint", C.c_int, [P(OrcSceneDesc), P(Camera), P(Settings), vp, vp, vp, C.c_int]),
    ("orc_post_process", C.c_int, [vp, vp, C.c_uint32, C.c_uint32, P(PostSettings)]),
    ("orc_scene_intersect", C.c_int, [P(OrcSceneDesc), vp, vp, vp, C.c_uint64]),
    ("orc_draft_render", C.c_int, [P(OrcSceneDesc), P(Camera), C.c_uint32, C.c_uint32, C.c_float, vp]),
    ("orc_alias_table", None, [vp, C.c_uint32, vp, vp]),
    ("orc_camera_ray", None, [P(Camera), P(Settings), C.c_uint32, C.c_uint32, C.c_float, C.c_float, vp, vp]),
    ("orc_sincos2pi", None, [C.c_float, P(C.c_float), P(C.c_float)]),
    ("orc_rand4", None, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, vp]),
    ("orc_morton3", C.c_uint32, [C.c_float, C.c_float, C.c_float]),
    ("orc_sample_sphere", None, [C.c_float, C.c_float, vp]),
    ("orc_build_local", None, [vp, vp, vp]),
    ("orc_ggx_d", C.c_float, [C.c_float, C.c_float]),
    ("orc_ggx_lambda", C.c_float, [vp, C.c_float]),
    ("orc_sample_vndf", None, [vp, C.c_float, C.c_float, C.c_float, vp]),
    ("orc_fresnel_dielectric", C.c_float, [C.c_float, C.c_float]),
    ("orc_sun_sample", None, [P(Sun), vp, C.c_float, C.c_float, vp, vp, vp]),
    ("orc_sun_visible", C.c_int, [P(Sun), vp]),
    ("orc_cos_hemp", None, [C.c_float, C.c_float, vp]),
]


def bind(lib: C.CDLL, sigs) -> C.CDLL:
    for name, res, args in sigs:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def ptr(a: np.ndarray | None):
    """Host address of a C-contiguous numpy array (None -> NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data
