"""ctypes binding of libkrr_gb300.so (the C ABI declared in include/krr_gb300.h).

There is no fallback: if the shared library is missing or does not load,
importing the package's GPU entry points raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libkrr_gb300.so"

KRR_OK = 0
KRR_MISS = 0xFFFFFFFF
NOALLOC_MAX_RAYS = 65536

MATERIAL_NULL, MATERIAL_DIFFUSE, MATERIAL_DIELECTRIC, MATERIAL_CONDUCTOR = 0, 1, 2, 3
QUEUES = ["RAY0", "RAY1", "MISS", "HIT_LIGHT", "SHADOW", "SCATTER", "MEDIUM_SAMPLE",
          "MEDIUM_SCATTER"]


class MaterialDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("diffuse", C.c_float * 3), ("specular", C.c_float * 3),
                ("roughness", C.c_float), ("specular_transmission", C.c_float),
                ("eta", C.c_float), ("anisotropic", C.c_float)]


class MeshDesc(C.Structure):
    _fields_ = [("h_positions", C.c_void_p), ("h_normals", C.c_void_p),
                ("h_texcoords", C.c_void_p), ("h_indices", C.c_void_p),
                ("n_vertices", C.c_int64), ("n_triangles", C.c_int64),
                ("material", C.c_int32), ("emission", C.c_float * 3),
                ("medium_inside", C.c_int32), ("medium_outside", C.c_int32)]


class InstanceDesc(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("transform", C.c_float * 12)]


class InfiniteLightDesc(C.Structure):
    _fields_ = [("tint", C.c_float * 3), ("scale", C.c_float), ("rotation", C.c_float * 9),
                ("h_image", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32)]


class MediumDesc(C.Structure):
    _fields_ = [("h_density", C.c_void_p), ("nx", C.c_int32), ("ny", C.c_int32),
                ("nz", C.c_int32), ("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3),
                ("sigma_t", C.c_float * 3), ("albedo", C.c_float * 3), ("g", C.c_float),
                ("scale", C.c_float), ("majorant_res", C.c_int32 * 3)]


class CameraDesc(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("rotation", C.c_float * 9),
                ("film_size", C.c_float * 2), ("focal_length", C.c_float),
                ("focal_distance", C.c_float), ("lens_radius", C.c_float),
                ("aspect_ratio", C.c_float), ("shutter_open", C.c_float),
                ("shutter_time", C.c_float), ("medium", C.c_int32)]


class WfTuning(C.Structure):
    _fields_ = [("block", C.c_int32), ("blocks_per_sm", C.c_int32), ("wave", C.c_int64),
                ("queue_capacity", C.c_int64), ("frame_ms", C.c_float),
                ("default_frame_ms", C.c_float), ("candidates", C.c_int32),
                ("reserved", C.c_int32)]


class ViewDesc(C.Structure):
    _fields_ = [("camera", CameraDesc), ("width", C.c_int32), ("height", C.c_int32),
                ("seed", C.c_uint32), ("scene", C.c_int32)]


class SceneDesc(C.Structure):
    _fields_ = [("meshes", C.POINTER(MeshDesc)), ("n_meshes", C.c_int32),
                ("instances", C.POINTER(InstanceDesc)), ("n_instances", C.c_int32),
                ("materials", C.POINTER(MaterialDesc)), ("n_materials", C.c_int32),
                ("infinite_lights", C.POINTER(InfiniteLightDesc)), ("n_infinite_lights", C.c_int32),
                ("media", C.POINTER(MediumDesc)), ("n_media", C.c_int32)]


class AccelStats(C.Structure):
    _fields_ = [("n_triangles", C.c_int64), ("n_nodes", C.c_int64), ("max_depth", C.c_int32),
                ("reserved", C.c_int32), ("build_ms", C.c_double), ("node_bytes", C.c_double),
                ("triangle_bytes", C.c_double)]


class StageTime(C.Structure):
    _fields_ = [("name", C.c_char * 40), ("calls", C.c_int64), ("ms", C.c_double)]


class NrcConfig(C.Structure):
    _fields_ = [("n_levels", C.c_int32), ("features_per_level", C.c_int32),
                ("log2_table_size", C.c_int32), ("base_resolution", C.c_int32),
                ("max_resolution", C.c_int32), ("hidden_layers", C.c_int32),
                ("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float),
                ("epsilon", C.c_float), ("loss_scale", C.c_float), ("batch_size", C.c_int32),
                ("train_pixel_stride", C.c_int32), ("seed", C.c_uint32),
                ("scene_lo", C.c_float * 3), ("scene_hi", C.c_float * 3),
                ("tensor_cores", C.c_int32), ("termination_spread", C.c_float),
                ("ema_decay", C.c_float)]


class NrcInfo(C.Structure):
    _fields_ = [("n_params_mlp", C.c_int64), ("n_table_entries", C.c_int64),
                ("n_levels", C.c_int32), ("resolution", C.c_int32 * 16),
                ("level_offset", C.c_uint32 * 16), ("level_size", C.c_uint32 * 16),
                ("step", C.c_int64)]


class WfParams(C.Structure):
    _fields_ = [("nee", C.c_int32), ("enable_medium", C.c_int32), ("max_depth", C.c_int32),
                ("rr", C.c_float), ("enable_clamp", C.c_int32), ("clamp_max", C.c_float),
                ("spp", C.c_int32), ("seed", C.c_uint32), ("independent_samples", C.c_int32)]


# name -> (restype, argtypes); every function declared in include/krr_gb300.h
_P = C.c_void_p
_I = C.c_int
SIGNATURES = {
    "krr_last_error": (C.c_char_p, []),
    "krr_status_string": (C.c_char_p, [_I]),
    "krr_version": (_I, []),
    "krr_accel_create_from_triangles": (_I, [_P, C.c_int64, C.POINTER(_P), _P]),
    "krr_set_bvh_node_format": (_I, [C.c_int32]),
    "krr_set_bvh_max_leaf": (_I, [C.c_int32]),
    "krr_set_bvh_full_node_leaf": (_I, [C.c_int32]),
    "krr_wf_group_create": (_I, [C.POINTER(_P), C.POINTER(_P), C.c_int32, C.POINTER(_P)]),
    "krr_wf_group_capture": (_I, [_P, _P]),
    "krr_wf_group_launch": (_I, [_P, C.c_int64, _P]),
    "krr_wf_group_destroy": (_I, [_P]),
    "krr_wf_update_instances": (_I, [_P, C.c_int32, _P, _P, _P]),
    "krr_wf_rebuild_bvh": (_I, [_P, _P]),
    "krr_tonemap": (_I, [_P, _P, C.c_int64, C.c_int32, C.c_float, C.c_int32, _P]),
    "krr_wf_render_megakernel": (_I, [_P, _P, _P]),
    "krr_wf_queue_view": (_I, [_P, C.c_int32, C.POINTER(_P), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "krr_accel_stats_get": (_I, [_P, C.POINTER(AccelStats)]),
    "krr_accel_destroy": (_I, [_P]),
    "krr_accel_refit_triangles": (_I, [_P, _P, C.c_int64, _P]),
    "krr_accel_trace_closest": (_I, [_P, _P, C.c_int64, _P, _P]),
    "krr_accel_trace_any": (_I, [_P, _P, C.c_int64, _P, _P]),
    "krr_accel_set_mask": (_I, [_P, _P]),
    "krr_accel_trace_closest_host": (_I, [_P, _P, C.c_int64, _P, _P]),
    "krr_accel_set_tuning": (_I, [_P, C.c_int32, C.c_int32]),
    "krr_set_bvh_builder": (_I, [C.c_int32]),
    "krr_set_bvh_collapse": (_I, [C.c_int32]),
    "krr_set_bvh_treelets": (_I, [C.c_int32]),
    "krr_accel_set_stack_limit": (_I, [_P, C.c_int32]),
    "krr_accel_create_instanced": (_I, [_P, _P, C.c_int32, _P, C.c_int32, _P, C.POINTER(_P), _P]),
    "krr_accel_update_instances": (_I, [_P, _P, _P]),
    "krr_accel_instance_inverse": (_I, [_P, _P, C.c_int32]),
    "krr_accel_device_errors": (_I, [_P, C.POINTER(C.c_uint32), _P]),
    "krr_accel_autotune": (_I, [_P, _P, C.c_int64, C.c_int32, C.POINTER(C.c_int32),
                                C.POINTER(C.c_int32), C.POINTER(C.c_float), _P]),
    "krr_accel_trace_stats": (_I, [_P, _P, C.c_int64, C.c_int32, C.POINTER(C.c_ulonglong), _P]),
    "krr_accel_trace_stats_noalloc": (_I, [_P, _P, C.c_int64, C.c_int32,
                                           C.POINTER(C.c_ulonglong), _P]),
    "krr_wf_params_default": (None, [C.POINTER(WfParams)]),
    "krr_wf_create": (_I, [C.POINTER(WfParams), C.POINTER(_P)]),
    "krr_wf_destroy": (_I, [_P]),
    "krr_wf_set_params": (_I, [_P, C.POINTER(WfParams)]),
    "krr_wf_get_params": (_I, [_P, C.POINTER(WfParams)]),
    "krr_wf_params_from_json": (_I, [C.c_char_p, C.POINTER(WfParams)]),
    "krr_wf_create_json": (_I, [C.c_char_p, C.POINTER(_P)]),
    "krr_wf_set_params_json": (_I, [_P, C.c_char_p]),
    "krr_wf_set_scene": (_I, [_P, C.POINTER(SceneDesc), _P]),
    "krr_wf_resize": (_I, [_P, C.c_int32, C.c_int32]),
    "krr_wf_begin_frame": (_I, [_P, C.c_int64, C.POINTER(CameraDesc), _P]),
    "krr_wf_render": (_I, [_P, _P, _P]),
    "krr_wf_generate_camera_rays": (_I, [_P, _P]),
    "krr_wf_resize_views": (_I, [_P, C.POINTER(ViewDesc), C.c_int32]),
    "krr_wf_begin_frame_views": (_I, [_P, C.c_int64, C.POINTER(ViewDesc), C.c_int32, _P]),
    "krr_wf_capture_frame": (_I, [_P, _P, _P]),
    "krr_wf_launch_frame": (_I, [_P, C.c_int64, C.POINTER(ViewDesc), C.c_int32, _P]),
    "krr_wf_trace_closest": (_I, [_P, C.c_int32, _P]),
    "krr_wf_handle_hit": (_I, [_P, _P]),
    "krr_wf_handle_miss": (_I, [_P, _P]),
    "krr_wf_generate_scatter_rays": (_I, [_P, C.c_int32, _P]),
    "krr_wf_trace_shadow": (_I, [_P, _P]),
    "krr_wf_sample_medium_interaction": (_I, [_P, C.c_int32, _P]),
    "krr_wf_sample_medium_scattering": (_I, [_P, C.c_int32, _P]),
    "krr_wf_reset_queues": (_I, [_P, C.c_int32, _P]),
    "krr_wf_queue_size": (_I, [_P, C.c_int32, C.POINTER(C.c_int32), _P]),
    "krr_wf_pixel_radiance": (_I, [_P, C.POINTER(_P)]),
    "krr_wf_read_radiance": (_I, [_P, _P, _P]),
    "krr_wf_ray_queue": (_I, [_P, C.c_int32, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P),
                              C.POINTER(C.c_int32)]),
    "krr_wf_device_errors": (_I, [_P, C.POINTER(C.c_uint32), _P]),
    "krr_wf_accel": (_I, [_P, C.POINTER(_P)]),
    "krr_wf_set_loop_limits": (_I, [_P, C.c_int32, C.c_int32]),
    "krr_wf_set_scenes": (_I, [_P, _P, C.c_int32, _P]),
    "krr_wf_set_launch": (_I, [_P, C.c_int32, C.c_int32, C.c_int64]),
    "krr_wf_set_scene_max_depth": (_I, [_P, C.c_int32, C.c_int32]),
    "krr_wf_set_accel_levels": (_I, [_P, C.c_int32]),
    "krr_wf_set_megakernel_reorder": (_I, [_P, C.c_int32]),
    "krr_wf_set_media_order": (_I, [_P, C.c_int32]),
    "krr_wf_set_camera_order": (_I, [_P, C.c_int32]),
    "krr_wf_set_profiling": (_I, [_P, C.c_int32]),
    "krr_wf_profile_read": (_I, [_P, _P, C.c_int32, C.POINTER(C.c_int32)]),
    "krr_wf_get_launch": (_I, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                               C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "krr_wf_autotune": (_I, [_P, _P, C.c_int32, C.POINTER(WfTuning), _P]),
    "krr_wf_cache_box": (_I, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "krr_accumulate_f64": (_I, [_P, _P, C.c_int64, _P]),
    "krr_nrc_config_default": (None, [C.POINTER(NrcConfig)]),
    "krr_nrc_create": (_I, [C.POINTER(NrcConfig), C.POINTER(_P)]),
    "krr_nrc_destroy": (_I, [_P]),
    "krr_nrc_info": (_I, [_P, C.POINTER(NrcInfo)]),
    "krr_nrc_query": (_I, [_P, _P, C.c_int64, _P, _P]),
    "krr_nrc_train_step": (_I, [_P, _P, _P, C.c_int64, C.POINTER(C.c_float), _P]),
    "krr_nrc_gradients": (_I, [_P, _P, _P, C.c_int64, _P, _P, C.POINTER(C.c_float)]),
    "krr_nrc_get_params": (_I, [_P, C.c_int32, _P, C.c_int64]),
    "krr_nrc_status": (_I, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_int32), _P]),
    "krr_nrc_save": (_I, [_P, C.c_char_p]),
    "krr_nrc_load": (_I, [_P, C.c_char_p]),
    "krr_nrc_set_params": (_I, [_P, C.c_int32, _P, C.c_int64]),
    "krr_wf_set_nrc": (_I, [_P, _P, C.c_int32]),
    "krr_image_error": (_I, [_P, C.c_double, _P, C.c_int64, C.c_int32, C.POINTER(C.c_double),
                             _P]),
}

_lib: C.CDLL | None = None


class KrrError(RuntimeError):
    pass


def load() -> C.CDLL:
    """Loads libkrr_gb300.so; raises if it is missing (no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise KrrError(f"{LIB_PATH.name} is not built; run kiraray_gb300.build.build() first")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue   # tests/test_abi.py checks that every declared symbol is exported
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, what: str = "") -> None:
    if status != KRR_OK:
        lib = load()
        msg = lib.krr_last_error().decode(errors="replace")
        kind = lib.krr_status_string(status).decode()
        raise KrrError(f"{what}: {kind} ({status}): {msg}")
