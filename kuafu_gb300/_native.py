"""ctypes binding of libkf's C-ABI (include/kf.h).

The shared library is built in-tree (``python -m kuafu_gb300.build``). Loading
fails loudly when it is missing: there is no CPU fallback for the render path.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libkf.so"

c_u8p = C.POINTER(C.c_uint8)
c_u32p = C.POINTER(C.c_uint32)
c_f32p = C.POINTER(C.c_float)


class kf_vertex(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("normal", C.c_float * 3), ("color", C.c_float * 3), ("uv", C.c_float * 2),
                ("pad", C.c_float)]


class kf_material_gpu(C.Structure):
    _fields_ = [("diffuse", C.c_float * 4), ("emission", C.c_float * 4), ("alpha", C.c_float),
                ("metallic", C.c_float), ("specular", C.c_float), ("roughness", C.c_float), ("ior", C.c_float),
                ("transmission", C.c_float), ("diffuse_tex", C.c_int32), ("metallic_tex", C.c_int32),
                ("roughness_tex", C.c_int32), ("transmission_tex", C.c_int32), ("pad0", C.c_int32),
                ("pad1", C.c_int32)]


class kf_dir_light_ubo(C.Structure):
    _fields_ = [("direction", C.c_float * 4), ("rgbs", C.c_float * 4)]


class kf_point_lights_ubo(C.Structure):
    _fields_ = [("posr", (C.c_float * 4) * 32), ("rgbs", (C.c_float * 4) * 32)]


class kf_active_lights_ubo(C.Structure):
    _fields_ = [("view", (C.c_float * 16) * 8), ("proj", (C.c_float * 16) * 8), ("front", (C.c_float * 4) * 8),
                ("rgbs", (C.c_float * 4) * 8), ("position", (C.c_float * 4) * 8), ("sftp", (C.c_float * 4) * 8)]


class kf_camera_ubo(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("proj", C.c_float * 16), ("view_inv", C.c_float * 16),
                ("proj_inv", C.c_float * 16), ("position", C.c_float * 4), ("front", C.c_float * 4),
                ("pad1", C.c_float * 4), ("pad2", C.c_float * 4)]


class kf_push_constants(C.Structure):
    _fields_ = [("clear_color", C.c_float * 4), ("frame_count", C.c_int32), ("spp", C.c_uint32),
                ("max_path_depth", C.c_uint32), ("use_env_map", C.c_uint32), ("russian_roulette", C.c_uint32),
                ("rr_min_bounces", C.c_uint32), ("nee", C.c_uint32), ("nee_min", C.c_uint32)]


class kf_texture_desc(C.Structure):
    _fields_ = [("rgba8", c_u8p), ("width", C.c_uint32), ("height", C.c_uint32), ("srgb", C.c_uint32),
                ("pad", C.c_uint32)]


class kf_flat_geometry(C.Structure):
    _fields_ = [("vertices", C.POINTER(kf_vertex)), ("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32),
                ("indices", c_u32p), ("mat_index", c_u32p), ("opaque", C.c_uint32), ("hide_render", C.c_uint32)]


class kf_flat_instance(C.Structure):
    _fields_ = [("transform", C.c_float * 16), ("world_to_object", C.c_float * 12), ("geometry_index", C.c_uint32),
                ("pad", C.c_uint32 * 3)]


class kf_flat_scene(C.Structure):
    _fields_ = [("geometries", C.POINTER(kf_flat_geometry)), ("num_geometries", C.c_uint32),
                ("num_instances", C.c_uint32), ("instances", C.POINTER(kf_flat_instance)),
                ("materials", C.POINTER(kf_material_gpu)), ("num_materials", C.c_uint32),
                ("num_textures", C.c_uint32), ("textures", C.POINTER(kf_texture_desc)),
                ("dlight", kf_dir_light_ubo), ("plights", kf_point_lights_ubo), ("alights", kf_active_lights_ubo),
                ("env_rgba32f", c_f32p), ("env_size", C.c_uint32), ("env_pad", C.c_uint32)]


class kf_hit(C.Structure):
    _fields_ = [("t", C.c_float), ("u", C.c_float), ("v", C.c_float), ("instance", C.c_uint32), ("prim", C.c_uint32),
                ("pad", C.c_uint32 * 3)]


class kf_config(C.Structure):
    _fields_ = [("initial_width", C.c_int32), ("initial_height", C.c_int32), ("spp", C.c_uint32),
                ("path_depth", C.c_uint32), ("max_path_depth", C.c_uint32), ("russian_roulette", C.c_uint32),
                ("rr_min_bounces", C.c_uint32), ("nee", C.c_uint32), ("nee_min_bounces", C.c_uint32),
                ("accumulate_frames", C.c_uint32), ("use_denoiser", C.c_uint32), ("present", C.c_uint32),
                ("max_geometries", C.c_uint32), ("max_instances", C.c_uint32), ("max_textures", C.c_uint32),
                ("max_materials", C.c_uint32), ("seed", C.c_uint32), ("blas_leaf_size", C.c_uint32),
                ("tlas_leaf_size", C.c_uint32), ("max_paths_in_flight", C.c_uint64), ("debug_outputs", C.c_uint32),
                ("profile", C.c_uint32), ("use_graph", C.c_uint32), ("device", C.c_uint32),
                ("host_only", C.c_uint32), ("traversal", C.c_uint32), ("bvh_builder", C.c_uint32),
                ("dyn_refill_below", C.c_uint32), ("dyn_steps", C.c_uint32), ("blas_share", C.c_uint32)]


class kf_stats(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("rays_primary", C.c_uint64), ("rays_extension", C.c_uint64),
                ("rays_shadow", C.c_uint64), ("node_visits", C.c_uint64), ("tri_tests", C.c_uint64),
                ("inst_visits", C.c_uint64), ("shadow_node_visits", C.c_uint64), ("shadow_tri_tests", C.c_uint64),
                ("shadow_inst_visits", C.c_uint64), ("extend_ms", C.c_double), ("shadow_ms", C.c_double),
                ("shade_ms", C.c_double), ("frame_ms", C.c_double), ("bvh_build_ms", C.c_double),
                ("frame_count", C.c_int32), ("last_spp", C.c_uint32), ("blas_nodes", C.c_uint32),
                ("tlas_nodes", C.c_uint32), ("tlas_refits", C.c_uint64)]


class kf_material(C.Structure):
    _fields_ = [("diffuse_color", C.c_float * 3), ("alpha", C.c_float), ("metallic", C.c_float),
                ("specular", C.c_float), ("roughness", C.c_float), ("ior", C.c_float), ("transmission", C.c_float),
                ("emission", C.c_float * 3), ("emission_strength", C.c_float), ("diffuse_tex", C.c_int32),
                ("metallic_tex", C.c_int32), ("roughness_tex", C.c_int32), ("transmission_tex", C.c_int32)]


class kf_directional_light(C.Structure):
    _fields_ = [("direction", C.c_float * 3), ("color", C.c_float * 3), ("strength", C.c_float),
                ("softness", C.c_float)]


class kf_point_light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("color", C.c_float * 3), ("radius", C.c_float), ("strength", C.c_float)]


class kf_active_light(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("color", C.c_float * 3), ("fov", C.c_float), ("strength", C.c_float),
                ("softness", C.c_float), ("tex_id", C.c_int32)]


class kf_batch_item(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", C.c_void_p), ("spp", C.c_uint32), ("pad", C.c_uint32)]


class kf_autotune_result(C.Structure):
    _fields_ = [("traversal", C.c_uint32), ("blas_leaf_size", C.c_uint32), ("max_paths_in_flight", C.c_uint64),
                ("grid_extend", C.c_uint32), ("grid_shade", C.c_uint32), ("candidates", C.c_uint32),
                ("best_ms", C.c_float), ("start_ms", C.c_float), ("start_traversal", C.c_uint32),
                ("start_blas_leaf_size", C.c_uint32), ("start_max_paths_in_flight", C.c_uint64),
                ("dyn_refill_below", C.c_uint32), ("dyn_steps", C.c_uint32)]


VP = C.c_void_p
I = C.c_int
U32 = C.c_uint32
F = C.c_float
F16 = C.c_float * 16
F3 = C.c_float * 3
F4 = C.c_float * 4

# name -> (restype, argtypes)
PROTOTYPES = {
    "kf_last_error": (C.c_char_p, []),
    "kf_version": (I, []),
    "kf_config_init": (None, [C.POINTER(kf_config)]),
    "kf_renderer_create": (I, [C.POINTER(kf_config), C.POINTER(VP)]),
    "kf_renderer_destroy": (I, [VP]),
    "kf_renderer_get_config": (I, [VP, C.POINTER(kf_config)]),
    "kf_renderer_set_config": (I, [VP, C.POINTER(kf_config)]),
    "kf_renderer_get_scene": (I, [VP, C.POINTER(VP)]),
    "kf_renderer_create_scene": (I, [VP, C.POINTER(VP)]),
    "kf_renderer_set_scene": (I, [VP, VP]),
    "kf_renderer_remove_scene": (I, [VP, VP]),
    "kf_renderer_is_running": (I, [VP, C.POINTER(I)]),
    "kf_renderer_run": (I, [VP]),
    "kf_renderer_synchronize": (I, [VP]),
    "kf_renderer_get_stream": (I, [VP, C.POINTER(VP)]),
    "kf_renderer_download_latest_frame": (I, [VP, VP, VP, C.c_size_t]),
    "kf_renderer_download_aov": (I, [VP, VP, I, VP, C.c_size_t]),
    "kf_renderer_get_stats": (I, [VP, C.POINTER(kf_stats)]),
    "kf_renderer_reset_stats": (I, [VP]),
    "kf_renderer_reset_frame": (I, [VP]),
    "kf_renderer_count_traversal": (I, [VP, I]),
    "kf_material_init": (None, [C.POINTER(kf_material)]),
    "kf_material_add": (I, [C.POINTER(kf_material), C.POINTER(U32)]),
    "kf_material_count": (U32, []),
    "kf_material_get": (I, [U32, C.POINTER(kf_material)]),
    "kf_material_clear": (I, []),
    "kf_texture_create": (I, [VP, U32, U32, I, C.POINTER(C.c_int32)]),
    "kf_texture_count": (U32, []),
    "kf_geometry_create": (I, [VP, U32, VP, U32, VP, U32, C.POINTER(VP)]),
    "kf_geometry_set_material": (I, [VP, C.POINTER(kf_material)]),
    "kf_geometry_set_flags": (I, [VP, I, I, I]),
    "kf_geometry_recalculate_normals": (I, [VP]),
    "kf_geometry_get_info": (I, [VP, C.POINTER(U32), C.POINTER(U32)]),
    "kf_geometry_get_data": (I, [VP, VP, VP, VP]),
    "kf_geometry_release": (I, [VP]),
    "kf_geometry_create_builtin": (I, [I, F, F, C.POINTER(kf_material), C.POINTER(VP)]),
    "kf_load_scene": (I, [C.c_char_p, I, C.POINTER(VP), U32, C.POINTER(U32)]),
    "kf_scene_submit_geometry": (I, [VP, VP]),
    "kf_scene_clear_geometries": (I, [VP]),
    "kf_scene_remove_geometry": (I, [VP, VP]),
    "kf_scene_submit_instance": (I, [VP, VP, F16, C.POINTER(VP)]),
    "kf_instance_set_transform": (I, [VP, F16]),
    "kf_scene_remove_instance": (I, [VP, VP]),
    "kf_scene_clear_instances": (I, [VP]),
    "kf_scene_instance_count": (I, [VP, C.POINTER(U32)]),
    "kf_scene_get_instance": (I, [VP, U32, C.POINTER(VP)]),
    "kf_instance_release": (I, [VP]),
    "kf_scene_set_clear_color": (I, [VP, F4]),
    "kf_scene_get_clear_color": (I, [VP, F4]),
    "kf_scene_set_environment_map": (I, [VP, VP, U32]),
    "kf_scene_set_environment_map_rgba8": (I, [VP, VP, U32, I]),
    "kf_scene_set_environment_map_file": (I, [VP, C.c_char_p]),
    "kf_scene_remove_environment_map": (I, [VP]),
    "kf_scene_mark_geometries_changed": (I, [VP]),
    "kf_scene_mark_instances_changed": (I, [VP]),
    "kf_scene_set_directional_light": (I, [VP, C.POINTER(kf_directional_light)]),
    "kf_scene_remove_directional_light": (I, [VP]),
    "kf_scene_add_point_light": (I, [VP, C.POINTER(kf_point_light), C.POINTER(VP)]),
    "kf_scene_add_active_light": (I, [VP, C.POINTER(kf_active_light), C.POINTER(VP)]),
    "kf_light_update_point": (I, [VP, C.POINTER(kf_point_light)]),
    "kf_light_update_active": (I, [VP, C.POINTER(kf_active_light)]),
    "kf_scene_remove_light": (I, [VP, VP]),
    "kf_scene_create_camera": (I, [VP, I, I, C.POINTER(VP)]),
    "kf_scene_remove_camera": (I, [VP, VP]),
    "kf_scene_set_camera": (I, [VP, VP]),
    "kf_scene_get_camera": (I, [VP, C.POINTER(VP)]),
    "kf_scene_export": (I, [VP, C.POINTER(kf_flat_scene)]),
    "kf_camera_set_position": (I, [VP, F3]),
    "kf_camera_set_front": (I, [VP, F3]),
    "kf_camera_set_up": (I, [VP, F3]),
    "kf_camera_set_pose": (I, [VP, F16]),
    "kf_camera_get_pose": (I, [VP, F16]),
    "kf_camera_set_full_perspective": (I, [VP, F, F, F, F, F, F, F]),
    "kf_camera_set_size": (I, [VP, I, I]),
    "kf_camera_reset_view": (I, [VP]),
    "kf_camera_get_size": (I, [VP, C.POINTER(I), C.POINTER(I)]),
    "kf_camera_get_ubo": (I, [VP, C.POINTER(kf_camera_ubo)]),
    "kf_renderer_run_batch": (I, [VP, C.POINTER(kf_batch_item), U32]),
    "kf_renderer_autotune": (I, [VP, C.POINTER(kf_batch_item), U32, U32, C.POINTER(kf_autotune_result)]),
    "kf_relmse": (I, [VP, VP, VP, C.c_uint64, C.c_double, C.POINTER(C.c_double)]),
    "kf_relmse_noalloc": (I, [VP, VP, C.c_uint64, C.c_double, VP, C.POINTER(C.c_double)]),
    "kf_renderer_measure_l2_read": (I, [VP, C.c_uint64, C.c_uint32, C.c_uint32, C.POINTER(C.c_double)]),
    "kf_conv3x3_bf16": (I, [VP, I, I, I, I, VP, I, VP, I, I, VP, I, I, VP]),
    "kf_gemm_bf16_tn": (I, [VP, I, VP, I, I, VP, I, I, VP]),
    "kf_tc_error": (I, [C.POINTER(U32)]),
    "kf_tc_wait_probe": (I, [C.c_uint64, VP]),
    "kf_denoiser_create": (I, [VP, U32, C.POINTER(VP)]),
    "kf_denoiser_destroy": (I, [VP]),
    "kf_denoiser_num_params": (I, [VP, C.POINTER(C.c_uint64)]),
    "kf_denoiser_get_params": (I, [VP, VP, C.c_uint64]),
    "kf_denoiser_set_params": (I, [VP, VP, C.c_uint64]),
    "kf_denoiser_save": (I, [VP, C.c_char_p]),
    "kf_denoiser_load": (I, [VP, C.c_char_p]),
    "kf_denoiser_add_view": (I, [VP, VP, VP, U32, U32, U32]),
    "kf_denoiser_add_view_inputs": (I, [VP, VP, VP, C.POINTER(U32), U32, U32, U32]),
    "kf_denoiser_num_views": (I, [VP, C.POINTER(U32)]),
    "kf_denoiser_train": (I, [VP, U32, U32, U32, F, C.POINTER(F)]),
    "kf_denoiser_apply": (I, [VP, VP]),
    "kf_renderer_set_denoiser": (I, [VP, VP]),
    "kf_denoiser_forward": (I, [VP, VP, VP, I, I, I, VP]),
    "kf_denoiser_camera_features": (I, [VP, VP, VP, VP, C.POINTER(I), C.POINTER(I)]),
    "kf_denoiser_train_step": (I, [VP, VP, VP, VP, I, I, I, F, VP, I, C.POINTER(F)]),
}

KF_AOV_RADIANCE_F32, KF_AOV_ALBEDO_F32, KF_AOV_NORMAL_F32, KF_AOV_DEPTH_F32 = 0, 1, 2, 3
KF_AOV_SUM_F64, KF_AOV_PATH_RADIANCE, KF_AOV_PRIMARY_HITS, KF_AOV_DENOISED_F32 = 4, 5, 6, 7
KF_AOV_SEGMENTATION = 8
KF_MESH_YZ_PLANE, KF_MESH_CUBE, KF_MESH_SPHERE, KF_MESH_CAPSULE, KF_MESH_ICOSPHERE = 0, 1, 2, 3, 4

ERRORS = {1: "invalid argument", 2: "out of range", 3: "limit exceeded", 4: "CUDA error", 5: "not implemented",
          6: "invalid state", 7: "no CUDA device", 8: "out of memory", 9: "internal error", 10: "timeout"}


class KfError(RuntimeError):
    """Raised for a non-zero kf_* status (kuafu throws std::runtime_error)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


_lib = None


def load(path: str | os.PathLike | None = None):
    """Loads libkf and declares every prototype of include/kf.h."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else _LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with `python -m kuafu_gb300.build` (no CPU fallback exists)")
    lib = C.CDLL(str(p))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int):
    if status != 0:
        raise KfError(status, load().kf_last_error().decode(errors="replace"))
    return status
