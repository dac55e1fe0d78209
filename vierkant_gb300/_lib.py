"""ctypes binding of libvkg.so (the C ABI declared in include/vkg.h).

The library is loaded from the package directory; a missing library is a hard error (there is no
CPU fallback for any GPU entry point). Build it with ``python -m vierkant_gb300.build``.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libvkg.so"

VKG_OK = 0
STATUS_NAMES = {0: "VKG_OK", 1: "VKG_ERR_INVALID_ARGUMENT", 2: "VKG_ERR_CUDA", 3: "VKG_ERR_OUT_OF_MEMORY",
                4: "VKG_ERR_NOT_SUPPORTED", 5: "VKG_ERR_TIMEOUT", 6: "VKG_ERR_STACK_OVERFLOW",
                7: "VKG_ERR_CAPACITY"}
VKG_MISS = 0xFFFFFFFF
REJECT, INTERSECT, INSIDE = 0, 1, 2
RAY_CULL_BACK_FACES = 1
RAY_COUNT_STATS = 2
RAY_KEEP_ORDER = 4
NORMALS_FLOAT3 = 0
NORMALS_OCT_SNORM16 = 1
TEXCOORD_FLOAT2 = 0
TEXCOORD_HALF2 = 1
WRAP_REPEAT, WRAP_CLAMP_TO_EDGE, WRAP_MIRRORED_REPEAT = 0, 1, 2
NO_TEXTURE = 0xFFFFFFFF
BLEND_OPAQUE, BLEND_BLEND, BLEND_MASK = 0, 1, 2


RNG_PCG32, RNG_REFERENCE = 0, 1


class VkgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class vkg_ray(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("tmin", C.c_float), ("direction", C.c_float * 3), ("tmax", C.c_float)]


class vkg_hit(C.Structure):
    _fields_ = [("prim", C.c_uint32), ("t", C.c_float), ("u", C.c_float), ("v", C.c_float)]


class vkg_ray_intersection(C.Structure):
    _fields_ = [("type", C.c_int), ("distance", C.c_float)]


class vkg_ray_triangle_intersection(C.Structure):
    _fields_ = [("type", C.c_int), ("distance", C.c_float), ("u", C.c_float), ("v", C.c_float)]


class vkg_material(C.Structure):
    _fields_ = [("base_color", C.c_float * 3), ("roughness", C.c_float), ("metalness", C.c_float),
                ("emission", C.c_float * 3), ("twosided", C.c_uint32), ("transmission", C.c_float),
                ("ior", C.c_float), ("clearcoat", C.c_float), ("clearcoat_roughness", C.c_float),
                ("sheen_color", C.c_float * 3), ("sheen_roughness", C.c_float), ("diffuse_transmission", C.c_float),
                ("diffuse_transmission_color", C.c_float * 3), ("iridescence", C.c_float),
                ("iridescence_ior", C.c_float), ("iridescence_thickness", C.c_float),
                ("attenuation_color", C.c_float * 3), ("attenuation_distance", C.c_float),
                ("scatter_color", C.c_float * 3), ("scatter_factor", C.c_float), ("phase_g", C.c_float),
                ("null_surface", C.c_uint32), ("dispersion", C.c_float), ("tex_color", C.c_uint32),
                ("tex_normal", C.c_uint32), ("tex_emission", C.c_uint32), ("tex_ao_rough_metal", C.c_uint32),
                ("tex_transmission", C.c_uint32), ("tex_diffuse_transmission", C.c_uint32),
                ("tex_diffuse_transmission_color", C.c_uint32), ("alpha", C.c_float),
                ("blend_mode", C.c_uint32), ("alpha_cutoff", C.c_float), ("has_uv_transform", C.c_uint32),
                ("uv_transform", C.c_float * 6)]


class vkg_texture_desc(C.Structure):
    _fields_ = [("h_rgba8", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("wrap_s", C.c_uint32),
                ("wrap_t", C.c_uint32)]


class vkg_camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("right", C.c_float * 3), ("up", C.c_float * 3), ("back", C.c_float * 3),
                ("tan_half_fovy", C.c_float), ("aspect", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32)]


class vkg_medium_params(C.Structure):
    _fields_ = [("attenuation_color", C.c_float * 3), ("attenuation_distance", C.c_float),
                ("scatter_factor", C.c_float), ("scatter_color", C.c_float * 3), ("phase_g", C.c_float),
                ("ior", C.c_float), ("emission_color", C.c_float * 3), ("emission_intensity", C.c_float)]


class vkg_settings(C.Structure):
    _fields_ = [("resolution", C.c_uint32 * 2), ("max_num_batches", C.c_uint32), ("num_samples", C.c_uint32),
                ("max_trace_depth", C.c_uint32), ("max_path_beta", C.c_float), ("suspend_trace_when_done", C.c_uint32),
                ("disable_material", C.c_uint32), ("mis_mode", C.c_uint32), ("draw_skybox", C.c_uint32),
                ("environment", C.c_float), ("rr_start_depth", C.c_uint32), ("crop", C.c_uint32 * 4),
                ("samples_per_wave", C.c_uint32), ("suppress_refractive_caustics", C.c_uint32),
                ("sun_color", C.c_float * 3), ("sun_intensity", C.c_float), ("sun_spherical_coords", C.c_float * 2),
                ("sun_angular_size", C.c_float), ("denoising", C.c_uint32), ("clip_near", C.c_float),
                ("camera_medium_mode", C.c_uint32), ("camera_medium", vkg_medium_params), ("rng_mode", C.c_uint32)]


class vkg_post_fx_settings(C.Structure):
    _fields_ = [("tonemap", C.c_uint32), ("bloom", C.c_uint32), ("exposure", C.c_float), ("gamma", C.c_float),
                ("brightness_thresh", C.c_float * 2), ("blur_iterations", C.c_uint32)]


class vkg_gltf_counts(C.Structure):
    _fields_ = [("num_meshes", C.c_uint32), ("num_instances", C.c_uint32), ("num_materials", C.c_uint32),
                ("num_lights", C.c_uint32), ("skipped_primitives", C.c_uint32), ("num_textures", C.c_uint32),
                ("skipped_textures", C.c_uint32)]


class vkg_wire_entry_info(C.Structure):
    _fields_ = [("buffer_index", C.c_uint32), ("base_index", C.c_uint32), ("vertex_offset", C.c_int32),
                ("aabb_min", C.c_float * 3), ("aabb_max", C.c_float * 3), ("has_uv_transform", C.c_uint32),
                ("uv_transform", C.c_float * 6)]


class vkg_pixel_data(C.Structure):
    _fields_ = [("radiance", C.c_float * 3), ("alpha", C.c_float), ("depth", C.c_float), ("normal", C.c_uint32),
                ("object_id", C.c_uint32), ("albedo", C.c_uint32)]


class vkg_light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("type", C.c_uint32), ("color", C.c_float * 3), ("intensity", C.c_float),
                ("direction", C.c_float * 3), ("range", C.c_float), ("spot_angle_scale", C.c_float),
                ("spot_angle_offset", C.c_float), ("angular_size", C.c_float), ("size_y", C.c_float),
                ("tangent", C.c_float * 3), ("size_x", C.c_float)]


class vkg_light_source(C.Structure):
    _fields_ = [("type", C.c_uint32), ("color", C.c_float * 3), ("intensity", C.c_float), ("range", C.c_float),
                ("inner_cone_angle", C.c_float), ("outer_cone_angle", C.c_float), ("size", C.c_float * 2)]


class vkg_tracer_create_info(C.Structure):
    _fields_ = [("seed", C.c_uint32), ("settings", vkg_settings)]


class vkg_tlas_info(C.Structure):
    _fields_ = [("num_instances", C.c_uint32), ("num_blas", C.c_uint32), ("num_nodes", C.c_uint32),
                ("depth", C.c_uint32), ("scene_min", C.c_float * 3), ("scene_max", C.c_float * 3),
                ("d_nodes", C.c_void_p), ("d_instances", C.c_void_p), ("d_instances_by_id", C.c_void_p),
                ("build_ms", C.c_float)]


class vkg_mesh_desc(C.Structure):
    _fields_ = [("d_xyz", C.c_void_p), ("num_vertices", C.c_uint32), ("d_indices", C.c_void_p),
                ("num_tris", C.c_uint32), ("twosided", C.c_uint32), ("vertex_stride", C.c_uint32)]


class vkg_instanced_scene_desc(C.Structure):
    _fields_ = [("meshes", C.POINTER(vkg_mesh_desc)), ("num_meshes", C.c_uint32), ("d_instances", C.c_void_p),
                ("num_instances", C.c_uint32), ("d_materials", C.c_void_p), ("num_materials", C.c_uint32),
                ("d_env_rgb", C.c_void_p), ("env_width", C.c_uint32), ("env_height", C.c_uint32),
                ("leaf_max", C.c_uint32)]


class vkg_batch_job(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", vkg_camera), ("settings", vkg_settings), ("seed", C.c_uint32),
                ("pad", C.c_uint32), ("d_rgb_out", C.c_void_p)]


class vkg_batch_tuning(C.Structure):
    _fields_ = [("extend_kernel", C.c_uint32), ("ctas_per_sm", C.c_uint32), ("wave_paths", C.c_uint32),
                ("use_graph", C.c_uint32), ("block_size", C.c_uint32), ("stack_depth", C.c_uint32)]


class vkg_batch_stats(C.Structure):
    _fields_ = [("render_ms", C.c_double), ("paths", C.c_uint64), ("extension_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("waves", C.c_uint32), ("batch", C.c_uint32)]


class vkg_tracer_stats(C.Structure):
    _fields_ = [("raytrace_ms", C.c_double), ("total_ms", C.c_double), ("paths", C.c_uint64),
                ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("batch", C.c_uint32),
                ("pad", C.c_uint32), ("train_ms", C.c_double), ("cache_queries", C.c_uint64),
                ("train_records", C.c_uint64)]


class vkg_scene_desc(C.Structure):
    _fields_ = [("d_xyz", C.c_void_p), ("num_vertices", C.c_uint32), ("d_indices", C.c_void_p),
                ("num_tris", C.c_uint32), ("d_tri_material", C.c_void_p), ("d_materials", C.c_void_p),
                ("num_materials", C.c_uint32), ("d_env_rgb", C.c_void_p), ("env_width", C.c_uint32),
                ("env_height", C.c_uint32), ("leaf_max", C.c_uint32)]


class vkg_nrc_config(C.Structure):
    _fields_ = [("levels", C.c_uint32), ("log2_table_size", C.c_uint32), ("base_resolution", C.c_uint32),
                ("max_resolution", C.c_uint32), ("learning_rate", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("epsilon", C.c_float), ("seed", C.c_uint32), ("scene_min", C.c_float * 3),
                ("scene_max", C.c_float * 3), ("batch_size", C.c_uint32), ("train_paths", C.c_uint32),
                ("terminate_depth", C.c_uint32), ("train_depth", C.c_uint32), ("train_steps", C.c_uint32),
                ("infer_kernel", C.c_uint32), ("train_kernel", C.c_uint32)]


class vkg_nrc_info_t(C.Structure):
    _fields_ = [("levels", C.c_uint32), ("table_size", C.c_uint32), ("growth", C.c_float),
                ("level_resolution", C.c_uint32 * 16), ("num_mlp_params", C.c_uint32),
                ("num_grid_params", C.c_uint64), ("d_mlp_params", C.c_void_p), ("d_grid_params", C.c_void_p),
                ("d_mlp_grads", C.c_void_p), ("d_grid_grads", C.c_void_p), ("step", C.c_uint32),
                ("kernel_error", C.c_uint32), ("infer_kernel", C.c_uint32), ("train_kernel", C.c_uint32)]


class vkg_bvh_build_options(C.Structure):
    _fields_ = [("leaf_max", C.c_uint32)]


class vkg_bvh_info(C.Structure):
    _fields_ = [("num_tris", C.c_uint32), ("num_nodes", C.c_uint32), ("depth", C.c_uint32), ("leaf_max", C.c_uint32),
                ("scene_min", C.c_float * 3), ("scene_max", C.c_float * 3), ("margin", C.c_float),
                ("bytes", C.c_size_t), ("d_nodes", C.c_void_p), ("d_tris", C.c_void_p), ("d_morton", C.c_void_p),
                ("d_sorted", C.c_void_p), ("build_ms", C.c_float)]


P = C.c_void_p
U32 = C.c_uint32
U64 = C.c_uint64
I32 = C.c_int
F32 = C.c_float
PF = C.POINTER(C.c_float)

# name -> (restype, argtypes); keep in sync with include/vkg.h
SIGNATURES = {
    "vkg_version": (C.c_char_p, []),
    "vkg_ctx_create": (I32, [I32, C.POINTER(P)]),
    "vkg_ctx_destroy": (I32, [P]),
    "vkg_last_error": (C.c_char_p, [P]),
    "vkg_intersect_ray_triangle": (I32, [P, P, P, C.POINTER(vkg_ray_triangle_intersection)]),
    "vkg_intersect_ray_aabb": (I32, [P, P, P, P, C.POINTER(vkg_ray_intersection)]),
    "vkg_intersect_ray_obb": (I32, [P, P, P, P, P, C.POINTER(vkg_ray_intersection)]),
    "vkg_intersect_ray_sphere": (I32, [P, P, P, F32, C.POINTER(vkg_ray_intersection)]),
    "vkg_intersect_ray_plane": (I32, [P, P, P, C.POINTER(vkg_ray_intersection)]),
    "vkg_intersect_triangle_aabb": (I32, [P, P, P, C.POINTER(U32)]),
    "vkg_intersect_triangle_triangle": (I32, [P, P, C.POINTER(U32)]),
    "vkg_geometry_icosphere_counts": (I32, [U32, C.POINTER(U32), C.POINTER(U32)]),
    "vkg_geometry_icosphere": (I32, [F32, U32, P, P]),
    "vkg_scene_cornell_counts": (I32, [U32, U32, C.POINTER(U32), C.POINTER(U32), C.POINTER(U32)]),
    "vkg_scene_cornell": (I32, [U64, U64, U32, U32, P, P, P, P]),
    "vkg_camera_lookat": (I32, [P, P, P, F32, U32, U32, C.POINTER(vkg_camera)]),
    "vkg_material_defaults": (I32, [C.POINTER(vkg_material)]),
    "vkg_camera_rays": (I32, [P, C.POINTER(vkg_camera), U64, U64, U32, P, P]),
    "vkg_bvh_build": (I32, [P, P, U32, P, U32, C.POINTER(vkg_bvh_build_options), C.POINTER(P), P]),
    "vkg_bvh_info_get": (I32, [P, C.POINTER(vkg_bvh_info)]),
    "vkg_bvh_destroy": (I32, [P, P]),
    "vkg_bvh_build_noalloc": (I32, [P, U32, P, U32, U32, P, U32, P, P, P]),
    "vkg_closest_hit": (I32, [P, P, P, U32, P, U32, P]),
    "vkg_any_hit": (I32, [P, P, P, U32, P, U32, P]),
    "vkg_closest_hit_host": (I32, [P, P, P, U32, P, U32, P]),
    "vkg_ray_stats_get": (I32, [P, C.POINTER(U64), C.POINTER(U64), I32]),
    "vkg_env_procedural_sky": (I32, [P, U32, U32, P, F32, F32, P, P]),
    "vkg_scene_create": (I32, [P, C.POINTER(vkg_scene_desc), C.POINTER(P), P]),
    "vkg_scene_destroy": (I32, [P, P]),
    "vkg_scene_set_lights": (I32, [P, P, P, U32]),
    "vkg_scene_set_normals": (I32, [P, P, U32, P, U32, U32, P]),
    "vkg_scene_set_tangents": (I32, [P, P, U32, P, U32, U32, P]),
    "vkg_scene_set_texcoords": (I32, [P, P, U32, P, U32, U32, P]),
    "vkg_scene_set_textures": (I32, [P, P, P, U32, P]),
    "vkg_tracer_pixel_data": (I32, [P, P, P]),
    "vkg_denoise": (I32, [P, P, U32, U32, P, P, P]),
    "vkg_post_fx_default": (I32, [C.POINTER(vkg_post_fx_settings)]),
    "vkg_gltf_load": (I32, [C.c_char_p, C.POINTER(P), C.c_char_p, C.c_size_t]),
    "vkg_gltf_counts_get": (I32, [P, C.POINTER(vkg_gltf_counts)]),
    "vkg_gltf_mesh": (I32, [P, U32, C.POINTER(C.POINTER(C.c_float)), C.POINTER(U32), C.POINTER(C.POINTER(U32)),
                            C.POINTER(U32)]),
    "vkg_gltf_mesh_normals": (I32, [P, U32, C.POINTER(C.POINTER(C.c_float))]),
    "vkg_gltf_mesh_texcoords": (I32, [P, U32, C.POINTER(C.POINTER(C.c_float))]),
    "vkg_gltf_mesh_tangents": (I32, [P, U32, C.POINTER(C.POINTER(C.c_float))]),
    "vkg_gltf_textures": (I32, [P, P]),
    "vkg_gltf_instances": (I32, [P, P]),
    "vkg_gltf_materials": (I32, [P, P]),
    "vkg_gltf_lights": (I32, [P, P]),
    "vkg_gltf_destroy": (I32, [P]),
    "vkg_post_fx": (I32, [P, P, U32, U32, C.POINTER(vkg_post_fx_settings), P, P]),
    "vkg_light_convert": (I32, [C.POINTER(vkg_light_source), P, P, C.POINTER(vkg_light)]),
    "vkg_scene_bvh": (I32, [P, C.POINTER(P)]),
    "vkg_scene_env_tables": (I32, [P, C.POINTER(P), C.POINTER(P), C.POINTER(U32), C.POINTER(U32)]),
    "vkg_settings_default": (I32, [C.POINTER(vkg_settings)]),
    "vkg_materials_from_wire": (I32, [P, U32, P, C.POINTER(U32)]),
    "vkg_instances_from_wire": (I32, [P, U32, P, P]),
    "vkg_medium_params_default": (I32, [C.POINTER(vkg_medium_params)]),
    "vkg_scene_camera_medium": (I32, [P, C.POINTER(C.c_float), C.POINTER(U32)]),
    "vkg_tracer_create": (I32, [P, C.POINTER(vkg_tracer_create_info), C.POINTER(P)]),
    "vkg_tracer_set_settings": (I32, [P, C.POINTER(vkg_settings)]),
    "vkg_tracer_get_settings": (I32, [P, C.POINTER(vkg_settings)]),
    "vkg_tracer_render": (I32, [P, P, C.POINTER(vkg_camera), P, P]),
    "vkg_tracer_reset_accumulator": (I32, [P]),
    "vkg_tracer_current_batch": (I32, [P, C.POINTER(U32)]),
    "vkg_tracer_statistics": (I32, [P, C.POINTER(vkg_tracer_stats)]),
    "vkg_tracer_destroy": (I32, [P]),
    "vkg_tracer_attach_cache": (I32, [P, P]),
    "vkg_scene_create_instanced": (I32, [P, C.POINTER(vkg_instanced_scene_desc), C.POINTER(P), P]),
    "vkg_scene_tlas": (I32, [P, C.POINTER(P)]),
    "vkg_geometry_cubesphere": (I32, [U32, C.c_float, P, P]),
    "vkg_geometry_terrain": (I32, [U32, C.c_float, C.c_float, C.c_float, U32, U32, P, P]),
    "vkg_instances_random": (I32, [C.c_uint64, C.c_uint64, U32, U32, U32, U32, P, P, C.c_float, C.c_float, P]),
    "vkg_tlas_build": (I32, [P, P, U32, P, U32, P, C.POINTER(P), P]),
    "vkg_tlas_info_get": (I32, [P, C.POINTER(vkg_tlas_info)]),
    "vkg_tlas_destroy": (I32, [P, P]),
    "vkg_tlas_closest_hit": (I32, [P, P, P, U32, P, U32, P]),
    "vkg_tlas_any_hit": (I32, [P, P, P, U32, P, U32, P]),
    "vkg_batch_tuning_default": (I32, [C.POINTER(vkg_batch_tuning)]),
    "vkg_batch_create": (I32, [P, C.POINTER(vkg_batch_job), U32, C.POINTER(vkg_batch_tuning), C.POINTER(P)]),
    "vkg_batch_autotune": (I32, [P, P, C.POINTER(vkg_batch_tuning)]),
    "vkg_batch_set_tuning": (I32, [P, C.POINTER(vkg_batch_tuning)]),
    "vkg_batch_render": (I32, [P, P]),
    "vkg_batch_reset_accumulator": (I32, [P]),
    "vkg_batch_statistics": (I32, [P, C.POINTER(vkg_batch_stats)]),
    "vkg_batch_destroy": (I32, [P]),
    "vkg_diag_tc_gemm": (I32, [P, P, P, U32, U32, P, P, P]),
    "vkg_diag_wait_timeout": (I32, [P, U32, U64, P, P, P]),
    "vkg_diag_tracer_uniforms": (I32, [P, P, U32]),
    "vkg_nrc_config_default": (I32, [C.POINTER(vkg_nrc_config)]),
    "vkg_nrc_create": (I32, [P, C.POINTER(vkg_nrc_config), C.POINTER(P)]),
    "vkg_nrc_destroy": (I32, [P]),
    "vkg_nrc_info": (I32, [P, C.POINTER(vkg_nrc_info_t)]),
    "vkg_nrc_infer": (I32, [P, P, U32, P, P]),
    "vkg_nrc_backward": (I32, [P, P, P, U32, P]),
    "vkg_nrc_adam_step": (I32, [P, P]),
    "vkg_nrc_train_step": (I32, [P, P, P, U32, C.POINTER(F32), P]),
    "vkg_nrc_load_params": (I32, [P, P, P, P]),
    "vkg_nrc_save": (I32, [P, C.c_char_p, P]),
    "vkg_nrc_load": (I32, [P, C.c_char_p, P]),
}

_lib = None


def lib() -> C.CDLL:
    """Load libvkg.so (once). Raises if the library has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m vierkant_gb300.build` "
                               "(the GPU path has no fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int, ctx=None, what: str = "") -> None:
    if status != VKG_OK:
        msg = lib().vkg_last_error(ctx).decode() if ctx else ""
        raise VkgError(status, f"{what}: {msg}" if what else msg)
