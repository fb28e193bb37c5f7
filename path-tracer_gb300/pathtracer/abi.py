"""ctypes mirror of include/pt.h and include/pt_world.h.

Struct layouts are checked against the C sizes by the tests; the library is
loaded from the in-tree build (path-tracer_gb300/_build/libpt.so) and nothing
else: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

c_f = C.c_float
c_u32 = C.c_uint32
c_i32 = C.c_int32
c_u64 = C.c_uint64

PT_OK = 0
PT_ERR_INVALID_ARG = 1
PT_ERR_OUT_OF_LIMITS = 2
PT_ERR_OOM = 3
PT_ERR_CUDA = 4
PT_ERR_TIMEOUT = 5
PT_ERR_STATE = 6
ERROR_NAMES = {0: "PT_OK", 1: "PT_ERR_INVALID_ARG", 2: "PT_ERR_OUT_OF_LIMITS", 3: "PT_ERR_OOM",
               4: "PT_ERR_CUDA", 5: "PT_ERR_TIMEOUT", 6: "PT_ERR_STATE"}

PT_ALPHA_MODE_OPAQUE = 0
PT_ALPHA_MODE_MASK = 1
PT_ALPHA_MODE_BLEND = 2
PT_ATLAS_SIZE = 8192
PT_DEFAULT_MAX_BOUNCES = 10
PT_MAX_BOUNCES_LIMIT = 16
PT_MAX_SAMPLES_PER_TRACE = 16
PT_KERNEL_WAVEFRONT = 0
PT_KERNEL_PLAIN = 1
PT_TILE_IMAGE = 0
PT_TILE_ACCUMULATION = 1
PT_TILE_COMPENSATION = 2
# include/pt_precision.h
PT_PRECISION_FP32 = 0
PT_PRECISION_WIDE_BVH = 1
PT_PRECISION_HALF_ATTRIBUTES = 2
PT_PRECISION_KAHAN = 4
PT_PRECISION_COMPRESSED = 7
PT_KERNEL_CLASS_COUNT = 7
KERNEL_CLASSES = ["raygen", "extend", "shade", "shadow", "accumulate", "plain", "sort"]
PT_RECORD_MAX_BOUNCES = 17
COUNT_FIELDS = ["extend_rays", "shadow_rays", "interior_visits", "leaf_visits", "triangle_tests",
                "shadow_interior_visits", "shadow_leaf_visits", "shadow_triangle_tests", "rand_draws",
                "hits", "sky_misses", "light_samples", "sky_light_samples"]
EXPOSURE = 0.00002604166


class TriangleGeometry(C.Structure):
    _fields_ = [("v0", c_f * 3), ("v1", c_f * 3), ("v2", c_f * 3)]


class TriangleAttribute(C.Structure):
    _fields_ = [("material_index", c_u32), ("n0", c_f * 3), ("n1", c_f * 3), ("n2", c_f * 3),
                ("uv0", c_f * 2), ("uv1", c_f * 2), ("uv2", c_f * 2),
                ("t0", c_f * 4), ("t1", c_f * 4), ("t2", c_f * 4)]


class BvhNode(C.Structure):
    _fields_ = [("aabb_min", c_f * 3), ("left_first", c_u32), ("aabb_max", c_f * 3), ("tri_count", c_u32)]


class Material(C.Structure):
    _fields_ = [("base_color", c_f * 4), ("base_weight", c_f), ("base_metalness", c_f),
                ("base_diffuse_roughness", c_f), ("emission_weight", c_f),
                ("emission_color_and_luminance", c_f * 4), ("specular_color_and_weight", c_f * 4),
                ("specular_roughness", c_f), ("specular_roughness_anisotropy", c_f), ("specular_haze", c_f),
                ("specular_haze_spread", c_f), ("specular_ior", c_f), ("specular_retroreflectivity", c_f),
                ("normal_scale", c_f), ("alpha_mode", c_u32), ("alpha_cutoff", c_f), ("pad", c_f),
                ("base_color_tex_layer", c_i32), ("normal_tex_layer", c_i32),
                ("metallic_roughness_tex_layer", c_i32), ("emission_tex_layer", c_i32),
                ("specular_color_tex_layer", c_i32), ("specular_weight_tex_layer", c_i32),
                ("base_color_uv", c_f * 4), ("normal_uv", c_f * 4), ("metallic_roughness_uv", c_f * 4),
                ("emission_uv", c_f * 4), ("specular_color_uv", c_f * 4), ("specular_weight_uv", c_f * 4)]


class Camera(C.Structure):
    _fields_ = [("position", c_f * 4), ("lower_left_corner_minus_position", c_f * 4),
                ("horizontal", c_f * 4), ("vertical", c_f * 4)]


class SceneUniforms(C.Structure):
    _fields_ = [("total_luminous_flux", c_f), ("emissive_triangles_count", c_u32),
                ("light_probabilities", c_f * 2)]


class SceneAliasEntry(C.Structure):
    _fields_ = [("threshold", c_f), ("alias_index", c_u32), ("triangle_index", c_u32),
                ("selection_probability", c_f)]


class SkyboxUniforms(C.Structure):
    _fields_ = [("total_luminous_flux", c_f), ("average_luminance", c_f), ("width", c_u32), ("height", c_u32)]


class SkyboxAliasEntry(C.Structure):
    _fields_ = [("threshold", c_f), ("alias_index", c_u32), ("selection_probability", c_f)]


class TraceParameters(C.Structure):
    _fields_ = [("image_size", c_u32 * 2), ("tile_origin", c_u32 * 2), ("max_bounces", c_u32),
                ("sample_count", c_u32), ("pad", c_u32 * 2)]


class SceneUpload(C.Structure):
    _fields_ = [("geometries", C.POINTER(TriangleGeometry)), ("attributes", C.POINTER(TriangleAttribute)),
                ("triangle_count", c_u64), ("materials", C.POINTER(Material)), ("material_count", c_u64),
                ("bvh_nodes", C.POINTER(BvhNode)), ("node_count", c_u64),
                ("srgb_texture_atlases", C.POINTER(C.c_uint8)), ("srgb_atlas_count", c_u32),
                ("linear_texture_atlases", C.POINTER(C.c_uint8)), ("linear_atlas_count", c_u32)]


class SkyboxUpload(C.Structure):
    _fields_ = [("rgba", C.POINTER(c_f)), ("uniforms", SkyboxUniforms),
                ("alias_table", C.POINTER(SkyboxAliasEntry)), ("alias_count", c_u64)]


class MaterialUpdate(C.Structure):
    _fields_ = [("index", c_u32), ("material", Material)]


class WorldUpdates(C.Structure):
    _fields_ = [("scene", C.POINTER(SceneUpload)), ("skybox", C.POINTER(SkyboxUpload)),
                ("camera", C.POINTER(Camera)), ("materials", C.POINTER(MaterialUpdate)),
                ("material_update_count", c_u64), ("scene_uniforms", C.POINTER(SceneUniforms)),
                ("scene_alias_table", C.POINTER(SceneAliasEntry)), ("scene_alias_count", c_u64),
                ("skybox_uniforms", C.POINTER(SkyboxUniforms)), ("reset_accumulation", c_i32)]


class PathRecord(C.Structure):
    _fields_ = [("visit_hash", c_u64), ("hit", c_i32 * PT_RECORD_MAX_BOUNCES), ("extend_rays", c_u32),
                ("shadow_rays", c_u32), ("interior_visits", c_u32), ("leaf_visits", c_u32),
                ("triangle_tests", c_u32), ("shadow_interior_visits", c_u32), ("shadow_leaf_visits", c_u32),
                ("shadow_triangle_tests", c_u32), ("rand_draws", c_u32), ("hits", c_u32), ("sky_misses", c_u32),
                ("light_samples", c_u32), ("sky_light_samples", c_u32), ("radiance", c_f * 3), ("pad", c_u32)]


class Mesh(C.Structure):
    _fields_ = [("positions", C.POINTER(c_f)), ("normals", C.POINTER(c_f)), ("uvs", C.POINTER(c_f)),
                ("tangents", C.POINTER(c_f)), ("vertex_count", c_u32), ("indices", C.POINTER(c_u32)),
                ("index_count", c_u32), ("material_index", c_u32)]


class ProceduralParams(C.Structure):
    _fields_ = [("seed", c_u64), ("grid_x", c_u32), ("grid_z", c_u32), ("boxes", c_u32), ("spheres", c_u32),
                ("sphere_subdivision", c_u32), ("emissive_triangles", c_u32), ("skybox_width", c_u32),
                ("skybox_height", c_u32), ("skybox_luminance", c_f), ("textured", c_i32), ("non_opaque", c_i32)]


class DeviceWorld(C.Structure):
    """pt_device_world: the world as device buffers owned by the caller."""
    _fields_ = [("geometries", C.c_void_p), ("attributes", C.c_void_p), ("triangle_count", c_u64),
                ("materials", C.c_void_p), ("material_count", c_u64), ("bvh_nodes", C.c_void_p),
                ("node_count", c_u64), ("srgb_texture_atlases", C.c_void_p), ("srgb_atlas_count", c_u32),
                ("linear_texture_atlases", C.c_void_p), ("linear_atlas_count", c_u32),
                ("skybox_rgba", C.c_void_p), ("skybox_aliases", C.c_void_p), ("scene_aliases", C.c_void_p),
                ("camera", Camera), ("scene_uniforms", SceneUniforms), ("skybox_uniforms", SkyboxUniforms),
                ("any_non_opaque", c_i32)]


class WideNode(C.Structure):
    """pt_wide_node: one 8-wide node of the precision form, 128 B."""
    _fields_ = [("origin", c_f * 3), ("exponent", C.c_uint8 * 3), ("child_count", C.c_uint8),
                ("lo", (C.c_uint8 * 8) * 3), ("hi", (C.c_uint8 * 8) * 3), ("child", c_u32 * 8),
                ("tri_count", C.c_uint16 * 8), ("source_node", c_u32), ("pad", c_u32 * 3)]


class HalfAttribute(C.Structure):
    """pt_half_attribute: FP16 shading attributes, 64 B."""
    _fields_ = [("n0", C.c_uint16 * 4), ("n1", C.c_uint16 * 4), ("n2", C.c_uint16 * 4), ("t0", C.c_uint16 * 4),
                ("t1", C.c_uint16 * 4), ("t2", C.c_uint16 * 4), ("uv0", C.c_uint16 * 2), ("uv1", C.c_uint16 * 2),
                ("uv2", C.c_uint16 * 2), ("material_index", c_u32)]


PT_NOALLOC_MAX_PATHS = 262144
PT_NOALLOC_SCRATCH_BYTES = 48 << 20

STRUCT_SIZES = {
    TriangleGeometry: 36, TriangleAttribute: 112, BvhNode: 32, Material: 224, Camera: 64,
    SceneUniforms: 16, SceneAliasEntry: 16, SkyboxUniforms: 16, SkyboxAliasEntry: 12,
    TraceParameters: 32, PathRecord: 144, WideNode: 128, HalfAttribute: 64, DeviceWorld: 216,
}

P = C.POINTER
_vp = C.c_void_p
# name: (restype, argtypes) of every entry point declared in include/pt.h, include/pt_precision.h
# and include/pt_world.h
SIGNATURES = {
    # pt.h
    "pt_create": (C.c_int, [C.c_int, P(WorldUpdates), c_u32, c_u32, P(_vp)]),
    "pt_destroy": (None, [_vp]),
    "pt_apply_updates": (C.c_int, [_vp, P(WorldUpdates)]),
    "pt_set_tile": (C.c_int, [_vp, P(c_u32), P(c_u32), P(c_u32)]),
    "pt_set_max_bounces": (C.c_int, [_vp, c_u32]),
    "pt_max_bounces": (c_u32, [_vp]),
    "pt_sample_count": (c_u32, [_vp]),
    "pt_trace": (C.c_int, [_vp, c_u32, P(c_u32)]),
    "pt_read_tile": (C.c_int, [_vp, C.c_int, _vp]),
    "pt_display_tile": (C.c_int, [_vp, _vp]),
    "pt_synchronize": (C.c_int, [_vp, c_u32]),
    "pt_last_error": (C.c_char_p, [_vp]),
    "pt_set_kernel": (C.c_int, [_vp, C.c_int]),
    "pt_get_stream": (C.c_int, [_vp, P(_vp)]),
    "pt_set_profiling": (C.c_int, [_vp, C.c_int]),
    "pt_get_kernel_times": (C.c_int, [_vp, P(c_u64), P(C.c_double)]),
    "pt_reset_kernel_times": (C.c_int, [_vp]),
    "pt_launch_count": (c_u64, [_vp]),
    "pt_trace_recorded": (C.c_int, [_vp, c_u32, P(c_u32), _vp]),
    "pt_trace_counted": (C.c_int, [_vp, c_u32, P(c_u32), P(c_u64)]),
    "pt_debug_intersect": (C.c_int, [_vp, c_u64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "pt_trace_noalloc": (C.c_int, [P(DeviceWorld), P(TraceParameters), c_u32, c_u32, c_u32, _vp, _vp, _vp,
                                   C.c_char_p, C.c_size_t]),
    # pt_precision.h
    "pt_build_wide_bvh": (C.c_int, [P(BvhNode), c_u64, c_u32, _vp, c_u64, P(c_u64), P(c_u32)]),
    "pt_half_attributes": (None, [P(TriangleAttribute), c_u64, _vp]),
    "pt_set_precision": (C.c_int, [_vp, c_u32]),
    "pt_precision": (c_u32, [_vp]),
    "pt_precision_active": (c_u32, [_vp]),
    "pt_render_fp64": (C.c_int, [_vp, c_u32, c_u32, _vp]),
    # pt_world.h
    "ptw_create": (C.c_int, [P(_vp)]),
    "ptw_destroy": (None, [_vp]),
    "ptw_last_error": (C.c_char_p, [_vp]),
    "ptw_default_material": (None, [P(Material)]),
    "ptw_add_material": (C.c_int, [_vp, P(Material), P(c_u32)]),
    "ptw_add_mesh": (C.c_int, [_vp, P(Mesh)]),
    "ptw_add_atlas_layer": (C.c_int, [_vp, C.c_int, _vp, P(c_i32)]),
    "ptw_load_gltf": (C.c_int, [_vp, C.c_char_p, C.c_char_p, C.c_size_t]),
    "ptw_load_gltf_bytes": (C.c_int, [_vp, _vp, C.c_size_t, C.c_char_p, C.c_size_t]),
    "ptw_set_skybox_bytes": (C.c_int, [_vp, _vp, C.c_size_t, C.c_char_p, C.c_size_t]),
    "ptw_edit_emission_scale": (C.c_int, [_vp, c_f]),
    "ptw_emission_scale": (c_f, [_vp]),
    "ptw_build": (C.c_int, [_vp]),
    "ptw_set_skybox_rgba": (C.c_int, [_vp, _vp, c_u32, c_u32]),
    "ptw_set_skybox_file": (C.c_int, [_vp, C.c_char_p, C.c_char_p, C.c_size_t]),
    "ptw_read_image_rgba": (C.c_int, [C.c_char_p, _vp, c_u64, P(c_u32), P(c_u32), C.c_char_p, C.c_size_t]),
    "ptw_write_image": (C.c_int, [C.c_char_p, _vp, c_u32, c_u32, C.c_char_p, C.c_size_t]),
    "ptw_decode_texture_rgba8": (C.c_int, [_vp, C.c_size_t, _vp, c_u64, P(c_u32), P(c_u32), C.c_char_p, C.c_size_t]),
    "ptw_set_procedural_skybox": (C.c_int, [_vp, c_u32, c_u32]),
    "ptw_edit_skybox_average_luminance": (C.c_int, [_vp, c_f]),
    "ptw_set_aspect_ratio": (C.c_int, [_vp, c_f]),
    "ptw_edit_camera": (C.c_int, [_vp, P(c_f), P(c_f), P(c_f), P(c_f)]),
    "ptw_edit_material": (C.c_int, [_vp, c_u32, P(Material)]),
    "ptw_take_updates": (C.c_int, [_vp, P(WorldUpdates)]),
    "ptw_triangle_count": (c_u64, [_vp]),
    "ptw_node_count": (c_u64, [_vp]),
    "ptw_material_count": (c_u64, [_vp]),
    "ptw_geometries": (P(TriangleGeometry), [_vp]),
    "ptw_attributes": (P(TriangleAttribute), [_vp]),
    "ptw_bvh_nodes": (P(BvhNode), [_vp]),
    "ptw_materials": (P(Material), [_vp]),
    "ptw_bvh_order": (P(c_u32), [_vp]),
    "ptw_bvh_max_depth": (c_u32, [_vp]),
    "ptw_alias_table": (c_u64, [_vp, c_u64, _vp]),
    "ptw_build_bvh": (c_u64, [_vp, c_u64, _vp, _vp]),
    "ptw_scene_cornell_box": (C.c_int, [P(_vp)]),
    "ptw_scene_cornell_box_textured": (C.c_int, [c_u64, P(_vp)]),
    "ptw_procedural_defaults": (None, [P(ProceduralParams)]),
    "ptw_scene_procedural": (C.c_int, [P(ProceduralParams), P(_vp)]),
}

_LIB: C.CDLL | None = None


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libpt.so (building it first if it is missing); raises if it cannot be loaded."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        if not build_if_missing:
            raise OSError(f"{path} is missing: run the build first")
        _build.build()
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


# ---------------------------------------------------------------- pt_batch.h

PT_JOB_QUEUED = 0
PT_JOB_RUNNING = 1
PT_JOB_DONE = 2


class EngineConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget_bytes", c_u64), ("wave_paths", c_u32), ("tile_size", c_u32),
                ("steps_per_refill", c_u32), ("use_graphs", c_u32), ("precision", c_u32), ("sort_min_hits", c_u32),
                ("traversal_threads", c_u32), ("shade_threads", c_u32)]


class JobDesc(C.Structure):
    _fields_ = [("scene_id", c_u64), ("camera", Camera), ("width", c_u32), ("height", c_u32),
                ("samples", c_u32), ("max_bounces", c_u32), ("continue_job", c_u64)]


class EngineStats(C.Structure):
    _fields_ = [("waves", c_u64), ("items", c_u64), ("paths", c_u64), ("jobs_submitted", c_u64),
                ("jobs_done", c_u64), ("scenes_cached", c_u64), ("scene_hits", c_u64), ("scenes_evicted", c_u64),
                ("hbm_used", c_u64), ("hbm_budget", c_u64), ("gpu_ms", C.c_double), ("wave_paths", c_u32),
                ("tile_size", c_u32), ("steps_per_refill", c_u32), ("use_graphs", c_u32), ("precision", c_u32),
                ("sort_min_hits", c_u32), ("traversal_threads", c_u32), ("shade_threads", c_u32)]


STRUCT_SIZES.update({EngineConfig: 48, JobDesc: 96, EngineStats: 120})


SIGNATURES.update({
    "pte_create": (C.c_int, [P(EngineConfig), P(_vp)]),
    "pte_destroy": (None, [_vp]),
    "pte_last_error": (C.c_char_p, [_vp]),
    "pte_scene_add": (C.c_int, [_vp, P(WorldUpdates), P(c_u64)]),
    "pte_scene_release": (C.c_int, [_vp, c_u64]),
    "pte_submit": (C.c_int, [_vp, P(JobDesc), P(c_u64)]),
    "pte_poll": (C.c_int, [_vp, c_u32, P(c_u64), c_u32, P(c_u32)]),
    "pte_wait_idle": (C.c_int, [_vp, c_u32]),
    "pte_job_status": (C.c_int, [_vp, c_u64, P(C.c_int), P(c_u32)]),
    "pte_job_read": (C.c_int, [_vp, c_u64, C.c_int, _vp]),
    "pte_job_release": (C.c_int, [_vp, c_u64]),
    "pte_stats": (C.c_int, [_vp, P(EngineStats)]),
    "pte_autotune": (C.c_int, [_vp, P(JobDesc), c_u32, P(EngineConfig)]),
})
