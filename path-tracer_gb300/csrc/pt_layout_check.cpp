// pt_layout_check.cpp - compile-time proof that the C ABI structs match the
// byte layouts of the reference's bytemuck GPU structs (world.rs:139-537,
// path_tracer.rs:45-57) and the shader's structs (trace.slang:48-152).
#include <cstddef>

#include "../../include/pt.h"
#include "../../include/pt_batch.h"

#define CHECK_SIZE(T, n) static_assert(sizeof(T) == (n), #T " size")
#define CHECK_OFF(T, f, n) static_assert(offsetof(T, f) == (n), #T "." #f " offset")

CHECK_SIZE(pt_triangle_geometry, 36);
CHECK_SIZE(pt_triangle_attribute, 112);
CHECK_OFF(pt_triangle_attribute, n0, 4);
CHECK_OFF(pt_triangle_attribute, uv0, 40);
CHECK_OFF(pt_triangle_attribute, t0, 64);
CHECK_OFF(pt_triangle_attribute, t2, 96);
CHECK_SIZE(pt_bvh_node, 32);
CHECK_OFF(pt_bvh_node, left_first, 12);
CHECK_OFF(pt_bvh_node, aabb_max, 16);
CHECK_OFF(pt_bvh_node, tri_count, 28);
CHECK_SIZE(pt_material, 224);
CHECK_OFF(pt_material, base_weight, 16);
CHECK_OFF(pt_material, emission_weight, 28);
CHECK_OFF(pt_material, emission_color_and_luminance, 32);
CHECK_OFF(pt_material, specular_color_and_weight, 48);
CHECK_OFF(pt_material, specular_roughness, 64);
CHECK_OFF(pt_material, specular_ior, 80);
CHECK_OFF(pt_material, normal_scale, 88);
CHECK_OFF(pt_material, alpha_mode, 92);
CHECK_OFF(pt_material, alpha_cutoff, 96);
CHECK_OFF(pt_material, base_color_tex_layer, 104);
CHECK_OFF(pt_material, specular_weight_tex_layer, 124);
CHECK_OFF(pt_material, base_color_uv, 128);
CHECK_OFF(pt_material, specular_color_uv, 192);
CHECK_OFF(pt_material, specular_weight_uv, 208);
CHECK_SIZE(pt_camera, 64);
CHECK_SIZE(pt_scene_uniforms, 16);
CHECK_SIZE(pt_scene_alias_entry, 16);
CHECK_SIZE(pt_skybox_uniforms, 16);
CHECK_SIZE(pt_skybox_alias_entry, 12);
CHECK_SIZE(pt_trace_parameters, 32);
CHECK_SIZE(pt_path_record, 144);
// the upload descriptors (64-bit pointers), mirrored by the Rust binding include/pt_ffi.rs
CHECK_SIZE(pt_scene_upload, 88);
CHECK_OFF(pt_scene_upload, srgb_atlas_count, 64);
CHECK_OFF(pt_scene_upload, linear_atlas_count, 80);
CHECK_SIZE(pt_skybox_upload, 40);
CHECK_OFF(pt_skybox_upload, alias_table, 24);
CHECK_SIZE(pt_material_update, 228);
CHECK_OFF(pt_material_update, material, 4);
CHECK_SIZE(pt_world_updates, 80);
CHECK_OFF(pt_world_updates, material_update_count, 32);
CHECK_OFF(pt_world_updates, skybox_uniforms, 64);
CHECK_OFF(pt_world_updates, reset_accumulation, 72);
// the caller-owned device world of pt_trace_noalloc (64-bit pointers)
CHECK_SIZE(pt_device_world, 216);
CHECK_OFF(pt_device_world, triangle_count, 16);
CHECK_OFF(pt_device_world, bvh_nodes, 40);
CHECK_OFF(pt_device_world, srgb_atlas_count, 64);
CHECK_OFF(pt_device_world, linear_texture_atlases, 72);
CHECK_OFF(pt_device_world, skybox_rgba, 88);
CHECK_OFF(pt_device_world, camera, 112);
CHECK_OFF(pt_device_world, scene_uniforms, 176);
CHECK_OFF(pt_device_world, skybox_uniforms, 192);
CHECK_OFF(pt_device_world, any_non_opaque, 208);
// the batched engine's structs, mirrored by the Python binding
CHECK_SIZE(pt_engine_config, 48);
CHECK_OFF(pt_engine_config, hbm_budget_bytes, 8);
CHECK_OFF(pt_engine_config, traversal_threads, 40);
CHECK_OFF(pt_engine_config, shade_threads, 44);
CHECK_SIZE(pt_job_desc, 96);
CHECK_OFF(pt_job_desc, continue_job, 88);
CHECK_SIZE(pt_engine_stats, 120);
CHECK_OFF(pt_engine_stats, gpu_ms, 80);
CHECK_OFF(pt_engine_stats, shade_threads, 116);

extern "C" int pt_layout_checked(void) { return 1; }
