/*
 * pt.h - C ABI of the GB300 path-trace compute pass.
 *
 * This is the drop-in boundary for the reference's trace dispatch
 * (src/render/path_tracer.rs + src/render/world_resources.rs driving
 * src/render/trace.slang).  Every struct below is byte-identical to the
 * reference's `#[repr(C)] bytemuck::Pod` GPU structs, so a host that already
 * builds those buffers (the reference's Rust world builder) can pass them
 * through unchanged.  Sizes and offsets are checked with static asserts in
 * path-tracer_gb300/csrc/pt_layout_check.cpp.
 *
 * Conventions
 *   - every entry point returns an int status (PT_OK on success) and never
 *     aborts; the message of the last failure is pt_last_error(ctx)
 *     (replaces the anyhow::ensure! errors of path_tracer.rs:294-297,361-382
 *     and world_resources.rs:607-642);
 *   - host pointers passed in are borrowed for the duration of the call only
 *     and copied to device memory owned by the context;
 *   - one context = one CUDA stream; a context is not thread-safe (the
 *     reference drives its PathTracer from one thread, headless.rs:130-133).
 */
#ifndef PT_H
#define PT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
#define PT_OK 0
#define PT_ERR_INVALID_ARG 1   /* argument outside its documented range      */
#define PT_ERR_OUT_OF_LIMITS 2 /* tile/world larger than the device limits    */
#define PT_ERR_OOM 3           /* device allocation failed                    */
#define PT_ERR_CUDA 4          /* a CUDA call failed                          */
#define PT_ERR_TIMEOUT 5       /* a bounded wait gave up                      */
#define PT_ERR_STATE 6         /* call not valid in the context's state       */

/* ------------------------------------------------------ GPU buffer layouts */

/* GpuTriangleGeometry, world.rs:139-146; TriangleGeometry trace.slang:48-56. 36 B */
typedef struct pt_triangle_geometry {
    float v0[3];
    float v1[3];
    float v2[3];
} pt_triangle_geometry;

/* GpuTriangleAttribute, world.rs:155-182; TriangleAttribute trace.slang:57-66. 112 B */
typedef struct pt_triangle_attribute {
    uint32_t material_index;
    float n0[3], n1[3], n2[3];
    float uv0[2], uv1[2], uv2[2];
    float t0[4], t1[4], t2[4];
} pt_triangle_attribute;

/* GpuBvhNode, world.rs:323-335; BvhNode trace.slang:68-73. 32 B.
 * Interior node: tri_count == 0, children at left_first and left_first + 1.
 * Leaf: triangles [left_first, left_first + tri_count). */
typedef struct pt_bvh_node {
    float aabb_min[3];
    uint32_t left_first;
    float aabb_max[3];
    uint32_t tri_count;
} pt_bvh_node;

/* alpha modes, world.rs:32-36 */
#define PT_ALPHA_MODE_OPAQUE 0u
#define PT_ALPHA_MODE_MASK 1u
#define PT_ALPHA_MODE_BLEND 2u

/* GpuMaterial, world.rs:199-309; Material trace.slang:76-106. 224 B.
 * Field names follow the shader (OpenPBR names). */
typedef struct pt_material {
    float base_color[4];
    float base_weight;
    float base_metalness;
    float base_diffuse_roughness;
    float emission_weight;
    float emission_color_and_luminance[4];
    float specular_color_and_weight[4];
    float specular_roughness;
    float specular_roughness_anisotropy;
    float specular_haze;
    float specular_haze_spread;
    float specular_ior;
    float specular_retroreflectivity;
    float normal_scale;
    uint32_t alpha_mode;
    float alpha_cutoff;
    float pad;
    int32_t base_color_tex_layer;
    int32_t normal_tex_layer;
    int32_t metallic_roughness_tex_layer;
    int32_t emission_tex_layer;
    int32_t specular_color_tex_layer;
    int32_t specular_weight_tex_layer;
    float base_color_uv[4];
    float normal_uv[4];
    float metallic_roughness_uv[4];
    float emission_uv[4];
    float specular_color_uv[4];
    float specular_weight_uv[4];
} pt_material;

/* GpuCamera, world.rs:389-398; Camera trace.slang:112-117. 64 B (w unused) */
typedef struct pt_camera {
    float position[4];
    float lower_left_corner_minus_position[4];
    float horizontal[4];
    float vertical[4];
} pt_camera;

/* GpuSceneUniforms, world.rs:476-482; SceneUniforms trace.slang:119-123. 16 B */
typedef struct pt_scene_uniforms {
    float total_luminous_flux;
    uint32_t emissive_triangles_count;
    float light_probabilities[2]; /* triangle lights, skybox */
} pt_scene_uniforms;

/* GpuSceneAliasEntry, world.rs:503-510. 16 B. Live prefix = emissive_triangles_count,
 * sorted by increasing triangle_index (world.rs:1695-1732). */
typedef struct pt_scene_alias_entry {
    float threshold;
    uint32_t alias_index;
    uint32_t triangle_index;
    float selection_probability;
} pt_scene_alias_entry;

/* GpuSkyboxUniforms, world.rs:522-529. 16 B */
typedef struct pt_skybox_uniforms {
    float total_luminous_flux;
    float average_luminance;
    uint32_t width;
    uint32_t height;
} pt_skybox_uniforms;

/* GpuSkyboxAliasEntry, world.rs:533-537. 12 B */
typedef struct pt_skybox_alias_entry {
    float threshold;
    uint32_t alias_index;
    float selection_probability;
} pt_skybox_alias_entry;

/* GpuTraceParameters, path_tracer.rs:45-57; TraceParameters trace.slang:146-152. 32 B */
typedef struct pt_trace_parameters {
    uint32_t image_size[2];
    uint32_t tile_origin[2];
    uint32_t max_bounces;
    uint32_t sample_count;
    uint32_t pad[2];
} pt_trace_parameters;

/* ------------------------------------------------------------ world upload */

/* texture atlas side, world.rs:29; each atlas layer is RGBA8, row-major */
#define PT_ATLAS_SIZE 8192u

/* SceneUpload, world.rs:87-94 */
typedef struct pt_scene_upload {
    const pt_triangle_geometry* geometries;   /* triangle_count entries, BVH order */
    const pt_triangle_attribute* attributes;  /* triangle_count entries         */
    uint64_t triangle_count;
    const pt_material* materials;
    uint64_t material_count;
    const pt_bvh_node* bvh_nodes;
    uint64_t node_count;
    const uint8_t* srgb_texture_atlases;      /* srgb_atlas_count layers        */
    uint32_t srgb_atlas_count;
    const uint8_t* linear_texture_atlases;    /* linear_atlas_count layers      */
    uint32_t linear_atlas_count;
} pt_scene_upload;

/* SkyboxUpload, world.rs:97-101 */
typedef struct pt_skybox_upload {
    const float* rgba;                        /* width * height * 4, row-major, top row first */
    pt_skybox_uniforms uniforms;
    const pt_skybox_alias_entry* alias_table; /* 0 or width * height entries    */
    uint64_t alias_count;
} pt_skybox_upload;

/* one (index, GpuMaterial) pair of WorldUpdates::materials */
typedef struct pt_material_update {
    uint32_t index;
    pt_material material;
} pt_material_update;

/* WorldUpdates, world.rs:75-84.  A NULL pointer means "unchanged". */
typedef struct pt_world_updates {
    const pt_scene_upload* scene;
    const pt_skybox_upload* skybox;
    const pt_camera* camera;
    const pt_material_update* materials;
    uint64_t material_update_count;
    const pt_scene_uniforms* scene_uniforms;
    const pt_scene_alias_entry* scene_alias_table; /* live prefix; NULL = unchanged */
    uint64_t scene_alias_count;
    const pt_skybox_uniforms* skybox_uniforms;
    int32_t reset_accumulation;
} pt_world_updates;

/* ----------------------------------------------------------------- context */

typedef struct pt_ctx pt_ctx;

/* PathTracer::DEFAULT_MAX_BOUNCES / MAX_BOUNCES_LIMIT / MAX_SAMPLES_PER_TRACE, path_tracer.rs:61-66 */
#define PT_DEFAULT_MAX_BOUNCES 10u
#define PT_MAX_BOUNCES_LIMIT 16u
#define PT_MAX_SAMPLES_PER_TRACE 16u

/* kernel organisation used by pt_trace */
#define PT_KERNEL_WAVEFRONT 0 /* raygen / extend / shade / shadow / accumulate queues (default) */
#define PT_KERNEL_PLAIN 1     /* one thread per pixel, one launch per sample */

/* PathTracer::new, path_tracer.rs:69-251.  `updates` must carry a full upload
 * (scene, skybox, camera, scene uniforms, scene alias table, skybox uniforms),
 * as the reference's WorldBindings::new requires (world_resources.rs:395-474).
 * The tile covers [0, tile) of an image of the same size until pt_set_tile. */
int pt_create(int device, const pt_world_updates* updates, uint32_t tile_width,
              uint32_t tile_height, pt_ctx** out);
void pt_destroy(pt_ctx* ctx);

/* PathTracer::apply_updates, path_tracer.rs:272-282: applies partial or full
 * updates; resets accumulation when updates->reset_accumulation != 0. */
int pt_apply_updates(pt_ctx* ctx, const pt_world_updates* updates);

/* PathTracer::set_tile, path_tracer.rs:287-313.  Errors with
 * PT_ERR_INVALID_ARG if the origin lies outside the image; reallocates the
 * tile buffers if the size changes; always resets the sample count. */
int pt_set_tile(pt_ctx* ctx, const uint32_t image_size[2], const uint32_t origin[2],
                const uint32_t size[2]);

/* PathTracer::set_max_bounces / max_bounces, path_tracer.rs:259-269.  Values
 * above PT_MAX_BOUNCES_LIMIT are rejected (the CLI range, headless.rs:43-48). */
int pt_set_max_bounces(pt_ctx* ctx, uint32_t max_bounces);
uint32_t pt_max_bounces(const pt_ctx* ctx);

/* PathTracer::sample_count, path_tracer.rs:254-256 */
uint32_t pt_sample_count(const pt_ctx* ctx);

/* PathTracer::trace, path_tracer.rs:316-351: traces min(sample_count,
 * PT_MAX_SAMPLES_PER_TRACE) samples of every tile pixel inside the image,
 * writing *traced.  Work is queued on the context stream; the call does not
 * wait for it (pt_synchronize does). */
int pt_trace(pt_ctx* ctx, uint32_t sample_count, uint32_t* traced);

/* which buffer pt_read_tile copies out (tile_w * tile_h * 4 floats, row stride tile_w) */
#define PT_TILE_IMAGE 0        /* storage texture: EXPOSURE * sum / n, alpha 1 (trace.slang:1308) */
#define PT_TILE_ACCUMULATION 1 /* accumulation buffer: running sum, w = 1 (trace.slang:1305)    */
int pt_read_tile(pt_ctx* ctx, int which, float* host_rgba);

/* PathTracer::display + TileReadback::read (path_tracer.rs:354-358,
 * headless.rs:330-384): ACES-fit tonemap and sRGB OETF of the storage texture
 * (display.wgsl:19-46) into tile_w * tile_h RGBA8 pixels. */
int pt_display_tile(pt_ctx* ctx, uint8_t* host_rgba8);

/* wait for all queued work; PT_ERR_TIMEOUT if it does not finish within
 * timeout_ms (0 = wait without a limit) */
int pt_synchronize(pt_ctx* ctx, uint32_t timeout_ms);

const char* pt_last_error(const pt_ctx* ctx);

/* select PT_KERNEL_WAVEFRONT or PT_KERNEL_PLAIN; both give identical bits */
int pt_set_kernel(pt_ctx* ctx, int kernel);

/* the cudaStream_t the context launches on (for CUDA-event timing by callers).
 * The wavefront kernels of a pt_trace run on streams of the library that
 * join this one: work queued here after a pt_trace call runs after that
 * call's samples are accumulated. */
int pt_get_stream(pt_ctx* ctx, void** stream);

/* --------------------------------------------------------- instrumentation */

/* per-kernel timing with CUDA events (0 = off).  While it is on, the
 * wavefront stages of pt_trace run one after another (consecutive groups and
 * a bounce's shadow stage otherwise overlap), so each kernel's time is its
 * own; the total time of a trace is then longer than with profiling off. */
#define PT_KERNEL_CLASS_COUNT 7
#define PT_KC_RAYGEN 0
#define PT_KC_EXTEND 1
#define PT_KC_SHADE 2
#define PT_KC_SHADOW 3
#define PT_KC_ACCUMULATE 4
#define PT_KC_PLAIN 5
#define PT_KC_SORT 6 /* ray and hit ordering of the wavefront method */
int pt_set_profiling(pt_ctx* ctx, int enabled);
/* per class: launches and summed milliseconds since the last reset */
int pt_get_kernel_times(pt_ctx* ctx, uint64_t launches[PT_KERNEL_CLASS_COUNT],
                        double milliseconds[PT_KERNEL_CLASS_COUNT]);
int pt_reset_kernel_times(pt_ctx* ctx);
/* number of kernels this context has launched since creation */
uint64_t pt_launch_count(const pt_ctx* ctx);

#define PT_RECORD_MAX_BOUNCES 17
/* Per-path record written by pt_trace_recorded.  Counters cover every
 * traversal of the path (extend and shadow); visit_hash is FNV-1a (64 bit)
 * over the node indices fetched at trace.slang:793 and :637, in path order. */
typedef struct pt_path_record {
    uint64_t visit_hash;
    int32_t hit[PT_RECORD_MAX_BOUNCES]; /* closest-hit triangle per bounce; -1 miss; -2 not reached */
    uint32_t extend_rays;
    uint32_t shadow_rays;
    uint32_t interior_visits;           /* interior nodes fetched (each tests 2 children), all traversals */
    uint32_t leaf_visits;
    uint32_t triangle_tests;
    uint32_t shadow_interior_visits;    /* the part of the three counters above spent in shadow rays */
    uint32_t shadow_leaf_visits;
    uint32_t shadow_triangle_tests;
    uint32_t rand_draws;
    uint32_t hits;                      /* extend rays that hit a triangle */
    uint32_t sky_misses;                /* extend rays that escaped */
    uint32_t light_samples;             /* sample_light calls that drew a triangle light */
    uint32_t sky_light_samples;         /* sample_light calls that drew the skybox */
    float radiance[3];                  /* final_color of this sample */
    uint32_t pad;
} pt_path_record;                       /* 144 B */

/* totals over every path of a pt_trace_counted call, in this order */
#define PT_COUNT_FIELDS 13
#define PT_COUNT_EXTEND_RAYS 0
#define PT_COUNT_SHADOW_RAYS 1
#define PT_COUNT_INTERIOR_VISITS 2
#define PT_COUNT_LEAF_VISITS 3
#define PT_COUNT_TRIANGLE_TESTS 4
#define PT_COUNT_SHADOW_INTERIOR_VISITS 5
#define PT_COUNT_SHADOW_LEAF_VISITS 6
#define PT_COUNT_SHADOW_TRIANGLE_TESTS 7
#define PT_COUNT_RAND_DRAWS 8
#define PT_COUNT_HITS 9
#define PT_COUNT_SKY_MISSES 10
#define PT_COUNT_LIGHT_SAMPLES 11
#define PT_COUNT_SKY_LIGHT_SAMPLES 12
/* Like pt_trace, with the counting kernel variants: adds the pt_path_record
 * counters of every traced path into totals[PT_COUNT_FIELDS] (not cleared). */
int pt_trace_counted(pt_ctx* ctx, uint32_t sample_count, uint32_t* traced, uint64_t totals[PT_COUNT_FIELDS]);

/* Like pt_trace, but with the recording kernel variants; writes
 * traced * tile_w * tile_h records to host_records, sample-major
 * ([sample][tile_y][tile_x]); pixels outside the image are zeroed. */
int pt_trace_recorded(pt_ctx* ctx, uint32_t sample_count, uint32_t* traced,
                      pt_path_record* host_records);

/* Closest-hit traversal (trace.slang:764-884) of n opaque rays given on the
 * host: origins and directions are 3 floats each, t_max the initial hit_t.
 * Writes the hit triangle (-1 = miss), the hit t, and the record fields
 * visit_hash, interior_visits, leaf_visits, triangle_tests of each ray.
 * With PT_PRECISION_WIDE_BVH selected (include/pt_precision.h), an opaque
 * world and records == NULL, the rays traverse the 8-wide BVH instead. */
int pt_debug_intersect(pt_ctx* ctx, uint64_t n, const float* origins, const float* directions,
                       const float* t_max, int32_t* hit, float* hit_t, pt_path_record* records);

/* ------------------------------------------------- allocation-free tracing */

/* The world as device buffers the caller already owns: the same layouts as
 * pt_scene_upload / pt_skybox_upload, but every pointer is a device address. */
typedef struct pt_device_world {
    const pt_triangle_geometry* geometries;   /* triangle_count entries */
    const pt_triangle_attribute* attributes;  /* triangle_count entries */
    uint64_t triangle_count;
    const pt_material* materials;
    uint64_t material_count;
    const pt_bvh_node* bvh_nodes;             /* 32-byte aligned (each node is one 32-byte load) */
    uint64_t node_count;
    const uint8_t* srgb_texture_atlases;      /* srgb_atlas_count layers, may be NULL if 0 */
    uint32_t srgb_atlas_count;
    const uint8_t* linear_texture_atlases;
    uint32_t linear_atlas_count;
    const float* skybox_rgba;                 /* width * height RGBA32F, 16-byte aligned */
    const pt_skybox_alias_entry* skybox_aliases;
    const pt_scene_alias_entry* scene_aliases;
    pt_camera camera;
    pt_scene_uniforms scene_uniforms;
    pt_skybox_uniforms skybox_uniforms;
    int32_t any_non_opaque;                   /* 1 if some material is not PT_ALPHA_MODE_OPAQUE */
} pt_device_world;

/* largest (visible tile pixels x samples) one pt_trace_noalloc call accepts */
#define PT_NOALLOC_MAX_PATHS 262144u
/* size of the library's static device scratch array (every GPU that loads
 * the library holds it until the process exits) */
#define PT_NOALLOC_SCRATCH_BYTES (48u << 20)

/* No counterpart in the reference: an extra entry point for callers that
 * cannot allocate device memory themselves or through this library - for
 * example a host application whose allocator owns all device memory and
 * hands plug-ins ready-made buffers, or a latency-critical render thread that
 * must not hit the device-wide synchronisation of cudaMalloc / cudaFree.
 *
 * Traces `samples` samples of one tile with the wavefront kernels and adds
 * them to the caller's accumulation buffer, exactly like pt_trace (same
 * bits), but allocates nothing: the world, `accum` and `image` (tile_width *
 * tile_height * 4 floats each, row stride tile_width, 16-byte aligned) are
 * the caller's device buffers, the queues live in a static device array of
 * PT_NOALLOC_SCRATCH_BYTES, and at most PT_NOALLOC_MAX_PATHS paths are
 * accepted per call (larger requests fail with PT_ERR_OUT_OF_LIMITS; split
 * them into several calls or tiles).  params->sample_count is the number of
 * samples already in `accum` (0 starts a new accumulation); image_size,
 * tile_origin and max_bounces mean what they mean for pt_set_tile and
 * pt_set_max_bounces.  Work is queued on `stream` (a cudaStream_t of the
 * current device; NULL = legacy default stream) and the call returns without
 * waiting.
 *
 * The first call on each device sets up the scratch array on that device
 * (looks up its device address and uploads a 1 KB sRGB table, a synchronous
 * copy); make that first call before any stream capture.  Every call on a
 * device shares the one scratch array, which keeps the previous call's
 * contents: calls that overlap on the GPU (different streams or threads
 * without ordering) race and corrupt each other.  The world is not
 * validated, so it must be a world pt_apply_updates would accept.  If
 * `error` is not NULL, a failure message is written there (at most
 * error_size bytes, NUL-terminated). */
int pt_trace_noalloc(const pt_device_world* world, const pt_trace_parameters* params, uint32_t tile_width,
                     uint32_t tile_height, uint32_t samples, float* accum, float* image, void* stream,
                     char* error, size_t error_size);

#ifdef __cplusplus
}
#endif

#endif /* PT_H */
