/*
 * oracle.h - C ABI of the CPU oracle of the path-trace compute pass.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library, and only
 * as the checker or as the timed CPU baseline - never as the product path.
 *
 * PARITY UNPINNED: the reference (Rust + Slang compiled to WGSL, run through
 * wgpu) cannot be built or run here and ships no golden vectors or tests of
 * this path, so the oracle is a line-by-line C++ restatement of
 * src/render/trace.slang and is pinned only by self-derived known answers
 * (RNG sequence, BVH and alias tables, transcendental accuracy).
 */
#ifndef PT_ORACLE_H
#define PT_ORACLE_H

#include "../include/pt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* the world as the trace pass sees it (bind group 1, trace.slang:163-190) */
typedef struct oracle_world {
    const pt_triangle_geometry* geometries;
    const pt_triangle_attribute* attributes;
    uint64_t triangle_count;
    const pt_material* materials;
    uint64_t material_count;
    const pt_bvh_node* bvh_nodes;
    uint64_t node_count;
    const uint8_t* srgb_atlases;
    uint32_t srgb_atlas_count;
    const uint8_t* linear_atlases;
    uint32_t linear_atlas_count;
    pt_camera camera;
    const float* skybox_rgba;
    pt_skybox_uniforms skybox;
    const pt_skybox_alias_entry* skybox_aliases;
    uint64_t skybox_alias_count;
    pt_scene_uniforms scene;
    const pt_scene_alias_entry* scene_aliases;
    uint64_t scene_alias_count;
} oracle_world;

#define ORACLE_FP32 32 /* parity mode: FP32, same bits as the CUDA kernels */
#define ORACLE_FP64 64 /* reference render: FP64 arithmetic, libm functions */

/* Traces sample_count samples (1-based sample indices sample_first ..) of the
 * given pixels (absolute image coordinates, 2 x uint32 each), one
 * compute_main invocation each (trace.slang:721-1297).  Outputs, any may be
 * NULL: radiance32 [sample][pixel][3] (FP32 mode), radiance64 (either mode,
 * widened), records [sample][pixel].  threads <= 0 uses all cores.
 * Returns 0, or -1 on bad arguments. */
int oracle_trace_paths(const oracle_world* world, const uint32_t image_size[2], uint32_t max_bounces,
                       const uint32_t* pixels, uint64_t pixel_count, uint32_t sample_first,
                       uint32_t sample_count, int precision, int threads, float* radiance32,
                       double* radiance64, pt_path_record* records);

/* closest-hit traversal of opaque rays (trace.slang:764-884) in FP32 */
int oracle_intersect(const oracle_world* world, uint64_t n, const float* origins, const float* directions,
                     const float* t_max, int32_t* hit, float* hit_t, pt_path_record* records);

/* the shader's rand() (trace.slang:195-202) from a state, `count` draws */
void oracle_rand_sequence(uint32_t state, uint32_t count, float* out);
/* the seed of compute_main (trace.slang:736-737) */
uint32_t oracle_seed(uint32_t px, uint32_t py, uint32_t sample_count);

/* Elementary operations of the FP32 parity mode, n elements each (vectors
 * are 3 floats): the semantic choices the restatement makes where WGSL
 * leaves them to the implementation, exposed for the pin tests. */
#define ORACLE_OP_NORMALIZE 0 /* a -> out (3)                                */
#define ORACLE_OP_DOT 1       /* a, b -> out                                 */
#define ORACLE_OP_MIX 2       /* a, b, c -> out                              */
#define ORACLE_OP_REFLECT 3   /* a (incident), b (normal) -> out (3)         */
#define ORACLE_OP_FRACT 4
#define ORACLE_OP_MIN 5
#define ORACLE_OP_MAX 6
#define ORACLE_OP_CLAMP 7     /* clamp(a, b, c)                              */
#define ORACLE_OP_RSQRT 8
#define ORACLE_OP_TO_U32 9    /* out holds the uint32 bits                   */
#define ORACLE_OP_SRGB 10     /* a = byte value -> decoded sRGB channel      */
#define ORACLE_OP_SLAB 11     /* a = box (6), b = origin + direction (6), c = hit_t -> intersect_aabb */
#define ORACLE_OP_CAMERA_RAY 12 /* a = pt_camera (16), b = px, py, width, height, c = RNG state bits -> direction (3) */
int oracle_elementary(int op, uint64_t n, const float* a, const float* b, const float* c, float* out);

/* One shading point of trace.slang:1097-1181 from its material inputs (after
 * texture fetches) and wo in the shading frame; rng is the state before
 * estimate_e_dielectric's 32 draws. */
typedef struct oracle_shade_case {
    float base_color[3], base_weight, base_metalness, base_diffuse_roughness;
    float specular_color[3], specular_weight, specular_roughness, specular_anisotropy, specular_ior;
    float wo[3], wi[3];
    uint32_t rng;
} oracle_shade_case;

/* E_dielectric, p_ggx, P_u, evaluate_lobes at case.wi, then a BSDF sample
 * (trace.slang:1212-1260, the next 3 draws) and evaluate_lobes at it. */
typedef struct oracle_shade_result {
    double e_dielectric[3], p_ggx, p_u, f[3], pdf, sampled_wi[3], sampled_f[3], sampled_pdf;
    uint32_t rng_after, pad;
} oracle_shade_result;
int oracle_shade_cases(int precision, const oracle_shade_case* cases, uint64_t n, oracle_shade_result* out);

/* sample_light (trace.slang:531-592) from each origin with its RNG state */
typedef struct oracle_light_result {
    double direction[3], distance, emission[3], pdf;
    int32_t triangle_index;
    uint32_t rng_after;
} oracle_light_result;
int oracle_sample_lights(const oracle_world* world, int precision, uint64_t n, const float* origins,
                         const uint32_t* rng_states, oracle_light_result* out);

/* FP32 transcendental functions shared with the kernels, for accuracy tests */
void oracle_fmath(int which, const float* x, const float* y, float* out, uint64_t n);

/* number of OpenMP threads the oracle would use */
int oracle_max_threads(void);

#ifdef __cplusplus
}
#endif

#endif
