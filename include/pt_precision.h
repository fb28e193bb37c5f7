/*
 * pt_precision.h - the compressed ("precision") form of the trace pass.
 *
 * No counterpart in the reference: its trace pass (src/render/trace.slang)
 * reads the 32-byte binary BVH nodes (world.rs:323-335), the 112-byte FP32
 * triangle attributes (world.rs:155-182) and the RGBA32F skybox
 * (world_resources.rs:451-456), and accumulates radiance with plain FP32
 * sums (trace.slang:1299-1305).  The precision form keeps every input of the
 * reference (the caller still uploads exactly those buffers) and derives
 * narrower copies on the device:
 *
 *   PT_PRECISION_WIDE_BVH   8-wide BVH collapsed from the caller's binary BVH;
 *                           child boxes quantised to 8 bits per coordinate
 *                           relative to a per-node FP32 frame and rounded
 *                           outward, so a box test never rejects a ray the
 *                           binary node's test accepts.  Traversal arithmetic
 *                           stays FP32 and uses the reference's watertight
 *                           triangle test, so each ray's closest hit (triangle,
 *                           t, barycentrics) is the binary traversal's; exact-t
 *                           ties go to the triangle the binary traversal
 *                           reaches first (decided from the binary tree's
 *                           parent links).  For a ray with a zero direction
 *                           component the reference's slab test is not a
 *                           bound (0 * inf); the wide test then returns the
 *                           same hit or a nearer one, never a farther one.
 *   PT_PRECISION_HALF_ATTRIBUTES  shading normals, tangents and UVs stored as
 *                           FP16 (64 B per triangle instead of 112 B) and
 *                           skybox texels as BF16 (8 B instead of 16 B).
 *   PT_PRECISION_KAHAN      per-pixel radiance sums with Kahan compensation.
 *
 * The precision form runs on the wavefront kernels, for scenes whose
 * materials are all opaque (non-opaque materials draw random numbers in
 * traversal order, trace.slang:446-454, which the wide order would change;
 * such scenes keep the binary traversal and report it through
 * pt_precision_active).
 */
#ifndef PT_PRECISION_H
#define PT_PRECISION_H

#include "pt.h"

#ifdef __cplusplus
extern "C" {
#endif

#define PT_PRECISION_FP32 0u
#define PT_PRECISION_WIDE_BVH 1u
#define PT_PRECISION_HALF_ATTRIBUTES 2u
#define PT_PRECISION_KAHAN 4u
#define PT_PRECISION_COMPRESSED 7u /* all three */

/* One 8-wide node, 128 B (one L2 line).  Child i < child_count has the box
 *   lo[a][i] decoded as origin[a] + lo[a][i] * 2^(exponent[a] - 127)
 *   hi[a][i] decoded as origin[a] + hi[a][i] * 2^(exponent[a] - 127)
 * with the product exact and one FP32 round-to-nearest addition; every
 * decoded box contains the binary node it stands for.  tri_count[i] == 0
 * marks an interior child (child[i] = its wide node index); otherwise the
 * child is a binary leaf, or a merged binary subtree, with triangles
 * [child[i], child[i] + tri_count[i]). */
typedef struct pt_wide_node {
    float origin[3];
    uint8_t exponent[3];
    uint8_t child_count;
    uint8_t lo[3][8];
    uint8_t hi[3][8];
    uint32_t child[8];
    uint16_t tri_count[8];
    uint32_t source_node; /* binary node this wide node was collapsed from */
    uint32_t pad[3];
} pt_wide_node;

/* Per-triangle shading attributes in FP16, 64 B (IEEE binary16 bit patterns,
 * round to nearest even from the FP32 attributes). */
typedef struct pt_half_attribute {
    uint16_t n0[4], n1[4], n2[4]; /* xyz, 0 */
    uint16_t t0[4], t1[4], t2[4]; /* xyzw   */
    uint16_t uv0[2], uv1[2], uv2[2];
    uint32_t material_index;
} pt_half_attribute;

/* Collapse a binary BVH (the reference's layout, root at 0) into 8-wide
 * nodes: each wide node starts from a binary interior node's two children
 * and repeatedly opens its interior child of largest surface area until it
 * has 8 children or only leaves.  The children are placed in slots so that
 * a ray visiting slot i ^ o (i = 0..7, o = its direction's sign bits) meets
 * them roughly nearest first.  A binary subtree of at most
 * max_leaf_triangles triangles (0: none) becomes one leaf child over its
 * contiguous triangle range.  Runs on the host.  `out` may be NULL to query
 * the count.  PT_ERR_INVALID_ARG for a malformed tree, non-finite boxes or
 * a leaf of more than 65535 triangles; PT_ERR_OUT_OF_LIMITS if `capacity`
 * is too small. */
int pt_build_wide_bvh(const pt_bvh_node* nodes, uint64_t node_count, uint32_t max_leaf_triangles,
                      pt_wide_node* out, uint64_t capacity, uint64_t* wide_count, uint32_t* wide_depth);

/* FP32 attributes -> FP16 (host-side reference of the device conversion). */
void pt_half_attributes(const pt_triangle_attribute* in, uint64_t count, pt_half_attribute* out);

/* Select the precision form of a context (PT_PRECISION_* bits).  Resets the
 * accumulation.  PT_ERR_STATE unless the wavefront kernels are selected. */
int pt_set_precision(pt_ctx* ctx, uint32_t flags);
uint32_t pt_precision(const pt_ctx* ctx);
/* The form the last pt_trace used (WIDE_BVH dropped for non-opaque scenes). */
uint32_t pt_precision_active(const pt_ctx* ctx);

/* Kahan compensation of the accumulation (tile_w * tile_h * 4 floats);
 * zeros unless PT_PRECISION_KAHAN is set. */
#define PT_TILE_COMPENSATION 2

/* FP64 reference render of the current tile: the image error of every form
 * above is stated against it.  Traces the samples sample_first ..
 * sample_first + sample_count - 1 (1-based sample indices n of the seed,
 * trace.slang:736-737) of every tile pixel inside the image, one thread per
 * path, in double arithmetic with CUDA's double-precision math functions,
 * from the same FP32 world buffers (binary BVH, FP32 attributes and skybox,
 * whatever precision form is selected), with the shader's own f32 random
 * numbers.  Writes per-pixel radiance SUMS over those samples to
 * host_rgb_sums (tile_w * tile_h * 3 doubles, row stride tile_w; pixels
 * outside the image are 0).  The accumulation buffer, storage texture and
 * sample count are not touched.  This is the only code of the library that
 * computes in FP64; no counterpart in the reference.
 * PT_ERR_INVALID_ARG for sample_first == 0, sample_count == 0 or a range
 * past 2^32 - 1; PT_ERR_STATE without a world. */
int pt_render_fp64(pt_ctx* ctx, uint32_t sample_first, uint32_t sample_count, double* host_rgb_sums);

#ifdef __cplusplus
}
#endif

#endif
