// trace_plain.cu - the plain CUDA form of the trace pass: one thread per tile
// pixel runs a whole path (compute_main, trace.slang:719-1309), one launch
// per sample, 8 x 8 blocks as the shader's [numthreads(8, 8, 1)].  This is
// the "one job per launch" baseline the wavefront path is measured against;
// both produce identical bits.
#include "pt_kernels.h"
#include "pt_path.cuh"

namespace ptd {

PTD void init_counters(Counters& c) {
    c.visit_hash = kFnvBasis;
    c.extend_rays = c.shadow_rays = c.interior_visits = c.leaf_visits = c.triangle_tests = c.rand_draws = 0;
    c.shadow_interior_visits = c.shadow_leaf_visits = c.shadow_triangle_tests = 0;
    c.hits = c.sky_misses = c.light_samples = c.sky_light_samples = 0;
}

PTD void write_record(pt_path_record* r, const Counters& c, const int32_t* hits, f3 color) {
    r->visit_hash = c.visit_hash;
    for (int i = 0; i < PT_RECORD_MAX_BOUNCES; ++i) r->hit[i] = hits[i];
    r->extend_rays = c.extend_rays;
    r->shadow_rays = c.shadow_rays;
    r->interior_visits = c.interior_visits;
    r->leaf_visits = c.leaf_visits;
    r->triangle_tests = c.triangle_tests;
    r->shadow_interior_visits = c.shadow_interior_visits;
    r->shadow_leaf_visits = c.shadow_leaf_visits;
    r->shadow_triangle_tests = c.shadow_triangle_tests;
    r->rand_draws = c.rand_draws;
    r->hits = c.hits;
    r->sky_misses = c.sky_misses;
    r->light_samples = c.light_samples;
    r->sky_light_samples = c.sky_light_samples;
    r->radiance[0] = color.x;
    r->radiance[1] = color.y;
    r->radiance[2] = color.z;
}

template <bool kRec>
__global__ void __launch_bounds__(64) plain_kernel(World w, ptk::Tile t, uint32_t n, ptk::Sinks sinks) {
    const uint32_t gx = blockIdx.x * 8u + threadIdx.x, gy = blockIdx.y * 8u + threadIdx.y;
    const uint32_t px = gx + t.origin_x, py = gy + t.origin_y;
    if (gx >= t.tile_w || gy >= t.tile_h || px >= t.image_w || py >= t.image_h) return;
    Counters c;
    int32_t hits[PT_RECORD_MAX_BOUNCES];
    if constexpr (kRec) {
        init_counters(c);
        for (int i = 0; i < PT_RECORD_MAX_BOUNCES; ++i) hits[i] = -2;
    }
    Rng<kRec> rng;
    rng.s = seed(px, py, n);
    if constexpr (kRec) rng.rec.c = &c;
    PathState ps;
    camera_ray(w, px, py, t.image_w, t.image_h, rng, ps);
    f3 rcp = 1.0f / ps.d;
    for (uint32_t bounce = 0; bounce <= t.max_bounces; ++bounce) {
        float hit_t = kFltMax, hv = 0.0f, hw = 0.0f;
        int32_t hit = -1;
        closest_hit(w, ps.o, ps.d, rcp, rng, &c, hit_t, hit, hv, hw);
        if constexpr (kRec) {
            if (bounce < PT_RECORD_MAX_BOUNCES) hits[bounce] = hit;
        }
        if (hit == -1) {
            if constexpr (kRec) c.sky_misses += 1;
            shade_miss(w, bounce, ps);
            break;
        }
        if constexpr (kRec) c.hits += 1;
        if (!shade_hit<kRec, true>(w, bounce, t.max_bounces, ps, hit_t, (uint32_t)hit, hv, hw, rng, &c, nullptr)) break;
        rcp = 1.0f / ps.d;
    }
    // accumulate, trace.slang:1299-1308
    const uint32_t idx = gy * t.tile_w + gx;
    f3 prev = mk(0.0f, 0.0f, 0.0f);
    if (n > 1u) {
        const float4 a = t.accum[idx];
        prev = mk(a.x, a.y, a.z);
    }
    const f3 acc = prev + ps.color;
    t.accum[idx] = make_float4(acc.x, acc.y, acc.z, 1.0f);
    const f3 out = kExposure * acc / (float)n;
    t.image[idx] = make_float4(out.x, out.y, out.z, 1.0f);
    if constexpr (kRec) {
        if (sinks.records) write_record(sinks.records + idx, c, hits, ps.color);
        if (sinks.totals) add_totals(sinks.totals, c);
    }
}

__global__ void debug_intersect_kernel(World w, uint64_t n, const float* origins, const float* directions,
                                       const float* t_max, int32_t* hit_out, float* hit_t_out, pt_path_record* records) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Counters c;
    init_counters(c);
    Rng<true> rng;
    rng.s = 1u;
    rng.rec.c = &c;
    const f3 o = mk(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]);
    const f3 d = mk(directions[3 * i], directions[3 * i + 1], directions[3 * i + 2]);
    float ht = t_max[i], hv = 0.0f, hw = 0.0f;
    int32_t h = -1;
    World opaque = w;
    opaque.any_alpha = 0;
    closest_hit(opaque, o, d, 1.0f / d, rng, &c, ht, h, hv, hw);
    hit_out[i] = h;
    hit_t_out[i] = ht;
    if (records) {
        int32_t hits[PT_RECORD_MAX_BOUNCES];
        for (int k = 0; k < PT_RECORD_MAX_BOUNCES; ++k) hits[k] = -2;
        hits[0] = h;
        write_record(records + i, c, hits, mk(0.0f, 0.0f, 0.0f));
    }
}

}  // namespace ptd

namespace ptk {

cudaError_t launch_plain(const ptd::World& w, const Tile& t, uint32_t n, Sinks sinks, cudaStream_t stream) {
    const uint32_t vw = t.tile_w < t.image_w - t.origin_x ? t.tile_w : t.image_w - t.origin_x;
    const uint32_t vh = t.tile_h < t.image_h - t.origin_y ? t.tile_h : t.image_h - t.origin_y;
    const dim3 grid((vw + 7u) / 8u, (vh + 7u) / 8u, 1u), block(8u, 8u, 1u);
    if (sinks.any())
        ptd::plain_kernel<true><<<grid, block, 0, stream>>>(w, t, n, sinks);
    else
        ptd::plain_kernel<false><<<grid, block, 0, stream>>>(w, t, n, sinks);
    return cudaGetLastError();
}

cudaError_t launch_debug_intersect(const ptd::World& w, uint64_t n, const float* origins, const float* directions,
                                   const float* t_max, int32_t* hit, float* hit_t, pt_path_record* records,
                                   cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint32_t block = 128;
    const uint64_t grid = (n + block - 1) / block;
    ptd::debug_intersect_kernel<<<(unsigned)grid, block, 0, stream>>>(w, n, origins, directions, t_max, hit, hit_t, records);
    return cudaGetLastError();
}

}  // namespace ptk
