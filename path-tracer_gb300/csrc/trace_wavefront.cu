// trace_wavefront.cu - wavefront kernels of the trace pass (see pt_wavefront.h).
//
// Layout in HBM
//   ray queues (ping-pong, slot order):  o = (origin xyz, path id bits)
//                                        d = (direction xyz, rng state bits)
//                                        T = (throughput xyz, previous BSDF pdf)
//   hit per slot:                        (t, triangle bits, v, w)
//   colour per path id:                  (final_color xyz, unused)
//   shadow queue (slot order):           (origin xyz, path id), (direction xyz, distance),
//                                        (contribution xyz, light triangle bits)
//   BVH nodes copied 32 bytes past a 256-byte boundary, so the two children
//   of every interior node (indices 2k+1, 2k+2) fill one aligned 64-byte
//   block read with four 16-byte loads; triangles padded to 3 x float4.
// Every path runs exactly the arithmetic of the plain kernel (pt_path.cuh),
// in the same order, so results are bit-identical.
#include <cmath>
#include <cstdio>
#include <mutex>
#include <type_traits>
#include <vector>

#include "../../include/pt_precision.h"
#include "pt_abi_guard.h"
#include "pt_links.h"
#include "pt_wave.cuh"
#include "pt_wavefront.h"

namespace ptd {

// per group: paths p = s * P + pixel, P = visible tile pixels
struct Group {
    uint32_t vis_w, vis_h;   // visible part of the tile
    uint32_t pixels;         // vis_w * vis_h
    uint32_t paths;          // pixels * samples
    uint32_t first_sample;   // 1-based n of sample 0 of the group
    uint32_t samples;
    uint32_t record_sample;  // sample offset of the group within the pt_trace call
};

// Path order within a group.  Pixel-major (PT_PIXEL_MAJOR 1): a pixel's
// samples are consecutive paths, so a warp's camera rays are 32 jittered
// rays through two pixels and traverse almost the same nodes; sample-major:
// consecutive pixels of one sample.  Only the order of work changes.
PTD void split_path(uint32_t p, const Group& g, uint32_t* s, uint32_t* pix) {
#if PT_PIXEL_MAJOR
    *pix = p / g.samples;
    *s = p - *pix * g.samples;
#else
    *s = p / g.pixels;
    *pix = p - *s * g.pixels;
#endif
}
PTD size_t path_of(uint32_t s, uint32_t pix, const Group& g) {
#if PT_PIXEL_MAJOR
    return (size_t)pix * g.samples + s;
#else
    return (size_t)s * g.pixels + pix;
#endif
}

template <bool kRec>
__global__ void __launch_bounds__(256) raygen_kernel(World w, ptk::Tile t, Group g, Queues q) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) {
        q.cnt[0] = g.paths;
        q.cnt[1] = 0u;
    }
    if (p >= g.paths) return;
    uint32_t s, pix;
    split_path(p, g, &s, &pix);
    const uint32_t gy = pix / g.vis_w, gx = pix - gy * g.vis_w;
    const uint32_t px = gx + t.origin_x, py = gy + t.origin_y;
    Counters c;
    if constexpr (kRec) {
        c.visit_hash = kFnvBasis;
        c.extend_rays = c.shadow_rays = c.interior_visits = c.leaf_visits = c.triangle_tests = c.rand_draws = 0;
        c.shadow_interior_visits = c.shadow_leaf_visits = c.shadow_triangle_tests = 0;
        c.hits = c.sky_misses = c.light_samples = c.sky_light_samples = 0;
    }
    Rng<kRec> rng;
    rng.s = seed(px, py, g.first_sample + s);
    if constexpr (kRec) rng.rec.c = &c;
    PathState ps;
    camera_ray(w, px, py, t.image_w, t.image_h, rng, ps);
    q.o[0][p] = make_float4(ps.o.x, ps.o.y, ps.o.z, __uint_as_float(p));
    q.d[0][p] = make_float4(ps.d.x, ps.d.y, ps.d.z, __uint_as_float(rng.s));
    q.T[0][p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    q.color[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if constexpr (kRec) {
        q.rec[p] = c;
        for (int i = 0; i < PT_RECORD_MAX_BOUNCES; ++i) q.rec_hits[(size_t)p * PT_RECORD_MAX_BOUNCES + i] = -2;
    }
}

// counters of one bounce: the next ray queue, the extend fetch, the hit and
// miss lists, the sort and order flags (shadow: true also the shadow queue,
// its fetch counter and order flag)
__global__ void bounce_reset_kernel(uint32_t* cnt, int next, bool shadow) {
    cnt[next] = 0u;
    cnt[3] = 0u;
    cnt[5] = 0u;
    cnt[6] = 0u;
    cnt[7] = 0u;
    cnt[8] = 0u;
    if (shadow) {
        cnt[2] = 0u;
        cnt[4] = 0u;
        cnt[9] = 0u;
    }
}
// the shadow queue's counters alone (before the shading kernel appends to it)
__global__ void shadow_reset_kernel(uint32_t* cnt) {
    cnt[2] = 0u;
    cnt[4] = 0u;
    cnt[9] = 0u;
}

// Persistent extend kernel: every lane traverses its own ray and takes a new
// one from the queue (one atomic per warp for all idle lanes) as soon as it
// finishes, so long and short rays do not leave lanes idle.  Finished rays
// are filed under hits or misses for the shading kernel.  kWide traverses the
// 8-wide BVH of the precision form instead of the binary one.
template <bool kRec, bool kAlpha, bool kTri36 = false, bool kWide = false>
__global__ void __launch_bounds__(kExtendThreads, kWide ? PT_WIDE_MIN_BLOCKS : PT_EXTEND_MIN_BLOCKS) extend_kernel(World w, Fast f, Queues q, int cur, uint32_t bounce) {
    static_assert(!(kWide && (kRec || kAlpha)), "the wide form keeps no records and runs opaque scenes only");
    const Stage st = stage_of(q, cur);
    const uint32_t count = *st.count;
    const bool ordered = PT_RAY_ORDER && q.cnt[8] != 0u;
    typename std::conditional<kWide, WideTraverser<false, kTri36>, Traverser<kRec, kAlpha, false, kTri36>>::type tr;
    constexpr uint32_t kShared = kWide ? kWideSmemStack : kSmemStack;
    __shared__ uint2 stack_top[kShared > 0u ? kShared * kExtendThreads : 1u];
    LaneStack<kExtendThreads, kShared> stack;
    stack.col = stack_top + threadIdx.x;
    uint32_t istack[kRec ? 64 : 1];
    uint32_t slot = 0, path = 0;
    __shared__ FilerSlots<kExtendThreads> filer_slots;
    ResultFiler filer = filer_slots.of_warp(lane_id());
    lane_refill_loop(
        &q.cnt[3], count, kWide ? kWideStepsPerRefill : kStepsPerRefill, kRefillBelow,
        [&](uint32_t i) {
            slot = ordered ? q.hit_sorted[i] : i;
            const float4 o4 = st.o[slot], d4 = st.d[slot];
            path = __float_as_uint(o4.w);
            tr.rng.s = __float_as_uint(d4.w);
            if constexpr (kRec) tr.c = q.rec[path];
            stack.reset();
            tr.init(f, mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z), kFltMax, -1);
        },
        [&]() {
            if (!tr.step(w, f, stack, istack)) return false;
            q.hit[slot] = make_float4(tr.hit_t, __int_as_float(tr.hit), tr.hv, tr.hw);
            if constexpr (kAlpha) st.d[slot].w = __uint_as_float(tr.rng.s);
            if constexpr (kRec) {
                q.rec[path] = tr.c;
                if (bounce < PT_RECORD_MAX_BOUNCES) q.rec_hits[(size_t)path * PT_RECORD_MAX_BOUNCES + bounce] = tr.hit;
            }
            filer.file(slot, tr.hit != -1, min((uint32_t)tr.hit >> q.key_shift, kSortBuckets - 1u));
            return true;
        },
        [&]() { filer.flush(q, lane_id()); }, step_kind<PT_MAJORITY_EXTEND && !kWide>(tr, [&]() -> const Fast& { return f; }));
}

template <bool kRec, bool kAlpha>
__global__ void __launch_bounds__(kShadeThreads, PT_SHADE_MIN_BLOCKS) shade_kernel(World w, Fast f, Queues q, int cur, uint32_t bounce,
                                                              uint32_t max_bounces) {
    const Stage st = stage_of(q, cur);
    const ShadeRange range(q);
    const uint32_t count = range.count();
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const unsigned lane = lane_id();
    for (uint32_t base = warp * 32u; base < count; base += warps * 32u) {
        const uint32_t i = range.slot(q, base + lane);
        bool cont = false;
        ShadowRay sr;
        sr.valid = false;
        PathState ps;
        uint32_t p = 0, rs = 0;
        if (i != 0xffffffffu) {
            // the entries before miss_span are misses (the extend kernel filed them so): no hit record to read
            const bool miss = base + lane < range.miss_span;
            const float4 o4 = st.o[i], d4 = st.d[i], t4 = st.T[i];
            const float4 h4 = miss ? make_float4(0.0f, __int_as_float(-1), 0.0f, 0.0f) : q.hit[i];
            p = __float_as_uint(o4.w);
            ps.o = mk(o4.x, o4.y, o4.z);
            ps.d = mk(d4.x, d4.y, d4.z);
            ps.throughput = mk(t4.x, t4.y, t4.z);
            ps.prev_pdf = t4.w;
            if constexpr (kColorDelta<kAlpha>) {
                ps.color = mk(0.0f, 0.0f, 0.0f);
            } else {
                const float4 c4 = q.color[p];
                ps.color = mk(c4.x, c4.y, c4.z);
            }
            Counters c;
            Rng<kRec> rng;
            rng.s = __float_as_uint(d4.w);
            if constexpr (kRec) {
                c = q.rec[p];
                rng.rec.c = &c;
            }
            const int32_t hit = __float_as_int(h4.y);
            if (hit == -1) {
                if constexpr (kRec) c.sky_misses += 1;
                shade_miss(w, bounce, ps);
            } else {
                if constexpr (kRec) c.hits += 1;
                cont = shade_hit<kRec, kAlpha>(w, bounce, max_bounces, ps, h4.x, (uint32_t)hit, h4.z, h4.w, rng, &c, &sr);
            }
            store_color<kAlpha>(q.color, p, ps.color);
            rs = rng.s;
            if constexpr (kRec) q.rec[p] = c;
        }
        const uint32_t slot = warp_append(cont, st.next_count, 0xffffffffu);
        if (cont) {
            st.no[slot] = make_float4(ps.o.x, ps.o.y, ps.o.z, __uint_as_float(p));
            st.nd[slot] = make_float4(ps.d.x, ps.d.y, ps.d.z, __uint_as_float(rs));
            st.nT[slot] = make_float4(ps.throughput.x, ps.throughput.y, ps.throughput.z, ps.prev_pdf);
        }
        if constexpr (!kAlpha) {
            const uint32_t sslot = warp_append(sr.valid, &q.cnt[2], 0xffffffffu);
            if (sr.valid) {
                q.so[sslot] = make_float4(sr.o.x, sr.o.y, sr.o.z, __uint_as_float(p));
                q.sd[sslot] = make_float4(sr.d.x, sr.d.y, sr.d.z, sr.dist);
                q.sc[sslot] = make_float4(sr.contribution.x, sr.contribution.y, sr.contribution.z, __int_as_float(sr.light_tri));
            }
        }
    }
}

// Persistent shadow kernel (opaque scenes): any-hit traversal of every queued
// shadow ray with the same lane refill; unoccluded rays add their light.
template <bool kRec, bool kTri36 = false, bool kWide = false>
__global__ void __launch_bounds__(kExtendThreads, kWide ? PT_WIDE_MIN_BLOCKS : PT_EXTEND_MIN_BLOCKS) shadow_kernel(World w, Fast f, Queues q) {
    static_assert(!(kWide && kRec), "the wide form keeps no records");
    const uint32_t count = q.cnt[2];
    const bool ordered = PT_SHADOW_ORDER && q.cnt[9] != 0u;
    typename std::conditional<kWide, WideTraverser<true, kTri36>,
                              Traverser<kRec, false, true, kTri36, PT_SHADOW_TRI_PER_STEP != 0>>::type tr;
    constexpr uint32_t kShared = kWide ? kWideSmemStack : kSmemStack;
    __shared__ uint2 stack_top[kShared > 0u ? kShared * kExtendThreads : 1u];
    LaneStack<kExtendThreads, kShared> stack;
    stack.col = stack_top + threadIdx.x;
    uint32_t istack[kRec ? 64 : 1];
    uint32_t path = 0;
    float4 contribution = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    lane_refill_loop(
        &q.cnt[4], count, kWide ? kWideStepsPerRefill : kStepsPerRefill, kRefillBelow,
        [&](uint32_t i) {
            const uint32_t slot = ordered ? q.hit_sorted[i] : i;
            const float4 o4 = q.so[slot], d4 = q.sd[slot];
            contribution = q.sc[slot];
            path = __float_as_uint(o4.w);
            if constexpr (kRec) tr.c = q.rec[path];
            stack.reset();
            tr.init(f, mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z), d4.w, __float_as_int(contribution.w));
        },
        [&]() {
            if (!tr.step(w, f, stack, istack)) return false;
            if (tr.hit != 1) {
                const float4 col = q.color[path];
                const f3 sum = mk(col.x, col.y, col.z) + mk(contribution.x, contribution.y, contribution.z);
                q.color[path] = make_float4(sum.x, sum.y, sum.z, 0.0f);
            }
            if constexpr (kRec) q.rec[path] = tr.c;
            return true;
        },
        NoRound(), step_kind<PT_MAJORITY_SHADOW && !kWide>(tr, [&]() -> const Fast& { return f; }));
}

// accumulate, trace.slang:1299-1308, samples of the group in order
__global__ void accumulate_kernel(ptk::Tile t, Group g, const float4* color) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= g.pixels) return;
    const uint32_t gy = pix / g.vis_w, gx = pix - gy * g.vis_w;
    const uint32_t idx = gy * t.tile_w + gx;
    f3 acc = mk(0.0f, 0.0f, 0.0f);
    if (g.first_sample > 1u) {
        const float4 a = t.accum[idx];
        acc = mk(a.x, a.y, a.z);
    }
    uint32_t n = g.first_sample;
    if (t.comp) {
        // Kahan-compensated sums (precision form); the first sample is 0 + L
        // with zero compensation, as in the plain sum
        f3 comp = mk(0.0f, 0.0f, 0.0f);
        if (g.first_sample > 1u) {
            const float4 k = t.comp[idx];
            comp = mk(k.x, k.y, k.z);
        }
        for (uint32_t s = 0; s < g.samples; ++s, ++n) {
            const float4 c = color[path_of(s, pix, g)];
            const f3 y = mk(c.x, c.y, c.z) - comp;
            const f3 sum = acc + y;
            comp = (sum - acc) - y;
            acc = sum;
        }
        t.comp[idx] = make_float4(comp.x, comp.y, comp.z, 0.0f);
    } else {
        for (uint32_t s = 0; s < g.samples; ++s, ++n) {
            const float4 c = color[path_of(s, pix, g)];
            acc = (n > 1u ? acc : mk(0.0f, 0.0f, 0.0f)) + mk(c.x, c.y, c.z);
        }
    }
    n -= 1u;
    t.accum[idx] = make_float4(acc.x, acc.y, acc.z, 1.0f);
    const f3 out = kExposure * acc / (float)n;
    t.image[idx] = make_float4(out.x, out.y, out.z, 1.0f);
}

__global__ void finalize_records_kernel(ptk::Tile t, Group g, Queues q, ptk::Sinks sinks) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= g.paths) return;
    uint32_t s, pix;
    split_path(p, g, &s, &pix);
    const uint32_t gy = pix / g.vis_w, gx = pix - gy * g.vis_w;
    const Counters c = q.rec[p];
    const float4 col = q.color[p];
    if (sinks.records) {
        pt_path_record* r = sinks.records + (size_t)(g.record_sample + s) * t.tile_w * t.tile_h + gy * t.tile_w + gx;
        r->visit_hash = c.visit_hash;
        for (int k = 0; k < PT_RECORD_MAX_BOUNCES; ++k) r->hit[k] = q.rec_hits[(size_t)p * PT_RECORD_MAX_BOUNCES + k];
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
        r->radiance[0] = col.x;
        r->radiance[1] = col.y;
        r->radiance[2] = col.z;
    }
    if (sinks.totals) add_totals(sinks.totals, c);
}

__global__ void pad_triangles_kernel(const pt_triangle_geometry* geo, uint64_t n, float4* tri4) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = geo[i].v0;
    tri4[kTriStride * i + 0] = make_float4(v[0], v[1], v[2], 0.0f);
    tri4[kTriStride * i + 1] = make_float4(v[3], v[4], v[5], 0.0f);
    tri4[kTriStride * i + 2] = make_float4(v[6], v[7], v[8], 0.0f);
    if (kTriStride == 4) tri4[kTriStride * i + 3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // read, never used
}

// FP32 attributes -> pt_half_attribute records (round to nearest even)
PTD uint32_t pack_half2(float x, float y) {
    return (uint32_t)__half_as_ushort(__float2half_rn(x)) | ((uint32_t)__half_as_ushort(__float2half_rn(y)) << 16);
}
__global__ void half_attributes_kernel(const pt_triangle_attribute* in, uint64_t n, uint2* out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const pt_triangle_attribute& a = in[i];
    uint2* o = out + 8 * i;
    o[0] = make_uint2(pack_half2(a.n0[0], a.n0[1]), pack_half2(a.n0[2], 0.0f));
    o[1] = make_uint2(pack_half2(a.n1[0], a.n1[1]), pack_half2(a.n1[2], 0.0f));
    o[2] = make_uint2(pack_half2(a.n2[0], a.n2[1]), pack_half2(a.n2[2], 0.0f));
    o[3] = make_uint2(pack_half2(a.t0[0], a.t0[1]), pack_half2(a.t0[2], a.t0[3]));
    o[4] = make_uint2(pack_half2(a.t1[0], a.t1[1]), pack_half2(a.t1[2], a.t1[3]));
    o[5] = make_uint2(pack_half2(a.t2[0], a.t2[1]), pack_half2(a.t2[2], a.t2[3]));
    o[6] = make_uint2(pack_half2(a.uv0[0], a.uv0[1]), pack_half2(a.uv1[0], a.uv1[1]));
    o[7] = make_uint2(pack_half2(a.uv2[0], a.uv2[1]), a.material_index);
}

// RGBA32F skybox texels -> BF16 RGBA (round to nearest even)
PTD uint32_t pack_bf162(float x, float y) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(y)) << 16);
}
__global__ void bf16_sky_kernel(const float4* in, uint64_t n, uint2* out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = in[i];
    out[i] = make_uint2(pack_bf162(p.x, p.y), pack_bf162(p.z, p.w));
}

// closest hit of given rays on the 8-wide BVH (hit-id parity of the precision form)
__global__ void debug_intersect_wide_kernel(World w, Fast f, uint64_t n, const float* origins, const float* directions,
                                            const float* t_max, int32_t* hit, float* hit_t) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    WideTraverser<false> tr;
    LocalStack stack;
    tr.init(f, mk(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]),
            mk(directions[3 * i], directions[3 * i + 1], directions[3 * i + 2]), t_max ? t_max[i] : kFltMax, -1);
    while (!tr.step(w, f, stack, nullptr)) {
    }
    hit[i] = tr.hit;
    hit_t[i] = tr.hit_t;
}

}  // namespace ptd

namespace ptw {

namespace {

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, n ? n : 16);
        if (e == cudaSuccess) bytes = n ? n : 16;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

constexpr uint64_t kMaxPaths = 1ull << 25;  // paths in flight per group

// 1: a group's shadow stage runs on a second stream of its lane, beside the
// next bounce's extend stage
#ifndef PT_SHADOW_SIDE
#define PT_SHADOW_SIDE 1
#endif

#define PTW_TRY(x)                          \
    do {                                    \
        const cudaError_t e_ = (x);         \
        if (e_ != cudaSuccess) return e_;   \
    } while (0)

}  // namespace

// the second stream of a lane for the shadow stage, with its two events
struct ShadowSide {
    cudaStream_t stream;
    cudaEvent_t shaded;  // a bounce's shading finished (recorded on the group's stream)
    cudaEvent_t traced;  // its shadow rays finished (recorded on `stream`)
};

// The queues of one group of paths and the stream it runs on.  Several lanes
// let consecutive groups overlap: one group's last bounces (few, long rays
// that leave most SMs idle) run beside the next group's first ones.  Three
// lanes: 256x256 x 16-spp Cornell images 3784 Mrays/s against 3529 with two
// and 2701 with one; the 1920x1080 x 64-spp procedural image 1812 against
// 1814 and 1738 (each lane holds the queues of a whole group of paths).
#ifndef PT_LANES
#define PT_LANES 3
#endif
static_assert(PT_LANES >= 1 && PT_LANES <= 4, "one to four queue lanes");
struct Lane {
    Buf o[2], d[2], T[2], hit, color, so, sd, sc, cnt;
    Buf lists;  // hit list, miss list, sorted hit list (capacity entries each), sort counts and offsets
    cudaStream_t stream = nullptr;
    ShadowSide side{};            // the stream the lane's shadow stage runs on (PT_SHADOW_SIDE)
    cudaEvent_t done = nullptr;   // the lane's group finished (recorded on the lane)
    cudaEvent_t freed = nullptr;  // its accumulation consumed the colours (recorded on the caller's stream)
    bool pending = false;         // `freed` was recorded and not yet waited for
};

struct Wavefront {
    Lane lane[PT_LANES];
    Buf rec, rec_hits;
    int next_lane = 0;
    cudaEvent_t start = nullptr;  // the caller's stream before the last group began
    bool have_start = false;
    Buf pairs, tri4;
    Buf wide, links, attr_h, sky_h;  // precision form copies (links: parent per node, leaf per triangle)
    bool stale = true;
    bool wide_ready = false, attr_h_ready = false, sky_h_ready = false;
    uint64_t wide_count = 0;
    uint64_t tri_count = 0;    // of the world the layouts were built for
    uint64_t links_nodes = 0;  // node count of the links array (leaf_of follows the parents)
    const void* layout_nodes = nullptr;  // world buffers the layouts were built from
    const void* layout_geo = nullptr;
    uint64_t capacity = 0;
    int sms = 0;
    int extend_blocks[2][2] = {{0, 0}, {0, 0}};
    int shade_blocks = 0;
};

int create(Wavefront** out) {
    Wavefront* wf = new Wavefront();
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&wf->sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaEventCreateWithFlags(&wf->start, cudaEventDisableTiming);
    for (Lane& l : wf->lane) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&l.freed, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&l.side.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&l.side.shaded, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&l.side.traced, cudaEventDisableTiming);
    }
    *out = wf;
    return e == cudaSuccess ? 0 : (int)e;
}

void destroy(Wavefront* wf) {
    if (!wf) return;
    for (Lane& l : wf->lane) {
        if (l.stream) cudaStreamSynchronize(l.stream);
        for (Buf* b : {&l.o[0], &l.o[1], &l.d[0], &l.d[1], &l.T[0], &l.T[1], &l.hit, &l.color, &l.so, &l.sd, &l.sc,
                       &l.cnt, &l.lists})
            b->release();
        if (l.side.stream) cudaStreamSynchronize(l.side.stream);
        if (l.done) cudaEventDestroy(l.done);
        if (l.freed) cudaEventDestroy(l.freed);
        if (l.side.shaded) cudaEventDestroy(l.side.shaded);
        if (l.side.traced) cudaEventDestroy(l.side.traced);
        if (l.side.stream) cudaStreamDestroy(l.side.stream);
        if (l.stream) cudaStreamDestroy(l.stream);
    }
    if (wf->start) cudaEventDestroy(wf->start);
    for (Buf* b : {&wf->rec, &wf->rec_hits, &wf->pairs, &wf->tri4, &wf->wide, &wf->links, &wf->attr_h, &wf->sky_h})
        b->release();
    delete wf;
}

void world_changed(Wavefront* wf) {
    if (wf) {
        wf->stale = true;
        wf->wide_ready = wf->attr_h_ready = false;
    }
}

void sky_changed(Wavefront* wf) {
    if (wf) wf->sky_h_ready = false;
}

namespace {

cudaError_t build_layouts(Wavefront* wf, const ptd::World& w, uint64_t nodes, uint64_t tris, cudaStream_t stream) {
    PTW_TRY(wf->pairs.reserve((nodes + 1) * 32 + 256));
    PTW_TRY(cudaMemcpyAsync(static_cast<char*>(wf->pairs.p) + 32, w.nodes, nodes * 32, cudaMemcpyDeviceToDevice, stream));
    PTW_TRY(wf->tri4.reserve(tris * 16 * ptd::kTriStride));
    ptd::pad_triangles_kernel<<<(unsigned)((tris + 255) / 256), 256, 0, stream>>>(w.geo, tris, static_cast<float4*>(wf->tri4.p));
    PTW_TRY(cudaGetLastError());
    wf->stale = false;
    wf->layout_nodes = w.nodes;
    wf->layout_geo = w.geo;
    wf->tri_count = tris;
    wf->wide_ready = wf->attr_h_ready = false;
    return cudaSuccess;
}

// the 8-wide BVH: binary nodes back from the device, collapsed and quantised
// on the host (pt_build_wide_bvh), uploaded
cudaError_t build_wide(Wavefront* wf, const ptd::World& w, uint64_t nodes, uint64_t tris, cudaStream_t stream) {
    std::vector<pt_bvh_node> host(nodes);
    PTW_TRY(cudaMemcpyAsync(host.data(), w.nodes, nodes * sizeof(pt_bvh_node), cudaMemcpyDeviceToHost, stream));
    PTW_TRY(cudaStreamSynchronize(stream));
    uint32_t depth = 0;
    std::vector<pt_wide_node> wide;
    if (ptw::build_wide_bvh(host.data(), nodes, ptd::kWideLeafMerge, wide, &depth) != PT_OK)
        return cudaErrorInvalidValue;
    const uint64_t count = wide.size();
    std::vector<uint32_t> links(nodes + tris);
    if (!ptw::build_bvh_links(host.data(), nodes, tris, links.data(), links.data() + nodes)) return cudaErrorInvalidValue;
    PTW_TRY(wf->wide.reserve(count * sizeof(pt_wide_node)));
    PTW_TRY(cudaMemcpyAsync(wf->wide.p, wide.data(), count * sizeof(pt_wide_node), cudaMemcpyHostToDevice, stream));
    PTW_TRY(wf->links.reserve(links.size() * 4));
    PTW_TRY(cudaMemcpyAsync(wf->links.p, links.data(), links.size() * 4, cudaMemcpyHostToDevice, stream));
    PTW_TRY(cudaStreamSynchronize(stream));  // the host vectors go out of scope
    wf->links_nodes = nodes;
    wf->wide_count = count;
    wf->wide_ready = true;
    return cudaSuccess;
}

cudaError_t reserve_paths(Wavefront* wf, uint64_t paths, bool record) {
    const size_t b = paths * 16;
    // earlier groups (on the lanes) and their accumulations (on the callers'
    // streams) may still use the buffers a larger reservation frees
    PTW_TRY(cudaDeviceSynchronize());
    for (Lane& l : wf->lane) {
        for (Buf* x : {&l.o[0], &l.o[1], &l.d[0], &l.d[1], &l.T[0], &l.T[1], &l.hit, &l.color, &l.so, &l.sd, &l.sc})
            PTW_TRY(x->reserve(b));
        PTW_TRY(l.cnt.reserve(64));
        // hit list, miss list, sorted hit list, sort counts and offsets, hit sort keys
        PTW_TRY(l.lists.reserve(paths * 16 + 2 * ptd::kSortBuckets * 4));
        PTW_TRY(cudaMemset(static_cast<uint32_t*>(l.lists.p) + 3 * paths, 0, ptd::kSortBuckets * 4));  // sort counts
    }
    if (record) {
        PTW_TRY(wf->rec.reserve(paths * sizeof(ptd::Counters)));
        PTW_TRY(wf->rec_hits.reserve(paths * PT_RECORD_MAX_BOUNCES * 4));
    }
    wf->capacity = paths;
    return cudaSuccess;
}

template <class K>
int occupancy(K kernel, int threads) {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, threads, 0);
    return blocks > 0 ? blocks : 1;
}

// hit sorting of one trace: counts[kSortBuckets] then offsets[kSortBuckets];
// min_hits == ~0u: no sorting
struct SortCfg {
    uint32_t* counts = nullptr;
    uint32_t min_hits = 0xffffffffu;
    uint32_t tri_shift = 0;
};

// hits are sorted before shading when a bounce has at least this many
// (0xffffffff: never); key 1 = triangle bucket, 0 = material index
#ifndef PT_SORT_MIN_HITS
#define PT_SORT_MIN_HITS 65536u
#endif
#ifndef PT_SORT_KEY
#define PT_SORT_KEY 1
#endif

// one group of paths through raygen, max_bounces + 1 rounds of extend /
// (hit sort) / shade / shadow, and accumulate; kTri36 reads the reference's
// 36-byte triangles instead of the padded copy
// One group of paths through every bounce on `stream`; the accumulation runs
// on `acc_stream` (null: `stream`) after `done` marks the group's end there.
template <bool kRec, bool kAlpha, bool kTri36, bool kWide = false, class TimerF>
cudaError_t run_group(int sms, const ptd::World& w, const ptd::Fast& f, const ptd::Queues& q,
                      const ptk::Tile& tile, const ptd::Group& g, ptk::Sinks sinks, cudaStream_t stream,
                      TimerF&& timer, const SortCfg& sort = SortCfg(), cudaStream_t acc_stream = nullptr,
                      cudaEvent_t done = nullptr, const ShadowSide* side = nullptr) {
    using namespace ptd;
    const int ext_blocks = sms * occupancy(extend_kernel<kRec, kAlpha, kTri36, kWide>, kExtendThreads);
    const int sha_blocks = sms * occupancy(shade_kernel<kRec, kAlpha>, kShadeThreads);
    const int shd_blocks = sms * occupancy(shadow_kernel<kRec, kTri36, kWide>, kExtendThreads);
    PTW_TRY(timer(PT_KC_RAYGEN, stream, [&] {
        raygen_kernel<kRec><<<(g.paths + 255u) / 256u, 256, 0, stream>>>(w, tile, g, q);
        return cudaGetLastError();
    }));
    int cur = 0;
    const bool sorting = sort.counts && sort.min_hits != 0xffffffffu;
    // octant order of a ray queue (current rays: flag 8, shadow rays: flag 9) into hit_sorted
    const auto order_rays = [&](const float4* dirs, const uint32_t* count, uint32_t flag) {
        ray_count_kernel<0><<<sms * 2, kSortThreads, 0, stream>>>(dirs, count, sort.counts, sort.min_hits);
        ray_scan_kernel<0><<<1, 1, 0, stream>>>(count, sort.counts, sort.counts + kSortBuckets, q.cnt + flag,
                                             sort.min_hits);
        ray_scatter_kernel<0><<<sms * 4, kSortThreads, 0, stream>>>(dirs, count, sort.counts + kSortBuckets,
                                                                  q.hit_sorted, sort.min_hits);
        return cudaGetLastError();
    };
    // With `side`, bounce k's shadow rays are traced on side->stream while
    // bounce k + 1's extend (and hit sort) run: neither touches what the other
    // reads or writes.  Bounce k + 1's shading waits for them (it adds to the
    // same path colours, in the reference's order, and refills the shadow queue).
    const bool split = side != nullptr && !kAlpha;
    for (uint32_t bounce = 0; bounce <= tile.max_bounces; ++bounce) {
        bounce_reset_kernel<<<1, 1, 0, stream>>>(q.cnt, cur ^ 1, !split);
        PTW_TRY(cudaGetLastError());
        if (PT_RAY_ORDER && sorting && bounce > 0) {  // camera rays are coherent already (pixel-major)
            PTW_TRY(timer(PT_KC_SORT, stream, [&] { return order_rays(cur ? q.d[1] : q.d[0], q.cnt + cur, 8u); }));
        }
        PTW_TRY(timer(PT_KC_EXTEND, stream, [&] {
            extend_kernel<kRec, kAlpha, kTri36, kWide><<<ext_blocks, kExtendThreads, 0, stream>>>(w, f, q, cur, bounce);
            return cudaGetLastError();
        }));
        if (sort.counts && sort.min_hits != 0xffffffffu) {
            PTW_TRY(timer(PT_KC_SORT, stream, [&] {
                sort_count_kernel<PT_SORT_KEY><<<sms * 4, kSortThreads, 0, stream>>>(w, q, sort.counts, sort.min_hits,
                                                                                    sort.tri_shift);
                sort_scan_kernel<0><<<1, 1024, 0, stream>>>(q, sort.counts, sort.counts + kSortBuckets, sort.min_hits);
                sort_scatter_kernel<PT_SORT_KEY><<<sms * 4, kSortThreads, 0, stream>>>(
                    w, q, sort.counts + kSortBuckets, sort.min_hits, sort.tri_shift);
                return cudaGetLastError();
            }));
        }
        if (split) {
            if (bounce > 0) PTW_TRY(cudaStreamWaitEvent(stream, side->traced, 0));
            shadow_reset_kernel<<<1, 1, 0, stream>>>(q.cnt);
            PTW_TRY(cudaGetLastError());
        }
        PTW_TRY(timer(PT_KC_SHADE, stream, [&] {
            shade_kernel<kRec, kAlpha><<<sha_blocks, kShadeThreads, 0, stream>>>(w, f, q, cur, bounce, tile.max_bounces);
            return cudaGetLastError();
        }));
        if constexpr (!kAlpha) {
            if (PT_SHADOW_ORDER && sorting) {
                PTW_TRY(timer(PT_KC_SORT, stream, [&] { return order_rays(q.sd, q.cnt + 2, 9u); }));
            }
            const cudaStream_t ss = split ? side->stream : stream;
            if (split) {
                PTW_TRY(cudaEventRecord(side->shaded, stream));
                PTW_TRY(cudaStreamWaitEvent(ss, side->shaded, 0));
            }
            PTW_TRY(timer(PT_KC_SHADOW, ss, [&] {
                shadow_kernel<kRec, kTri36, kWide><<<shd_blocks, kExtendThreads, 0, ss>>>(w, f, q);
                return cudaGetLastError();
            }));
            if (split) PTW_TRY(cudaEventRecord(side->traced, ss));
        }
        cur ^= 1;
    }
    if (split) PTW_TRY(cudaStreamWaitEvent(stream, side->traced, 0));  // the last bounce's shadow rays
    const cudaStream_t as = acc_stream ? acc_stream : stream;
    if (as != stream) {
        PTW_TRY(cudaEventRecord(done, stream));
        PTW_TRY(cudaStreamWaitEvent(as, done, 0));
    }
    PTW_TRY(timer(PT_KC_ACCUMULATE, as, [&] {
        accumulate_kernel<<<(g.pixels + 255u) / 256u, 256, 0, as>>>(tile, g, q.color);
        return cudaGetLastError();
    }));
    if constexpr (kRec) {
        finalize_records_kernel<<<(g.paths + 255u) / 256u, 256, 0, stream>>>(tile, g, q, sinks);
        PTW_TRY(cudaGetLastError());
    }
    return cudaSuccess;
}

}  // namespace

cudaError_t trace(Wavefront* wf, const ptd::World& w_in, const ptk::Tile& tile, uint32_t first, uint32_t samples,
                  ptk::Sinks sinks, cudaStream_t stream, const Timer& timer, uint32_t precision, bool overlap,
                  bool serial) {
    precision = effective_precision(w_in, precision, sinks.any());
    ptd::World w = w_in;
    if (precision & PT_PRECISION_HALF_ATTRIBUTES) {
        if (!wf->attr_h_ready || !wf->sky_h_ready) return cudaErrorNotReady;  // prepare() first
        w.attr_h = static_cast<const uint2*>(wf->attr_h.p);
        w.sky_h = static_cast<const uint2*>(wf->sky_h.p);
    }
    const bool wide = (precision & PT_PRECISION_WIDE_BVH) != 0;
    if (wide && !wf->wide_ready) return cudaErrorNotReady;
    const uint32_t vis_w = tile.tile_w < tile.image_w - tile.origin_x ? tile.tile_w : tile.image_w - tile.origin_x;
    const uint32_t vis_h = tile.tile_h < tile.image_h - tile.origin_y ? tile.tile_h : tile.image_h - tile.origin_y;
    const uint64_t pixels = (uint64_t)vis_w * vis_h;
    if (pixels == 0 || samples == 0) return cudaSuccess;
    if (wf->stale || wf->layout_nodes != w.nodes || wf->layout_geo != w.geo) return cudaErrorNotReady;  // prepare() first
    if (ptd::kTriStride == 4) w.tri64 = static_cast<const float4*>(wf->tri4.p);  // the shading frame's vertices
    uint32_t group = (uint32_t)(kMaxPaths / pixels);
    if (group == 0) group = 1;
    if (group > samples) group = samples;
    const uint64_t paths = pixels * group;
    const bool record = sinks.any();
    if (paths > wf->capacity || (record && wf->rec.bytes < paths * sizeof(ptd::Counters))) {
        PTW_TRY(reserve_paths(wf, paths > wf->capacity ? paths : wf->capacity, record));
        wf->have_start = false;
    }
    ptd::Fast f;
    f.pairs = reinterpret_cast<const float4*>(static_cast<const char*>(wf->pairs.p) + 32);
    f.tri4 = static_cast<const float4*>(wf->tri4.p);
    f.wide = static_cast<const float4*>(wf->wide.p);
    f.parent = static_cast<const uint32_t*>(wf->links.p);
    f.leaf_of = f.parent ? f.parent + wf->links_nodes : nullptr;
    for (uint32_t s0 = 0; s0 < samples; s0 += group) {
        ptd::Group g;
        g.vis_w = vis_w;
        g.vis_h = vis_h;
        g.pixels = (uint32_t)pixels;
        g.samples = samples - s0 < group ? samples - s0 : group;
        g.paths = (uint32_t)(pixels * g.samples);
        g.first_sample = first + s0;
        g.record_sample = s0;
        // The recording variants run in order on the caller's stream with lane
        // 0's queues.  Otherwise the group runs on the next lane: it starts after
        // the caller's stream reaches this call (or, when `overlap` says nothing
        // was queued there since the previous group began, after that group's
        // starting point) and after the lane's previous accumulation; its own
        // accumulation runs on the caller's stream, so the samples of a pixel
        // are still summed in order and any later work there sees the result.
        Lane& l = record ? wf->lane[0] : wf->lane[wf->next_lane];
        const cudaStream_t gs = record ? stream : l.stream;
        if (!record) {
            wf->next_lane = (wf->next_lane + 1) % PT_LANES;
            if (serial || !(overlap && wf->have_start)) {
                PTW_TRY(cudaEventRecord(wf->start, stream));
                wf->have_start = true;
            }
            overlap = true;  // the call's later groups start from the same point (unless serial)
            PTW_TRY(cudaStreamWaitEvent(gs, wf->start, 0));
            if (l.pending) PTW_TRY(cudaStreamWaitEvent(gs, l.freed, 0));
        }
        ptd::Queues q;
        for (int k = 0; k < 2; ++k) {
            q.o[k] = static_cast<float4*>(l.o[k].p);
            q.d[k] = static_cast<float4*>(l.d[k].p);
            q.T[k] = static_cast<float4*>(l.T[k].p);
        }
        q.hit = static_cast<float4*>(l.hit.p);
        q.color = static_cast<float4*>(l.color.p);
        q.so = static_cast<float4*>(l.so.p);
        q.sd = static_cast<float4*>(l.sd.p);
        q.sc = static_cast<float4*>(l.sc.p);
        q.cnt = static_cast<uint32_t*>(l.cnt.p);
        q.hit_list = static_cast<uint32_t*>(l.lists.p);
        q.miss_list = q.hit_list + wf->capacity;
        q.hit_sorted = q.miss_list + wf->capacity;
        q.rec = static_cast<ptd::Counters*>(wf->rec.p);
        q.rec_hits = static_cast<int32_t*>(wf->rec_hits.p);
        SortCfg sort;
        sort.counts = q.hit_sorted + wf->capacity;  // kSortBuckets counts, then kSortBuckets offsets
        sort.min_hits = PT_SORT_MIN_HITS;
        while (((uint64_t)ptd::kSortBuckets << sort.tri_shift) < wf->tri_count && sort.tri_shift < 31u) sort.tri_shift += 1u;
        if (PT_SORT_KEY == 1) {  // the extend kernel files each hit's bucket beside the hit list
            q.hit_keys = sort.counts + 2 * ptd::kSortBuckets;
            q.key_shift = sort.tri_shift;
        }
        const cudaStream_t as = record ? nullptr : stream;
        const ShadowSide* side = (!record && !serial && PT_SHADOW_SIDE) ? &l.side : nullptr;
        cudaError_t e;
        if (record)
            e = w.any_alpha ? run_group<true, true, false>(wf->sms, w, f, q, tile, g, sinks, gs, timer)
                            : run_group<true, false, false>(wf->sms, w, f, q, tile, g, sinks, gs, timer);
        else if (wide)
            e = run_group<false, false, false, true>(wf->sms, w, f, q, tile, g, sinks, gs, timer, sort, as, l.done, side);
        else
            e = w.any_alpha ? run_group<false, true, false>(wf->sms, w, f, q, tile, g, sinks, gs, timer, sort, as, l.done)
                            : run_group<false, false, false>(wf->sms, w, f, q, tile, g, sinks, gs, timer, sort, as, l.done,
                                                             side);
        PTW_TRY(e);
        if (!record) {
            PTW_TRY(cudaEventRecord(l.freed, stream));
            l.pending = true;
        } else {
            wf->have_start = false;  // a later group must start after this one, which used lane 0 on `stream`
        }
    }
    return cudaSuccess;
}

cudaError_t prepare(Wavefront* wf, const ptd::World& w, uint64_t nodes, uint64_t tris, uint32_t precision,
                    cudaStream_t stream, bool* queued) {
    const bool work = wf->stale || wf->layout_nodes != w.nodes || wf->layout_geo != w.geo ||
                      ((precision & PT_PRECISION_WIDE_BVH) && !wf->wide_ready) ||
                      ((precision & PT_PRECISION_HALF_ATTRIBUTES) && (!wf->attr_h_ready || !wf->sky_h_ready));
    if (queued) *queued = work;
    if (work) {
        // groups still running on the lanes read the layouts about to be rebuilt
        for (Lane& l : wf->lane) PTW_TRY(cudaStreamWaitEvent(stream, l.done, 0));
        wf->have_start = false;
    }
    if (wf->stale || wf->layout_nodes != w.nodes || wf->layout_geo != w.geo)
        PTW_TRY(build_layouts(wf, w, nodes, tris, stream));
    if ((precision & PT_PRECISION_WIDE_BVH) && !wf->wide_ready) PTW_TRY(build_wide(wf, w, nodes, tris, stream));
    if ((precision & PT_PRECISION_HALF_ATTRIBUTES) && !wf->attr_h_ready) {
        PTW_TRY(wf->attr_h.reserve(tris * sizeof(pt_half_attribute)));
        PTW_TRY(convert_half_attributes(w.attr, tris, static_cast<uint2*>(wf->attr_h.p), stream));
        wf->attr_h_ready = true;
    }
    if ((precision & PT_PRECISION_HALF_ATTRIBUTES) && !wf->sky_h_ready) {
        const uint64_t texels = (uint64_t)w.sky_u.width * w.sky_u.height;
        PTW_TRY(wf->sky_h.reserve(texels * 8));
        PTW_TRY(convert_bf16_sky(w.sky, texels, static_cast<uint2*>(wf->sky_h.p), stream));
        wf->sky_h_ready = true;
    }
    return cudaSuccess;
}

cudaError_t convert_half_attributes(const pt_triangle_attribute* in, uint64_t n, uint2* out, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    ptd::half_attributes_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(in, n, out);
    return cudaGetLastError();
}

cudaError_t convert_bf16_sky(const float4* in, uint64_t n, uint2* out, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    ptd::bf16_sky_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(in, n, out);
    return cudaGetLastError();
}

uint32_t effective_precision(const ptd::World& w, uint32_t precision, bool record) {
    if (w.any_alpha || record) precision &= ~PT_PRECISION_WIDE_BVH;
    return precision;
}

cudaError_t debug_intersect_wide(Wavefront* wf, const ptd::World& w, uint64_t n, const float* origins,
                                 const float* directions, const float* t_max, int32_t* hit, float* hit_t,
                                 cudaStream_t stream) {
    if (!wf->wide_ready) return cudaErrorNotReady;
    ptd::Fast f;
    f.pairs = reinterpret_cast<const float4*>(static_cast<const char*>(wf->pairs.p) + 32);
    f.tri4 = static_cast<const float4*>(wf->tri4.p);
    f.wide = static_cast<const float4*>(wf->wide.p);
    f.parent = static_cast<const uint32_t*>(wf->links.p);
    f.leaf_of = f.parent + wf->links_nodes;
    if (n == 0) return cudaSuccess;
    ptd::debug_intersect_wide_kernel<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(w, f, n, origins, directions,
                                                                                      t_max, hit, hit_t);
    return cudaGetLastError();
}

}  // namespace ptw

// ---------------------------------------------------------------------------
// pt_trace_noalloc: the wavefront trace for callers that cannot allocate.
// Its queues, counters and sRGB table live in the static device array below;
// in host code the array's name is only a stand-in, so its device address is
// looked up once per device with cudaGetSymbolAddress.
namespace {

constexpr uint64_t kNoAllocPaths = PT_NOALLOC_MAX_PATHS;
constexpr size_t kNoAllocQueueBytes = 11ull * 16ull * kNoAllocPaths;  // o, d, T (x2), hit, colour, shadow o/d/c
constexpr size_t kNoAllocCountersOffset = kNoAllocQueueBytes;
constexpr size_t kNoAllocLutOffset = kNoAllocCountersOffset + 256;
constexpr size_t kNoAllocListOffset = kNoAllocLutOffset + 1024;  // hit list, miss list
static_assert(kNoAllocListOffset + 2 * 4 * kNoAllocPaths <= PT_NOALLOC_SCRATCH_BYTES, "static scratch too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[PT_NOALLOC_SCRATCH_BYTES];

constexpr int kNoAllocMaxDevices = 64;
struct NoAllocDevice {
    bool ready;
    unsigned char* scratch;  // device address of g_noalloc_scratch on this device
    int sms;
};
NoAllocDevice g_noalloc_devices[kNoAllocMaxDevices];
std::mutex g_noalloc_mutex;

int noalloc_fail(char* error, size_t size, int code, const char* msg) {
    if (error && size) snprintf(error, size, "%s", msg);
    return code;
}

int noalloc_cuda(char* error, size_t size, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return PT_OK;
    if (error && size) snprintf(error, size, "%s: %s", what, cudaGetErrorString(e));
    return PT_ERR_CUDA;
}

// once per device, with that device current
int noalloc_setup(int dev, char* error, size_t size) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoAllocDevice& d = g_noalloc_devices[dev];
    if (d.ready) return PT_OK;
    unsigned char* ptr = nullptr;
    int rc = noalloc_cuda(error, size, cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch), "cudaGetSymbolAddress");
    if (rc) return rc;
    float lut[256];
    for (int i = 0; i < 256; ++i) {
        const double v = (double)i / 255.0;
        lut[i] = (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
    }
    rc = noalloc_cuda(error, size, cudaMemcpy(ptr + kNoAllocLutOffset, lut, sizeof lut, cudaMemcpyHostToDevice),
                      "sRGB table upload");
    if (rc) return rc;
    int sms = 0;
    rc = noalloc_cuda(error, size, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    if (rc) return rc;
    d.scratch = ptr;
    d.sms = sms;
    d.ready = true;
    return PT_OK;
}

}  // namespace

extern "C" int pt_trace_noalloc(const pt_device_world* world, const pt_trace_parameters* params, uint32_t tile_width,
                                uint32_t tile_height, uint32_t samples, float* accum, float* image, void* stream,
                                char* error, size_t error_size) try {
    if (!world || !params || !accum || !image)
        return noalloc_fail(error, error_size, PT_ERR_INVALID_ARG, "world, params, accum and image are required");
    if (!world->geometries || !world->attributes || !world->materials || !world->bvh_nodes || !world->skybox_rgba ||
        world->triangle_count == 0 || world->node_count == 0)
        return noalloc_fail(error, error_size, PT_ERR_INVALID_ARG, "the world needs triangles, materials, BVH nodes and a skybox");
    if (((uintptr_t)world->skybox_rgba | (uintptr_t)accum | (uintptr_t)image) & 15u)
        return noalloc_fail(error, error_size, PT_ERR_INVALID_ARG, "skybox, accum and image must be 16-byte aligned");
    if ((uintptr_t)world->bvh_nodes & 31u)  // nodes are read in place with 32-byte loads
        return noalloc_fail(error, error_size, PT_ERR_INVALID_ARG, "BVH nodes must be 32-byte aligned");
    if (tile_width == 0 || tile_height == 0)
        return noalloc_fail(error, error_size, PT_ERR_OUT_OF_LIMITS, "tile size must be positive");
    if (!(params->tile_origin[0] < params->image_size[0] && params->tile_origin[1] < params->image_size[1]))
        return noalloc_fail(error, error_size, PT_ERR_INVALID_ARG, "tile origin must be within the image");
    if (params->max_bounces > PT_MAX_BOUNCES_LIMIT)
        return noalloc_fail(error, error_size, PT_ERR_INVALID_ARG, "max bounces must be at most 16");
    const uint32_t vis_w = tile_width < params->image_size[0] - params->tile_origin[0]
                               ? tile_width : params->image_size[0] - params->tile_origin[0];
    const uint32_t vis_h = tile_height < params->image_size[1] - params->tile_origin[1]
                               ? tile_height : params->image_size[1] - params->tile_origin[1];
    const uint64_t pixels = (uint64_t)vis_w * vis_h;  // >= 1: the origin lies inside the image
    // two comparisons, so that no product can wrap before the check
    if (pixels > kNoAllocPaths || samples > kNoAllocPaths / pixels) {
        char msg[200];
        snprintf(msg, sizeof msg, "%u x %u visible pixels x %u samples exceed the %u paths one call can hold",
                 vis_w, vis_h, samples, PT_NOALLOC_MAX_PATHS);
        return noalloc_fail(error, error_size, PT_ERR_OUT_OF_LIMITS, msg);
    }
    if (samples == 0) return PT_OK;
    int dev = 0;
    int rc = noalloc_cuda(error, error_size, cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return noalloc_fail(error, error_size, PT_ERR_OUT_OF_LIMITS, "device index too large");
    if ((rc = noalloc_setup(dev, error, error_size))) return rc;
    unsigned char* base = g_noalloc_devices[dev].scratch;

    ptd::World w;
    w.geo = world->geometries;
    w.attr = world->attributes;
    w.mat = world->materials;
    w.nodes = world->bvh_nodes;
    w.srgb = world->srgb_texture_atlases;
    w.linear = world->linear_texture_atlases;
    w.srgb_count = world->srgb_texture_atlases ? world->srgb_atlas_count : 0u;
    w.linear_count = world->linear_texture_atlases ? world->linear_atlas_count : 0u;
    w.sky = reinterpret_cast<const float4*>(world->skybox_rgba);
    w.sky_alias = world->skybox_aliases;
    w.scene_alias = world->scene_aliases;
    w.sky_u = world->skybox_uniforms;
    w.scene = world->scene_uniforms;
    w.camera = world->camera;
    w.srgb_lut = reinterpret_cast<const float*>(base + kNoAllocLutOffset);
    w.any_alpha = world->any_non_opaque ? 1 : 0;
    w.attr16 = ((uintptr_t)world->attributes & 15u) == 0u ? 1 : 0;  // the caller's buffer: any alignment

    ptd::Queues q;
    float4* slots = reinterpret_cast<float4*>(base);
    float4* arrays[11];
    for (int k = 0; k < 11; ++k) arrays[k] = slots + (size_t)k * kNoAllocPaths;
    q.o[0] = arrays[0];
    q.o[1] = arrays[1];
    q.d[0] = arrays[2];
    q.d[1] = arrays[3];
    q.T[0] = arrays[4];
    q.T[1] = arrays[5];
    q.hit = arrays[6];
    q.color = arrays[7];
    q.so = arrays[8];
    q.sd = arrays[9];
    q.sc = arrays[10];
    q.cnt = reinterpret_cast<uint32_t*>(base + kNoAllocCountersOffset);
    q.hit_list = reinterpret_cast<uint32_t*>(base + kNoAllocListOffset);
    q.miss_list = q.hit_list + kNoAllocPaths;
    q.rec = nullptr;
    q.rec_hits = nullptr;

    ptd::Fast f;
    f.pairs = reinterpret_cast<const float4*>(world->bvh_nodes);  // child pairs read in place
    f.tri4 = nullptr;                                              // triangles read in the 36-byte layout

    ptk::Tile t;
    t.image_w = params->image_size[0];
    t.image_h = params->image_size[1];
    t.origin_x = params->tile_origin[0];
    t.origin_y = params->tile_origin[1];
    t.tile_w = tile_width;
    t.tile_h = tile_height;
    t.max_bounces = params->max_bounces;
    t.accum = reinterpret_cast<float4*>(accum);
    t.image = reinterpret_cast<float4*>(image);

    ptd::Group g;
    g.vis_w = vis_w;
    g.vis_h = vis_h;
    g.pixels = (uint32_t)pixels;
    g.samples = samples;
    g.paths = (uint32_t)(pixels * samples);
    g.first_sample = params->sample_count + 1u;
    g.record_sample = 0;

    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    auto untimed = [](int, cudaStream_t, auto&& launch) { return launch(); };
    const cudaError_t e = w.any_alpha
                              ? ptw::run_group<false, true, true>(g_noalloc_devices[dev].sms, w, f, q, t, g, ptk::Sinks{nullptr, nullptr}, s, untimed)
                              : ptw::run_group<false, false, true>(g_noalloc_devices[dev].sms, w, f, q, t, g, ptk::Sinks{nullptr, nullptr}, s, untimed);
    return noalloc_cuda(error, error_size, e, "trace launch");
} catch (...) {
    std::string message;
    const int rc = pt_abi_current_status(&message);
    return noalloc_fail(error, error_size, rc, message.c_str());
}
