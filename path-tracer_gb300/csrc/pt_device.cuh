// pt_device.cuh - device-side building blocks of the path-trace pass.
//
// Each function restates the trace.slang function named in its comment.
// Everything here is compiled with -fmad=false -prec-div=true
// -prec-sqrt=true -ftz=false, so +, -, *, / and sqrt round exactly like IEEE
// binary32; fma appears only where the shader writes fma.  Vector helpers fix
// one evaluation order (dot = (x*x' + y*y') + z*z', normalize = v * (1 /
// sqrt(dot)), mix(a, b, t) = a*(1-t) + b*t, reflect(i, n) = i - (2 dot(n,i)) n,
// fract(x) = x - floor(x)), and min/max drop NaN operands; the CPU oracle uses
// the same definitions, which is what makes per-ray results bit-identical.
#pragma once

#include <stdint.h>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "../../include/pt.h"
#include "pt_fmath.h"

namespace ptd {

#define PTD __device__ __forceinline__

constexpr float kPi = 3.14159265359f;
constexpr float kInvPi = 0.31830988618f;
constexpr float kInv2Pi = 0.15915494309189535f;
constexpr float kTwoPi = 2.0f * 3.14159265359f;
constexpr float kExposure = 0.00002604166f;
constexpr float kFltMax = 0x1.fffffep+127f;
constexpr uint64_t kFnvBasis = 0xcbf29ce484222325ull;
constexpr uint64_t kFnvPrime = 0x100000001b3ull;

struct f2 {
    float x, y;
};
struct f3 {
    float x, y, z;
};

PTD f3 mk(float x, float y, float z) { return f3{x, y, z}; }
PTD f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
PTD f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
PTD f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
PTD f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
PTD f3 operator/(f3 a, f3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
PTD f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
PTD f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
PTD f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
PTD f3 operator/(float s, f3 a) { return {s / a.x, s / a.y, s / a.z}; }
PTD f3 operator+(f3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
PTD f3 operator-(float s, f3 a) { return {s - a.x, s - a.y, s - a.z}; }
PTD f3 operator-(f3 a, float s) { return {a.x - s, a.y - s, a.z - s}; }
PTD float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PTD f3 cross(f3 a, f3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
PTD float rsqrt_(float x) { return 1.0f / sqrtf(x); }
PTD float length(f3 v) { return sqrtf(dot(v, v)); }
PTD f3 normalize(f3 v) { return v * rsqrt_(dot(v, v)); }
PTD float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
PTD f3 mix(f3 a, f3 b, float t) { return {mix(a.x, b.x, t), mix(a.y, b.y, t), mix(a.z, b.z, t)}; }
PTD float saturate(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
PTD f3 saturate(f3 v) { return {saturate(v.x), saturate(v.y), saturate(v.z)}; }
PTD float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
PTD float fract(float x) { return x - floorf(x); }
PTD float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
PTD f3 reflect(f3 i, f3 n) { return i - (2.0f * dot(n, i)) * n; }
PTD bool any_positive(f3 v) { return v.x > 0.0f || v.y > 0.0f || v.z > 0.0f; }
PTD float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
PTD float comp(f3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// WGSL u32(f32): truncation, saturating, NaN -> 0
PTD uint32_t to_u32(float x) { return __float2uint_rz(x); }

// rand(), trace.slang:195-202
PTD float rand_next(uint32_t& s) {
    s = s * 747796405u + 2891336453u;
    const uint32_t word = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return __uint_as_float(0x3f800000u | (((word >> 22u) ^ word) >> 9u)) - 1.0f;
}

// seed of compute_main, trace.slang:736-737 (global_id.z is always 0)
PTD uint32_t seed(uint32_t px, uint32_t py, uint32_t sample_count) {
    uint32_t s = (px * 0x9E3779B9u) ^ (py * 0x85EBCA6Bu) ^ (sample_count * 0x27D4EB2Du) ^ 0xA511E9B3u;
    return s | 1u;
}

// the world bind group (trace.slang:163-190) as device pointers
struct World {
    const pt_triangle_geometry* geo;
    const pt_triangle_attribute* attr;
    const pt_material* mat;
    const pt_bvh_node* nodes;
    const uint8_t* srgb;
    const uint8_t* linear;
    uint32_t srgb_count;
    uint32_t linear_count;
    const float4* sky;
    const pt_skybox_alias_entry* sky_alias;
    const pt_scene_alias_entry* scene_alias;
    pt_skybox_uniforms sky_u;
    pt_scene_uniforms scene;
    pt_camera camera;
    const float* srgb_lut;  // sRGB EOTF per byte (Rgba8UnormSrgb decode), 256 floats
    int any_alpha;          // some material is not opaque
    // compressed copies (precision form); null: read attr / sky
    const uint2* attr_h = nullptr;  // pt_half_attribute records, 8 x uint2 each
    const uint2* sky_h = nullptr;   // skybox texels as BF16 RGBA
    // the triangles padded to 64 bytes (the wavefront traversal's copy), read
    // by the shading code with two vector loads; null: geo
    const float4* tri64 = nullptr;
    int attr16 = 0;  // attr is 16-byte aligned: records are read in 16-byte pieces
};

// per-path instrumentation (pt_path_record) kept in registers while tracing
struct Counters {
    uint64_t visit_hash;
    uint32_t extend_rays, shadow_rays, interior_visits, leaf_visits, triangle_tests;
    uint32_t shadow_interior_visits, shadow_leaf_visits, shadow_triangle_tests, rand_draws;
    uint32_t hits, sky_misses, light_samples, sky_light_samples;
};

// add one path's counters into device totals (one atomic per field per warp;
// __reduce_add_sync sums over exactly the lanes in the active mask)
PTD void add_totals(unsigned long long* totals, const Counters& c) {
    const uint32_t v[PT_COUNT_FIELDS] = {c.extend_rays, c.shadow_rays, c.interior_visits, c.leaf_visits,
                                         c.triangle_tests, c.shadow_interior_visits, c.shadow_leaf_visits,
                                         c.shadow_triangle_tests, c.rand_draws, c.hits, c.sky_misses,
                                         c.light_samples, c.sky_light_samples};
    const unsigned mask = __activemask();
    unsigned lane;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(lane));
    const unsigned leader = (unsigned)(__ffs(mask) - 1);
#pragma unroll
    for (int f = 0; f < PT_COUNT_FIELDS; ++f) {
        const unsigned sum = __reduce_add_sync(mask, v[f]);
        if (lane == leader) atomicAdd(totals + f, (unsigned long long)sum);
    }
}

template <bool kRec>
struct Rec {
    PTD void visit(uint32_t) {}
    PTD void interior() {}
    PTD void leaf() {}
    PTD void tri() {}
    PTD void draw() {}
};
template <>
struct Rec<true> {
    Counters* c;
    bool shadow = false;  // counting inside an any-hit (shadow) traversal
    PTD void visit(uint32_t i) { c->visit_hash = (c->visit_hash ^ i) * kFnvPrime; }
    PTD void interior() {
        c->interior_visits += 1;
        if (shadow) c->shadow_interior_visits += 1;
    }
    PTD void leaf() {
        c->leaf_visits += 1;
        if (shadow) c->shadow_leaf_visits += 1;
    }
    PTD void tri() {
        c->triangle_tests += 1;
        if (shadow) c->shadow_triangle_tests += 1;
    }
    PTD void draw() { c->rand_draws += 1; }
};

template <bool kRec>
struct Rng {
    uint32_t s;
    Rec<kRec> rec;
    PTD float operator()() {
        rec.draw();
        return rand_next(s);
    }
};

PTD f3 vert(const World& w, uint32_t tri, int k) {
    const float* v = w.geo[tri].v0 + 3 * k;
    return mk(__ldg(v), __ldg(v + 1), __ldg(v + 2));
}

struct Tri {
    f3 v0, v1, v2;
};
PTD Tri load_tri(const World& w, uint32_t tri) {
    const float* p = w.geo[tri].v0;
    Tri t;
    t.v0 = mk(__ldg(p + 0), __ldg(p + 1), __ldg(p + 2));
    t.v1 = mk(__ldg(p + 3), __ldg(p + 4), __ldg(p + 5));
    t.v2 = mk(__ldg(p + 6), __ldg(p + 7), __ldg(p + 8));
    return t;
}
// The hit triangle for the shading frame: with the 64-byte padded copy one
// 256-bit and one 128-bit load instead of nine 32-bit loads (same values)
PTD Tri load_hit_tri(const World& w, uint32_t tri) {
    if (!w.tri64) return load_tri(w, tri);
    const float4* p = w.tri64 + 4 * (size_t)tri;
    float4 a, b;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
    const float4 c = __ldg(p + 2);
    Tri t;
    t.v0 = mk(a.x, a.y, a.z);
    t.v1 = mk(b.x, b.y, b.z);
    t.v2 = mk(c.x, c.y, c.z);
    return t;
}

// nearest + clamp-to-edge atlas fetch (default sampler, world_resources.rs:447-450)
PTD float4 atlas(const World& w, bool srgb, int32_t layer, f2 uv) {
    const uint32_t count = srgb ? w.srgb_count : w.linear_count;
    const uint8_t* base = srgb ? w.srgb : w.linear;
    if (count == 0u) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const uint32_t l = layer < 0 ? 0u : ((uint32_t)layer >= count ? count - 1u : (uint32_t)layer);
    const float fx = floorf(uv.x * 8192.0f), fy = floorf(uv.y * 8192.0f);
    const uint32_t ix = fx >= 8191.0f ? 8191u : to_u32(fx);
    const uint32_t iy = fy >= 8191.0f ? 8191u : to_u32(fy);
    const uchar4 p = __ldg(reinterpret_cast<const uchar4*>(base) + ((uint64_t)l * PT_ATLAS_SIZE + iy) * PT_ATLAS_SIZE + ix);
    if (srgb)
        return make_float4(__ldg(w.srgb_lut + p.x), __ldg(w.srgb_lut + p.y), __ldg(w.srgb_lut + p.z), (float)p.w / 255.0f);
    return make_float4((float)p.x / 255.0f, (float)p.y / 255.0f, (float)p.z / 255.0f, (float)p.w / 255.0f);
}

PTD f2 atlas_uv(f2 uv, const float* os) { return {fma_(uv.x, os[2], os[0]), fma_(uv.y, os[3], os[1])}; }

// bilinear + clamp-to-edge skybox fetch (skybox sampler, world_resources.rs:451-456)
PTD uint32_t sky_index(float f, uint32_t n, int off) {
    if (!(f == f)) return 0u;
    int64_t i = f < -1e9f ? -1000000000ll : (f > 1e9f ? 1000000000ll : (int64_t)f);
    i += off;
    if (i < 0) i = 0;
    if (i > (int64_t)n - 1) i = (int64_t)n - 1;
    return (uint32_t)i;
}
PTD f3 sky_px(const World& w, uint32_t ix, uint32_t iy) {
    const uint64_t i = (uint64_t)iy * w.sky_u.width + ix;
    if (w.sky_h) {
        const uint2 p = __ldg(w.sky_h + i);
        const __nv_bfloat162 rg = *reinterpret_cast<const __nv_bfloat162*>(&p.x);
        return mk(__low2float(rg), __high2float(rg), __bfloat162float(__ushort_as_bfloat16((unsigned short)(p.y & 0xffffu))));
    }
    const float4 p = __ldg(w.sky + i);
    return mk(p.x, p.y, p.z);
}
PTD f3 skybox_bilinear(const World& w, f2 uv) {
    const uint32_t W = w.sky_u.width, H = w.sky_u.height;
    const float x = uv.x * (float)W - 0.5f, y = uv.y * (float)H - 0.5f;
    const float x0 = floorf(x), y0 = floorf(y);
    const float fx = x - x0, fy = y - y0;
    const uint32_t ix0 = sky_index(x0, W, 0), ix1 = sky_index(x0, W, 1);
    const uint32_t iy0 = sky_index(y0, H, 0), iy1 = sky_index(y0, H, 1);
    const f3 top = mix(sky_px(w, ix0, iy0), sky_px(w, ix1, iy0), fx);
    const f3 bottom = mix(sky_px(w, ix0, iy1), sky_px(w, ix1, iy1), fx);
    return mix(top, bottom, fy);
}

// orthonormal_tangent, trace.slang:207-218
PTD f3 orthonormal_tangent(f3 tangent, f3 normal) {
    const f3 projected = tangent - dot(normal, tangent) * normal;
    const float ls = dot(projected, projected);
    if (ls > 1e-12f) return projected * rsqrt_(ls);
    const float s = normal.z >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (s + normal.z);
    return mk(fma_(s * normal.x * normal.x, a, 1.0f), s * normal.x * normal.y * a, -s * normal.x);
}

PTD float fifth_power(float x) { return x * x * x * x * x; }

// fresnel_exact, trace.slang:330-341, with ior2 = ior * ior given
PTD float fresnel_exact_sq(float ior, float ior2, float cos_i) {
    const float s = fma_(-cos_i, cos_i, 1.0f) / ior2;
    if (s >= 1.0f) return 1.0f;
    const float cos_t = sqrtf(1.0f - s);
    const float rs = fma_(-ior, cos_t, cos_i) / fma_(ior, cos_t, cos_i);
    const float rp = fma_(-ior, cos_i, cos_t) / fma_(ior, cos_i, cos_t);
    return 0.5f * (rs * rs + rp * rp);
}
PTD float fresnel_exact(float ior, float cos_i) { return fresnel_exact_sq(ior, ior * ior, cos_i); }

// ggx_lambda, trace.slang:347-352, with the squared roughnesses ax2 = a.x * a.x, ay2 = a.y * a.y given
PTD float ggx_lambda_sq(f3 v, float ax2, float ay2) {
    return fma_(0.5f, sqrtf(1.0f + (ax2 * v.x * v.x + ay2 * v.y * v.y) / (v.z * v.z)), -0.5f);
}
PTD float ggx_lambda(f3 v, f2 a) { return ggx_lambda_sq(v, a.x * a.x, a.y * a.y); }

// sample_VNDF, trace.slang:356-364, with sin / cos of 2 pi r given and the
// view vector's part computed: ww = normalize((wo.x a.x, wo.y a.y, wo.z)),
// ww1 = 1 + ww.z
PTD f3 sample_vndf_ww(f3 ww, float ww1, f2 a, float r, float sin_2pr, float cos_2pr) {
    const float z = fma_(1.0f - r, ww1, -ww.z);
    const float sin_theta = sqrtf(saturate(fma_(-z, z, 1.0f)));
    const float x = sin_theta * cos_2pr;
    const float y = sin_theta * sin_2pr;
    const f3 h = mk(x, y, z) + ww;
    return normalize(mk(h.x * a.x, h.y * a.y, h.z));
}
PTD f3 vndf_view(f3 wo, f2 a) { return normalize(mk(wo.x * a.x, wo.y * a.y, wo.z)); }
PTD f3 sample_vndf_sc(f3 wo, f2 a, float r, float sin_2pr, float cos_2pr) {
    const f3 ww = vndf_view(wo, a);
    return sample_vndf_ww(ww, 1.0f + ww.z, a, r, sin_2pr, cos_2pr);
}
// 1: sin and cos of one argument share one reduction (same bits either way)
#ifndef PT_SHARED_SINCOS
#define PT_SHARED_SINCOS 1
#endif
PTD f3 sample_vndf(f3 wo, f2 a, float r, float two_pi_r) {
    float sn, cs;
#if PT_SHARED_SINCOS
    ptm::sincosf_(two_pi_r, &sn, &cs);
#else
    sn = ptm::sinf_(two_pi_r);
    cs = ptm::cosf_(two_pi_r);
#endif
    return sample_vndf_sc(wo, a, r, sn, cs);
}

// alpha_anisotropic, trace.slang:369-375
PTD f2 alpha_anisotropic(float roughness, float anisotropy) {
    const float iso = 1.0f - anisotropy;
    const float at = roughness * roughness * 1.41421356237f * rsqrt_(fma_(iso, iso, 1.0f));
    return {fmaxf(at, 1e-4f), fmaxf(at * iso, 1e-4f)};
}

// specular_ior_modulated, trace.slang:379-391
PTD float specular_ior_modulated(float ior, float weight) {
    const float num = ior - 1.0f;
    const float den = ior + 1.0f;
    const float f0 = num * num / (den * den);
    const float f0s = signf(ior - 1.0f) * sqrtf(fminf(weight * f0, __uint_as_float(0x3f800000u - 1u)));
    return (1.0f + f0s) / (1.0f - f0s);
}

// power_heuristic, trace.slang:416-424
PTD float power_heuristic(float pdf, float other) {
    const float scale = fmaxf(pdf, other);
    if (scale <= 0.0f) return 0.0f;
    const float p = pdf / scale;
    const float q = other / scale;
    return p * p / (p * p + q * q);
}

// Triangle attributes (TriangleAttribute, trace.slang:57-66) from the FP32
// records, or from the FP16 records of the precision form (pt_half_attribute:
// n0..n2 at uint2 0..2, t0..t2 at 3..5, uv0..uv2 in words 12..14, material
// in word 15).
PTD f3 half3_of(uint2 p) {
    const __half2 a = *reinterpret_cast<const __half2*>(&p.x);
    return mk(__low2float(a), __high2float(a), __half2float(__ushort_as_half((unsigned short)(p.y & 0xffffu))));
}
PTD uint32_t attr_material(const World& w, uint32_t tri) {
    if (w.attr_h) return __ldg(reinterpret_cast<const uint32_t*>(w.attr_h + 8 * (size_t)tri) + 15);
    return __ldg(&w.attr[tri].material_index);
}
PTD f3 attr_normal(const World& w, uint32_t tri, int k) {
    if (w.attr_h) return half3_of(__ldg(w.attr_h + 8 * (size_t)tri + k));
    const float* n = k == 0 ? w.attr[tri].n0 : (k == 1 ? w.attr[tri].n1 : w.attr[tri].n2);
    return mk(__ldg(n), __ldg(n + 1), __ldg(n + 2));
}
// xyz of tangent k; w of tangent 0 through attr_tangent0_w
PTD f3 attr_tangent(const World& w, uint32_t tri, int k) {
    if (w.attr_h) return half3_of(__ldg(w.attr_h + 8 * (size_t)tri + 3 + k));
    const float* t = k == 0 ? w.attr[tri].t0 : (k == 1 ? w.attr[tri].t1 : w.attr[tri].t2);
    return mk(__ldg(t), __ldg(t + 1), __ldg(t + 2));
}
PTD float attr_tangent0_w(const World& w, uint32_t tri) {
    if (w.attr_h) return __half2float(__ushort_as_half((unsigned short)(__ldg(&w.attr_h[8 * (size_t)tri + 3].y) >> 16)));
    return __ldg(&w.attr[tri].t0[3]);
}
PTD f2 attr_uv(const World& w, uint32_t tri, int k) {
    if (w.attr_h) {
        const uint32_t bits = __ldg(reinterpret_cast<const uint32_t*>(w.attr_h + 8 * (size_t)tri) + 12 + k);
        const __half2 a = *reinterpret_cast<const __half2*>(&bits);
        return {__low2float(a), __high2float(a)};
    }
    const float* uv = k == 0 ? w.attr[tri].uv0 : (k == 1 ? w.attr[tri].uv1 : w.attr[tri].uv2);
    return {__ldg(uv), __ldg(uv + 1)};
}

// The FP32 attribute record (112 bytes) in 16-byte pieces, when the buffer is
// 16-byte aligned: [0] material, n0 | [1] n1, n2.x | [2] n2.yz, uv0 |
// [3] uv1, uv2 | [4] t0 | [5] t1 | [6] t2.  Three normals, three tangents or
// three UVs then take two or three 128-bit loads instead of six to ten
// 32-bit loads (same values).
#ifndef PT_VEC_ATTR
#define PT_VEC_ATTR 1
#endif
PTD bool attr_pieces(const World& w) { return PT_VEC_ATTR && w.attr16 && !w.attr_h; }
PTD float4 attr_piece(const World& w, uint32_t tri, int k) {
    return __ldg(reinterpret_cast<const float4*>(w.attr + tri) + k);
}
PTD void attr_normals(const World& w, uint32_t tri, f3& n0, f3& n1, f3& n2) {
    if (attr_pieces(w)) {
        const float4 a = attr_piece(w, tri, 0), b = attr_piece(w, tri, 1), c = attr_piece(w, tri, 2);
        n0 = mk(a.y, a.z, a.w);
        n1 = mk(b.x, b.y, b.z);
        n2 = mk(b.w, c.x, c.y);
        return;
    }
    n0 = attr_normal(w, tri, 0);
    n1 = attr_normal(w, tri, 1);
    n2 = attr_normal(w, tri, 2);
}
PTD void attr_tangents(const World& w, uint32_t tri, f3& t0, f3& t1, f3& t2, float& t0w) {
    if (attr_pieces(w)) {
        const float4 a = attr_piece(w, tri, 4), b = attr_piece(w, tri, 5), c = attr_piece(w, tri, 6);
        t0 = mk(a.x, a.y, a.z);
        t0w = a.w;
        t1 = mk(b.x, b.y, b.z);
        t2 = mk(c.x, c.y, c.z);
        return;
    }
    t0 = attr_tangent(w, tri, 0);
    t1 = attr_tangent(w, tri, 1);
    t2 = attr_tangent(w, tri, 2);
    t0w = attr_tangent0_w(w, tri);
}

PTD f2 interp_uv(const World& w, uint32_t tri, float u, float v, float w2) {
    f2 a, b, c;
    if (attr_pieces(w)) {
        const float4 p = attr_piece(w, tri, 2), q = attr_piece(w, tri, 3);
        a = {p.z, p.w};
        b = {q.x, q.y};
        c = {q.z, q.w};
    } else {
        a = attr_uv(w, tri, 0);
        b = attr_uv(w, tri, 1);
        c = attr_uv(w, tri, 2);
    }
    return {fract(u * a.x + v * b.x + w2 * c.x), fract(u * a.y + v * b.y + w2 * c.y)};
}

// coverage, trace.slang:426-443
PTD float coverage(const World& w, const pt_material& m, f2 uv) {
    if (m.alpha_mode == PT_ALPHA_MODE_OPAQUE) return 1.0f;
    float alpha = m.base_color[3];
    if (m.base_color_tex_layer >= 0) alpha *= atlas(w, true, m.base_color_tex_layer, atlas_uv(uv, m.base_color_uv)).w;
    if (m.alpha_mode == PT_ALPHA_MODE_MASK) return alpha >= m.alpha_cutoff ? 1.0f : 0.0f;
    return alpha;
}

// passes_through, trace.slang:446-454
template <bool kRec>
PTD bool passes_through(const World& w, uint32_t tri, float v, float w2, Rng<kRec>& rng) {
    const pt_material& m = w.mat[attr_material(w, tri)];
    if (m.alpha_mode == PT_ALPHA_MODE_OPAQUE) return false;
    const f2 uv = interp_uv(w, tri, 1.0f - v - w2, v, w2);
    return coverage(w, m, uv) <= rng();
}

// evaluate_emission, trace.slang:455-466
PTD f3 evaluate_emission(const World& w, const pt_material& m, f2 uv) {
    f3 color = mk(m.emission_color_and_luminance[0], m.emission_color_and_luminance[1], m.emission_color_and_luminance[2]);
    if (m.emission_tex_layer >= 0) {
        const float4 t = atlas(w, true, m.emission_tex_layer, atlas_uv(uv, m.emission_uv));
        color = color * mk(t.x, t.y, t.z);
    }
    return m.emission_weight * m.emission_color_and_luminance[3] * color;
}

// skybox_uv, trace.slang:467-472
PTD f2 skybox_uv(f3 d) {
    return {fract(fma_(ptm::atan2f_(d.z, d.x), kInv2Pi, 0.5f)), ptm::atan2f_(sqrtf(d.x * d.x + d.z * d.z), d.y) * kInvPi};
}

// evaluate_skybox, trace.slang:473-475
PTD f3 evaluate_skybox(const World& w, f3 d) { return skybox_bilinear(w, skybox_uv(d)) * w.sky_u.average_luminance; }

// skybox_texel_solid_angle, trace.slang:476-481
PTD float skybox_texel_solid_angle(const World& w, uint32_t row) {
    const float step = kPi / (float)w.sky_u.height;
    const uint32_t other = w.sky_u.height - 1u - row;
    const uint32_t pole_row = row < other ? row : other;
    return (kTwoPi / (float)w.sky_u.width) * 2.0f * ptm::sinf_(((float)pole_row + 0.5f) * step) * ptm::sinf_(0.5f * step);
}

// skybox_light_pdf, trace.slang:482-489
PTD float skybox_light_pdf(const World& w, f3 d, float prob) {
    if (prob <= 0.0f) return 0.0f;
    const f2 uv = skybox_uv(d);
    uint32_t px = to_u32(uv.x * (float)w.sky_u.width);
    uint32_t py = to_u32(uv.y * (float)w.sky_u.height);
    if (px > w.sky_u.width - 1u) px = w.sky_u.width - 1u;
    if (py > w.sky_u.height - 1u) py = w.sky_u.height - 1u;
    return prob * __ldg(&w.sky_alias[(uint64_t)py * w.sky_u.width + px].selection_probability) /
           skybox_texel_solid_angle(w, py);
}

// triangle_selection_probability, trace.slang:490-507
PTD float triangle_selection_probability(const World& w, uint32_t tri) {
    uint32_t first = 0u, end = w.scene.emissive_triangles_count;
    while (first < end) {
        const uint32_t middle = first + (end - first) / 2u;
        const uint32_t ti = __ldg(&w.scene_alias[middle].triangle_index);
        if (ti < tri) first = middle + 1u;
        else if (ti > tri) end = middle;
        else return __ldg(&w.scene_alias[middle].selection_probability);
    }
    return 0.0f;
}

// triangle_light_pdf, trace.slang:508-523
PTD float triangle_light_pdf(const World& w, uint32_t tri, f3 d, float dist2, float prob) {
    if (prob <= 0.0f) return 0.0f;
    const Tri t = load_tri(w, tri);
    const float area = 0.5f * fabsf(dot(cross(t.v1 - t.v0, t.v2 - t.v0), d));
    if (area <= 0.0f) return 0.0f;
    return prob * dist2 / area;
}

struct LightSample {
    f3 direction;
    float distance;
    f3 emission;
    float pdf;
    int32_t triangle_index;
};

// sample_light, trace.slang:531-592
template <bool kRec>
PTD LightSample sample_light(const World& w, f3 origin, Rng<kRec>& rng, Counters* c) {
    LightSample r;
    r.direction = mk(0.0f, 0.0f, 0.0f);
    r.distance = 0.0f;
    r.emission = mk(0.0f, 0.0f, 0.0f);
    r.pdf = 0.0f;
    r.triangle_index = -1;
    const float p0 = w.scene.light_probabilities[0], p1 = w.scene.light_probabilities[1];
    if (p0 + p1 <= 0.0f) return r;
    if (rng() < p0) {
        if (kRec) c->light_samples += 1;
        const uint32_t count = w.scene.emissive_triangles_count;
        uint32_t slot = to_u32(rng() * (float)count);
        if (slot > count - 1u) slot = count - 1u;
        const pt_scene_alias_entry cand = w.scene_alias[slot];
        const pt_scene_alias_entry entry = w.scene_alias[rng() < cand.threshold ? slot : cand.alias_index];
        const Tri t = load_tri(w, entry.triangle_index);
        const float root = sqrtf(rng());
        const float u = 1.0f - root;
        const float v = root * (1.0f - rng());
        const float wb = 1.0f - u - v;
        const f3 delta = u * t.v0 + v * t.v1 + wb * t.v2 - origin;
        const float d2 = dot(delta, delta);
        if (d2 <= 0.0f) return r;
        r.distance = sqrtf(d2);
        r.direction = delta / r.distance;
        r.triangle_index = (int32_t)entry.triangle_index;
        r.pdf = triangle_light_pdf(w, entry.triangle_index, r.direction, d2, p0 * entry.selection_probability);
        const f2 uv = interp_uv(w, entry.triangle_index, u, v, wb);
        const pt_material& m = w.mat[attr_material(w, entry.triangle_index)];
        r.emission = coverage(w, m, uv) * evaluate_emission(w, m, uv);
    } else {
        if (kRec) c->sky_light_samples += 1;
        const uint32_t W = w.sky_u.width, H = w.sky_u.height;
        const uint32_t count = W * H;
        uint32_t slot = to_u32(rng() * (float)count);
        if (slot > count - 1u) slot = count - 1u;
        const pt_skybox_alias_entry cand = w.sky_alias[slot];
        const uint32_t index = rng() < cand.threshold ? slot : cand.alias_index;
        const uint32_t row = index / W, column = index % W;
        const float phi = (((float)column + rng()) / (float)W - 0.5f) * kTwoPi;
        const bool north = row < H / 2u;
        const uint32_t pole_row = north ? row : H - 1u - row;
        const float half_step = 0.5f * kPi / (float)H;
        const float a = ptm::sinf_((float)pole_row * half_step);
        const float b = ptm::sinf_((float)(pole_row + 1u) * half_step);
        const float shs = mix(a * a, b * b, rng());
        const float cos_theta = 1.0f - 2.0f * shs;
        const float sin_theta = 2.0f * sqrtf(fmaxf(0.0f, shs * (1.0f - shs)));
        float sin_phi, cos_phi;
        ptm::sincosf_(phi, &sin_phi, &cos_phi);
        r.direction = mk(sin_theta * cos_phi, north ? cos_theta : -cos_theta, sin_theta * sin_phi);
        r.distance = kFltMax;
        r.pdf = skybox_light_pdf(w, r.direction, p1);
        r.emission = evaluate_skybox(w, r.direction);
    }
    return r;
}

// three-input minimum / maximum (one instruction on sm_100 and later; NaN
// inputs are ignored as by nested fminf / fmaxf, and the result is exact, so
// it equals the nested two-input form except possibly in the sign of a zero)
PTD float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
PTD float min3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// 1: the slab test takes its entry and exit distances with three-input
// min/max; 0: nested two-input fminf / fmaxf.  The three-input form gives the
// same visits (the parity tests pass with it) but measured slower (extend
// 387 against 369 ms over three 64-spp images of the 2.1M-triangle scene)
#ifndef PT_MINMAX3
#define PT_MINMAX3 0
#endif
// the same choice for the 8-wide traversal's child test
#ifndef PT_WIDE_MINMAX3
#define PT_WIDE_MINMAX3 1
#endif

// intersect_aabb, trace.slang:597-609, on a node's bounds.  A zero's sign
// never matters here: the results are only compared, and the returned
// distance is max(0, t_near).
PTD float intersect_aabb(const float* bmin, const float* bmax, f3 nod, f3 rcp, float hit_t) {
    const float t0x = fma_(bmin[0], rcp.x, nod.x), t0y = fma_(bmin[1], rcp.y, nod.y), t0z = fma_(bmin[2], rcp.z, nod.z);
    const float t1x = fma_(bmax[0], rcp.x, nod.x), t1y = fma_(bmax[1], rcp.y, nod.y), t1z = fma_(bmax[2], rcp.z, nod.z);
#if PT_MINMAX3
    const float t_near = max3f(fminf(t0x, t1x), fminf(t0y, t1y), fminf(t0z, t1z));
    const float t_far = min3f(fmaxf(t0x, t1x), fmaxf(t0y, t1y), fmaxf(t0z, t1z));
#else
    const float t_near = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
    const float t_far = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
#endif
    return (t_near <= t_far && t_far > 0.0f && t_near < hit_t) ? fmaxf(0.0f, t_near) : -1.0f;
}

// watertight shear setup, trace.slang:769-783
struct Shear {
    int kx, ky, kz;
    float sx, sy, sz;
};
PTD Shear make_shear(f3 d, f3 rcp) {
    const float adx = fabsf(d.x), ady = fabsf(d.y), adz = fabsf(d.z);
    const int kxy = adx > ady ? 0 : 1;
    const int kz = (kxy == 0 ? adx : ady) > adz ? kxy : 2;
    const int kx_val = kz == 2 ? 0 : kz + 1;
    const int ky_val = kx_val == 2 ? 0 : kx_val + 1;
    const bool is_neg = comp(d, kz) < 0.0f;
    Shear s;
    s.kz = kz;
    s.kx = is_neg ? ky_val : kx_val;
    s.ky = is_neg ? kx_val : ky_val;
    s.sz = comp(rcp, kz);
    s.sx = -comp(d, s.kx) * s.sz;
    s.sy = -comp(d, s.ky) * s.sz;
    return s;
}

// watertight ray-triangle test, trace.slang:807-834 (false = rejected)
PTD bool triangle_test(const Tri& t, f3 o, const Shear& s, float* t_out, float* v_out, float* w_out) {
    const f3 A = t.v0 - o, B = t.v1 - o, C = t.v2 - o;
    const float akz = comp(A, s.kz), bkz = comp(B, s.kz), ckz = comp(C, s.kz);
    const float ax = fma_(s.sx, akz, comp(A, s.kx));
    const float ay = fma_(s.sy, akz, comp(A, s.ky));
    const float bx = fma_(s.sx, bkz, comp(B, s.kx));
    const float by = fma_(s.sy, bkz, comp(B, s.ky));
    const float cx = fma_(s.sx, ckz, comp(C, s.kx));
    const float cy = fma_(s.sy, ckz, comp(C, s.ky));
    const float U = fma_(cx, by, -cy * bx);
    const float V = fma_(ax, cy, -ay * cx);
    const float W = fma_(bx, ay, -by * ax);
    if (fminf(U, fminf(V, W)) < 0.0f && fmaxf(U, fmaxf(V, W)) > 0.0f) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float inv_det = 1.0f / det;
    *t_out = s.sz * fma_(U, akz, fma_(V, bkz, W * ckz)) * inv_det;
    *v_out = V * inv_det;
    *w_out = W * inv_det;
    return true;
}

// E_FON_exact, trace.slang:318-323
// with af = 1 / (1 + 0.28779340921 r) given
PTD float e_fon_af(float mu, float r, float af) {
    const float si = sqrtf(fma_(-mu, mu, 1.0f));
    const float g = si * (ptm::acosf_(mu) - si * mu) + 0x1.555556p-1f * ((si / mu) * (1.0f - (si * si * si)) - si);
    return af + r * af * kInvPi * g;
}
PTD float e_fon_exact(float mu, float r) { return e_fon_af(mu, r, 1.0f / fma_(0.28779340921f, r, 1.0f)); }

// state of one shading point shared by both lobe evaluations (trace.slang:1097-1181)
struct Bsdf {
    float p_ggx, p_diffuse;
    f3 base_color;
    float base_weight, base_metalness, base_diffuse_roughness;
    f3 specular_color;
    float specular_weight, ior_m;
    f2 alpha;
    float opl;
    f3 f0;
    f3 e_dielectric;
    float la, lb, lc, ld;  // ltc_coefficients
    f3 bx, by;             // rows 0 and 1 of orthonormal_basis_ltc_wo (row 2 = z axis)
    float p_u, p_c;
};

struct Lobes {
    f3 f;
    float pdf;
};

// evaluate_lobes, trace.slang:229-315
PTD Lobes evaluate_lobes(f3 wo, f3 wi, const Bsdf& b) {
    const f3 h = normalize(wo + wi);
    const float hdotw = dot(h, wo);
    const float g1 = 1.0f / b.opl;
    const float g2 = 1.0f / (b.opl + ggx_lambda(wi, b.alpha));
    const float dh = (h.x * h.x) / (b.alpha.x * b.alpha.x) + (h.y * h.y) / (b.alpha.y * b.alpha.y) + h.z * h.z;
    const float D = kInvPi / (b.alpha.x * b.alpha.y * dh * dh);
    const float ts = D * g2 / (4.0f * wi.z * wo.z);
    const float omh = 1.0f - hdotw;
    const float p5 = fifth_power(omh);
    const f3 fa = (0.00105024005f * hdotw * omh) * (1.0f - b.specular_color);
    const f3 fb = 9031.0f * b.f0 + 7776.0f;
    const f3 fc = b.f0 - 1.0f;
    const f3 fm = mk(fma_(fa.x, fb.x, fc.x), fma_(fa.y, fb.y, fc.y), fma_(fa.z, fb.z, fc.z));
    const f3 f82 = b.f0 - p5 * fm;
    const f3 f_conductor = saturate(b.specular_weight * f82) * ts;
    const f3 f_dielectric = b.specular_color * fresnel_exact(b.ior_m, hdotw) * ts;
    const f3 rho = b.base_color;
    const float r = b.base_diffuse_roughness;
    const float s_f = wi.x * wo.x + wi.y * wo.y;
    const float sovert_f = s_f > 0.0f ? s_f / fmaxf(wo.z, wi.z) : s_f;
    const float af = 1.0f / fma_(0.28779340921f, r, 1.0f);
    const f3 f_ss = rho * kInvPi * af * fma_(r, sovert_f, 1.0f);
    const float efo = e_fon_exact(wo.z, r);
    const float efi = e_fon_exact(wi.z, r);
    const float avg_ef = af * fma_(0.07248821245f, r, 1.0f);
    const f3 rho_ms = rho * rho * avg_ef / (1.0f - rho * (1.0f - avg_ef));
    const f3 f_ms = (rho_ms * kInvPi) * fmaxf(1.0e-7f, 1.0f - efo) * fmaxf(1.0e-7f, 1.0f - efi) / fmaxf(1.0e-7f, 1.0f - avg_ef);
    const f3 f_diffuse = b.base_weight * (f_ss + f_ms);
    const f3 f_glossy_diffuse = f_dielectric + (1.0f - b.e_dielectric) * f_diffuse;
    const f3 f_total = mix(f_glossy_diffuse, f_conductor, b.base_metalness);
    const float pdf_ggx = D * g1 / (4.0f * wo.z);
    const f3 wl = mk(dot(b.bx, wi), dot(b.by, wi), dot(mk(0.0f, 0.0f, 1.0f), wi));
    const float a = b.la, bb = b.lb, c = b.lc, d = b.ld;
    const float det_m = c * fma_(-bb, d, a);
    const f3 wh = mk(c * (wl.x - bb * wl.z), (a - bb * d) * wl.y, -c * (d * wl.x - a * wl.z));
    const float len_sqr = dot(wh, wh);
    const float s_pdf = fma_(0.5f, rsqrt_(fma_(d, d, 1.0f)), 0.5f);
    const float pdf_c = (det_m * det_m) / (len_sqr * len_sqr) * fmaxf(wh.z, 0.0f) / (kPi * s_pdf);
    const float pdf_eon = b.p_u * 0.15915494309f + b.p_c * pdf_c;
    return {f_total, b.p_ggx * pdf_ggx + b.p_diffuse * pdf_eon};
}

// The parts of evaluate_lobes that depend on the shading point and wo but not
// on wi (the G1 term, the Oren-Nayar single- and multiple-scattering factors
// with E_FON(wo), the LTC determinant and normalisation), for the two
// evaluations of one shading point (next-event and BSDF sample).  Each is the
// same operations in the same order as inside evaluate_lobes, so
// evaluate_lobes_t gives evaluate_lobes's bits.  Measured slower on the
// 2.1M-triangle scene (1920x1080x64: 1814 against 1817 Mrays/s, shade 201.7
// against 199.5 ms over three images: the 14 values kept live between the
// two evaluations raise the shading kernel's spills from 280 to 332 bytes),
// so off by default.
#ifndef PT_LOBE_TERMS
#define PT_LOBE_TERMS 0
#endif
struct LobeTerms {
    float g1, af, ms_den, det2, pi_s, four_woz, amb;
    f3 ss, ms;
};
PTD LobeTerms lobe_terms(f3 wo, const Bsdf& b) {
    LobeTerms t;
    t.g1 = 1.0f / b.opl;
    const float r = b.base_diffuse_roughness;
    const f3 rho = b.base_color;
    t.af = 1.0f / fma_(0.28779340921f, r, 1.0f);
    t.ss = rho * kInvPi * t.af;
    const float efo = e_fon_af(wo.z, r, t.af);
    const float avg_ef = t.af * fma_(0.07248821245f, r, 1.0f);
    const f3 rho_ms = rho * rho * avg_ef / (1.0f - rho * (1.0f - avg_ef));
    t.ms = (rho_ms * kInvPi) * fmaxf(1.0e-7f, 1.0f - efo);
    t.ms_den = fmaxf(1.0e-7f, 1.0f - avg_ef);
    const float a = b.la, bb = b.lb, c = b.lc, d = b.ld;
    const float det_m = c * fma_(-bb, d, a);
    t.det2 = det_m * det_m;
    t.amb = a - bb * d;
    t.pi_s = kPi * fma_(0.5f, rsqrt_(fma_(d, d, 1.0f)), 0.5f);
    t.four_woz = 4.0f * wo.z;
    return t;
}
PTD Lobes evaluate_lobes_t(f3 wo, f3 wi, const Bsdf& b, const LobeTerms& t) {
    const f3 h = normalize(wo + wi);
    const float hdotw = dot(h, wo);
    const float g2 = 1.0f / (b.opl + ggx_lambda(wi, b.alpha));
    const float dh = (h.x * h.x) / (b.alpha.x * b.alpha.x) + (h.y * h.y) / (b.alpha.y * b.alpha.y) + h.z * h.z;
    const float D = kInvPi / (b.alpha.x * b.alpha.y * dh * dh);
    const float ts = D * g2 / (4.0f * wi.z * wo.z);
    const float omh = 1.0f - hdotw;
    const float p5 = fifth_power(omh);
    const f3 fa = (0.00105024005f * hdotw * omh) * (1.0f - b.specular_color);
    const f3 fb = 9031.0f * b.f0 + 7776.0f;
    const f3 fc = b.f0 - 1.0f;
    const f3 fm = mk(fma_(fa.x, fb.x, fc.x), fma_(fa.y, fb.y, fc.y), fma_(fa.z, fb.z, fc.z));
    const f3 f82 = b.f0 - p5 * fm;
    const f3 f_conductor = saturate(b.specular_weight * f82) * ts;
    const f3 f_dielectric = b.specular_color * fresnel_exact(b.ior_m, hdotw) * ts;
    const float r = b.base_diffuse_roughness;
    const float s_f = wi.x * wo.x + wi.y * wo.y;
    const float sovert_f = s_f > 0.0f ? s_f / fmaxf(wo.z, wi.z) : s_f;
    const f3 f_ss = t.ss * fma_(r, sovert_f, 1.0f);
    const float efi = e_fon_af(wi.z, r, t.af);
    const f3 f_ms = t.ms * fmaxf(1.0e-7f, 1.0f - efi) / t.ms_den;
    const f3 f_diffuse = b.base_weight * (f_ss + f_ms);
    const f3 f_glossy_diffuse = f_dielectric + (1.0f - b.e_dielectric) * f_diffuse;
    const f3 f_total = mix(f_glossy_diffuse, f_conductor, b.base_metalness);
    const float pdf_ggx = D * t.g1 / t.four_woz;
    const f3 wl = mk(dot(b.bx, wi), dot(b.by, wi), dot(mk(0.0f, 0.0f, 1.0f), wi));
    const float a = b.la, bb = b.lb, c = b.lc, d = b.ld;
    const f3 wh = mk(c * (wl.x - bb * wl.z), t.amb * wl.y, -c * (d * wl.x - a * wl.z));
    const float len_sqr = dot(wh, wh);
    const float pdf_c = t.det2 / (len_sqr * len_sqr) * fmaxf(wh.z, 0.0f) / t.pi_s;
    const float pdf_eon = b.p_u * 0.15915494309f + b.p_c * pdf_c;
    return {f_total, b.p_ggx * pdf_ggx + b.p_diffuse * pdf_eon};
}

// estimate_e_dielectric, trace.slang:396-411.  With PT_HOIST_INVARIANTS the
// parts of sample_VNDF, fresnel_exact and ggx_lambda that do not change
// between the 16 samples (the stretched view vector, ior^2, the squared
// roughnesses) are evaluated once before the loop, by the same operations in
// the same order, so every sample's bits are those of the plain loop
// (1920x1080x64 on the 2.1M-triangle scene: 1817 against 1797 Mrays/s, shade
// 199.5 against 207.8 ms over three images).
#ifndef PT_HOIST_INVARIANTS
#define PT_HOIST_INVARIANTS 1
#endif
// unroll factor of that loop (1: a rolled loop; 2 and 4 measured slower on
// the 2.1M-triangle scene, 1798 and 1789 against 1818 Mrays/s)
#ifndef PT_EDIEL_UNROLL
#define PT_EDIEL_UNROLL 1
#endif
#define PT_STRINGIFY(x) #x
#define PT_PRAGMA(x) _Pragma(PT_STRINGIFY(x))
template <bool kRec>
PTD f3 estimate_e_dielectric(f3 wo, float opl, f2 alpha, float ior_m, f3 spec_color, Rng<kRec>& rng) {
    float sum = 0.0f;
#if PT_HOIST_INVARIANTS
    const f3 ww = vndf_view(wo, alpha);
    const float ww1 = 1.0f + ww.z;
    const float ior2 = ior_m * ior_m;
    const float ax2 = alpha.x * alpha.x, ay2 = alpha.y * alpha.y;
    PT_PRAGMA(unroll PT_EDIEL_UNROLL)
    for (int i = 0; i < 16; ++i) {
        const float r1 = rng();
        const float tpr = kTwoPi * rng();
        float sn, cs;
#if PT_SHARED_SINCOS
        ptm::sincosf_(tpr, &sn, &cs);
#else
        sn = ptm::sinf_(tpr);
        cs = ptm::cosf_(tpr);
#endif
        const f3 h = sample_vndf_ww(ww, ww1, alpha, r1, sn, cs);
        const f3 wi = reflect(-wo, h);
        if (wi.z <= 0.0f) continue;
        const float f = fresnel_exact_sq(ior_m, ior2, dot(h, wo));
        sum += f * opl / (opl + ggx_lambda_sq(wi, ax2, ay2));
    }
#else
#pragma unroll 1
    for (int i = 0; i < 16; ++i) {
        const float r1 = rng();
        const float tpr = kTwoPi * rng();
        const f3 h = sample_vndf(wo, alpha, r1, tpr);
        const f3 wi = reflect(-wo, h);
        if (wi.z <= 0.0f) continue;
        const float f = fresnel_exact(ior_m, dot(h, wo));
        sum += f * opl / (opl + ggx_lambda(wi, alpha));
    }
#endif
    return spec_color * sum / 16.0f;
}

}  // namespace ptd
