// trace_oracle.cpp - CPU oracle of the path-trace compute pass.
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/, by __graft_entry__.smoke() and
// by bench.py's CPU-baseline and reference legs, never by the product path.
//
// PARITY UNPINNED: the reference cannot run here and has no golden vectors
// for this path; this file restates src/render/trace.slang function by
// function (each cites the lines it follows).  T = float is the parity mode
// (same operation order, fma where the shader writes fma, IEEE division and
// square root, the shared transcendentals of pt_fmath.h), T = double the
// FP64 reference render (libm transcendentals).
//
// Build: g++ -O3 -ffp-contract=off -fopenmp (no -ffast-math: it would change
// the rounding the parity mode depends on).
#include <omp.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#include "../path-tracer_gb300/csrc/pt_fmath.h"
#include "oracle.h"

namespace {

template <class T>
struct M;
template <>
struct M<float> {
    static float fma(float a, float b, float c) { return __builtin_fmaf(a, b, c); }
    static float sqrt(float x) { return __builtin_sqrtf(x); }
    static float sin(float x) { return ptm::sinf_(x); }
    static float cos(float x) { return ptm::cosf_(x); }
    static float acos(float x) { return ptm::acosf_(x); }
    static float atan2(float y, float x) { return ptm::atan2f_(y, x); }
    static float pow(float x, float y) { return ptm::powf_(x, y); }
    static float floor(float x) { return __builtin_floorf(x); }
    static float fmin(float a, float b) { return __builtin_fminf(a, b); }
    static float fmax(float a, float b) { return __builtin_fmaxf(a, b); }
    static float abs(float x) { return __builtin_fabsf(x); }
};
template <>
struct M<double> {
    static double fma(double a, double b, double c) { return std::fma(a, b, c); }
    static double sqrt(double x) { return std::sqrt(x); }
    static double sin(double x) { return std::sin(x); }
    static double cos(double x) { return std::cos(x); }
    static double acos(double x) { return std::acos(x); }
    static double atan2(double y, double x) { return std::atan2(y, x); }
    static double pow(double x, double y) { return std::pow(x, y); }
    static double floor(double x) { return std::floor(x); }
    static double fmin(double a, double b) { return std::fmin(a, b); }
    static double fmax(double a, double b) { return std::fmax(a, b); }
    static double abs(double x) { return std::fabs(x); }
};

// shader constants are f32 literals; both modes use the f32 values
#define K(x) T(x##f)

template <class T>
struct V2 {
    T x, y;
};
template <class T>
struct V3 {
    T x, y, z;
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T>
struct V4 {
    T x, y, z, w;
};
template <class T> V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> V3<T> operator/(T s, V3<T> a) { return {s / a.x, s / a.y, s / a.z}; }
template <class T> V3<T> operator+(V3<T> a, T s) { return {a.x + s, a.y + s, a.z + s}; }
template <class T> V3<T> operator-(T s, V3<T> a) { return {s - a.x, s - a.y, s - a.z}; }
template <class T> V3<T> operator-(V3<T> a, T s) { return {a.x - s, a.y - s, a.z - s}; }
template <class T> V3<T> splat(T s) { return {s, s, s}; }
template <class T> T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> T rsqrt(T x) { return T(1) / M<T>::sqrt(x); }
template <class T> T length(V3<T> v) { return M<T>::sqrt(dot(v, v)); }
template <class T> V3<T> normalize(V3<T> v) { return v * rsqrt(dot(v, v)); }
template <class T> T lerp(T a, T b, T t) { return a * (T(1) - t) + b * t; }
template <class T> V3<T> lerp(V3<T> a, V3<T> b, T t) {
    return {lerp(a.x, b.x, t), lerp(a.y, b.y, t), lerp(a.z, b.z, t)};
}
template <class T> T saturate(T x) { return M<T>::fmin(M<T>::fmax(x, T(0)), T(1)); }
template <class T> V3<T> saturate(V3<T> v) { return {saturate(v.x), saturate(v.y), saturate(v.z)}; }
template <class T> T clamp(T x, T lo, T hi) { return M<T>::fmin(M<T>::fmax(x, lo), hi); }
template <class T> T frac(T x) { return x - M<T>::floor(x); }
template <class T> T sign(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0)); }
template <class T> V3<T> reflect(V3<T> i, V3<T> n) { return i - (T(2) * dot(n, i)) * n; }
template <class T> bool any_positive(V3<T> v) { return v.x > T(0) || v.y > T(0) || v.z > T(0); }

// float -> u32 as WGSL u32(): truncation, saturating, NaN -> 0
template <class T> uint32_t to_u32(T x) {
    if (!(x > T(0))) return 0u;
    if (x >= T(4294967296.0)) return 0xffffffffu;
    return (uint32_t)x;
}

constexpr float kPi = 3.14159265359f;
constexpr float kInvPi = 0.31830988618f;
constexpr float kInv2Pi = 0.15915494309189535f;
constexpr float kExposure = 0.00002604166f;
constexpr float kFltMax = 0x1.fffffep+127f;

inline uint64_t fnv_step(uint64_t h, uint32_t word) { return (h ^ word) * 0x100000001b3ull; }
constexpr uint64_t kFnvBasis = 0xcbf29ce484222325ull;

// sRGB EOTF table for Rgba8UnormSrgb sampling (world_resources.rs:86), computed
// in double and rounded once to float
struct SrgbTable {
    float v[256];
    SrgbTable() {
        for (int i = 0; i < 256; ++i) {
            const double c = (double)i / 255.0;
            v[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
        }
    }
};
const SrgbTable kSrgb;

template <class T>
struct Tracer {
    const oracle_world& w;
    uint32_t rng = 0;
    pt_path_record* rec = nullptr;
    bool in_shadow = false;  // counting inside occluded()

    explicit Tracer(const oracle_world& world) : w(world) {}

    // rand(), trace.slang:195-202
    T rand() {
        rng = rng * 747796405u + 2891336453u;
        const uint32_t word = ((rng >> ((rng >> 28u) + 4u)) ^ rng) * 277803737u;
        const float f = ptm::u2f(0x3f800000u | (((word >> 22u) ^ word) >> 9u)) - 1.0f;
        if (rec) rec->rand_draws += 1;
        return T(f);
    }

    V3<T> vert(uint32_t tri, int k) const {
        const pt_triangle_geometry& g = w.geometries[tri];
        const float* v = k == 0 ? g.v0 : (k == 1 ? g.v1 : g.v2);
        return {T(v[0]), T(v[1]), T(v[2])};
    }

    // Texture2DArray SampleLevel with the default (nearest, clamp-to-edge)
    // sampler, world_resources.rs:447-450
    V4<T> atlas(bool srgb, int32_t layer, V2<T> uv) const {
        const uint32_t count = srgb ? w.srgb_atlas_count : w.linear_atlas_count;
        const uint8_t* base = srgb ? w.srgb_atlases : w.linear_atlases;
        if (count == 0 || base == nullptr) return {T(0), T(0), T(0), T(0)};
        const uint32_t l = layer < 0 ? 0u : ((uint32_t)layer >= count ? count - 1 : (uint32_t)layer);
        const T fx = M<T>::floor(uv.x * T(8192.0f)), fy = M<T>::floor(uv.y * T(8192.0f));
        const uint32_t ix = fx >= T(8191) ? 8191u : to_u32(fx);
        const uint32_t iy = fy >= T(8191) ? 8191u : to_u32(fy);
        const uint8_t* p = base + (((uint64_t)l * PT_ATLAS_SIZE + iy) * PT_ATLAS_SIZE + ix) * 4;
        if (srgb) return {T(kSrgb.v[p[0]]), T(kSrgb.v[p[1]]), T(kSrgb.v[p[2]]), T((float)p[3] / 255.0f)};
        return {T((float)p[0] / 255.0f), T((float)p[1] / 255.0f), T((float)p[2] / 255.0f),
                T((float)p[3] / 255.0f)};
    }

    V2<T> atlas_uv(V2<T> uv, const float* offset_scale) const {
        return {M<T>::fma(uv.x, T(offset_scale[2]), T(offset_scale[0])),
                M<T>::fma(uv.y, T(offset_scale[3]), T(offset_scale[1]))};
    }

    // skybox SampleLevel with the linear clamp-to-edge sampler, world_resources.rs:451-456
    V3<T> skybox_bilinear(V2<T> uv) const {
        const uint32_t W = w.skybox.width, H = w.skybox.height;
        const T x = uv.x * T((float)W) - T(0.5f), y = uv.y * T((float)H) - T(0.5f);
        const T x0 = M<T>::floor(x), y0 = M<T>::floor(y);
        const T fx = x - x0, fy = y - y0;
        auto idx = [](T f, uint32_t n, int off) -> uint32_t {
            if (!(f == f)) return 0u;
            int64_t i = f < T(-1e9) ? -1000000000ll : (f > T(1e9) ? 1000000000ll : (int64_t)f);
            i += off;
            if (i < 0) i = 0;
            if (i > (int64_t)n - 1) i = (int64_t)n - 1;
            return (uint32_t)i;
        };
        const uint32_t ix0 = idx(x0, W, 0), ix1 = idx(x0, W, 1), iy0 = idx(y0, H, 0), iy1 = idx(y0, H, 1);
        auto px = [&](uint32_t ix, uint32_t iy) {
            const float* p = w.skybox_rgba + ((uint64_t)iy * W + ix) * 4;
            return V3<T>{T(p[0]), T(p[1]), T(p[2])};
        };
        const V3<T> top = lerp(px(ix0, iy0), px(ix1, iy0), fx);
        const V3<T> bottom = lerp(px(ix0, iy1), px(ix1, iy1), fx);
        return lerp(top, bottom, fy);
    }

    // orthonormal_tangent, trace.slang:207-218
    static V3<T> orthonormal_tangent(V3<T> tangent, V3<T> normal) {
        const V3<T> projected = tangent - dot(normal, tangent) * normal;
        const T ls = dot(projected, projected);
        if (ls > K(1e-12)) return projected * rsqrt(ls);
        const T s = normal.z >= T(0) ? T(1) : T(-1);
        const T a = T(-1) / (s + normal.z);
        return {M<T>::fma(s * normal.x * normal.x, a, T(1)), s * normal.x * normal.y * a, -s * normal.x};
    }

    static T fifth_power(T x) { return x * x * x * x * x; }

    // fresnel_exact, trace.slang:330-341
    static T fresnel_exact(T ior, T cos_i) {
        const T s = M<T>::fma(-cos_i, cos_i, T(1)) / (ior * ior);
        if (s >= T(1)) return T(1);
        const T cos_t = M<T>::sqrt(T(1) - s);
        const T rs = M<T>::fma(-ior, cos_t, cos_i) / M<T>::fma(ior, cos_t, cos_i);
        const T rp = M<T>::fma(-ior, cos_i, cos_t) / M<T>::fma(ior, cos_i, cos_t);
        return K(0.5) * (rs * rs + rp * rp);
    }

    // ggx_lambda, trace.slang:347-352
    static T ggx_lambda(V3<T> v, V2<T> a) {
        return M<T>::fma(K(0.5),
                         M<T>::sqrt(T(1) + (a.x * a.x * v.x * v.x + a.y * a.y * v.y * v.y) / (v.z * v.z)),
                         K(-0.5));
    }

    // sample_VNDF, trace.slang:356-364
    static V3<T> sample_vndf(V3<T> wo, V2<T> a, T r, T two_pi_r) {
        const V3<T> ww = normalize(V3<T>{wo.x * a.x, wo.y * a.y, wo.z});
        const T z = M<T>::fma(T(1) - r, T(1) + ww.z, -ww.z);
        const T sin_theta = M<T>::sqrt(saturate(M<T>::fma(-z, z, T(1))));
        const T x = sin_theta * M<T>::cos(two_pi_r);
        const T y = sin_theta * M<T>::sin(two_pi_r);
        const V3<T> h = V3<T>{x, y, z} + ww;
        return normalize(V3<T>{h.x * a.x, h.y * a.y, h.z});
    }

    // alpha_anisotropic, trace.slang:369-375
    static V2<T> alpha_anisotropic(T roughness, T anisotropy) {
        const T iso = T(1) - anisotropy;
        const T at = roughness * roughness * K(1.41421356237) * rsqrt(M<T>::fma(iso, iso, T(1)));
        return {M<T>::fmax(at, K(1e-4)), M<T>::fmax(at * iso, K(1e-4))};
    }

    // specular_ior_modulated, trace.slang:379-391
    static T specular_ior_modulated(T ior, T weight) {
        const T num = ior - T(1);
        const T den = ior + T(1);
        const T f0 = num * num / (den * den);
        const T f0s = sign(ior - T(1)) * M<T>::sqrt(M<T>::fmin(weight * f0, T(ptm::u2f(0x3f800000u - 1u))));
        return (T(1) + f0s) / (T(1) - f0s);
    }

    // estimate_e_dielectric, trace.slang:396-411
    V3<T> estimate_e_dielectric(V3<T> wo, T opl, V2<T> alpha, T ior_m, V3<T> spec_color) {
        T sum = T(0);
        for (int i = 0; i < 16; ++i) {
            const T r1 = rand();
            const T tpr = T(2.0f * kPi) * rand();
            const V3<T> h = sample_vndf(wo, alpha, r1, tpr);
            const V3<T> wi = reflect(-wo, h);
            if (wi.z <= T(0)) continue;
            const T f = fresnel_exact(ior_m, dot(h, wo));
            sum += f * opl / (opl + ggx_lambda(wi, alpha));
        }
        return spec_color * sum / K(16.0);
    }

    // power_heuristic, trace.slang:416-424
    static T power_heuristic(T pdf, T other) {
        const T scale = M<T>::fmax(pdf, other);
        if (scale <= T(0)) return T(0);
        const T p = pdf / scale;
        const T q = other / scale;
        return p * p / (p * p + q * q);
    }

    // coverage, trace.slang:426-443
    T coverage(const pt_material& m, V2<T> uv) const {
        if (m.alpha_mode == PT_ALPHA_MODE_OPAQUE) return T(1);
        T alpha = T(m.base_color[3]);
        if (m.base_color_tex_layer >= 0) alpha *= atlas(true, m.base_color_tex_layer, atlas_uv(uv, m.base_color_uv)).w;
        if (m.alpha_mode == PT_ALPHA_MODE_MASK) return alpha >= T(m.alpha_cutoff) ? T(1) : T(0);
        return alpha;
    }

    static V2<T> interp_uv(const pt_triangle_attribute& a, T u, T v, T w2) {
        return {frac(u * T(a.uv0[0]) + v * T(a.uv1[0]) + w2 * T(a.uv2[0])),
                frac(u * T(a.uv0[1]) + v * T(a.uv1[1]) + w2 * T(a.uv2[1]))};
    }

    // passes_through, trace.slang:446-454
    bool passes_through(uint32_t tri, T v, T w2) {
        const pt_triangle_attribute& attr = w.attributes[tri];
        const pt_material& m = w.materials[attr.material_index];
        if (m.alpha_mode == PT_ALPHA_MODE_OPAQUE) return false;
        const V2<T> uv = interp_uv(attr, T(1) - v - w2, v, w2);
        return coverage(m, uv) <= rand();
    }

    // evaluate_emission, trace.slang:455-466
    V3<T> evaluate_emission(const pt_material& m, V2<T> uv) const {
        V3<T> color{T(m.emission_color_and_luminance[0]), T(m.emission_color_and_luminance[1]),
                    T(m.emission_color_and_luminance[2])};
        if (m.emission_tex_layer >= 0) {
            const V4<T> t = atlas(true, m.emission_tex_layer, atlas_uv(uv, m.emission_uv));
            color = color * V3<T>{t.x, t.y, t.z};
        }
        return T(m.emission_weight) * T(m.emission_color_and_luminance[3]) * color;
    }

    // skybox_uv, trace.slang:467-472
    static V2<T> skybox_uv(V3<T> d) {
        return {frac(M<T>::fma(M<T>::atan2(d.z, d.x), T(kInv2Pi), K(0.5))),
                M<T>::atan2(M<T>::sqrt(d.x * d.x + d.z * d.z), d.y) * T(kInvPi)};
    }

    // evaluate_skybox, trace.slang:473-475
    V3<T> evaluate_skybox(V3<T> d) const { return skybox_bilinear(skybox_uv(d)) * T(w.skybox.average_luminance); }

    // skybox_texel_solid_angle, trace.slang:476-481
    T skybox_texel_solid_angle(uint32_t row) const {
        const T step = T(kPi) / T((float)w.skybox.height);
        const uint32_t pole_row = row < w.skybox.height - 1u - row ? row : w.skybox.height - 1u - row;
        return (T(2.0f * kPi) / T((float)w.skybox.width)) * T(2) * M<T>::sin((T((float)pole_row) + K(0.5)) * step) *
               M<T>::sin(K(0.5) * step);
    }

    // skybox_light_pdf, trace.slang:482-489
    T skybox_light_pdf(V3<T> d, T prob) const {
        if (prob <= T(0)) return T(0);
        const V2<T> uv = skybox_uv(d);
        uint32_t px = to_u32(uv.x * T((float)w.skybox.width));
        uint32_t py = to_u32(uv.y * T((float)w.skybox.height));
        if (px > w.skybox.width - 1u) px = w.skybox.width - 1u;
        if (py > w.skybox.height - 1u) py = w.skybox.height - 1u;
        return prob * T(w.skybox_aliases[(uint64_t)py * w.skybox.width + px].selection_probability) /
               skybox_texel_solid_angle(py);
    }

    // triangle_selection_probability, trace.slang:490-507
    T triangle_selection_probability(uint32_t tri) const {
        uint32_t first = 0, end = w.scene.emissive_triangles_count;
        while (first < end) {
            const uint32_t middle = first + (end - first) / 2u;
            const pt_scene_alias_entry& e = w.scene_aliases[middle];
            if (e.triangle_index < tri) first = middle + 1u;
            else if (e.triangle_index > tri) end = middle;
            else return T(e.selection_probability);
        }
        return T(0);
    }

    // triangle_light_pdf, trace.slang:508-523
    T triangle_light_pdf(uint32_t tri, V3<T> d, T dist2, T prob) const {
        if (prob <= T(0)) return T(0);
        const V3<T> v0 = vert(tri, 0), v1 = vert(tri, 1), v2 = vert(tri, 2);
        const T area = K(0.5) * M<T>::abs(dot(cross(v1 - v0, v2 - v0), d));
        if (area <= T(0)) return T(0);
        return prob * dist2 / area;
    }

    struct LightSample {
        V3<T> direction{T(0), T(0), T(0)};
        T distance = T(0);
        V3<T> emission{T(0), T(0), T(0)};
        T pdf = T(0);
        int32_t triangle_index = -1;
    };

    // sample_light, trace.slang:531-592
    LightSample sample_light(V3<T> origin) {
        LightSample r;
        const T p0 = T(w.scene.light_probabilities[0]), p1 = T(w.scene.light_probabilities[1]);
        if (p0 + p1 <= T(0)) return r;
        if (rand() < p0) {
            if (rec) rec->light_samples += 1;
            const uint32_t count = w.scene.emissive_triangles_count;
            uint32_t slot = to_u32(rand() * T((float)count));
            if (slot > count - 1u) slot = count - 1u;
            const pt_scene_alias_entry cand = w.scene_aliases[slot];
            const pt_scene_alias_entry entry = w.scene_aliases[rand() < T(cand.threshold) ? slot : cand.alias_index];
            const V3<T> v0 = vert(entry.triangle_index, 0), v1 = vert(entry.triangle_index, 1),
                        v2 = vert(entry.triangle_index, 2);
            const T root = M<T>::sqrt(rand());
            const T u = T(1) - root;
            const T v = root * (T(1) - rand());
            const T wb = T(1) - u - v;
            const V3<T> delta = u * v0 + v * v1 + wb * v2 - origin;
            const T d2 = dot(delta, delta);
            if (d2 <= T(0)) return r;
            r.distance = M<T>::sqrt(d2);
            r.direction = delta / r.distance;
            r.triangle_index = (int32_t)entry.triangle_index;
            r.pdf = triangle_light_pdf(entry.triangle_index, r.direction, d2, p0 * T(entry.selection_probability));
            const pt_triangle_attribute& attr = w.attributes[entry.triangle_index];
            const V2<T> uv = interp_uv(attr, u, v, wb);
            const pt_material& m = w.materials[attr.material_index];
            r.emission = coverage(m, uv) * evaluate_emission(m, uv);
        } else {
            if (rec) rec->sky_light_samples += 1;
            const uint32_t W = w.skybox.width, H = w.skybox.height;
            const uint32_t count = W * H;
            uint32_t slot = to_u32(rand() * T((float)count));
            if (slot > count - 1u) slot = count - 1u;
            const pt_skybox_alias_entry cand = w.skybox_aliases[slot];
            const uint32_t index = rand() < T(cand.threshold) ? slot : cand.alias_index;
            const uint32_t row = index / W, column = index % W;
            const T phi = ((T((float)column) + rand()) / T((float)W) - K(0.5)) * T(2.0f * kPi);
            const bool north = row < H / 2u;
            const uint32_t pole_row = north ? row : H - 1u - row;
            const T half_step = K(0.5) * T(kPi) / T((float)H);
            const T a = M<T>::sin(T((float)pole_row) * half_step);
            const T b = M<T>::sin(T((float)(pole_row + 1u)) * half_step);
            const T shs = lerp(a * a, b * b, rand());
            const T cos_theta = T(1) - T(2) * shs;
            const T sin_theta = T(2) * M<T>::sqrt(M<T>::fmax(T(0), shs * (T(1) - shs)));
            r.direction = {sin_theta * M<T>::cos(phi), north ? cos_theta : -cos_theta, sin_theta * M<T>::sin(phi)};
            r.distance = T(kFltMax);
            r.pdf = skybox_light_pdf(r.direction, p1);
            r.emission = evaluate_skybox(r.direction);
        }
        return r;
    }

    const pt_bvh_node& node(uint32_t i) {
        if (rec) rec->visit_hash = fnv_step(rec->visit_hash, i);
        return w.bvh_nodes[i];
    }

    // intersect_aabb, trace.slang:597-609
    static T intersect_aabb(const pt_bvh_node& n, V3<T> nod, V3<T> rcp, T hit_t) {
        const V3<T> t0{M<T>::fma(T(n.aabb_min[0]), rcp.x, nod.x), M<T>::fma(T(n.aabb_min[1]), rcp.y, nod.y),
                       M<T>::fma(T(n.aabb_min[2]), rcp.z, nod.z)};
        const V3<T> t1{M<T>::fma(T(n.aabb_max[0]), rcp.x, nod.x), M<T>::fma(T(n.aabb_max[1]), rcp.y, nod.y),
                       M<T>::fma(T(n.aabb_max[2]), rcp.z, nod.z)};
        const V3<T> tmin{M<T>::fmin(t0.x, t1.x), M<T>::fmin(t0.y, t1.y), M<T>::fmin(t0.z, t1.z)};
        const V3<T> tmax{M<T>::fmax(t0.x, t1.x), M<T>::fmax(t0.y, t1.y), M<T>::fmax(t0.z, t1.z)};
        const T t_near = M<T>::fmax(M<T>::fmax(tmin.x, tmin.y), tmin.z);
        const T t_far = M<T>::fmin(M<T>::fmin(tmax.x, tmax.y), tmax.z);
        return (t_near <= t_far && t_far > T(0) && t_near < hit_t) ? M<T>::fmax(T(0), t_near) : T(-1);
    }

    // watertight setup shared by both traversals, trace.slang:769-783 / 617-630
    struct Shear {
        int kx, ky, kz;
        T sx, sy, sz;
    };
    static Shear shear(V3<T> d, V3<T> rcp) {
        const V3<T> ad{M<T>::abs(d.x), M<T>::abs(d.y), M<T>::abs(d.z)};
        const int kxy = ad.x > ad.y ? 0 : 1;
        const int kz = ad[kxy] > ad.z ? kxy : 2;
        const int kx_val = kz == 2 ? 0 : kz + 1;
        const int ky_val = kx_val == 2 ? 0 : kx_val + 1;
        const bool is_neg = d[kz] < T(0);
        Shear s;
        s.kz = kz;
        s.kx = is_neg ? ky_val : kx_val;
        s.ky = is_neg ? kx_val : ky_val;
        s.sz = rcp[kz];
        s.sx = -d[s.kx] * s.sz;
        s.sy = -d[s.ky] * s.sz;
        return s;
    }

    // watertight ray-triangle test, trace.slang:807-834; returns false when rejected
    bool triangle_test(uint32_t tri, V3<T> o, const Shear& s, T* t_out, T* v_out, T* w_out) {
        if (rec) {
            rec->triangle_tests += 1;
            if (in_shadow) rec->shadow_triangle_tests += 1;
        }
        const V3<T> A = vert(tri, 0) - o, B = vert(tri, 1) - o, C = vert(tri, 2) - o;
        const T ax = M<T>::fma(s.sx, A[s.kz], A[s.kx]);
        const T ay = M<T>::fma(s.sy, A[s.kz], A[s.ky]);
        const T bx = M<T>::fma(s.sx, B[s.kz], B[s.kx]);
        const T by = M<T>::fma(s.sy, B[s.kz], B[s.ky]);
        const T cx = M<T>::fma(s.sx, C[s.kz], C[s.kx]);
        const T cy = M<T>::fma(s.sy, C[s.kz], C[s.ky]);
        const T U = M<T>::fma(cx, by, -cy * bx);
        const T V = M<T>::fma(ax, cy, -ay * cx);
        const T W = M<T>::fma(bx, ay, -by * ax);
        if (M<T>::fmin(U, M<T>::fmin(V, W)) < T(0) && M<T>::fmax(U, M<T>::fmax(V, W)) > T(0)) return false;
        const T det = U + V + W;
        if (det == T(0)) return false;
        const T inv_det = T(1) / det;
        *t_out = s.sz * M<T>::fma(U, A[s.kz], M<T>::fma(V, B[s.kz], W * C[s.kz])) * inv_det;
        *v_out = V * inv_det;
        *w_out = W * inv_det;
        return true;
    }

    // closest-hit traversal, trace.slang:764-884
    void closest_hit(V3<T> o, V3<T> d, V3<T> rcp, bool alpha_test, T* hit_t, int32_t* hit_index, T* hit_v,
                     T* hit_w) {
        if (rec) rec->extend_rays += 1;
        const Shear s = shear(d, rcp);
        uint32_t stack[64];
        uint32_t node_index = 0, sp = 0;
        const V3<T> nod = -o * rcp;
        for (;;) {
            const pt_bvh_node& n = node(node_index);
            if (n.tri_count > 0u) {
                if (rec) {
                    rec->leaf_visits += 1;
                    if (in_shadow) rec->shadow_leaf_visits += 1;
                }
                for (uint32_t i = 0; i < n.tri_count; ++i) {
                    const uint32_t tri = n.left_first + i;
                    T t, v, wb;
                    if (!triangle_test(tri, o, s, &t, &v, &wb)) continue;
                    if (t > T(0) && t < *hit_t) {
                        if (alpha_test && passes_through(tri, v, wb)) continue;
                        *hit_t = t;
                        *hit_index = (int32_t)tri;
                        *hit_v = v;
                        *hit_w = wb;
                    }
                }
            } else {
                if (rec) {
                    rec->interior_visits += 1;
                    if (in_shadow) rec->shadow_interior_visits += 1;
                }
                const uint32_t li = n.left_first, ri = n.left_first + 1u;
                const T dl = intersect_aabb(w.bvh_nodes[li], nod, rcp, *hit_t);
                const T dr = intersect_aabb(w.bvh_nodes[ri], nod, rcp, *hit_t);
                const bool hl = dl >= T(0), hr = dr >= T(0);
                if (hl && hr) {
                    const bool left_closer = dl < dr;
                    stack[sp++ & 63u] = left_closer ? ri : li;
                    node_index = left_closer ? li : ri;
                    continue;
                } else if (hl) {
                    node_index = li;
                    continue;
                } else if (hr) {
                    node_index = ri;
                    continue;
                }
            }
            if (sp == 0u) break;
            sp -= 1u;
            node_index = stack[sp & 63u];
        }
    }

    // occluded, trace.slang:614-717
    bool occluded(V3<T> o, V3<T> d, T hit_t, int32_t light_tri) {
        in_shadow = true;
        const bool r = occluded_impl(o, d, hit_t, light_tri);
        in_shadow = false;
        return r;
    }

    bool occluded_impl(V3<T> o, V3<T> d, T hit_t, int32_t light_tri) {
        if (rec) rec->shadow_rays += 1;
        const V3<T> rcp = T(1) / d;
        const Shear s = shear(d, rcp);
        uint32_t stack[64];
        uint32_t node_index = 0, sp = 0;
        const V3<T> nod = -o * rcp;
        for (;;) {
            const pt_bvh_node& n = node(node_index);
            if (n.tri_count > 0u) {
                if (rec) {
                    rec->leaf_visits += 1;
                    if (in_shadow) rec->shadow_leaf_visits += 1;
                }
                for (uint32_t i = 0; i < n.tri_count; ++i) {
                    const uint32_t tri = n.left_first + i;
                    if ((int32_t)tri == light_tri) continue;
                    T t, v, wb;
                    if (!triangle_test(tri, o, s, &t, &v, &wb)) continue;
                    if (t > T(0) && t < hit_t && !passes_through(tri, v, wb)) return true;
                }
            } else {
                if (rec) {
                    rec->interior_visits += 1;
                    if (in_shadow) rec->shadow_interior_visits += 1;
                }
                const uint32_t li = n.left_first, ri = n.left_first + 1u;
                const T dl = intersect_aabb(w.bvh_nodes[li], nod, rcp, hit_t);
                const T dr = intersect_aabb(w.bvh_nodes[ri], nod, rcp, hit_t);
                const bool hl = dl >= T(0), hr = dr >= T(0);
                if (hl && hr) {
                    const bool left_closer = dl < dr;
                    stack[sp++ & 63u] = left_closer ? ri : li;
                    node_index = left_closer ? li : ri;
                    continue;
                } else if (hl) {
                    node_index = li;
                    continue;
                } else if (hr) {
                    node_index = ri;
                    continue;
                }
            }
            if (sp == 0u) break;
            sp -= 1u;
            node_index = stack[sp & 63u];
        }
        return false;
    }

    struct Lobes {
        V3<T> f;
        T pdf;
    };

    // E_FON_exact, trace.slang:318-323
    static T e_fon_exact(T mu, T r) {
        const T af = T(1) / M<T>::fma(K(0.28779340921), r, T(1));
        const T si = M<T>::sqrt(M<T>::fma(-mu, mu, T(1)));
        const T g = si * (M<T>::acos(mu) - si * mu) + T(0x1.555556p-1f) * ((si / mu) * (T(1) - (si * si * si)) - si);
        return af + r * af * T(kInvPi) * g;
    }

    // evaluate_lobes, trace.slang:229-315
    struct Bsdf {
        T p_ggx, p_diffuse;
        V3<T> base_color;
        T base_weight, base_metalness, base_diffuse_roughness;
        V3<T> specular_color;
        T specular_weight, ior_m;
        V2<T> alpha;
        T opl;
        V3<T> f0;
        V3<T> e_dielectric;
        V4<T> ltc;
        V3<T> bx, by, bz;  // rows of orthonormal_basis_ltc_wo
        T p_u, p_c;
    };

    static Lobes evaluate_lobes(V3<T> wo, V3<T> wi, const Bsdf& b) {
        const V3<T> h = normalize(wo + wi);
        const T hdotw = dot(h, wo);
        const T g1 = T(1) / b.opl;
        const T g2 = T(1) / (b.opl + ggx_lambda(wi, b.alpha));
        const T dh = (h.x * h.x) / (b.alpha.x * b.alpha.x) + (h.y * h.y) / (b.alpha.y * b.alpha.y) + h.z * h.z;
        const T D = T(kInvPi) / (b.alpha.x * b.alpha.y * dh * dh);
        const T ts = D * g2 / (K(4.0) * wi.z * wo.z);
        const T omh = T(1) - hdotw;
        const T p5 = fifth_power(omh);
        const V3<T> fa = (K(0.00105024005) * hdotw * omh) * (T(1) - b.specular_color);
        const V3<T> fb = K(9031.0) * b.f0 + K(7776.0);
        const V3<T> fc = b.f0 - T(1);
        const V3<T> fm{M<T>::fma(fa.x, fb.x, fc.x), M<T>::fma(fa.y, fb.y, fc.y), M<T>::fma(fa.z, fb.z, fc.z)};
        const V3<T> f82 = b.f0 - p5 * fm;
        const V3<T> f_conductor = saturate(b.specular_weight * f82) * ts;
        const V3<T> f_dielectric = b.specular_color * fresnel_exact(b.ior_m, hdotw) * ts;
        const V3<T> rho = b.base_color;
        const T r = b.base_diffuse_roughness;
        const T s_f = wi.x * wo.x + wi.y * wo.y;
        const T sovert_f = s_f > T(0) ? s_f / M<T>::fmax(wo.z, wi.z) : s_f;
        const T af = T(1) / M<T>::fma(K(0.28779340921), r, T(1));
        const V3<T> f_ss = rho * T(kInvPi) * af * M<T>::fma(r, sovert_f, T(1));
        const T efo = e_fon_exact(wo.z, r);
        const T efi = e_fon_exact(wi.z, r);
        const T avg_ef = af * M<T>::fma(K(0.07248821245), r, T(1));
        const V3<T> rho_ms = rho * rho * avg_ef / (T(1) - rho * (T(1) - avg_ef));
        const V3<T> f_ms = (rho_ms * T(kInvPi)) * M<T>::fmax(K(1.0e-7), T(1) - efo) *
                           M<T>::fmax(K(1.0e-7), T(1) - efi) / M<T>::fmax(K(1.0e-7), T(1) - avg_ef);
        const V3<T> f_diffuse = b.base_weight * (f_ss + f_ms);
        const V3<T> f_glossy_diffuse = f_dielectric + (T(1) - b.e_dielectric) * f_diffuse;
        const V3<T> f_total = lerp(f_glossy_diffuse, f_conductor, b.base_metalness);
        const T pdf_ggx = D * g1 / (K(4.0) * wo.z);
        const V3<T> wl{dot(b.bx, wi), dot(b.by, wi), dot(b.bz, wi)};
        const T a = b.ltc.x, bb = b.ltc.y, c = b.ltc.z, d = b.ltc.w;
        const T det_m = c * M<T>::fma(-bb, d, a);
        const V3<T> wh{c * (wl.x - bb * wl.z), (a - bb * d) * wl.y, -c * (d * wl.x - a * wl.z)};
        const T len_sqr = dot(wh, wh);
        const T s_pdf = M<T>::fma(K(0.5), rsqrt(M<T>::fma(d, d, T(1))), K(0.5));
        const T pdf_c = (det_m * det_m) / (len_sqr * len_sqr) * M<T>::fmax(wh.z, T(0)) / (T(kPi) * s_pdf);
        const T pdf_eon = b.p_u * K(0.15915494309) + b.p_c * pdf_c;
        return {f_total, b.p_ggx * pdf_ggx + b.p_diffuse * pdf_eon};
    }

    // OpenPBR setup of one shading point, trace.slang:1097-1181 (draws the 32
    // random numbers of estimate_e_dielectric)
    Bsdf setup_bsdf(V3<T> base_color, T base_weight, T base_metalness, T base_diffuse_roughness, V3<T> specular_color,
                    T specular_weight, T specular_roughness, T specular_anisotropy, T specular_ior, V3<T> wo) {
        Bsdf b;
        b.alpha = alpha_anisotropic(specular_roughness, specular_anisotropy);
        b.ior_m = specular_ior_modulated(specular_ior, specular_weight);
        b.f0 = base_weight * base_color;
        b.opl = T(1) + ggx_lambda(wo, b.alpha);
        const T r = base_diffuse_roughness;
        const T z = wo.z;
        b.ltc.x = T(1) + r * (K(0.303392) + (K(-0.518982) + K(0.111709) * z) * z + (K(-0.276266) + K(0.335918) * z) * r);
        b.ltc.y = r * (K(-1.16407) + K(1.15859) * z + (K(0.150815) - K(0.150105) * z) * r) / (z * z * z - K(1.43545));
        b.ltc.z = T(1) + r * (K(0.20013) + (K(-0.506373) + K(0.261777) * z) * z);
        b.ltc.w = r * (K(0.540852) + (K(-1.01625) + K(0.475392) * z) * z) / (K(-1.0743) + (K(0.0725628) + z) * z);
        const T ls = wo.x * wo.x + wo.y * wo.y;
        V3<T> bx{T(1), T(0), T(0)};
        if (ls > T(0)) bx = V3<T>{wo.x, wo.y, T(0)} * rsqrt(ls);
        b.bx = bx;
        b.by = V3<T>{-bx.y, bx.x, T(0)};
        b.bz = V3<T>{T(0), T(0), T(1)};
        b.e_dielectric = estimate_e_dielectric(wo, b.opl, b.alpha, b.ior_m, specular_color);
        const V3<T> luma{K(0.2126), K(0.7152), K(0.0722)};
        const T albedo_gloss = dot(b.e_dielectric, luma);
        const T albedo_diffuse = (T(1) - albedo_gloss) * base_weight * dot(base_color, luma);
        const V3<T> fsm = b.f0 + (T(1) - b.f0) * fifth_power(T(1) - wo.z);
        const T albedo_metal = dot(fsm, luma);
        const T w_ggx = lerp(albedo_gloss, albedo_metal, base_metalness);
        const T w_diffuse = (T(1) - base_metalness) * albedo_diffuse;
        b.p_ggx = clamp(w_ggx / M<T>::fmax(w_ggx + w_diffuse, K(1e-7)), K(0.1), K(0.9));
        b.p_diffuse = T(1) - b.p_ggx;
        b.p_u = M<T>::pow(r, K(0.1)) * (K(0.162925) + (K(-0.372058) + (K(0.538233) - K(0.290822) * z) * z) * z);
        b.p_c = T(1) - b.p_u;
        b.base_color = base_color;
        b.base_weight = base_weight;
        b.base_metalness = base_metalness;
        b.base_diffuse_roughness = base_diffuse_roughness;
        b.specular_color = specular_color;
        b.specular_weight = specular_weight;
        return b;
    }

    // BSDF sampling, trace.slang:1212-1260 (3 random numbers)
    V3<T> sample_bsdf(V3<T> wo, const Bsdf& b) {
        const T two_pi_r = T(2.0f * kPi) * rand();
        const T r1 = rand();
        V3<T> wi;
        if (rand() < b.p_ggx) {
            wi = reflect(-wo, sample_vndf(wo, b.alpha, r1, two_pi_r));
        } else if (r1 < b.p_u) {
            const T u1 = r1 / b.p_u;
            const T sin_theta = M<T>::sqrt(T(1) - u1 * u1);
            wi = {sin_theta * M<T>::cos(two_pi_r), sin_theta * M<T>::sin(two_pi_r), u1};
        } else {
            const T u1 = (r1 - b.p_u) / b.p_c;
            const T a = b.ltc.x, bb = b.ltc.y, c = b.ltc.z, dd = b.ltc.w;
            const T R = M<T>::sqrt(u1);
            const T y = R * M<T>::sin(two_pi_r);
            const T s = M<T>::fma(K(0.5), rsqrt(M<T>::fma(dd, dd, T(1))), K(0.5));
            const T x = -lerp(M<T>::sqrt(M<T>::fma(-y, y, T(1))), R * M<T>::cos(two_pi_r), s);
            const V3<T> wh{x, y, M<T>::sqrt(M<T>::fmax(T(1) - (x * x + y * y), T(0)))};
            const V3<T> wu{a * wh.x + bb * wh.z, c * wh.y, dd * wh.x + wh.z};
            wi = normalize(wu.x * b.bx + wu.y * b.by + wu.z * b.bz);
        }
        return wi;
    }

    // camera ray, trace.slang:739-748: the jitter takes the first two draws,
    // x then y (float2(rand(), rand()) evaluated left to right)
    void camera_ray(const pt_camera& cam, uint32_t px, uint32_t py, const uint32_t image_size[2], V3<T>* o,
                    V3<T>* d) {
        const T jx = rand();
        const T jy = rand();
        const V2<T> puv{(T((float)px) + jx) / T((float)image_size[0]), (T((float)py) + jy) / T((float)image_size[1])};
        *o = V3<T>{T(cam.position[0]), T(cam.position[1]), T(cam.position[2])};
        const V3<T> llc{T(cam.lower_left_corner_minus_position[0]), T(cam.lower_left_corner_minus_position[1]),
                        T(cam.lower_left_corner_minus_position[2])};
        const V3<T> hor{T(cam.horizontal[0]), T(cam.horizontal[1]), T(cam.horizontal[2])};
        const V3<T> ver{T(cam.vertical[0]), T(cam.vertical[1]), T(cam.vertical[2])};
        *d = normalize(llc + puv.x * hor + puv.y * ver);
    }

    // compute_main, trace.slang:721-1297: radiance of one sample
    V3<T> trace(uint32_t px, uint32_t py, const uint32_t image_size[2], uint32_t sample_count, uint32_t max_bounces) {
        rng = (px * 0x9E3779B9u) ^ (py * 0x85EBCA6Bu) ^ (0u * 0xC2B2AE35u) ^ (sample_count * 0x27D4EB2Du) ^ 0xA511E9B3u;
        rng |= 1u;
        V3<T> o, d;
        camera_ray(w.camera, px, py, image_size, &o, &d);
        V3<T> rcp = T(1) / d;
        V3<T> throughput{T(1), T(1), T(1)};
        V3<T> color{T(0), T(0), T(0)};
        T prev_pdf = T(0);
        const bool any_alpha = true;
        for (uint32_t bounce = 0; bounce <= max_bounces; ++bounce) {
            T hit_t = T(kFltMax);
            int32_t hit = -1;
            T hv = T(0), hw = T(0);
            closest_hit(o, d, rcp, any_alpha, &hit_t, &hit, &hv, &hw);
            if (rec && bounce < PT_RECORD_MAX_BOUNCES) rec->hit[bounce] = hit;
            if (hit == -1) {
                if (rec) rec->sky_misses += 1;
                T mis = T(1);
                if (bounce > 0u) mis = power_heuristic(prev_pdf, skybox_light_pdf(d, T(w.scene.light_probabilities[1])));
                color = color + throughput * evaluate_skybox(d) * mis;
                break;
            }
            if (rec) rec->hits += 1;
            const uint32_t h = (uint32_t)hit;
            const pt_triangle_attribute& attr = w.attributes[h];
            const T hu = T(1) - hv - hw;
            const V2<T> iuv = interp_uv(attr, hu, hv, hw);
            const pt_material& m = w.materials[attr.material_index];
            V3<T> base_color{T(m.base_color[0]), T(m.base_color[1]), T(m.base_color[2])};
            const T base_weight = T(m.base_weight);
            T base_metalness = T(m.base_metalness);
            T base_diffuse_roughness = T(m.base_diffuse_roughness);
            V3<T> specular_color{T(m.specular_color_and_weight[0]), T(m.specular_color_and_weight[1]),
                                 T(m.specular_color_and_weight[2])};
            T specular_weight = T(m.specular_color_and_weight[3]);
            const T specular_roughness = T(m.specular_roughness);
            const T specular_anisotropy = T(m.specular_roughness_anisotropy);
            const T specular_ior = T(m.specular_ior);
            if (m.base_color_tex_layer >= 0) {
                const V4<T> t = atlas(true, m.base_color_tex_layer, atlas_uv(iuv, m.base_color_uv));
                base_color = base_color * V3<T>{t.x, t.y, t.z};
            }
            if (m.metallic_roughness_tex_layer >= 0) {
                const V4<T> t = atlas(false, m.metallic_roughness_tex_layer, atlas_uv(iuv, m.metallic_roughness_uv));
                base_metalness *= t.z;
                base_diffuse_roughness *= t.y;
            }
            if (m.specular_color_tex_layer >= 0) {
                const V4<T> t = atlas(true, m.specular_color_tex_layer, atlas_uv(iuv, m.specular_color_uv));
                specular_color = specular_color * V3<T>{t.x, t.y, t.z};
            }
            if (m.specular_weight_tex_layer >= 0) {
                const V4<T> t = atlas(false, m.specular_weight_tex_layer, atlas_uv(iuv, m.specular_weight_uv));
                specular_weight *= t.w;
            }
            // emission with MIS, trace.slang:984-991
            const V3<T> emission = evaluate_emission(m, iuv);
            T emission_mis = T(1);
            if (bounce > 0u && T(w.scene.light_probabilities[0]) > T(0) && any_positive(emission)) {
                const T lpdf = triangle_light_pdf(h, d, hit_t * hit_t,
                                                  T(w.scene.light_probabilities[0]) * triangle_selection_probability(h));
                emission_mis = power_heuristic(prev_pdf, lpdf);
            }
            color = color + throughput * emission * emission_mis;

            // shading frame, trace.slang:993-1091
            const V3<T> hit_point = d * hit_t + o;
            const V3<T> V = -d;
            const V3<T> v0 = vert(h, 0), v1 = vert(h, 1), v2 = vert(h, 2);
            const V3<T> flat_raw = normalize(cross(v1 - v0, v2 - v0));
            const T bfm = dot(V, flat_raw) > T(0) ? T(1) : T(-1);
            const V3<T> flat_n = flat_raw * bfm;
            const V3<T> n0{T(attr.n0[0]), T(attr.n0[1]), T(attr.n0[2])};
            const V3<T> n1{T(attr.n1[0]), T(attr.n1[1]), T(attr.n1[2])};
            const V3<T> n2{T(attr.n2[0]), T(attr.n2[1]), T(attr.n2[2])};
            V3<T> N = normalize(hu * n0 + hv * n1 + hw * n2) * bfm;
            const V3<T> t0{T(attr.t0[0]), T(attr.t0[1]), T(attr.t0[2])};
            const V3<T> t1{T(attr.t1[0]), T(attr.t1[1]), T(attr.t1[2])};
            const V3<T> t2{T(attr.t2[0]), T(attr.t2[1]), T(attr.t2[2])};
            const T t0w = T(attr.t0[3]);
            V3<T> Tn = orthonormal_tangent(hu * t0 + hv * t1 + hw * t2, N) * bfm;
            V3<T> Bn = cross(N, Tn) * t0w * bfm;
            bool n_changed = false;
            if (m.normal_tex_layer >= 0) {
                const V4<T> t = atlas(false, m.normal_tex_layer, atlas_uv(iuv, m.normal_uv));
                V3<T> ln{t.x * T(2) - T(1), t.y * T(2) - T(1), t.z * T(2) - T(1)};
                ln = normalize(V3<T>{ln.x * T(m.normal_scale), ln.y * T(m.normal_scale), ln.z});
                N = normalize(ln.x * Tn + ln.y * Bn + ln.z * N);
                n_changed = true;
            }
            const T flat_ndotv = dot(flat_n, V);
            const T threshold = K(0.5) * flat_ndotv;
            T ndotv = dot(N, V);
            if (ndotv < threshold) {
                N = normalize(lerp(N, flat_n, (threshold - ndotv) / (flat_ndotv - ndotv)));
                ndotv = dot(N, V);
                n_changed = true;
            }
            if (n_changed) {
                Tn = orthonormal_tangent(Tn, N);
                Bn = cross(N, Tn) * t0w * bfm;
            }

            // OpenPBR setup, trace.slang:1097-1181
            const V3<T> wo{dot(Tn, V), dot(Bn, V), ndotv};
            const Bsdf b = setup_bsdf(base_color, base_weight, base_metalness, base_diffuse_roughness, specular_color,
                                      specular_weight, specular_roughness, specular_anisotropy, specular_ior, wo);

            // next-event estimation, trace.slang:1187-1206
            const V3<T> next_origin = hit_point + flat_n * M<T>::fmax(K(1e-4), K(1e-4) * length(hit_point));
            const LightSample light = sample_light(next_origin);
            const V3<T> lwi{dot(Tn, light.direction), dot(Bn, light.direction), dot(N, light.direction)};
            if (light.pdf > T(0) && lwi.z > T(0) && any_positive(light.emission)) {
                const Lobes lobes = evaluate_lobes(wo, lwi, b);
                if (!occluded(next_origin, light.direction, light.distance, light.triangle_index)) {
                    const T weight = bounce < max_bounces ? power_heuristic(light.pdf, lobes.pdf) : T(1);
                    color = color + throughput * lobes.f * lwi.z * light.emission * (weight / light.pdf);
                }
            }
            if (bounce == max_bounces) break;

            // BSDF sampling, trace.slang:1212-1260
            const V3<T> wi = sample_bsdf(wo, b);
            if (wi.z <= T(0)) break;
            const Lobes lobes = evaluate_lobes(wo, wi, b);
            if (lobes.pdf <= T(0)) break;
            throughput = throughput * (lobes.f * wi.z / lobes.pdf);
            prev_pdf = lobes.pdf;
            if (bounce > 3u) {
                const T p_survive = clamp(M<T>::fmax(throughput.x, M<T>::fmax(throughput.y, throughput.z)), K(0.05), K(0.95));
                if (rand() > p_survive) break;
                throughput = throughput / p_survive;
            }
            o = next_origin;
            d = wi.x * Tn + wi.y * Bn + wi.z * N;
            rcp = T(1) / d;
        }
        return color;
    }
};

void init_record(pt_path_record* r) {
    std::memset(r, 0, sizeof(*r));
    r->visit_hash = kFnvBasis;
    for (int i = 0; i < PT_RECORD_MAX_BOUNCES; ++i) r->hit[i] = -2;
}

// one shading point per case: setup (32 draws), the lobes at case.wi, and a
// BSDF sample (the next 3 draws) with its lobes
template <class T>
void shade_case(const oracle_shade_case& k, oracle_shade_result* r) {
    oracle_world dummy{};
    Tracer<T> t(dummy);
    t.rng = k.rng;
    auto v = [](const float* p) { return V3<T>{T(p[0]), T(p[1]), T(p[2])}; };
    const V3<T> wo = v(k.wo);
    const typename Tracer<T>::Bsdf b =
        t.setup_bsdf(v(k.base_color), T(k.base_weight), T(k.base_metalness), T(k.base_diffuse_roughness),
                     v(k.specular_color), T(k.specular_weight), T(k.specular_roughness), T(k.specular_anisotropy),
                     T(k.specular_ior), wo);
    const auto lobes = Tracer<T>::evaluate_lobes(wo, v(k.wi), b);
    const V3<T> ws = t.sample_bsdf(wo, b);
    const auto slobes = Tracer<T>::evaluate_lobes(wo, ws, b);
    const T ed[3] = {b.e_dielectric.x, b.e_dielectric.y, b.e_dielectric.z};
    const T f[3] = {lobes.f.x, lobes.f.y, lobes.f.z};
    const T sw[3] = {ws.x, ws.y, ws.z};
    const T sf[3] = {slobes.f.x, slobes.f.y, slobes.f.z};
    for (int j = 0; j < 3; ++j) {
        r->e_dielectric[j] = (double)ed[j];
        r->f[j] = (double)f[j];
        r->sampled_wi[j] = (double)sw[j];
        r->sampled_f[j] = (double)sf[j];
    }
    r->p_ggx = (double)b.p_ggx;
    r->p_u = (double)b.p_u;
    r->pdf = (double)lobes.pdf;
    r->sampled_pdf = (double)slobes.pdf;
    r->rng_after = t.rng;
}

template <class T>
void light_case(const oracle_world& w, const float* origin, uint32_t rng, oracle_light_result* r) {
    Tracer<T> t(w);
    t.rng = rng;
    const auto s = t.sample_light(V3<T>{T(origin[0]), T(origin[1]), T(origin[2])});
    const T d[3] = {s.direction.x, s.direction.y, s.direction.z};
    const T e[3] = {s.emission.x, s.emission.y, s.emission.z};
    for (int j = 0; j < 3; ++j) {
        r->direction[j] = (double)d[j];
        r->emission[j] = (double)e[j];
    }
    r->distance = (double)s.distance;
    r->pdf = (double)s.pdf;
    r->triangle_index = s.triangle_index;
    r->rng_after = t.rng;
}

}  // namespace

extern "C" {

int oracle_max_threads(void) { return omp_get_max_threads(); }

uint32_t oracle_seed(uint32_t px, uint32_t py, uint32_t n) {
    uint32_t s = (px * 0x9E3779B9u) ^ (py * 0x85EBCA6Bu) ^ (0u * 0xC2B2AE35u) ^ (n * 0x27D4EB2Du) ^ 0xA511E9B3u;
    return s | 1u;
}

void oracle_rand_sequence(uint32_t state, uint32_t count, float* out) {
    oracle_world dummy{};
    Tracer<float> t(dummy);
    t.rng = state;
    for (uint32_t i = 0; i < count; ++i) out[i] = t.rand();
}

int oracle_trace_paths(const oracle_world* world, const uint32_t image_size[2], uint32_t max_bounces,
                       const uint32_t* pixels, uint64_t pixel_count, uint32_t sample_first, uint32_t sample_count,
                       int precision, int threads, float* radiance32, double* radiance64, pt_path_record* records) {
    if (!world || !image_size || !pixels || sample_first == 0 || (precision != 32 && precision != 64)) return -1;
    if (precision == 64 && radiance32) return -1;
    const int64_t total = (int64_t)pixel_count * (int64_t)sample_count;
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
    for (int64_t k = 0; k < total; ++k) {
        const uint64_t s = (uint64_t)k / pixel_count, p = (uint64_t)k % pixel_count;
        const uint32_t px = pixels[2 * p], py = pixels[2 * p + 1];
        pt_path_record* rec = records ? &records[k] : nullptr;
        if (rec) init_record(rec);
        double out[3];
        if (precision == 32) {
            Tracer<float> t(*world);
            t.rec = rec;
            const V3<float> c = t.trace(px, py, image_size, sample_first + (uint32_t)s, max_bounces);
            if (radiance32) {
                radiance32[3 * k] = c.x;
                radiance32[3 * k + 1] = c.y;
                radiance32[3 * k + 2] = c.z;
            }
            if (rec) {
                rec->radiance[0] = c.x;
                rec->radiance[1] = c.y;
                rec->radiance[2] = c.z;
            }
            out[0] = c.x;
            out[1] = c.y;
            out[2] = c.z;
        } else {
            Tracer<double> t(*world);
            t.rec = rec;
            const V3<double> c = t.trace(px, py, image_size, sample_first + (uint32_t)s, max_bounces);
            if (rec) {
                rec->radiance[0] = (float)c.x;
                rec->radiance[1] = (float)c.y;
                rec->radiance[2] = (float)c.z;
            }
            out[0] = c.x;
            out[1] = c.y;
            out[2] = c.z;
        }
        if (radiance64) {
            radiance64[3 * k] = out[0];
            radiance64[3 * k + 1] = out[1];
            radiance64[3 * k + 2] = out[2];
        }
    }
    return 0;
}

int oracle_intersect(const oracle_world* world, uint64_t n, const float* origins, const float* directions,
                     const float* t_max, int32_t* hit, float* hit_t, pt_path_record* records) {
    if (!world || !origins || !directions || !t_max || !hit || !hit_t) return -1;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        Tracer<float> t(*world);
        pt_path_record local;
        init_record(&local);
        t.rec = &local;
        const V3<float> o{origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]};
        const V3<float> d{directions[3 * i], directions[3 * i + 1], directions[3 * i + 2]};
        const V3<float> rcp = 1.0f / d;
        float ht = t_max[i], hv = 0.0f, hw = 0.0f;
        int32_t h = -1;
        t.closest_hit(o, d, rcp, false, &ht, &h, &hv, &hw);
        hit[i] = h;
        hit_t[i] = ht;
        if (records) records[i] = local;
    }
    return 0;
}

// elementary operations of the parity mode, for the semantic pin tests
int oracle_elementary(int op, uint64_t n, const float* a, const float* b, const float* c, float* out) {
    if (!a || !out) return -1;
    using F = float;
    auto v3 = [](const float* p, uint64_t i) { return V3<F>{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; };
    auto put3 = [&](uint64_t i, V3<F> v) {
        out[3 * i] = v.x;
        out[3 * i + 1] = v.y;
        out[3 * i + 2] = v.z;
    };
    for (uint64_t i = 0; i < n; ++i) {
        switch (op) {
            case ORACLE_OP_NORMALIZE: put3(i, normalize(v3(a, i))); break;
            case ORACLE_OP_DOT: out[i] = dot(v3(a, i), v3(b, i)); break;
            case ORACLE_OP_MIX: out[i] = lerp(a[i], b[i], c[i]); break;
            case ORACLE_OP_REFLECT: put3(i, reflect(v3(a, i), v3(b, i))); break;
            case ORACLE_OP_FRACT: out[i] = frac(a[i]); break;
            case ORACLE_OP_MIN: out[i] = M<F>::fmin(a[i], b[i]); break;
            case ORACLE_OP_MAX: out[i] = M<F>::fmax(a[i], b[i]); break;
            case ORACLE_OP_CLAMP: out[i] = clamp(a[i], b[i], c[i]); break;
            case ORACLE_OP_RSQRT: out[i] = rsqrt(a[i]); break;
            case ORACLE_OP_TO_U32: {
                const uint32_t u = to_u32(a[i]);
                std::memcpy(&out[i], &u, 4);
                break;
            }
            case ORACLE_OP_SRGB: out[i] = kSrgb.v[(uint8_t)a[i]]; break;
            case ORACLE_OP_SLAB: {  // a: node min xyz, max xyz (6); b: origin xyz, direction xyz (6); c: hit_t
                pt_bvh_node node{};
                for (int k = 0; k < 3; ++k) {
                    node.aabb_min[k] = a[6 * i + k];
                    node.aabb_max[k] = a[6 * i + 3 + k];
                }
                const V3<F> o{b[6 * i], b[6 * i + 1], b[6 * i + 2]}, d{b[6 * i + 3], b[6 * i + 4], b[6 * i + 5]};
                const V3<F> rcp = F(1) / d;
                out[i] = Tracer<F>::intersect_aabb(node, -o * rcp, rcp, c[i]);
                break;
            }
            case ORACLE_OP_CAMERA_RAY: {  // a = camera (16 floats); b = px, py, width, height; c = RNG state bits
                pt_camera cam;
                std::memcpy(&cam, a + 16 * i, sizeof cam);
                uint32_t st;
                std::memcpy(&st, c + i, 4);
                oracle_world dummy{};
                Tracer<F> t(dummy);
                t.rng = st;
                const uint32_t img[2] = {(uint32_t)b[4 * i + 2], (uint32_t)b[4 * i + 3]};
                V3<F> o, d;
                t.camera_ray(cam, (uint32_t)b[4 * i], (uint32_t)b[4 * i + 1], img, &o, &d);
                put3(i, d);
                break;
            }
            default: return -1;
        }
    }
    return 0;
}

int oracle_shade_cases(int precision, const oracle_shade_case* cases, uint64_t n, oracle_shade_result* out) {
    if (!cases || !out || (precision != 32 && precision != 64)) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        if (precision == 32) shade_case<float>(cases[i], &out[i]);
        else shade_case<double>(cases[i], &out[i]);
    }
    return 0;
}

int oracle_sample_lights(const oracle_world* world, int precision, uint64_t n, const float* origins,
                         const uint32_t* rng_states, oracle_light_result* out) {
    if (!world || !origins || !rng_states || !out || (precision != 32 && precision != 64)) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        if (precision == 32) light_case<float>(*world, origins + 3 * i, rng_states[i], &out[i]);
        else light_case<double>(*world, origins + 3 * i, rng_states[i], &out[i]);
    }
    return 0;
}

void oracle_fmath(int which, const float* x, const float* y, float* out, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) {
        switch (which) {
            case 0: out[i] = ptm::sinf_(x[i]); break;
            case 1: out[i] = ptm::cosf_(x[i]); break;
            case 2: out[i] = ptm::acosf_(x[i]); break;
            case 3: out[i] = ptm::atan2f_(y[i], x[i]); break;
            case 4: out[i] = ptm::powf_(x[i], y[i]); break;
            case 5: out[i] = ptm::log2f_(x[i]); break;
            case 6: out[i] = ptm::exp2f_(x[i]); break;
            case 7: {  // sin through the shared-reduction sincos of the kernels
                float sn, cs;
                ptm::sincosf_(x[i], &sn, &cs);
                out[i] = sn;
                break;
            }
            case 8: {
                float sn, cs;
                ptm::sincosf_(x[i], &sn, &cs);
                out[i] = cs;
                break;
            }
            default: out[i] = 0.0f; break;
        }
    }
}

}  // extern "C"
