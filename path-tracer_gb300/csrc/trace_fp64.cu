// trace_fp64.cu - the FP64 reference render on the GPU.
//
// One thread runs one whole path (compute_main, trace.slang:719-1297) in
// double arithmetic: every quantity the shader computes in f32 is a double
// here, the shader's f32 literals are widened exactly, the world's FP32
// buffers are read as uploaded and widened, and the transcendentals are
// CUDA's double-precision sin / cos / acos / atan2 / pow.  The random numbers
// are the shader's own f32 draws (trace.slang:195-202) from the same per-pixel
// seeds (trace.slang:736-737), so a path here makes the decisions the FP32
// path makes unless the FP32 rounding moves a comparison, and the difference
// between the two renders measures the FP32 arithmetic error of the image.
//
// This is the only FP64 code of the library and it is not a rendering path:
// pt_render_fp64 (include/pt_precision.h) runs it to produce the reference
// image that the FP32 and compressed forms are measured against.  It reads
// the binary BVH and the FP32 attributes, whatever precision form the
// context has selected.
#include "pt_kernels.h"

namespace ptx64 {

#define PTX __device__ __forceinline__

// shader f32 literals, widened without rounding
#define KF(x) ((double)(x##f))

constexpr double kPi = (double)3.14159265359f;
constexpr double kInvPi = (double)0.31830988618f;
constexpr double kInv2Pi = (double)0.15915494309189535f;
constexpr double kTwoPi = (double)(2.0f * 3.14159265359f);
constexpr double kFltMax = (double)0x1.fffffep+127f;

struct d2 {
    double x, y;
};
struct d3 {
    double x, y, z;
};

PTX d3 mk(double x, double y, double z) { return d3{x, y, z}; }
PTX d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
PTX d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
PTX d3 operator-(d3 a) { return {-a.x, -a.y, -a.z}; }
PTX d3 operator*(d3 a, d3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
PTX d3 operator/(d3 a, d3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
PTX d3 operator*(d3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
PTX d3 operator*(double s, d3 a) { return {s * a.x, s * a.y, s * a.z}; }
PTX d3 operator/(d3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
PTX d3 operator/(double s, d3 a) { return {s / a.x, s / a.y, s / a.z}; }
PTX d3 operator+(d3 a, double s) { return {a.x + s, a.y + s, a.z + s}; }
PTX d3 operator-(double s, d3 a) { return {s - a.x, s - a.y, s - a.z}; }
PTX d3 operator-(d3 a, double s) { return {a.x - s, a.y - s, a.z - s}; }
PTX double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PTX d3 cross(d3 a, d3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
PTX double rsq(double x) { return 1.0 / sqrt(x); }
PTX double length(d3 v) { return sqrt(dot(v, v)); }
PTX d3 normalize(d3 v) { return v * rsq(dot(v, v)); }
PTX double mix(double a, double b, double t) { return a * (1.0 - t) + b * t; }
PTX d3 mix(d3 a, d3 b, double t) { return {mix(a.x, b.x, t), mix(a.y, b.y, t), mix(a.z, b.z, t)}; }
PTX double saturate(double x) { return fmin(fmax(x, 0.0), 1.0); }
PTX d3 saturate(d3 v) { return {saturate(v.x), saturate(v.y), saturate(v.z)}; }
PTX double clampd(double x, double lo, double hi) { return fmin(fmax(x, lo), hi); }
PTX double fract(double x) { return x - floor(x); }
PTX double signd(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }
PTX d3 reflect(d3 i, d3 n) { return i - (2.0 * dot(n, i)) * n; }
PTX bool any_positive(d3 v) { return v.x > 0.0 || v.y > 0.0 || v.z > 0.0; }
PTX double comp(d3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
PTX d3 f3of(const float* p) { return mk(__ldg(p), __ldg(p + 1), __ldg(p + 2)); }
PTX double fifth_power(double x) { return x * x * x * x * x; }

// WGSL u32(): truncation toward zero, saturating, NaN -> 0
PTX uint32_t to_u32(double x) {
    if (!(x > 0.0)) return 0u;
    if (x >= 4294967296.0) return 0xffffffffu;
    return (uint32_t)x;
}

struct Path {
    const ptd::World& w;
    uint32_t s;
    // rand(), trace.slang:195-202: the shader's f32 draw, widened
    PTX double rnd() { return (double)ptd::rand_next(s); }
};

// nearest + clamp-to-edge atlas fetch (world_resources.rs:447-450); sRGB
// layers decode through the library's FP32 table as the FP32 path does
PTX void atlas(const ptd::World& w, bool srgb, int32_t layer, d2 uv, double out[4]) {
    const uint32_t count = srgb ? w.srgb_count : w.linear_count;
    const uint8_t* base = srgb ? w.srgb : w.linear;
    if (count == 0u) {
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return;
    }
    const uint32_t l = layer < 0 ? 0u : ((uint32_t)layer >= count ? count - 1u : (uint32_t)layer);
    const double fx = floor(uv.x * 8192.0), fy = floor(uv.y * 8192.0);
    const uint32_t ix = fx >= 8191.0 ? 8191u : to_u32(fx);
    const uint32_t iy = fy >= 8191.0 ? 8191u : to_u32(fy);
    const uchar4 p = __ldg(reinterpret_cast<const uchar4*>(base) + ((uint64_t)l * PT_ATLAS_SIZE + iy) * PT_ATLAS_SIZE + ix);
    if (srgb) {
        out[0] = __ldg(w.srgb_lut + p.x);
        out[1] = __ldg(w.srgb_lut + p.y);
        out[2] = __ldg(w.srgb_lut + p.z);
    } else {
        out[0] = (double)((float)p.x / 255.0f);
        out[1] = (double)((float)p.y / 255.0f);
        out[2] = (double)((float)p.z / 255.0f);
    }
    out[3] = (double)((float)p.w / 255.0f);
}

PTX d2 atlas_uv(d2 uv, const float* os) {
    return {fma(uv.x, (double)os[2], (double)os[0]), fma(uv.y, (double)os[3], (double)os[1])};
}

// bilinear + clamp-to-edge skybox fetch (world_resources.rs:451-456)
PTX uint32_t sky_index(double f, uint32_t n, int off) {
    if (!(f == f)) return 0u;
    int64_t i = f < -1e9 ? -1000000000ll : (f > 1e9 ? 1000000000ll : (int64_t)f);
    i += off;
    if (i < 0) i = 0;
    if (i > (int64_t)n - 1) i = (int64_t)n - 1;
    return (uint32_t)i;
}
PTX d3 sky_px64(const ptd::World& w, uint32_t ix, uint32_t iy) {
    const float4 p = __ldg(w.sky + (uint64_t)iy * w.sky_u.width + ix);
    return mk(p.x, p.y, p.z);
}
PTX d3 skybox_bilinear(const ptd::World& w, d2 uv) {
    const uint32_t W = w.sky_u.width, H = w.sky_u.height;
    const double x = uv.x * (double)(float)W - 0.5, y = uv.y * (double)(float)H - 0.5;
    const double x0 = floor(x), y0 = floor(y);
    const double fx = x - x0, fy = y - y0;
    const uint32_t ix0 = sky_index(x0, W, 0), ix1 = sky_index(x0, W, 1);
    const uint32_t iy0 = sky_index(y0, H, 0), iy1 = sky_index(y0, H, 1);
    const d3 top = mix(sky_px64(w, ix0, iy0), sky_px64(w, ix1, iy0), fx);
    const d3 bottom = mix(sky_px64(w, ix0, iy1), sky_px64(w, ix1, iy1), fx);
    return mix(top, bottom, fy);
}

// orthonormal_tangent, trace.slang:207-218
PTX d3 orthonormal_tangent(d3 tangent, d3 normal) {
    const d3 projected = tangent - dot(normal, tangent) * normal;
    const double ls = dot(projected, projected);
    if (ls > KF(1e-12)) return projected * rsq(ls);
    const double s = normal.z >= 0.0 ? 1.0 : -1.0;
    const double a = -1.0 / (s + normal.z);
    return mk(fma(s * normal.x * normal.x, a, 1.0), s * normal.x * normal.y * a, -s * normal.x);
}

// fresnel_exact, trace.slang:330-341
PTX double fresnel_exact(double ior, double cos_i) {
    const double s = fma(-cos_i, cos_i, 1.0) / (ior * ior);
    if (s >= 1.0) return 1.0;
    const double cos_t = sqrt(1.0 - s);
    const double rs = fma(-ior, cos_t, cos_i) / fma(ior, cos_t, cos_i);
    const double rp = fma(-ior, cos_i, cos_t) / fma(ior, cos_i, cos_t);
    return 0.5 * (rs * rs + rp * rp);
}

// ggx_lambda, trace.slang:347-352
PTX double ggx_lambda(d3 v, d2 a) {
    return fma(0.5, sqrt(1.0 + (a.x * a.x * v.x * v.x + a.y * a.y * v.y * v.y) / (v.z * v.z)), -0.5);
}

// sample_VNDF, trace.slang:356-364
PTX d3 sample_vndf(d3 wo, d2 a, double r, double two_pi_r) {
    const d3 ww = normalize(mk(wo.x * a.x, wo.y * a.y, wo.z));
    const double z = fma(1.0 - r, 1.0 + ww.z, -ww.z);
    const double sin_theta = sqrt(saturate(fma(-z, z, 1.0)));
    double sn, cs;
    sincos(two_pi_r, &sn, &cs);
    const d3 h = mk(sin_theta * cs, sin_theta * sn, z) + ww;
    return normalize(mk(h.x * a.x, h.y * a.y, h.z));
}

// alpha_anisotropic, trace.slang:369-375
PTX d2 alpha_anisotropic(double roughness, double anisotropy) {
    const double iso = 1.0 - anisotropy;
    const double at = roughness * roughness * KF(1.41421356237) * rsq(fma(iso, iso, 1.0));
    return {fmax(at, KF(1e-4)), fmax(at * iso, KF(1e-4))};
}

// specular_ior_modulated, trace.slang:379-391 (the clamp is the f32 just below 1)
PTX double specular_ior_modulated(double ior, double weight) {
    const double num = ior - 1.0;
    const double den = ior + 1.0;
    const double f0 = num * num / (den * den);
    const double f0s = signd(ior - 1.0) * sqrt(fmin(weight * f0, (double)__uint_as_float(0x3f800000u - 1u)));
    return (1.0 + f0s) / (1.0 - f0s);
}

// power_heuristic, trace.slang:416-424
PTX double power_heuristic(double pdf, double other) {
    const double scale = fmax(pdf, other);
    if (scale <= 0.0) return 0.0;
    const double p = pdf / scale;
    const double q = other / scale;
    return p * p / (p * p + q * q);
}

PTX d2 interp_uv(const pt_triangle_attribute& a, double u, double v, double w2) {
    return {fract(u * (double)__ldg(&a.uv0[0]) + v * (double)__ldg(&a.uv1[0]) + w2 * (double)__ldg(&a.uv2[0])),
            fract(u * (double)__ldg(&a.uv0[1]) + v * (double)__ldg(&a.uv1[1]) + w2 * (double)__ldg(&a.uv2[1]))};
}

// coverage, trace.slang:426-443
PTX double coverage(const ptd::World& w, const pt_material& m, d2 uv) {
    if (m.alpha_mode == PT_ALPHA_MODE_OPAQUE) return 1.0;
    double alpha = m.base_color[3];
    if (m.base_color_tex_layer >= 0) {
        double t[4];
        atlas(w, true, m.base_color_tex_layer, atlas_uv(uv, m.base_color_uv), t);
        alpha *= t[3];
    }
    if (m.alpha_mode == PT_ALPHA_MODE_MASK) return alpha >= (double)m.alpha_cutoff ? 1.0 : 0.0;
    return alpha;
}

// passes_through, trace.slang:446-454
PTX bool passes_through(Path& p, uint32_t tri, double v, double w2) {
    const pt_triangle_attribute& a = p.w.attr[tri];
    const pt_material& m = p.w.mat[__ldg(&a.material_index)];
    if (m.alpha_mode == PT_ALPHA_MODE_OPAQUE) return false;
    const d2 uv = interp_uv(a, 1.0 - v - w2, v, w2);
    return coverage(p.w, m, uv) <= p.rnd();
}

// evaluate_emission, trace.slang:455-466
PTX d3 evaluate_emission(const ptd::World& w, const pt_material& m, d2 uv) {
    d3 color = f3of(m.emission_color_and_luminance);
    if (m.emission_tex_layer >= 0) {
        double t[4];
        atlas(w, true, m.emission_tex_layer, atlas_uv(uv, m.emission_uv), t);
        color = color * mk(t[0], t[1], t[2]);
    }
    return (double)m.emission_weight * (double)m.emission_color_and_luminance[3] * color;
}

// skybox_uv, trace.slang:467-472
PTX d2 skybox_uv(d3 d) {
    return {fract(fma(atan2(d.z, d.x), kInv2Pi, 0.5)), atan2(sqrt(d.x * d.x + d.z * d.z), d.y) * kInvPi};
}

// evaluate_skybox, trace.slang:473-475
PTX d3 evaluate_skybox(const ptd::World& w, d3 d) {
    return skybox_bilinear(w, skybox_uv(d)) * (double)w.sky_u.average_luminance;
}

// skybox_texel_solid_angle, trace.slang:476-481
PTX double sky_texel_solid_angle64(const ptd::World& w, uint32_t row) {
    const double step = kPi / (double)(float)w.sky_u.height;
    const uint32_t other = w.sky_u.height - 1u - row;
    const uint32_t pole_row = row < other ? row : other;
    return (kTwoPi / (double)(float)w.sky_u.width) * 2.0 * sin(((double)(float)pole_row + 0.5) * step) * sin(0.5 * step);
}

// skybox_light_pdf, trace.slang:482-489
PTX double skybox_light_pdf(const ptd::World& w, d3 d, double prob) {
    if (prob <= 0.0) return 0.0;
    const d2 uv = skybox_uv(d);
    uint32_t px = to_u32(uv.x * (double)(float)w.sky_u.width);
    uint32_t py = to_u32(uv.y * (double)(float)w.sky_u.height);
    if (px > w.sky_u.width - 1u) px = w.sky_u.width - 1u;
    if (py > w.sky_u.height - 1u) py = w.sky_u.height - 1u;
    return prob * (double)__ldg(&w.sky_alias[(uint64_t)py * w.sky_u.width + px].selection_probability) /
           sky_texel_solid_angle64(w, py);
}

// triangle_selection_probability, trace.slang:490-507
PTX double tri_selection_probability64(const ptd::World& w, uint32_t tri) {
    uint32_t first = 0u, end = w.scene.emissive_triangles_count;
    while (first < end) {
        const uint32_t middle = first + (end - first) / 2u;
        const uint32_t ti = __ldg(&w.scene_alias[middle].triangle_index);
        if (ti < tri) first = middle + 1u;
        else if (ti > tri) end = middle;
        else return (double)__ldg(&w.scene_alias[middle].selection_probability);
    }
    return 0.0;
}

PTX d3 vert64(const ptd::World& w, uint32_t tri, int k) { return f3of(w.geo[tri].v0 + 3 * k); }

// triangle_light_pdf, trace.slang:508-523
PTX double triangle_light_pdf(const ptd::World& w, uint32_t tri, d3 d, double dist2, double prob) {
    if (prob <= 0.0) return 0.0;
    const d3 v0 = vert64(w, tri, 0), v1 = vert64(w, tri, 1), v2 = vert64(w, tri, 2);
    const double area = 0.5 * fabs(dot(cross(v1 - v0, v2 - v0), d));
    if (area <= 0.0) return 0.0;
    return prob * dist2 / area;
}

struct LightSample {
    d3 direction, emission;
    double distance, pdf;
    int32_t triangle_index;
};

// sample_light, trace.slang:531-592
PTX LightSample sample_light(Path& p, d3 origin) {
    const ptd::World& w = p.w;
    LightSample r;
    r.direction = mk(0.0, 0.0, 0.0);
    r.emission = mk(0.0, 0.0, 0.0);
    r.distance = 0.0;
    r.pdf = 0.0;
    r.triangle_index = -1;
    const double p0 = w.scene.light_probabilities[0], p1 = w.scene.light_probabilities[1];
    if (p0 + p1 <= 0.0) return r;
    if (p.rnd() < p0) {
        const uint32_t count = w.scene.emissive_triangles_count;
        uint32_t slot = to_u32(p.rnd() * (double)(float)count);
        if (slot > count - 1u) slot = count - 1u;
        const pt_scene_alias_entry cand = w.scene_alias[slot];
        const pt_scene_alias_entry entry = w.scene_alias[p.rnd() < (double)cand.threshold ? slot : cand.alias_index];
        const uint32_t lt = entry.triangle_index;
        const d3 v0 = vert64(w, lt, 0), v1 = vert64(w, lt, 1), v2 = vert64(w, lt, 2);
        const double root = sqrt(p.rnd());
        const double u = 1.0 - root;
        const double v = root * (1.0 - p.rnd());
        const double wb = 1.0 - u - v;
        const d3 delta = u * v0 + v * v1 + wb * v2 - origin;
        const double d2v = dot(delta, delta);
        if (d2v <= 0.0) return r;
        r.distance = sqrt(d2v);
        r.direction = delta / r.distance;
        r.triangle_index = (int32_t)lt;
        r.pdf = triangle_light_pdf(w, lt, r.direction, d2v, p0 * (double)entry.selection_probability);
        const pt_triangle_attribute& a = w.attr[lt];
        const d2 uv = interp_uv(a, u, v, wb);
        const pt_material& m = w.mat[__ldg(&a.material_index)];
        r.emission = coverage(w, m, uv) * evaluate_emission(w, m, uv);
    } else {
        const uint32_t W = w.sky_u.width, H = w.sky_u.height;
        const uint32_t count = W * H;
        uint32_t slot = to_u32(p.rnd() * (double)(float)count);
        if (slot > count - 1u) slot = count - 1u;
        const pt_skybox_alias_entry cand = w.sky_alias[slot];
        const uint32_t index = p.rnd() < (double)cand.threshold ? slot : cand.alias_index;
        const uint32_t row = index / W, column = index % W;
        const double phi = (((double)(float)column + p.rnd()) / (double)(float)W - 0.5) * kTwoPi;
        const bool north = row < H / 2u;
        const uint32_t pole_row = north ? row : H - 1u - row;
        const double half_step = 0.5 * kPi / (double)(float)H;
        const double a = sin((double)(float)pole_row * half_step);
        const double b = sin((double)(float)(pole_row + 1u) * half_step);
        const double shs = mix(a * a, b * b, p.rnd());
        const double cos_theta = 1.0 - 2.0 * shs;
        const double sin_theta = 2.0 * sqrt(fmax(0.0, shs * (1.0 - shs)));
        double sn, cs;
        sincos(phi, &sn, &cs);
        r.direction = mk(sin_theta * cs, north ? cos_theta : -cos_theta, sin_theta * sn);
        r.distance = kFltMax;
        r.pdf = skybox_light_pdf(w, r.direction, p1);
        r.emission = evaluate_skybox(w, r.direction);
    }
    return r;
}

// intersect_aabb, trace.slang:597-609, on the FP32 node bounds widened
PTX double intersect_aabb(const pt_bvh_node* node, d3 nod, d3 rcp, double hit_t) {
    const float4* q = reinterpret_cast<const float4*>(node);
    const float4 lo = __ldg(q), hi = __ldg(q + 1);
    const double t0x = fma((double)lo.x, rcp.x, nod.x), t0y = fma((double)lo.y, rcp.y, nod.y),
                 t0z = fma((double)lo.z, rcp.z, nod.z);
    const double t1x = fma((double)hi.x, rcp.x, nod.x), t1y = fma((double)hi.y, rcp.y, nod.y),
                 t1z = fma((double)hi.z, rcp.z, nod.z);
    const double t_near = fmax(fmax(fmin(t0x, t1x), fmin(t0y, t1y)), fmin(t0z, t1z));
    const double t_far = fmin(fmin(fmax(t0x, t1x), fmax(t0y, t1y)), fmax(t0z, t1z));
    return (t_near <= t_far && t_far > 0.0 && t_near < hit_t) ? fmax(0.0, t_near) : -1.0;
}

// watertight shear setup, trace.slang:769-783
struct Shear {
    int kx, ky, kz;
    double sx, sy, sz;
};
PTX Shear make_shear(d3 d, d3 rcp) {
    const double adx = fabs(d.x), ady = fabs(d.y), adz = fabs(d.z);
    const int kxy = adx > ady ? 0 : 1;
    const int kz = (kxy == 0 ? adx : ady) > adz ? kxy : 2;
    const int kx_val = kz == 2 ? 0 : kz + 1;
    const int ky_val = kx_val == 2 ? 0 : kx_val + 1;
    const bool is_neg = comp(d, kz) < 0.0;
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
PTX bool triangle_test(const ptd::World& w, uint32_t tri, d3 o, const Shear& s, double* t_out, double* v_out,
                       double* w_out) {
    const d3 A = vert64(w, tri, 0) - o, B = vert64(w, tri, 1) - o, C = vert64(w, tri, 2) - o;
    const double akz = comp(A, s.kz), bkz = comp(B, s.kz), ckz = comp(C, s.kz);
    const double ax = fma(s.sx, akz, comp(A, s.kx));
    const double ay = fma(s.sy, akz, comp(A, s.ky));
    const double bx = fma(s.sx, bkz, comp(B, s.kx));
    const double by = fma(s.sy, bkz, comp(B, s.ky));
    const double cx = fma(s.sx, ckz, comp(C, s.kx));
    const double cy = fma(s.sy, ckz, comp(C, s.ky));
    const double U = fma(cx, by, -cy * bx);
    const double V = fma(ax, cy, -ay * cx);
    const double W = fma(bx, ay, -by * ax);
    if (fmin(U, fmin(V, W)) < 0.0 && fmax(U, fmax(V, W)) > 0.0) return false;
    const double det = U + V + W;
    if (det == 0.0) return false;
    const double inv_det = 1.0 / det;
    *t_out = s.sz * fma(U, akz, fma(V, bkz, W * ckz)) * inv_det;
    *v_out = V * inv_det;
    *w_out = W * inv_det;
    return true;
}

// Both traversals of the shader (closest hit, trace.slang:764-884; any hit,
// trace.slang:614-717): the same short stack, nearer child first, ties to the
// right.  kAny: stop at the first accepted triangle, skip light_tri.
template <bool kAny>
PTX bool traverse(Path& p, d3 o, d3 d, d3 rcp, double& hit_t, int32_t& hit, double& hv, double& hw,
                  int32_t light_tri) {
    const ptd::World& w = p.w;
    const Shear s = make_shear(d, rcp);
    const d3 nod = -o * rcp;
    uint32_t stack[64];
    uint32_t node_index = 0u, sp = 0u;
    for (;;) {
        const float4 nb = __ldg(reinterpret_cast<const float4*>(w.nodes + node_index) + 1);
        const uint32_t tri_count = __float_as_uint(nb.w);
        const uint32_t left_first = __ldg(&w.nodes[node_index].left_first);
        if (tri_count > 0u) {
            for (uint32_t i = 0; i < tri_count; ++i) {
                const uint32_t tri = left_first + i;
                if (kAny && (int32_t)tri == light_tri) continue;
                double t, v, wb;
                if (!triangle_test(w, tri, o, s, &t, &v, &wb)) continue;
                if (t > 0.0 && t < hit_t) {
                    const bool skip = w.any_alpha && passes_through(p, tri, v, wb);
                    if (kAny) {
                        if (!skip) return true;
                        continue;
                    }
                    if (skip) continue;
                    hit_t = t;
                    hit = (int32_t)tri;
                    hv = v;
                    hw = wb;
                }
            }
        } else {
            const uint32_t li = left_first, ri = left_first + 1u;
            const double dl = intersect_aabb(w.nodes + li, nod, rcp, hit_t);
            const double dr = intersect_aabb(w.nodes + ri, nod, rcp, hit_t);
            const bool hl = dl >= 0.0, hr = dr >= 0.0;
            if (hl && hr) {
                const bool left_closer = dl < dr;
                stack[sp & 63u] = left_closer ? ri : li;
                sp += 1u;
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

// E_FON_exact, trace.slang:318-323
PTX double e_fon_exact(double mu, double r) {
    const double af = 1.0 / fma(KF(0.28779340921), r, 1.0);
    const double si = sqrt(fma(-mu, mu, 1.0));
    const double g = si * (acos(mu) - si * mu) + (double)0x1.555556p-1f * ((si / mu) * (1.0 - (si * si * si)) - si);
    return af + r * af * kInvPi * g;
}

struct Bsdf {
    double p_ggx, p_diffuse;
    d3 base_color;
    double base_weight, base_metalness, base_diffuse_roughness;
    d3 specular_color;
    double specular_weight, ior_m;
    d2 alpha;
    double opl;
    d3 f0, e_dielectric;
    double la, lb, lc, ld;
    d3 bx, by;
    double p_u, p_c;
};

struct Lobes {
    d3 f;
    double pdf;
};

// evaluate_lobes, trace.slang:229-315
PTX Lobes evaluate_lobes(d3 wo, d3 wi, const Bsdf& b) {
    const d3 h = normalize(wo + wi);
    const double hdotw = dot(h, wo);
    const double g1 = 1.0 / b.opl;
    const double g2 = 1.0 / (b.opl + ggx_lambda(wi, b.alpha));
    const double dh = (h.x * h.x) / (b.alpha.x * b.alpha.x) + (h.y * h.y) / (b.alpha.y * b.alpha.y) + h.z * h.z;
    const double D = kInvPi / (b.alpha.x * b.alpha.y * dh * dh);
    const double ts = D * g2 / (4.0 * wi.z * wo.z);
    const double omh = 1.0 - hdotw;
    const double p5 = fifth_power(omh);
    const d3 fa = (KF(0.00105024005) * hdotw * omh) * (1.0 - b.specular_color);
    const d3 fb = 9031.0 * b.f0 + 7776.0;
    const d3 fc = b.f0 - 1.0;
    const d3 fm = mk(fma(fa.x, fb.x, fc.x), fma(fa.y, fb.y, fc.y), fma(fa.z, fb.z, fc.z));
    const d3 f82 = b.f0 - p5 * fm;
    const d3 f_conductor = saturate(b.specular_weight * f82) * ts;
    const d3 f_dielectric = b.specular_color * fresnel_exact(b.ior_m, hdotw) * ts;
    const d3 rho = b.base_color;
    const double r = b.base_diffuse_roughness;
    const double s_f = wi.x * wo.x + wi.y * wo.y;
    const double sovert_f = s_f > 0.0 ? s_f / fmax(wo.z, wi.z) : s_f;
    const double af = 1.0 / fma(KF(0.28779340921), r, 1.0);
    const d3 f_ss = rho * kInvPi * af * fma(r, sovert_f, 1.0);
    const double efo = e_fon_exact(wo.z, r);
    const double efi = e_fon_exact(wi.z, r);
    const double avg_ef = af * fma(KF(0.07248821245), r, 1.0);
    const d3 rho_ms = rho * rho * avg_ef / (1.0 - rho * (1.0 - avg_ef));
    const d3 f_ms = (rho_ms * kInvPi) * fmax(KF(1.0e-7), 1.0 - efo) * fmax(KF(1.0e-7), 1.0 - efi) /
                    fmax(KF(1.0e-7), 1.0 - avg_ef);
    const d3 f_diffuse = b.base_weight * (f_ss + f_ms);
    const d3 f_glossy_diffuse = f_dielectric + (1.0 - b.e_dielectric) * f_diffuse;
    const d3 f_total = mix(f_glossy_diffuse, f_conductor, b.base_metalness);
    const double pdf_ggx = D * g1 / (4.0 * wo.z);
    const d3 wl = mk(dot(b.bx, wi), dot(b.by, wi), wi.z);
    const double a = b.la, bb = b.lb, c = b.lc, d = b.ld;
    const double det_m = c * fma(-bb, d, a);
    const d3 wh = mk(c * (wl.x - bb * wl.z), (a - bb * d) * wl.y, -c * (d * wl.x - a * wl.z));
    const double len_sqr = dot(wh, wh);
    const double s_pdf = fma(0.5, rsq(fma(d, d, 1.0)), 0.5);
    const double pdf_c = (det_m * det_m) / (len_sqr * len_sqr) * fmax(wh.z, 0.0) / (kPi * s_pdf);
    const double pdf_eon = b.p_u * KF(0.15915494309) + b.p_c * pdf_c;
    return {f_total, b.p_ggx * pdf_ggx + b.p_diffuse * pdf_eon};
}

// estimate_e_dielectric, trace.slang:396-411
PTX d3 estimate_e_dielectric(Path& p, d3 wo, double opl, d2 alpha, double ior_m, d3 spec_color) {
    double sum = 0.0;
#pragma unroll 1
    for (int i = 0; i < 16; ++i) {
        const double r1 = p.rnd();
        const double tpr = kTwoPi * p.rnd();
        const d3 h = sample_vndf(wo, alpha, r1, tpr);
        const d3 wi = reflect(-wo, h);
        if (wi.z <= 0.0) continue;
        const double f = fresnel_exact(ior_m, dot(h, wo));
        sum += f * opl / (opl + ggx_lambda(wi, alpha));
    }
    return spec_color * sum / 16.0;
}

// compute_main, trace.slang:721-1297, for one (pixel, sample)
PTX d3 trace_path(const ptd::World& w, uint32_t px, uint32_t py, uint32_t img_w, uint32_t img_h, uint32_t n,
                  uint32_t max_bounces) {
    Path p{w, ptd::seed(px, py, n)};
    const double jx = p.rnd();
    const double jy = p.rnd();
    const d2 puv = {((double)(float)px + jx) / (double)(float)img_w, ((double)(float)py + jy) / (double)(float)img_h};
    const pt_camera& cam = w.camera;
    d3 o = mk(cam.position[0], cam.position[1], cam.position[2]);
    const d3 llc = mk(cam.lower_left_corner_minus_position[0], cam.lower_left_corner_minus_position[1],
                      cam.lower_left_corner_minus_position[2]);
    const d3 hor = mk(cam.horizontal[0], cam.horizontal[1], cam.horizontal[2]);
    const d3 ver = mk(cam.vertical[0], cam.vertical[1], cam.vertical[2]);
    d3 d = normalize(llc + puv.x * hor + puv.y * ver);
    d3 rcp = 1.0 / d;
    d3 throughput = mk(1.0, 1.0, 1.0);
    d3 color = mk(0.0, 0.0, 0.0);
    double prev_pdf = 0.0;
    const double lp0 = w.scene.light_probabilities[0], lp1 = w.scene.light_probabilities[1];
    for (uint32_t bounce = 0; bounce <= max_bounces; ++bounce) {
        double hit_t = kFltMax, hv = 0.0, hw = 0.0;
        int32_t hit = -1;
        traverse<false>(p, o, d, rcp, hit_t, hit, hv, hw, -1);
        if (hit == -1) {
            // escaped ray, trace.slang:887-927
            double mis = 1.0;
            if (bounce > 0u) mis = power_heuristic(prev_pdf, skybox_light_pdf(w, d, lp1));
            color = color + throughput * evaluate_skybox(w, d) * mis;
            break;
        }
        const uint32_t h = (uint32_t)hit;
        const pt_triangle_attribute& attr = w.attr[h];
        const double hu = 1.0 - hv - hw;
        const d2 iuv = interp_uv(attr, hu, hv, hw);
        const pt_material& m = w.mat[__ldg(&attr.material_index)];
        d3 base_color = f3of(m.base_color);
        const double base_weight = m.base_weight;
        double base_metalness = m.base_metalness;
        double base_diffuse_roughness = m.base_diffuse_roughness;
        d3 specular_color = f3of(m.specular_color_and_weight);
        double specular_weight = m.specular_color_and_weight[3];
        double t4[4];
        if (m.base_color_tex_layer >= 0) {
            atlas(w, true, m.base_color_tex_layer, atlas_uv(iuv, m.base_color_uv), t4);
            base_color = base_color * mk(t4[0], t4[1], t4[2]);
        }
        if (m.metallic_roughness_tex_layer >= 0) {
            atlas(w, false, m.metallic_roughness_tex_layer, atlas_uv(iuv, m.metallic_roughness_uv), t4);
            base_metalness *= t4[2];
            base_diffuse_roughness *= t4[1];
        }
        if (m.specular_color_tex_layer >= 0) {
            atlas(w, true, m.specular_color_tex_layer, atlas_uv(iuv, m.specular_color_uv), t4);
            specular_color = specular_color * mk(t4[0], t4[1], t4[2]);
        }
        if (m.specular_weight_tex_layer >= 0) {
            atlas(w, false, m.specular_weight_tex_layer, atlas_uv(iuv, m.specular_weight_uv), t4);
            specular_weight *= t4[3];
        }
        // emission with MIS, trace.slang:984-991
        const d3 emission = evaluate_emission(w, m, iuv);
        double emission_mis = 1.0;
        if (bounce > 0u && lp0 > 0.0 && any_positive(emission)) {
            const double lpdf = triangle_light_pdf(w, h, d, hit_t * hit_t, lp0 * tri_selection_probability64(w, h));
            emission_mis = power_heuristic(prev_pdf, lpdf);
        }
        color = color + throughput * emission * emission_mis;

        // shading frame, trace.slang:993-1091
        const d3 hit_point = d * hit_t + o;
        const d3 V = -d;
        const d3 v0 = vert64(w, h, 0), v1 = vert64(w, h, 1), v2 = vert64(w, h, 2);
        const d3 flat_raw = normalize(cross(v1 - v0, v2 - v0));
        const double bfm = dot(V, flat_raw) > 0.0 ? 1.0 : -1.0;
        const d3 flat_n = flat_raw * bfm;
        d3 N = normalize(hu * f3of(attr.n0) + hv * f3of(attr.n1) + hw * f3of(attr.n2)) * bfm;
        const double t0w = __ldg(&attr.t0[3]);
        d3 Tn = orthonormal_tangent(hu * f3of(attr.t0) + hv * f3of(attr.t1) + hw * f3of(attr.t2), N) * bfm;
        d3 Bn = cross(N, Tn) * t0w * bfm;
        bool n_changed = false;
        if (m.normal_tex_layer >= 0) {
            atlas(w, false, m.normal_tex_layer, atlas_uv(iuv, m.normal_uv), t4);
            d3 ln = mk(t4[0] * 2.0 - 1.0, t4[1] * 2.0 - 1.0, t4[2] * 2.0 - 1.0);
            ln = normalize(mk(ln.x * (double)m.normal_scale, ln.y * (double)m.normal_scale, ln.z));
            N = normalize(ln.x * Tn + ln.y * Bn + ln.z * N);
            n_changed = true;
        }
        const double flat_ndotv = dot(flat_n, V);
        const double threshold = 0.5 * flat_ndotv;
        double ndotv = dot(N, V);
        if (ndotv < threshold) {
            N = normalize(mix(N, flat_n, (threshold - ndotv) / (flat_ndotv - ndotv)));
            ndotv = dot(N, V);
            n_changed = true;
        }
        if (n_changed) {
            Tn = orthonormal_tangent(Tn, N);
            Bn = cross(N, Tn) * t0w * bfm;
        }

        // OpenPBR setup, trace.slang:1097-1181
        Bsdf b;
        b.alpha = alpha_anisotropic(m.specular_roughness, m.specular_roughness_anisotropy);
        b.ior_m = specular_ior_modulated(m.specular_ior, specular_weight);
        b.f0 = base_weight * base_color;
        const d3 wo = mk(dot(Tn, V), dot(Bn, V), ndotv);
        b.opl = 1.0 + ggx_lambda(wo, b.alpha);
        const double r = base_diffuse_roughness;
        const double z = wo.z;
        b.la = 1.0 + r * (KF(0.303392) + (KF(-0.518982) + KF(0.111709) * z) * z + (KF(-0.276266) + KF(0.335918) * z) * r);
        b.lb = r * (KF(-1.16407) + KF(1.15859) * z + (KF(0.150815) - KF(0.150105) * z) * r) / (z * z * z - KF(1.43545));
        b.lc = 1.0 + r * (KF(0.20013) + (KF(-0.506373) + KF(0.261777) * z) * z);
        b.ld = r * (KF(0.540852) + (KF(-1.01625) + KF(0.475392) * z) * z) / (KF(-1.0743) + (KF(0.0725628) + z) * z);
        const double ls = wo.x * wo.x + wo.y * wo.y;
        d3 bx = mk(1.0, 0.0, 0.0);
        if (ls > 0.0) bx = mk(wo.x, wo.y, 0.0) * rsq(ls);
        b.bx = bx;
        b.by = mk(-bx.y, bx.x, 0.0);
        b.e_dielectric = estimate_e_dielectric(p, wo, b.opl, b.alpha, b.ior_m, specular_color);
        const d3 luma = mk(KF(0.2126), KF(0.7152), KF(0.0722));
        const double albedo_gloss = dot(b.e_dielectric, luma);
        const double albedo_diffuse = (1.0 - albedo_gloss) * base_weight * dot(base_color, luma);
        const d3 fsm = b.f0 + (1.0 - b.f0) * fifth_power(1.0 - wo.z);
        const double albedo_metal = dot(fsm, luma);
        const double w_ggx = mix(albedo_gloss, albedo_metal, base_metalness);
        const double w_diffuse = (1.0 - base_metalness) * albedo_diffuse;
        b.p_ggx = clampd(w_ggx / fmax(w_ggx + w_diffuse, KF(1e-7)), KF(0.1), KF(0.9));
        b.p_diffuse = 1.0 - b.p_ggx;
        b.p_u = pow(r, KF(0.1)) * (KF(0.162925) + (KF(-0.372058) + (KF(0.538233) - KF(0.290822) * z) * z) * z);
        b.p_c = 1.0 - b.p_u;
        b.base_color = base_color;
        b.base_weight = base_weight;
        b.base_metalness = base_metalness;
        b.base_diffuse_roughness = base_diffuse_roughness;
        b.specular_color = specular_color;
        b.specular_weight = specular_weight;

        // next-event estimation, trace.slang:1187-1206
        const d3 next_origin = hit_point + flat_n * fmax(KF(1e-4), KF(1e-4) * length(hit_point));
        const LightSample light = sample_light(p, next_origin);
        const d3 lwi = mk(dot(Tn, light.direction), dot(Bn, light.direction), dot(N, light.direction));
        if (light.pdf > 0.0 && lwi.z > 0.0 && any_positive(light.emission)) {
            const Lobes lobes = evaluate_lobes(wo, lwi, b);
            double st = light.distance, sv = 0.0, sw = 0.0;
            int32_t sh = -1;
            if (!traverse<true>(p, next_origin, light.direction, 1.0 / light.direction, st, sh, sv, sw,
                                light.triangle_index)) {
                const double weight = bounce < max_bounces ? power_heuristic(light.pdf, lobes.pdf) : 1.0;
                color = color + throughput * lobes.f * lwi.z * light.emission * (weight / light.pdf);
            }
        }
        if (bounce == max_bounces) break;

        // BSDF sampling, trace.slang:1212-1260
        const double two_pi_r = kTwoPi * p.rnd();
        const double r1 = p.rnd();
        double sn, cs;
        sincos(two_pi_r, &sn, &cs);
        d3 wi;
        if (p.rnd() < b.p_ggx) {
            wi = reflect(-wo, sample_vndf(wo, b.alpha, r1, two_pi_r));
        } else if (r1 < b.p_u) {
            const double u1 = r1 / b.p_u;
            const double sin_theta = sqrt(1.0 - u1 * u1);
            wi = mk(sin_theta * cs, sin_theta * sn, u1);
        } else {
            const double u1 = (r1 - b.p_u) / b.p_c;
            const double R = sqrt(u1);
            const double y = R * sn;
            const double s = fma(0.5, rsq(fma(b.ld, b.ld, 1.0)), 0.5);
            const double x = -mix(sqrt(fma(-y, y, 1.0)), R * cs, s);
            const d3 wh = mk(x, y, sqrt(fmax(1.0 - (x * x + y * y), 0.0)));
            const d3 wu = mk(b.la * wh.x + b.lb * wh.z, b.lc * wh.y, b.ld * wh.x + wh.z);
            wi = normalize(wu.x * b.bx + wu.y * b.by + wu.z * mk(0.0, 0.0, 1.0));
        }
        if (wi.z <= 0.0) break;
        const Lobes lobes = evaluate_lobes(wo, wi, b);
        if (lobes.pdf <= 0.0) break;
        throughput = throughput * (lobes.f * wi.z / lobes.pdf);
        prev_pdf = lobes.pdf;
        if (bounce > 3u) {
            const double p_survive = clampd(fmax(throughput.x, fmax(throughput.y, throughput.z)), KF(0.05), KF(0.95));
            if (p.rnd() > p_survive) break;
            throughput = throughput / p_survive;
        }
        o = next_origin;
        d = wi.x * Tn + wi.y * Bn + wi.z * N;
        rcp = 1.0 / d;
    }
    return color;
}

// one launch per sample n: every visible tile pixel adds its radiance to
// sums[3 * (y * tile_w + x) ..]
__global__ void __launch_bounds__(128) fp64_kernel(ptd::World w, ptk::Tile t, uint32_t vis_w, uint32_t vis_h,
                                                   uint32_t n, double* sums) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= vis_w * vis_h) return;
    const uint32_t gx = i % vis_w, gy = i / vis_w;
    const d3 c = trace_path(w, gx + t.origin_x, gy + t.origin_y, t.image_w, t.image_h, n, t.max_bounces);
    double* s = sums + 3 * ((size_t)gy * t.tile_w + gx);
    s[0] += c.x;
    s[1] += c.y;
    s[2] += c.z;
}

}  // namespace ptx64

namespace ptk {

cudaError_t launch_fp64(const ptd::World& w, const Tile& t, uint32_t sample, double* sums, cudaStream_t stream) {
    if (t.origin_x >= t.image_w || t.origin_y >= t.image_h) return cudaErrorInvalidValue;
    const uint32_t vw = t.tile_w < t.image_w - t.origin_x ? t.tile_w : t.image_w - t.origin_x;
    const uint32_t vh = t.tile_h < t.image_h - t.origin_y ? t.tile_h : t.image_h - t.origin_y;
    const uint32_t paths = vw * vh;  // tile dimensions are at most 16384 each
    if (paths == 0) return cudaSuccess;
    ptx64::fp64_kernel<<<(paths + 127u) / 128u, 128, 0, stream>>>(w, t, vw, vh, sample, sums);
    return cudaGetLastError();
}

}  // namespace ptk
