// world.cpp - host-side world builder: the parts of the reference's
// src/render/world.rs that produce the GPU buffers read by the trace pass.
//
// Floating-point rules: compiled with -ffp-contract=off, so every a * b + c
// below rounds twice exactly like the reference's Rust (which never
// contracts), and every Rust `mul_add` is spelled as a correctly rounded fma.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "../../include/pt_world.h"
#include "pt_fmath.h"
#include "pt_abi_guard.h"
#include "pt_mikktspace.h"

namespace {

struct Vec3 {
    float x, y, z;
};
inline Vec3 v3(float x, float y, float z) { return Vec3{x, y, z}; }
inline Vec3 operator+(Vec3 a, Vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline Vec3 operator-(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec3 operator*(Vec3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline Vec3 operator/(Vec3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float get(Vec3 v, int axis) { return axis == 0 ? v.x : (axis == 1 ? v.y : v.z); }
// glam Vec3::min / max: per-component f32::min / max (IEEE minNum / maxNum)
inline Vec3 vmin(Vec3 a, Vec3 b) { return {std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)}; }
inline Vec3 vmax(Vec3 a, Vec3 b) { return {std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)}; }
// glam dot / cross / normalize (length_recip = 1 / sqrt(dot))
inline float dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3 cross(Vec3 a, Vec3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
inline Vec3 normalize(Vec3 v) { return v * (1.0f / std::sqrt(dot(v, v))); }

struct DVec3 {
    double x, y, z;
};
inline DVec3 dv(Vec3 v) { return {v.x, v.y, v.z}; }
inline DVec3 operator-(DVec3 a, DVec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double ddot(DVec3 a, DVec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline DVec3 dcross(DVec3 a, DVec3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}

// Aabb, world.rs:402-423
struct Aabb {
    Vec3 min{INFINITY, INFINITY, INFINITY};
    Vec3 max{-INFINITY, -INFINITY, -INFINITY};
    void unite(const Aabb& o) {
        min = vmin(min, o.min);
        max = vmax(max, o.max);
    }
    float surface_area_half() const {
        Vec3 e = max - min;
        return std::fma(e.z, e.x, std::fma(e.x, e.y, e.y * e.z));
    }
};

// BvhTriangle, world.rs:425-429
struct BvhTriangle {
    Aabb aabb;
    Vec3 centroid;
    uint32_t original_index;
};

constexpr int kBins = 8;  // BVH_BINS, world.rs:437

// `as usize` of a non-negative f32 (saturating, NaN -> 0), then .min(BVH_BINS - 1)
inline int bin_of(float scaled) {
    if (!(scaled > 0.0f)) return 0;
    if (scaled >= (float)(kBins - 1)) return kBins - 1;
    return (int)scaled;
}

void update_aabb(pt_bvh_node& node, const BvhTriangle* tris, size_t count) {
    Aabb a;
    for (size_t i = 0; i < count; ++i) a.unite(tris[i].aabb);
    node.aabb_min[0] = a.min.x;
    node.aabb_min[1] = a.min.y;
    node.aabb_min[2] = a.min.z;
    node.aabb_max[0] = a.max.x;
    node.aabb_max[1] = a.max.y;
    node.aabb_max[2] = a.max.z;
}

// Scene::subdivide, world.rs:1430-1591.  The recursion (left child fully,
// then right child) is replayed with an explicit LIFO so deep trees cannot
// overflow the call stack; node indices come out identical because children
// are still allocated when their parent is processed.
void subdivide_all(std::vector<pt_bvh_node>& nodes, std::vector<BvhTriangle>& tris) {
    struct Job {
        size_t node, start, end;
    };
    std::vector<Job> stack;
    stack.push_back({0, 0, tris.size()});
    while (!stack.empty()) {
        Job job = stack.back();
        stack.pop_back();
        const size_t node_index = job.node, start = job.start, end = job.end;
        const size_t tri_count = end - start;
        if (tri_count <= 2) {
            nodes[node_index].left_first = (uint32_t)start;
            nodes[node_index].tri_count = (uint32_t)tri_count;
            continue;
        }
        Vec3 cmin{INFINITY, INFINITY, INFINITY}, cmax{-INFINITY, -INFINITY, -INFINITY};
        for (size_t i = start; i < end; ++i) {
            cmin = vmin(cmin, tris[i].centroid);
            cmax = vmax(cmax, tris[i].centroid);
        }
        int best_axis = 0;
        int best_split = 0;
        float best_cost = std::numeric_limits<float>::max();
        for (int axis = 0; axis < 3; ++axis) {
            const float amin = get(cmin, axis), amax = get(cmax, axis);
            if (amin == amax) continue;
            Aabb bin_box[kBins];
            uint32_t bin_count[kBins] = {0};
            const float scale = (float)kBins / (amax - amin);
            for (size_t i = start; i < end; ++i) {
                const int b = bin_of((get(tris[i].centroid, axis) - amin) * scale);
                bin_count[b] += 1;
                bin_box[b].unite(tris[i].aabb);
            }
            float left_area[kBins - 1], right_area[kBins - 1];
            uint32_t left_count[kBins - 1], right_count[kBins - 1];
            Aabb left_box, right_box;
            uint32_t left_sum = 0, right_sum = 0;
            for (int i = 0; i < kBins - 1; ++i) {
                left_sum += bin_count[i];
                left_box.unite(bin_box[i]);
                left_count[i] = left_sum;
                left_area[i] = left_box.surface_area_half();
            }
            for (int i = kBins - 1; i >= 1; --i) {
                right_sum += bin_count[i];
                right_box.unite(bin_box[i]);
                right_count[i - 1] = right_sum;
                right_area[i - 1] = right_box.surface_area_half();
            }
            for (int i = 0; i < kBins - 1; ++i) {
                const float cost = std::fma((float)left_count[i], left_area[i],
                                            (float)right_count[i] * right_area[i]);
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = axis;
                    best_split = i;
                }
            }
        }
        const pt_bvh_node& n = nodes[node_index];
        const Vec3 e = v3(n.aabb_max[0], n.aabb_max[1], n.aabb_max[2]) -
                       v3(n.aabb_min[0], n.aabb_min[1], n.aabb_min[2]);
        const float leaf_cost = (float)tri_count * std::fma(e.z, e.x, std::fma(e.x, e.y, e.y * e.z));
        if (best_cost >= leaf_cost) {
            nodes[node_index].left_first = (uint32_t)start;
            nodes[node_index].tri_count = (uint32_t)tri_count;
            continue;
        }
        const float amin = get(cmin, best_axis), amax = get(cmax, best_axis);
        const float scale = (float)kBins / (amax - amin);
        auto get_bin = [&](size_t i) {
            return bin_of((get(tris[i].centroid, best_axis) - amin) * scale);
        };
        // modified Hoare partition, world.rs:1555-1575
        int64_t left = (int64_t)start, right = (int64_t)end - 1;
        for (;;) {
            while (left <= right && get_bin((size_t)left) <= best_split) left += 1;
            while (right > left && get_bin((size_t)right) > best_split) right -= 1;
            if (left >= right) break;
            std::swap(tris[(size_t)left], tris[(size_t)right]);
            left += 1;
            right -= 1;
        }
        const size_t split = (size_t)left;
        const size_t lc = nodes.size(), rc = lc + 1;
        nodes.push_back(pt_bvh_node{});
        nodes.push_back(pt_bvh_node{});
        update_aabb(nodes[lc], tris.data() + start, split - start);
        update_aabb(nodes[rc], tris.data() + split, end - split);
        nodes[node_index].left_first = (uint32_t)lc;
        nodes[node_index].tri_count = 0;
        stack.push_back({rc, split, end});
        stack.push_back({lc, start, split});
    }
}

void build_bvh(const std::vector<pt_triangle_geometry>& geos, std::vector<pt_bvh_node>& nodes,
               std::vector<uint32_t>& order) {
    std::vector<BvhTriangle> tris(geos.size());
    for (size_t i = 0; i < geos.size(); ++i) {
        const auto& g = geos[i];
        const Vec3 a = v3(g.v0[0], g.v0[1], g.v0[2]);
        const Vec3 b = v3(g.v1[0], g.v1[1], g.v1[2]);
        const Vec3 c = v3(g.v2[0], g.v2[1], g.v2[2]);
        tris[i].aabb.min = vmin(vmin(a, b), c);
        tris[i].aabb.max = vmax(vmax(a, b), c);
        tris[i].centroid = (a + b + c) / 3.0f;
        tris[i].original_index = (uint32_t)i;
    }
    nodes.clear();
    nodes.reserve(geos.empty() ? 1 : 2 * geos.size());
    nodes.push_back(pt_bvh_node{});
    if (!geos.empty()) {
        update_aabb(nodes[0], tris.data(), tris.size());
        subdivide_all(nodes, tris);
    }
    order.resize(tris.size());
    for (size_t i = 0; i < tris.size(); ++i) order[i] = tris[i].original_index;
}

// deepest stack use of the reference traversal: the number of deferred
// siblings is at most the depth of the tree
uint32_t bvh_depth(const std::vector<pt_bvh_node>& nodes) {
    if (nodes.empty()) return 0;
    uint32_t best = 0;
    std::vector<std::pair<uint32_t, uint32_t>> st{{0u, 0u}};
    while (!st.empty()) {
        auto [i, d] = st.back();
        st.pop_back();
        best = std::max(best, d);
        if (nodes[i].tri_count == 0) {
            st.push_back({nodes[i].left_first, d + 1});
            st.push_back({nodes[i].left_first + 1, d + 1});
        }
    }
    return best;
}

// luminance via Rec. 709, world.rs:578-581
double luminance(float r, float g, float b) {
    const double x = std::fmax((double)r, 0.0), y = std::fmax((double)g, 0.0), z = std::fmax((double)b, 0.0);
    return x * 0.2126 + y * 0.7152 + z * 0.0722;
}

// exact equirectangular row solid angle without the longitude factor, world.rs:584-587
double row_weight(uint32_t y, uint32_t height) {
    const double step = 3.14159265358979323846 / (double)height;
    return std::cos((double)y * step) - std::cos((double)(y + 1) * step);
}

// Vose's alias method, world.rs:542-575
std::vector<pt_skybox_alias_entry> alias_table(const double* w, size_t n) {
    double total = 0.0;
    for (size_t i = 0; i < n; ++i) total += w[i];
    std::vector<pt_skybox_alias_entry> entries;
    if (!(total > 0.0)) return entries;
    entries.resize(n);
    std::vector<double> scaled(n);
    std::vector<uint32_t> small, large;
    for (size_t i = 0; i < n; ++i) {
        entries[i].threshold = 1.0f;
        entries[i].alias_index = (uint32_t)i;
        entries[i].selection_probability = (float)(w[i] / total);
        scaled[i] = w[i] / total * (double)n;
    }
    for (size_t i = 0; i < n; ++i) (scaled[i] < 1.0 ? small : large).push_back((uint32_t)i);
    while (!small.empty() && !large.empty()) {
        const uint32_t low = small.back(), high = large.back();
        small.pop_back();
        large.pop_back();
        entries[low].threshold = (float)std::min(std::max(scaled[low], 0.0), 1.0);
        entries[low].alias_index = high;
        scaled[high] = (scaled[high] + scaled[low]) - 1.0;
        (scaled[high] < 1.0 ? small : large).push_back(high);
    }
    return entries;
}

// Camera, world.rs:360-376 (movement speeds are UI-only and left out)
struct Camera {
    Vec3 position{0, 0, 0};
    float yaw = 0, pitch = 0, fov = 0, aspect_ratio = 1;
    bool operator==(const Camera& o) const {
        return position.x == o.position.x && position.y == o.position.y &&
               position.z == o.position.z && yaw == o.yaw && pitch == o.pitch && fov == o.fov &&
               aspect_ratio == o.aspect_ratio;
    }
};

// Camera::new, world.rs:2178-2193
Camera auto_camera(Vec3 mn, Vec3 mx) {
    Camera c;
    const Vec3 center = (mn + mx) * 0.5f;
    c.position = v3(center.x, center.y, std::fma(std::fmax(mx.x - mn.x, mx.y - mn.y), 0.6f, mx.z));
    c.yaw = 0.0f;
    c.pitch = 0.0f;
    c.fov = 1.57079632679489661923f;  // FRAC_PI_2
    c.aspect_ratio = 1.0f;
    return c;
}

// glam Mat3 * Vec3 with columns cx, cy, cz
inline Vec3 mat_mul(Vec3 cx, Vec3 cy, Vec3 cz, Vec3 v) {
    Vec3 r = cx * v.x;
    r = r + cy * v.y;
    r = r + cz * v.z;
    return r;
}

// Camera::gpu_camera, world.rs:2159-2173.  Angles go through the same
// deterministic sin/cos as the kernels so the camera is identical on every host.
pt_camera gpu_camera(const Camera& c) {
    const float sy = ptm::sinf_(c.yaw), cy = ptm::cosf_(c.yaw);
    const float sp = ptm::sinf_(c.pitch), cp = ptm::cosf_(c.pitch);
    // from_rotation_y(yaw) columns
    const Vec3 ry0 = v3(cy, 0, -sy), ry1 = v3(0, 1, 0), ry2 = v3(sy, 0, cy);
    // from_rotation_x(pitch) columns
    const Vec3 rx0 = v3(1, 0, 0), rx1 = v3(0, cp, sp), rx2 = v3(0, -sp, cp);
    // rotation = Ry * Rx (column j = Ry * Rx.col_j)
    const Vec3 m0 = mat_mul(ry0, ry1, ry2, rx0);
    const Vec3 m1 = mat_mul(ry0, ry1, ry2, rx1);
    const Vec3 m2 = mat_mul(ry0, ry1, ry2, rx2);
    const float half = c.fov * 0.5f;
    const float height = 2.0f * (ptm::sinf_(half) / ptm::cosf_(half));
    const Vec3 horizontal = (mat_mul(m0, m1, m2, v3(1, 0, 0)) * c.aspect_ratio) * height;
    const Vec3 vertical = mat_mul(m0, m1, m2, v3(0, -1, 0)) * height;
    const Vec3 llc = mat_mul(m0, m1, m2, v3(0, 0, -1)) - (horizontal + vertical) * 0.5f;
    pt_camera g{};
    g.position[0] = c.position.x;
    g.position[1] = c.position.y;
    g.position[2] = c.position.z;
    g.lower_left_corner_minus_position[0] = llc.x;
    g.lower_left_corner_minus_position[1] = llc.y;
    g.lower_left_corner_minus_position[2] = llc.z;
    g.horizontal[0] = horizontal.x;
    g.horizontal[1] = horizontal.y;
    g.horizontal[2] = horizontal.z;
    g.vertical[0] = vertical.x;
    g.vertical[1] = vertical.y;
    g.vertical[2] = vertical.z;
    return g;
}

struct Skybox {
    std::vector<float> rgba{0, 0, 0, 0};
    pt_skybox_uniforms uniforms{0.0f, 0.0f, 1, 1};
    std::vector<pt_skybox_alias_entry> alias;
};

// Skybox::new on decoded RGBA32F pixels, world.rs:1872-1957
Skybox make_skybox(const float* px, uint32_t width, uint32_t height) {
    Skybox s;
    std::vector<float> pixels(px, px + (size_t)width * height * 4);
    double total_luma = 0.0;
    const double total_weight = 2.0 * (double)width;
    for (uint32_t y = 0; y < height; ++y) {
        const double w = row_weight(y, height);
        for (uint32_t x = 0; x < width; ++x) {
            const float* p = &pixels[((size_t)y * width + x) * 4];
            total_luma = std::fma(luminance(p[0], p[1], p[2]), w, total_luma);
        }
    }
    if (total_luma == 0.0) return s;  // black 1x1 skybox
    const double avg = total_luma / total_weight;
    const double scale = 1.0 / avg;
    for (size_t i = 0; i < (size_t)width * height; ++i)
        for (int ch = 0; ch < 3; ++ch) pixels[i * 4 + ch] = (float)((double)pixels[i * 4 + ch] * scale);
    s.rgba = std::move(pixels);
    s.uniforms.total_luminous_flux = 0.0f;
    s.uniforms.average_luminance = (float)avg;
    s.uniforms.width = width;
    s.uniforms.height = height;
    return s;
}

// Skybox::update_alias_table, world.rs:1959-1975
void skybox_update_alias(Skybox& s) {
    const uint32_t w = s.uniforms.width, h = s.uniforms.height;
    std::vector<double> weights((size_t)w * h);
    for (uint32_t y = 0; y < h; ++y) {
        const double rw = row_weight(y, h);
        for (uint32_t x = 0; x < w; ++x) {
            const float* p = &s.rgba[((size_t)y * w + x) * 4];
            weights[(size_t)y * w + x] = luminance(p[0], p[1], p[2]) * rw;
        }
    }
    s.alias = alias_table(weights.data(), weights.size());
}

// Skybox::update_total_luminous_flux, world.rs:1977-1987
void skybox_update_flux(Skybox& s, double radius_squared) {
    const double pi = 3.14159265358979323846;
    s.uniforms.total_luminous_flux =
        s.alias.empty()
            ? 0.0f
            : (float)std::min(4.0 * (pi * pi) * radius_squared * (double)s.uniforms.average_luminance,
                              (double)std::numeric_limits<float>::max());
}

// GpuSceneUniforms::update_light_probabilities, world.rs:484-498
void update_light_probabilities(pt_scene_uniforms& u, float sky_flux) {
    const float geometry = u.emissive_triangles_count > 0 ? u.total_luminous_flux : 0.0f;
    const float scale = std::fmax(geometry, sky_flux);
    if (scale > 0.0f) {
        const float g = geometry / scale, s = sky_flux / scale;
        u.light_probabilities[0] = g / (g + s);
        u.light_probabilities[1] = s / (g + s);
    } else {
        u.light_probabilities[0] = 0.0f;
        u.light_probabilities[1] = 0.0f;
    }
}

constexpr size_t kEditablePrefix = offsetof(pt_material, alpha_mode);  // world.rs:771

}  // namespace

struct ptw_world {
    std::string error;
    // scene inputs before the build
    std::vector<pt_triangle_geometry> in_geos;
    std::vector<pt_triangle_attribute> in_attrs;
    // built scene (BVH order)
    std::vector<pt_triangle_geometry> geos;
    std::vector<pt_triangle_attribute> attrs;
    std::vector<pt_material> materials;
    std::vector<pt_bvh_node> nodes;
    std::vector<uint32_t> order;
    std::vector<std::vector<uint8_t>> srgb_layers, linear_layers;
    std::vector<uint8_t> srgb_flat, linear_flat;
    bool built = false;
    uint32_t depth = 0;
    Camera camera;
    Skybox skybox;
    pt_scene_uniforms scene_uniforms{};
    std::vector<pt_scene_alias_entry> scene_alias;
    // pending changes (PendingChanges, world.rs:63-71)
    bool full_upload = false;
    bool pending_skybox = false;
    Skybox next_skybox;
    bool pending_camera = false;
    Camera next_camera;
    bool pending_luminance = false;
    float next_luminance = 0.0f;
    std::map<uint32_t, pt_material> pending_materials;
    std::vector<float> initial_strength;  // emission strength of every material when built
    float emission_scale = 1.0f;
    bool taken_once = false;
    // storage behind the pointers returned by take_updates
    pt_scene_upload scene_upload{};
    pt_skybox_upload skybox_upload{};
    pt_camera camera_upload{};
    std::vector<pt_material_update> material_updates;
    pt_scene_uniforms scene_uniforms_upload{};
    pt_skybox_uniforms skybox_uniforms_upload{};
    pt_scene_alias_entry empty_alias{};  // non-NULL marker for "changed, now empty"

    int fail(int code, const std::string& msg) {
        error = msg;
        return code;
    }
};

namespace {

// Scene::uniforms_and_alias_table, world.rs:1691-1735
void scene_uniforms_and_alias(ptw_world* w) {
    std::vector<uint32_t> indices;
    std::vector<double> weights;
    for (size_t i = 0; i < w->geos.size(); ++i) {
        const pt_material& m = w->materials[w->attrs[i].material_index];
        const double emission = luminance(m.emission_color_and_luminance[0], m.emission_color_and_luminance[1],
                                          m.emission_color_and_luminance[2]) *
                                (double)std::fmax(m.emission_color_and_luminance[3], 0.0f) *
                                (double)std::fmax(m.emission_weight, 0.0f);
        if (emission == 0.0) continue;
        const auto& g = w->geos[i];
        const DVec3 a = dv(v3(g.v0[0], g.v0[1], g.v0[2]));
        const DVec3 b = dv(v3(g.v1[0], g.v1[1], g.v1[2]));
        const DVec3 c = dv(v3(g.v2[0], g.v2[1], g.v2[2]));
        const DVec3 cr = dcross(b - a, c - a);
        const double area = std::sqrt(ddot(cr, cr)) * 0.5;
        const double flux = 6.28318530717958647692 * area * emission;
        if (flux > 0.0 && std::isfinite(flux)) {
            indices.push_back((uint32_t)i);
            weights.push_back(flux);
        }
    }
    double total = 0.0;
    for (double x : weights) total += x;
    w->scene_uniforms.total_luminous_flux = (float)std::min(total, (double)std::numeric_limits<float>::max());
    w->scene_uniforms.emissive_triangles_count = (uint32_t)indices.size();
    w->scene_uniforms.light_probabilities[0] = 0.0f;
    w->scene_uniforms.light_probabilities[1] = 0.0f;
    auto table = alias_table(weights.data(), weights.size());
    w->scene_alias.resize(table.size());
    for (size_t i = 0; i < table.size(); ++i) {
        w->scene_alias[i].threshold = table[i].threshold;
        w->scene_alias[i].alias_index = table[i].alias_index;
        w->scene_alias[i].triangle_index = indices[i];
        w->scene_alias[i].selection_probability = table[i].selection_probability;
    }
}

double radius_squared(const ptw_world* w) {
    const pt_bvh_node& r = w->nodes[0];
    const double dx = (double)r.aabb_max[0] - (double)r.aabb_min[0];
    const double dy = (double)r.aabb_max[1] - (double)r.aabb_min[1];
    const double dz = (double)r.aabb_max[2] - (double)r.aabb_min[2];
    return (dx * dx + dy * dy + dz * dz) * 0.25;
}

Vec3 tri_normal(Vec3 a, Vec3 b, Vec3 c) { return normalize(cross(b - a, c - a)); }

}  // namespace

extern "C" {

int ptw_create(ptw_world** out) try {
    if (!out) return PT_ERR_INVALID_ARG;
    *out = new ptw_world();
    return PT_OK;
} catch (...) {
    return pt_abi_current_status(nullptr);
}

void ptw_destroy(ptw_world* w) { delete w; }

const char* ptw_last_error(const ptw_world* w) { return w ? w->error.c_str() : "null world"; }

void ptw_default_material(pt_material* m) {
    if (!m) return;
    std::memset(m, 0, sizeof(*m));
    for (int i = 0; i < 4; ++i) m->base_color[i] = 1.0f;
    m->base_weight = 1.0f;
    m->base_metalness = 1.0f;
    m->base_diffuse_roughness = 1.0f;
    m->emission_weight = 1.0f;
    m->emission_color_and_luminance[3] = 1.0f;
    for (int i = 0; i < 4; ++i) m->specular_color_and_weight[i] = 1.0f;
    m->specular_roughness = 0.3f;
    m->specular_roughness_anisotropy = 0.0f;
    m->specular_haze = 0.0f;
    m->specular_haze_spread = 0.3f;
    m->specular_ior = 1.5f;
    m->specular_retroreflectivity = 0.0f;
    m->normal_scale = 1.0f;
    m->alpha_mode = PT_ALPHA_MODE_OPAQUE;
    m->alpha_cutoff = 0.5f;
    m->base_color_tex_layer = -1;
    m->normal_tex_layer = -1;
    m->metallic_roughness_tex_layer = -1;
    m->emission_tex_layer = -1;
    m->specular_color_tex_layer = -1;
    m->specular_weight_tex_layer = -1;
}

int ptw_add_material(ptw_world* w, const pt_material* m, uint32_t* index) try {
    if (!w || !m) return PT_ERR_INVALID_ARG;
    if (w->built) return w->fail(PT_ERR_STATE, "materials must be added before ptw_build");
    if (index) *index = (uint32_t)w->materials.size();
    w->materials.push_back(*m);
    return PT_OK;
} catch (...) {
    return pt_abi_status(w);
}

int ptw_add_atlas_layer(ptw_world* w, int srgb, const uint8_t* rgba8, int32_t* layer) try {
    if (!w || !rgba8) return PT_ERR_INVALID_ARG;
    if (w->built) return w->fail(PT_ERR_STATE, "atlas layers must be added before ptw_build");
    auto& layers = srgb ? w->srgb_layers : w->linear_layers;
    const size_t bytes = (size_t)PT_ATLAS_SIZE * PT_ATLAS_SIZE * 4;
    layers.emplace_back(rgba8, rgba8 + bytes);
    if (layer) *layer = (int32_t)layers.size() - 1;
    return PT_OK;
} catch (...) {
    return pt_abi_status(w);
}

// triangle intake, world.rs:1152-1331
int ptw_add_mesh(ptw_world* w, const ptw_mesh* mesh) try {
    if (!w || !mesh || !mesh->positions) return PT_ERR_INVALID_ARG;
    if (w->built) return w->fail(PT_ERR_STATE, "meshes must be added before ptw_build");
    if (mesh->material_index >= w->materials.size())
        return w->fail(PT_ERR_INVALID_ARG, "mesh material index out of range");
    const uint32_t nv = mesh->vertex_count;
    std::vector<uint32_t> idx;
    if (mesh->indices) {
        if (mesh->index_count % 3 != 0) return w->fail(PT_ERR_INVALID_ARG, "index count not a multiple of 3");
        idx.assign(mesh->indices, mesh->indices + mesh->index_count);
        for (uint32_t i : idx)
            if (i >= nv) return w->fail(PT_ERR_INVALID_ARG, "mesh index out of range");
    } else {
        if (nv % 3 != 0) return w->fail(PT_ERR_INVALID_ARG, "vertex count not a multiple of 3");
        idx.resize(nv);
        for (uint32_t i = 0; i < nv; ++i) idx[i] = i;
    }
    auto P = [&](uint32_t i) { return v3(mesh->positions[3 * i], mesh->positions[3 * i + 1], mesh->positions[3 * i + 2]); };
    std::vector<Vec3> normals(nv);
    bool computed_tangents = mesh->tangents == nullptr || mesh->normals == nullptr;
    if (mesh->normals) {
        // normals are normalised after the (here identity) transform, world.rs:1182-1187
        for (uint32_t i = 0; i < nv; ++i)
            normals[i] = normalize(v3(mesh->normals[3 * i], mesh->normals[3 * i + 1], mesh->normals[3 * i + 2]));
        if (mesh->tangents) {
            // placeholder tangents and mixed handedness fall back to computed tangents, world.rs:1188-1217
            for (uint32_t i = 0; i < nv && !computed_tangents; ++i) {
                const float* t = mesh->tangents + 4 * i;
                if (t[0] == 1.0f && t[1] == 0.0f && t[2] == 0.0f && t[3] == 1.0f) computed_tangents = true;
            }
            for (size_t t = 0; t + 2 < idx.size() && !computed_tangents; t += 3) {
                const float w0 = mesh->tangents[4 * idx[t] + 3], w1 = mesh->tangents[4 * idx[t + 1] + 3],
                            w2 = mesh->tangents[4 * idx[t + 2] + 3];
                if (w0 != w1 || w0 != w2) computed_tangents = true;
            }
        }
    } else {
        // flat normals, later triangles overwrite shared vertices (world.rs:1224-1234)
        for (size_t t = 0; t + 2 < idx.size(); t += 3) {
            const Vec3 n = tri_normal(P(idx[t]), P(idx[t + 1]), P(idx[t + 2]));
            normals[idx[t]] = n;
            normals[idx[t + 1]] = n;
            normals[idx[t + 2]] = n;
        }
    }
    static const float dummy_uv[3][2] = {{0, 0}, {1, 0}, {0, 1}};
    auto UV = [&](uint32_t i, int c) {
        return mesh->uvs ? mesh->uvs[2 * i + c] : dummy_uv[i % 3][c];
    };
    // MikkTSpace frames per corner where the mesh has no usable tangents (world.rs:1238-1260)
    std::vector<float> mikk;
    if (computed_tangents) {
        const size_t tris = idx.size() / 3;
        std::vector<float> cp(tris * 9), cn(tris * 9), cu(tris * 6);
        for (size_t c = 0; c < idx.size(); ++c) {
            const uint32_t v = idx[c];
            for (int k = 0; k < 3; ++k) cp[3 * c + k] = mesh->positions[3 * v + k];
            cn[3 * c] = normals[v].x;
            cn[3 * c + 1] = normals[v].y;
            cn[3 * c + 2] = normals[v].z;
            cu[2 * c] = UV(v, 0);
            cu[2 * c + 1] = UV(v, 1);
        }
        mikk.resize(tris * 12);
        ptw::mikktspace_tangents(tris, cp.data(), cn.data(), cu.data(), mikk.data());
    }
    for (size_t t = 0; t + 2 < idx.size(); t += 3) {
        const uint32_t i0 = idx[t], i1 = idx[t + 1], i2 = idx[t + 2];
        const Vec3 a = P(i0), b = P(i1), c = P(i2);
        pt_triangle_geometry g;
        g.v0[0] = a.x; g.v0[1] = a.y; g.v0[2] = a.z;
        g.v1[0] = b.x; g.v1[1] = b.y; g.v1[2] = b.z;
        g.v2[0] = c.x; g.v2[1] = c.y; g.v2[2] = c.z;
        pt_triangle_attribute at;
        std::memset(&at, 0, sizeof(at));
        at.material_index = mesh->material_index;
        const uint32_t vi[3] = {i0, i1, i2};
        float* ns[3] = {at.n0, at.n1, at.n2};
        float* uvs[3] = {at.uv0, at.uv1, at.uv2};
        float* ts[3] = {at.t0, at.t1, at.t2};
        for (int k = 0; k < 3; ++k) {
            ns[k][0] = normals[vi[k]].x;
            ns[k][1] = normals[vi[k]].y;
            ns[k][2] = normals[vi[k]].z;
            uvs[k][0] = UV(vi[k], 0);
            uvs[k][1] = UV(vi[k], 1);
        }
        if (!computed_tangents) {
            for (int k = 0; k < 3; ++k) {
                const float* src = mesh->tangents + 4 * vi[k];
                const Vec3 tn = normalize(v3(src[0], src[1], src[2]));
                ts[k][0] = tn.x;
                ts[k][1] = tn.y;
                ts[k][2] = tn.z;
                ts[k][3] = src[3];
            }
        } else {
            // the handedness is negated after MikkTSpace, world.rs:1252-1259
            for (int k = 0; k < 3; ++k) {
                const float* m = &mikk[4 * (t + (size_t)k)];
                ts[k][0] = m[0];
                ts[k][1] = m[1];
                ts[k][2] = m[2];
                ts[k][3] = -m[3];
            }
        }
        w->in_geos.push_back(g);
        w->in_attrs.push_back(at);
    }
    return PT_OK;
} catch (...) {
    return pt_abi_status(w);
}

int ptw_build(ptw_world* w) try {
    if (!w) return PT_ERR_INVALID_ARG;
    if (w->built) return w->fail(PT_ERR_STATE, "world already built");
    if (w->in_geos.empty()) return w->fail(PT_ERR_INVALID_ARG, "scene has no triangles");
    if (w->in_geos.size() > 0xffffffffull / 2) return w->fail(PT_ERR_OUT_OF_LIMITS, "too many triangles");
    build_bvh(w->in_geos, w->nodes, w->order);
    w->geos.resize(w->in_geos.size());
    w->attrs.resize(w->in_attrs.size());
    for (size_t i = 0; i < w->order.size(); ++i) {
        w->geos[i] = w->in_geos[w->order[i]];
        w->attrs[i] = w->in_attrs[w->order[i]];
    }
    std::vector<pt_triangle_geometry>().swap(w->in_geos);
    std::vector<pt_triangle_attribute>().swap(w->in_attrs);
    const pt_bvh_node& r = w->nodes[0];
    Camera cam = auto_camera(v3(r.aabb_min[0], r.aabb_min[1], r.aabb_min[2]),
                             v3(r.aabb_max[0], r.aabb_max[1], r.aabb_max[2]));
    cam.aspect_ratio = w->camera.aspect_ratio;
    w->camera = cam;
    w->depth = bvh_depth(w->nodes);
    // the reference keeps at least one (zeroed) atlas per kind (world.rs:931-934)
    const size_t layer_bytes = (size_t)PT_ATLAS_SIZE * PT_ATLAS_SIZE * 4;
    w->srgb_flat.clear();
    for (auto& l : w->srgb_layers) w->srgb_flat.insert(w->srgb_flat.end(), l.begin(), l.end());
    w->linear_flat.clear();
    for (auto& l : w->linear_layers) w->linear_flat.insert(w->linear_flat.end(), l.begin(), l.end());
    (void)layer_bytes;
    w->initial_strength.resize(w->materials.size());
    for (size_t i = 0; i < w->materials.size(); ++i) w->initial_strength[i] = w->materials[i].emission_color_and_luminance[3];
    w->built = true;
    w->full_upload = true;
    return PT_OK;
} catch (...) {
    return pt_abi_status(w);
}

int ptw_set_skybox_rgba(ptw_world* w, const float* rgba, uint32_t width, uint32_t height) try {
    if (!w || !rgba || width == 0 || height == 0) return PT_ERR_INVALID_ARG;
    Skybox s = make_skybox(rgba, width, height);
    if (!w->taken_once) {
        w->skybox = std::move(s);  // World::new
    } else {
        // World::replace_skybox, world.rs:635-643
        s.uniforms.average_luminance = w->pending_luminance ? w->next_luminance : w->skybox.uniforms.average_luminance;
        w->next_skybox = std::move(s);
        w->pending_skybox = true;
    }
    return PT_OK;
} catch (...) {
    return pt_abi_status(w);
}

int ptw_edit_skybox_average_luminance(ptw_world* w, float luminance) try {
    if (!w) return PT_ERR_INVALID_ARG;
    w->pending_luminance = true;
    w->next_luminance = std::fmax(luminance, 0.0f);
    return PT_OK;
} catch (...) {
    return pt_abi_status(w);
}

int ptw_set_aspect_ratio(ptw_world* w, float aspect) try {
    if (!w) return PT_ERR_INVALID_ARG;
    if (!(std::isfinite(aspect) && aspect > 0.0f))
        return w->fail(PT_ERR_INVALID_ARG, "Aspect ratio must be finite and positive.");
    if (!w->taken_once) w->camera.aspect_ratio = aspect;  // World::new resizes the scene camera
    if (w->taken_once || w->pending_camera) {
        if (!w->pending_camera) {
            w->next_camera = w->camera;
            w->pending_camera = true;
        }
        w->next_camera.aspect_ratio = aspect;
    }
    return PT_OK;
} catch (...) {
    return pt_abi_status(w);
}

int ptw_edit_camera(ptw_world* w, const float* position, const float* yaw, const float* pitch, const float* fov) try {
    if (!w) return PT_ERR_INVALID_ARG;
    if (!w->pending_camera) {
        w->next_camera = w->camera;
        w->pending_camera = true;
    }
    Camera& c = w->next_camera;
    if (position) c.position = v3(position[0], position[1], position[2]);
    if (yaw) c.yaw = *yaw;
    const float half_pi = 1.57079632679489661923f;
    if (pitch) c.pitch = std::fmin(std::fmax(*pitch, -half_pi), half_pi);
    else c.pitch = std::fmin(std::fmax(c.pitch, -half_pi), half_pi);
    if (fov) c.fov = std::fmin(std::fmax(*fov, 0.0f), 3.14159265358979323846f - std::numeric_limits<float>::epsilon());
    return PT_OK;
} catch (...) {
    return pt_abi_status(w);
}

int ptw_edit_material(ptw_world* w, uint32_t index, const pt_material* m) try {
    if (!w || !m) return PT_ERR_INVALID_ARG;
    if (index >= w->materials.size()) return w->fail(PT_ERR_INVALID_ARG, "material index out of range");
    const float* f = reinterpret_cast<const float*>(m);
    for (size_t i = 0; i < kEditablePrefix / 4; ++i)
        if (!std::isfinite(f[i])) return w->fail(PT_ERR_INVALID_ARG, "material values must be finite");
    auto it = w->pending_materials.find(index);
    pt_material accepted = it != w->pending_materials.end() ? it->second : w->materials[index];
    std::memcpy(&accepted, m, kEditablePrefix);
    if (std::memcmp(&accepted, &w->materials[index], sizeof(pt_material)) == 0)
        w->pending_materials.erase(index);
    else
        w->pending_materials[index] = accepted;
    return PT_OK;
} catch (...) {
    return pt_abi_status(w);
}

// World::edit_emission_scale, world.rs:655-692: every emissive material
// (emission colour luminance times emission weight above 0) gets its initial
// emission strength times `scale`, replacing edits of that value
int ptw_edit_emission_scale(ptw_world* w, float scale) try {
    if (!w) return PT_ERR_INVALID_ARG;
    if (!w->built) return w->fail(PT_ERR_STATE, "ptw_build has not run");
    if (std::isnan(scale)) return w->fail(PT_ERR_INVALID_ARG, "scale must not be NaN");
    scale = std::max(scale, 0.0f);
    w->emission_scale = scale;
    for (uint32_t i = 0; i < (uint32_t)w->materials.size(); ++i) {
        auto it = w->pending_materials.find(i);
        pt_material edited = it != w->pending_materials.end() ? it->second : w->materials[i];
        const float* e = edited.emission_color_and_luminance;
        if (luminance(e[0], e[1], e[2]) * (double)edited.emission_weight <= 0.0) continue;
        edited.emission_color_and_luminance[3] = w->initial_strength[i] * scale;
        if (std::memcmp(&edited, &w->materials[i], sizeof(pt_material)) == 0)
            w->pending_materials.erase(i);
        else
            w->pending_materials[i] = edited;
    }
    return PT_OK;
} catch (...) {
    return pt_abi_status(w);
}

float ptw_emission_scale(const ptw_world* w) { return w ? w->emission_scale : 0.0f; }

// World::take_updates, world.rs:790-884
int ptw_take_updates(ptw_world* w, pt_world_updates* out) try {
    if (!w || !out) return PT_ERR_INVALID_ARG;
    if (!w->built) return w->fail(PT_ERR_STATE, "ptw_build has not run");
    std::memset(out, 0, sizeof(*out));
    const bool scene_replaced = w->full_upload;
    const bool skybox_replaced = w->pending_skybox || w->full_upload;
    if (w->pending_skybox) w->skybox = std::move(w->next_skybox);
    bool camera_changed = scene_replaced;
    if (w->pending_camera) {
        camera_changed |= !(w->next_camera == w->camera);
        w->camera = w->next_camera;
    }
    bool luminance_changed = skybox_replaced;
    if (w->pending_luminance) {
        luminance_changed |= w->next_luminance != w->skybox.uniforms.average_luminance;
        w->skybox.uniforms.average_luminance = w->next_luminance;
    }
    bool lighting_changed = scene_replaced;
    w->material_updates.clear();
    for (auto& [index, mat] : w->pending_materials) {
        pt_material& old = w->materials[index];
        lighting_changed |= old.emission_weight != mat.emission_weight ||
                            std::memcmp(old.emission_color_and_luminance, mat.emission_color_and_luminance, 16) != 0;
        old = mat;
        if (!scene_replaced) {
            pt_material_update u;
            u.index = index;
            u.material = mat;
            w->material_updates.push_back(u);
        }
    }
    if (lighting_changed) scene_uniforms_and_alias(w);
    if (skybox_replaced) skybox_update_alias(w->skybox);
    const bool skybox_uniforms_changed = scene_replaced || luminance_changed;
    if (skybox_uniforms_changed) skybox_update_flux(w->skybox, radius_squared(w));
    const bool scene_uniforms_changed = lighting_changed || skybox_uniforms_changed;
    if (scene_uniforms_changed) update_light_probabilities(w->scene_uniforms, w->skybox.uniforms.total_luminous_flux);
    const bool reset = scene_replaced || skybox_replaced || camera_changed || luminance_changed ||
                       !w->material_updates.empty();

    if (scene_replaced) {
        w->scene_upload.geometries = w->geos.data();
        w->scene_upload.attributes = w->attrs.data();
        w->scene_upload.triangle_count = w->geos.size();
        w->scene_upload.materials = w->materials.data();
        w->scene_upload.material_count = w->materials.size();
        w->scene_upload.bvh_nodes = w->nodes.data();
        w->scene_upload.node_count = w->nodes.size();
        w->scene_upload.srgb_texture_atlases = w->srgb_flat.empty() ? nullptr : w->srgb_flat.data();
        w->scene_upload.srgb_atlas_count = (uint32_t)w->srgb_layers.size();
        w->scene_upload.linear_texture_atlases = w->linear_flat.empty() ? nullptr : w->linear_flat.data();
        w->scene_upload.linear_atlas_count = (uint32_t)w->linear_layers.size();
        out->scene = &w->scene_upload;
    }
    if (skybox_replaced) {
        w->skybox_upload.rgba = w->skybox.rgba.data();
        w->skybox_upload.uniforms = w->skybox.uniforms;
        w->skybox_upload.alias_table = w->skybox.alias.empty() ? nullptr : w->skybox.alias.data();
        w->skybox_upload.alias_count = w->skybox.alias.size();
        out->skybox = &w->skybox_upload;
    }
    if (camera_changed) {
        w->camera_upload = gpu_camera(w->camera);
        out->camera = &w->camera_upload;
    }
    out->materials = w->material_updates.empty() ? nullptr : w->material_updates.data();
    out->material_update_count = w->material_updates.size();
    if (scene_uniforms_changed) {
        w->scene_uniforms_upload = w->scene_uniforms;
        out->scene_uniforms = &w->scene_uniforms_upload;
    }
    if (lighting_changed) {
        out->scene_alias_table = w->scene_alias.empty() ? &w->empty_alias : w->scene_alias.data();
        out->scene_alias_count = w->scene_alias.size();
    }
    if (skybox_uniforms_changed) {
        w->skybox_uniforms_upload = w->skybox.uniforms;
        out->skybox_uniforms = &w->skybox_uniforms_upload;
    }
    out->reset_accumulation = reset ? 1 : 0;

    w->full_upload = false;
    w->pending_skybox = false;
    w->pending_camera = false;
    w->pending_luminance = false;
    w->pending_materials.clear();
    w->taken_once = true;
    return PT_OK;
} catch (...) {
    return pt_abi_status(w);
}

uint64_t ptw_triangle_count(const ptw_world* w) { return w ? w->geos.size() : 0; }
uint64_t ptw_node_count(const ptw_world* w) { return w ? w->nodes.size() : 0; }
uint64_t ptw_material_count(const ptw_world* w) { return w ? w->materials.size() : 0; }
const pt_triangle_geometry* ptw_geometries(const ptw_world* w) { return w ? w->geos.data() : nullptr; }
const pt_triangle_attribute* ptw_attributes(const ptw_world* w) { return w ? w->attrs.data() : nullptr; }
const pt_bvh_node* ptw_bvh_nodes(const ptw_world* w) { return w ? w->nodes.data() : nullptr; }
const pt_material* ptw_materials(const ptw_world* w) { return w ? w->materials.data() : nullptr; }
const uint32_t* ptw_bvh_order(const ptw_world* w) { return w ? w->order.data() : nullptr; }
uint32_t ptw_bvh_max_depth(const ptw_world* w) { return w ? w->depth : 0; }

uint64_t ptw_alias_table(const double* weights, uint64_t count, pt_skybox_alias_entry* out) try {
    if (!weights || !out) return 0;
    auto t = alias_table(weights, (size_t)count);
    std::copy(t.begin(), t.end(), out);
    return t.size();
} catch (...) {
    return 0;  // an allocation failed: nothing produced
}

uint64_t ptw_build_bvh(const pt_triangle_geometry* triangles, uint64_t count, pt_bvh_node* nodes_out,
                       uint32_t* order_out) try {
    if (!triangles || count == 0 || !nodes_out || !order_out) return 0;
    std::vector<pt_triangle_geometry> g(triangles, triangles + count);
    std::vector<pt_bvh_node> nodes;
    std::vector<uint32_t> order;
    build_bvh(g, nodes, order);
    std::copy(nodes.begin(), nodes.end(), nodes_out);
    std::copy(order.begin(), order.end(), order_out);
    return nodes.size();
} catch (...) {
    return 0;  // an allocation failed: nothing produced
}

}  // extern "C"
