// scenes.cpp - seeded procedural scenes fed to the world builder.
//
// The reference loads glTF files (world.rs:890-1337); the workloads of this
// project are synthetic, so they are generated here in memory with explicit
// normals, UVs and tangents (no MikkTSpace needed).  Generation uses only
// integer hashing, IEEE arithmetic and the deterministic functions of
// pt_fmath.h, so a seed produces the same bytes on every host.
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "pt_abi_guard.h"
#include "../../include/pt_world.h"
#include "pt_fmath.h"

namespace {

struct V3 {
    float x, y, z;
};
V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V3 normalize(V3 v) { return v * (1.0f / ptm::sqrt_(dot(v, v))); }

constexpr float kPi = 3.14159265358979323846f;

// splitmix64
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    float uniform() { return (float)(next() >> 40) * 0x1p-24f; }  // [0, 1)
    float range(float a, float b) { return a + (b - a) * uniform(); }
};

// a triangle mesh under construction
struct Mesh {
    std::vector<float> p, n, uv, t;
    std::vector<uint32_t> idx;
    uint32_t vertex(V3 pos, V3 nor, float u, float v, V3 tan, float w) {
        const uint32_t i = (uint32_t)(p.size() / 3);
        p.insert(p.end(), {pos.x, pos.y, pos.z});
        n.insert(n.end(), {nor.x, nor.y, nor.z});
        uv.insert(uv.end(), {u, v});
        t.insert(t.end(), {tan.x, tan.y, tan.z, w});
        return i;
    }
    void tri(uint32_t a, uint32_t b, uint32_t c) { idx.insert(idx.end(), {a, b, c}); }
    // planar quad a b c d (counter-clockwise seen from `nor`)
    void quad(V3 a, V3 b, V3 c, V3 d, V3 nor) {
        const V3 tan = normalize(b - a);
        const uint32_t i0 = vertex(a, nor, 0, 0, tan, 1.0f), i1 = vertex(b, nor, 1, 0, tan, 1.0f);
        const uint32_t i2 = vertex(c, nor, 1, 1, tan, 1.0f), i3 = vertex(d, nor, 0, 1, tan, 1.0f);
        tri(i0, i1, i2);
        tri(i0, i2, i3);
    }
    int add_to(ptw_world* w, uint32_t material) const {
        ptw_mesh m;
        m.positions = p.data();
        m.normals = n.data();
        m.uvs = uv.data();
        m.tangents = t.data();
        m.vertex_count = (uint32_t)(p.size() / 3);
        m.indices = idx.data();
        m.index_count = (uint32_t)idx.size();
        m.material_index = material;
        return ptw_add_mesh(w, &m);
    }
};

// box with half extents h, rotated by yaw about y then tilt about x, centred at c
void add_box(Mesh& m, V3 c, V3 h, float yaw, float tilt) {
    const float sy = ptm::sinf_(yaw), cy = ptm::cosf_(yaw);
    const float st = ptm::sinf_(tilt), ct = ptm::cosf_(tilt);
    auto rot = [&](V3 v) {
        // tilt about x, then yaw about y
        const V3 a{v.x, v.y * ct - v.z * st, v.y * st + v.z * ct};
        return V3{a.x * cy + a.z * sy, a.y, -a.x * sy + a.z * cy};
    };
    const V3 ax = rot({1, 0, 0}), ay = rot({0, 1, 0}), az = rot({0, 0, 1});
    auto corner = [&](float sx, float sy2, float sz) {
        return c + ax * (sx * h.x) + ay * (sy2 * h.y) + az * (sz * h.z);
    };
    const V3 p000 = corner(-1, -1, -1), p100 = corner(1, -1, -1), p110 = corner(1, 1, -1), p010 = corner(-1, 1, -1);
    const V3 p001 = corner(-1, -1, 1), p101 = corner(1, -1, 1), p111 = corner(1, 1, 1), p011 = corner(-1, 1, 1);
    m.quad(p001, p101, p111, p011, az);            // +z
    m.quad(p100, p000, p010, p110, az * -1.0f);    // -z
    m.quad(p101, p100, p110, p111, ax);            // +x
    m.quad(p000, p001, p011, p010, ax * -1.0f);    // -x
    m.quad(p011, p111, p110, p010, ay);            // +y
    m.quad(p000, p100, p101, p001, ay * -1.0f);    // -y
}

pt_material base_only(float r, float g, float b) {
    pt_material m;
    ptw_default_material(&m);
    m.base_color[0] = r;
    m.base_color[1] = g;
    m.base_color[2] = b;
    m.base_color[3] = 1.0f;
    m.base_metalness = 0.0f;
    m.base_diffuse_roughness = 0.0f;
    m.specular_color_and_weight[3] = 0.0f;  // base-only: specular weight 0
    return m;
}

// integer hash -> [0, 1)
float hash01(uint32_t x, uint32_t y, uint32_t z, uint64_t seed) {
    uint64_t h = seed ^ (0x9E3779B97F4A7C15ull * (x + 1)) ^ (0xC2B2AE3D27D4EB4Full * (y + 7)) ^
                 (0x165667B19E3779F9ull * (z + 13));
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
    h *= 0xc4ceb9fe1a85ec53ull;
    h ^= h >> 33;
    return (float)(h >> 40) * 0x1p-24f;
}

// 2D value noise with smoothstep interpolation
float value_noise(float x, float z, uint32_t octave, uint64_t seed) {
    const float fx0 = ptm::floor_(x), fz0 = ptm::floor_(z);
    const float fx = x - fx0, fz = z - fz0;
    const uint32_t ix = (uint32_t)(int32_t)fx0 + 0x40000000u, iz = (uint32_t)(int32_t)fz0 + 0x40000000u;
    const float a = hash01(ix, iz, octave, seed), b = hash01(ix + 1, iz, octave, seed);
    const float c = hash01(ix, iz + 1, octave, seed), d = hash01(ix + 1, iz + 1, octave, seed);
    const float sx = fx * fx * (3.0f - 2.0f * fx), sz = fz * fz * (3.0f - 2.0f * fz);
    const float ab = a + (b - a) * sx, cd = c + (d - c) * sx;
    return ab + (cd - ab) * sz;
}

struct Terrain {
    uint64_t seed;
    float amplitude = 4.0f, frequency = 0.125f;
    float height(float x, float z) const {
        float h = 0.0f, amp = amplitude, f = frequency;
        for (uint32_t o = 0; o < 4; ++o) {
            h += amp * value_noise(x * f, z * f, o, seed);
            amp *= 0.5f;
            f *= 2.0f;
        }
        return h;
    }
};

pt_material random_material(Rng& r) {
    pt_material m;
    ptw_default_material(&m);
    m.base_color[0] = r.uniform();
    m.base_color[1] = r.uniform();
    m.base_color[2] = r.uniform();
    m.base_color[3] = 1.0f;
    m.specular_roughness = r.range(0.05f, 1.0f);
    m.base_metalness = r.uniform() < 0.3f ? 1.0f : 0.0f;
    m.base_diffuse_roughness = r.uniform();
    return m;
}

// icosphere of subdivision `level` with smooth normals
void add_icosphere(Mesh& m, V3 c, float radius, uint32_t level) {
    const float t = (1.0f + ptm::sqrt_(5.0f)) * 0.5f;
    std::vector<V3> verts = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                             {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    for (auto& v : verts) v = normalize(v);
    std::vector<uint32_t> faces = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                                   11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                                   3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    for (uint32_t l = 0; l < level; ++l) {
        std::map<uint64_t, uint32_t> mid;
        auto midpoint = [&](uint32_t a, uint32_t b) {
            const uint64_t key = a < b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            verts.push_back(normalize((verts[a] + verts[b]) * 0.5f));
            const uint32_t i = (uint32_t)verts.size() - 1;
            mid[key] = i;
            return i;
        };
        std::vector<uint32_t> next;
        next.reserve(faces.size() * 4);
        for (size_t f = 0; f < faces.size(); f += 3) {
            const uint32_t a = faces[f], b = faces[f + 1], cc = faces[f + 2];
            const uint32_t ab = midpoint(a, b), bc = midpoint(b, cc), ca = midpoint(cc, a);
            next.insert(next.end(), {a, ab, ca, b, bc, ab, cc, ca, bc, ab, bc, ca});
        }
        faces.swap(next);
    }
    const uint32_t base = (uint32_t)(m.p.size() / 3);
    for (const V3& n : verts) {
        V3 tan = cross(V3{0, 1, 0}, n);
        tan = dot(tan, tan) > 1e-12f ? normalize(tan) : V3{1, 0, 0};
        const float u = 0.5f + ptm::atan2f_(n.z, n.x) * (0.5f / kPi);
        const float v = ptm::acosf_(std::fmax(-1.0f, std::fmin(1.0f, n.y))) * (1.0f / kPi);
        m.vertex(c + n * radius, n, u, v, tan, 1.0f);
    }
    for (size_t f = 0; f < faces.size(); f += 3) m.tri(base + faces[f], base + faces[f + 1], base + faces[f + 2]);
}

// Procedural RGBA8 textures: 1024 x 1024 each, 64 per 8192 x 8192 atlas
// layer in an 8 x 8 grid of slots.  Even kinds are checkers (8 x 8 squares
// of two seeded colours), odd kinds value noise (4 octaves, grey-tinted).
constexpr uint32_t kTexSize = 1024, kTexPerRow = PT_ATLAS_SIZE / kTexSize;
constexpr uint32_t kTexPerLayer = kTexPerRow * kTexPerRow;

struct TextureAtlas {
    std::vector<uint8_t> layer;  // allocated on first use
    uint32_t used = 0;
    uint64_t seed;

    // points the material's base colour at texture number `used` (the first
    // 64 are generated, later ones reuse them in turn)
    void texture(pt_material& m) {
        if (layer.empty()) layer.assign((size_t)PT_ATLAS_SIZE * PT_ATLAS_SIZE * 4, 0);
        const uint32_t slot = used % kTexPerLayer, kind = slot;
        const bool fresh = used < kTexPerLayer;
        used += 1;
        const uint32_t x0 = (slot % kTexPerRow) * kTexSize, y0 = (slot / kTexPerRow) * kTexSize;
        const float c0[3] = {hash01(kind, 0, 1, seed), hash01(kind, 0, 2, seed), hash01(kind, 0, 3, seed)};
        const float c1[3] = {hash01(kind, 1, 1, seed), hash01(kind, 1, 2, seed), hash01(kind, 1, 3, seed)};
        for (uint32_t y = 0; fresh && y < kTexSize; ++y) {
            uint8_t* row = layer.data() + ((size_t)(y0 + y) * PT_ATLAS_SIZE + x0) * 4;
            for (uint32_t x = 0; x < kTexSize; ++x) {
                float r, g, b;
                if (kind % 2 == 0) {
                    const bool odd = (((x >> 7) ^ (y >> 7)) & 1u) != 0;
                    r = odd ? c1[0] : c0[0];
                    g = odd ? c1[1] : c0[1];
                    b = odd ? c1[2] : c0[2];
                } else {
                    float n = 0.0f, amp = 0.5f, f = 1.0f / 64.0f;
                    for (uint32_t o = 0; o < 4; ++o) {
                        n += amp * value_noise((float)x * f, (float)y * f, 16 + o, seed ^ (uint64_t)kind * 0x9E37ull);
                        amp *= 0.5f;
                        f *= 2.0f;
                    }
                    r = 0.25f + 0.75f * n * (0.6f + 0.4f * c0[0]);
                    g = 0.25f + 0.75f * n * (0.6f + 0.4f * c0[1]);
                    b = 0.25f + 0.75f * n * (0.6f + 0.4f * c0[2]);
                }
                row[4 * x + 0] = (uint8_t)(r * 255.0f + 0.5f);
                row[4 * x + 1] = (uint8_t)(g * 255.0f + 0.5f);
                row[4 * x + 2] = (uint8_t)(b * 255.0f + 0.5f);
                row[4 * x + 3] = 255u;
            }
        }
        m.base_color_tex_layer = 0;
        m.base_color_uv[0] = (float)x0 / (float)PT_ATLAS_SIZE;
        m.base_color_uv[1] = (float)y0 / (float)PT_ATLAS_SIZE;
        m.base_color_uv[2] = (float)kTexSize / (float)PT_ATLAS_SIZE;
        m.base_color_uv[3] = (float)kTexSize / (float)PT_ATLAS_SIZE;
    }
    int add_to(ptw_world* w) const {
        if (layer.empty()) return PT_OK;
        int32_t index = 0;
        return ptw_add_atlas_layer(w, 1, layer.data(), &index);
    }
};

}  // namespace

extern "C" {

int ptw_scene_cornell_box(ptw_world** out) try {
    if (!out) return PT_ERR_INVALID_ARG;
    ptw_world* w = nullptr;
    ptw_create(&w);
    uint32_t white, red, green, light;
    pt_material m = base_only(0.73f, 0.73f, 0.73f);
    ptw_add_material(w, &m, &white);
    m = base_only(0.65f, 0.05f, 0.05f);
    ptw_add_material(w, &m, &red);
    m = base_only(0.12f, 0.45f, 0.15f);
    ptw_add_material(w, &m, &green);
    m = base_only(0.73f, 0.73f, 0.73f);
    m.emission_color_and_luminance[0] = 17.0f;
    m.emission_color_and_luminance[1] = 12.0f;
    m.emission_color_and_luminance[2] = 4.0f;
    m.emission_color_and_luminance[3] = 1.0f;
    m.emission_weight = 1.0f;
    ptw_add_material(w, &m, &light);

    Mesh walls, left, right, boxes, lamp;
    // unit room, open towards +z
    walls.quad({0, 0, 1}, {1, 0, 1}, {1, 0, 0}, {0, 0, 0}, {0, 1, 0});   // floor
    walls.quad({0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}, {0, -1, 0});  // ceiling
    walls.quad({0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1});   // back
    left.quad({0, 0, 0}, {0, 1, 0}, {0, 1, 1}, {0, 0, 1}, {1, 0, 0});
    right.quad({1, 0, 1}, {1, 1, 1}, {1, 1, 0}, {1, 0, 0}, {-1, 0, 0});
    // short box (0.3 tall) front right, tall box (0.6 tall) back left
    add_box(boxes, {0.66f, 0.15f, 0.64f}, {0.15f, 0.15f, 0.15f}, -0.30f, 0.0f);
    add_box(boxes, {0.34f, 0.30f, 0.36f}, {0.15f, 0.30f, 0.15f}, 0.29f, 0.0f);
    // 0.25 x 0.25 emissive quad just below the ceiling
    lamp.quad({0.375f, 0.999f, 0.375f}, {0.625f, 0.999f, 0.375f}, {0.625f, 0.999f, 0.625f},
              {0.375f, 0.999f, 0.625f}, {0, -1, 0});
    int rc = walls.add_to(w, white);
    if (!rc) rc = left.add_to(w, red);
    if (!rc) rc = right.add_to(w, green);
    if (!rc) rc = boxes.add_to(w, white);
    if (!rc) rc = lamp.add_to(w, light);
    if (!rc) rc = ptw_build(w);
    if (rc) {
        ptw_destroy(w);
        return rc;
    }
    *out = w;
    return PT_OK;
} catch (...) {
    return pt_abi_current_status(nullptr);
}

int ptw_scene_cornell_box_textured(uint64_t seed, ptw_world** out) try {
    if (!out) return PT_ERR_INVALID_ARG;
    ptw_world* w = nullptr;
    ptw_create(&w);
    TextureAtlas atlas;
    atlas.seed = seed;
    // eight meshes; floor, back wall, short box and tall box (4 of 8) textured
    const float colors[8][3] = {{0.73f, 0.73f, 0.73f}, {0.73f, 0.73f, 0.73f}, {0.73f, 0.73f, 0.73f},
                                {0.65f, 0.05f, 0.05f}, {0.12f, 0.45f, 0.15f}, {0.73f, 0.73f, 0.73f},
                                {0.73f, 0.73f, 0.73f}, {0.73f, 0.73f, 0.73f}};
    const bool textured[8] = {true, false, true, false, false, true, true, false};
    uint32_t mat[8];
    for (int i = 0; i < 8; ++i) {
        pt_material m = base_only(colors[i][0], colors[i][1], colors[i][2]);
        if (textured[i]) atlas.texture(m);
        if (i == 7) {
            m.emission_color_and_luminance[0] = 17.0f;
            m.emission_color_and_luminance[1] = 12.0f;
            m.emission_color_and_luminance[2] = 4.0f;
            m.emission_color_and_luminance[3] = 1.0f;
            m.emission_weight = 1.0f;
        }
        ptw_add_material(w, &m, &mat[i]);
    }
    Mesh floor_, ceiling, back, left, right, short_box, tall_box, lamp;
    floor_.quad({0, 0, 1}, {1, 0, 1}, {1, 0, 0}, {0, 0, 0}, {0, 1, 0});
    ceiling.quad({0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}, {0, -1, 0});
    back.quad({0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1});
    left.quad({0, 0, 0}, {0, 1, 0}, {0, 1, 1}, {0, 0, 1}, {1, 0, 0});
    right.quad({1, 0, 1}, {1, 1, 1}, {1, 1, 0}, {1, 0, 0}, {-1, 0, 0});
    add_box(short_box, {0.66f, 0.15f, 0.64f}, {0.15f, 0.15f, 0.15f}, -0.30f, 0.0f);
    add_box(tall_box, {0.34f, 0.30f, 0.36f}, {0.15f, 0.30f, 0.15f}, 0.29f, 0.0f);
    lamp.quad({0.375f, 0.999f, 0.375f}, {0.625f, 0.999f, 0.375f}, {0.625f, 0.999f, 0.625f},
              {0.375f, 0.999f, 0.625f}, {0, -1, 0});
    const Mesh* meshes[8] = {&floor_, &ceiling, &back, &left, &right, &short_box, &tall_box, &lamp};
    int rc = PT_OK;
    for (int i = 0; i < 8 && !rc; ++i) rc = meshes[i]->add_to(w, mat[i]);
    if (!rc) rc = atlas.add_to(w);
    if (!rc) rc = ptw_build(w);
    if (rc) {
        ptw_destroy(w);
        return rc;
    }
    *out = w;
    return PT_OK;
} catch (...) {
    return pt_abi_current_status(nullptr);
}

// sky: vertical gradient plus a Gaussian sun lobe, equirectangular, top row up
int ptw_set_procedural_skybox(ptw_world* w, uint32_t W, uint32_t H) try {
    if (!w || W == 0 || H == 0) return PT_ERR_INVALID_ARG;
    std::vector<float> px((size_t)W * H * 4);
    const V3 sun = normalize(V3{-0.45f, 0.64f, -0.62f});
    const float sigma2 = 0.0015f;
    for (uint32_t y = 0; y < H; ++y) {
        const float theta = ((float)y + 0.5f) / (float)H * kPi;
        const float st = ptm::sinf_(theta), ct = ptm::cosf_(theta);
        for (uint32_t x = 0; x < W; ++x) {
            const float phi = (((float)x + 0.5f) / (float)W - 0.5f) * (2.0f * kPi);
            const V3 d{st * ptm::cosf_(phi), ct, st * ptm::sinf_(phi)};
            float r, g, b;
            if (ct > 0.0f) {
                const float s = ptm::sqrt_(ct);
                r = 0.9f + (0.25f - 0.9f) * s;
                g = 0.85f + (0.45f - 0.85f) * s;
                b = 0.8f + (0.9f - 0.8f) * s;
            } else {
                const float s = 1.0f + ct;
                r = 0.25f * s;
                g = 0.22f * s;
                b = 0.2f * s;
            }
            const float sd = 1.0f - dot(d, sun);
            const float lobe = 2000.0f * ptm::exp2f_(-(sd / sigma2) * 1.44269504f);
            float* o = &px[((size_t)y * W + x) * 4];
            o[0] = r + lobe;
            o[1] = g + 0.95f * lobe;
            o[2] = b + 0.85f * lobe;
            o[3] = 1.0f;
        }
    }
    return ptw_set_skybox_rgba(w, px.data(), W, H);
} catch (...) {
    return pt_abi_current_status(nullptr);  // the world is opaque here: the status alone
}

void ptw_procedural_defaults(ptw_procedural_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->seed = 1;
    p->grid_x = 1024;
    p->grid_z = 512;
    p->boxes = 2000;
    p->spheres = 200;
    p->sphere_subdivision = 4;
    p->emissive_triangles = 64;
    p->skybox_width = 1024;
    p->skybox_height = 512;
    p->skybox_luminance = 1.0f;
    p->textured = 0;
    p->non_opaque = 0;
}

int ptw_scene_procedural(const ptw_procedural_params* params, ptw_world** out) try {
    if (!params || !out) return PT_ERR_INVALID_ARG;
    const ptw_procedural_params& P = *params;
    if (P.grid_x == 0 || P.grid_z == 0 || P.sphere_subdivision > 7) return PT_ERR_INVALID_ARG;
    ptw_world* w = nullptr;
    ptw_create(&w);
    Rng rng{P.seed * 0x2545F4914F6CDD1Dull + 0x1234567ull};
    // texture and alpha choices draw from their own stream, so the geometry
    // and materials of a seed do not depend on these options
    Rng look{P.seed * 0x9E3779B97F4A7C15ull + 0xABCDEFull};
    TextureAtlas atlas;
    atlas.seed = P.seed;
    const auto decorate = [&](pt_material& m, bool may_blend) {
        if (P.textured && look.uniform() < 0.5f) atlas.texture(m);
        if (P.non_opaque && may_blend && look.uniform() < 0.1f) {
            m.alpha_mode = PT_ALPHA_MODE_BLEND;
            m.base_color[3] = look.range(0.3f, 0.9f);
        }
    };
    const float ext_x = 64.0f, ext_z = 32.0f;
    Terrain terrain{P.seed};
    int rc = PT_OK;

    // heightfield
    {
        pt_material m = random_material(rng);
        decorate(m, false);
        uint32_t mi;
        ptw_add_material(w, &m, &mi);
        Mesh hf;
        const uint32_t nx = P.grid_x, nz = P.grid_z;
        const float dx = ext_x / (float)nx, dz = ext_z / (float)nz;
        hf.p.reserve((size_t)(nx + 1) * (nz + 1) * 3);
        for (uint32_t j = 0; j <= nz; ++j) {
            for (uint32_t i = 0; i <= nx; ++i) {
                const float x = -0.5f * ext_x + dx * (float)i, z = -0.5f * ext_z + dz * (float)j;
                const float y = terrain.height(x, z);
                const float hx = terrain.height(x + dx, z) - terrain.height(x - dx, z);
                const float hz = terrain.height(x, z + dz) - terrain.height(x, z - dz);
                const V3 n = normalize(V3{-hx, 2.0f * dx, -hz * (dx / dz)});
                const V3 t = normalize(V3{2.0f * dx, hx, 0.0f});
                hf.vertex({x, y, z}, n, (float)i / (float)nx, (float)j / (float)nz, t, 1.0f);
            }
        }
        for (uint32_t j = 0; j < nz; ++j) {
            for (uint32_t i = 0; i < nx; ++i) {
                const uint32_t a = j * (nx + 1) + i, b = a + 1, c = a + (nx + 1), d = c + 1;
                hf.tri(a, c, b);
                hf.tri(b, c, d);
            }
        }
        rc = hf.add_to(w, mi);
    }
    // boxes, one material each
    for (uint32_t k = 0; k < P.boxes && !rc; ++k) {
        pt_material m = random_material(rng);
        decorate(m, true);
        uint32_t mi;
        ptw_add_material(w, &m, &mi);
        const float x = rng.range(-0.47f * ext_x, 0.47f * ext_x), z = rng.range(-0.47f * ext_z, 0.47f * ext_z);
        const V3 h{rng.range(0.1f, 0.6f), rng.range(0.1f, 0.6f), rng.range(0.1f, 0.6f)};
        const float yaw = rng.range(0.0f, 2.0f * kPi), tilt = rng.range(-0.3f, 0.3f);
        Mesh b;
        add_box(b, {x, terrain.height(x, z) + 0.8f * h.y, z}, h, yaw, tilt);
        rc = b.add_to(w, mi);
    }
    // icospheres
    for (uint32_t k = 0; k < P.spheres && !rc; ++k) {
        pt_material m = random_material(rng);
        decorate(m, true);
        uint32_t mi;
        ptw_add_material(w, &m, &mi);
        const float x = rng.range(-0.45f * ext_x, 0.45f * ext_x), z = rng.range(-0.45f * ext_z, 0.45f * ext_z);
        const float r = rng.range(0.3f, 1.5f);
        const float y = terrain.height(x, z) + r * rng.range(0.5f, 2.5f);
        Mesh s;
        add_icosphere(s, {x, y, z}, r, P.sphere_subdivision);
        rc = s.add_to(w, mi);
    }
    // small emissive triangles, radiance log-uniform in [1, 100]
    for (uint32_t k = 0; k < P.emissive_triangles && !rc; ++k) {
        pt_material m = base_only(0.8f, 0.8f, 0.8f);
        const float radiance = ptm::exp2f_(rng.uniform() * 6.64385619f);  // 100^u
        m.emission_color_and_luminance[0] = 1.0f;
        m.emission_color_and_luminance[1] = 1.0f;
        m.emission_color_and_luminance[2] = 1.0f;
        m.emission_color_and_luminance[3] = radiance;
        uint32_t mi;
        ptw_add_material(w, &m, &mi);
        const float x = rng.range(-0.44f * ext_x, 0.44f * ext_x), z = rng.range(-0.44f * ext_z, 0.44f * ext_z);
        const V3 c{x, terrain.height(x, z) + rng.range(1.5f, 5.0f), z};
        const float cz = rng.range(-1.0f, 1.0f), phi = rng.range(0.0f, 2.0f * kPi);
        const float sz = ptm::sqrt_(std::fmax(0.0f, 1.0f - cz * cz));
        const V3 n{sz * ptm::cosf_(phi), cz, sz * ptm::sinf_(phi)};
        V3 t = cross(std::fabs(n.y) < 0.9f ? V3{0, 1, 0} : V3{1, 0, 0}, n);
        t = normalize(t);
        const V3 bt = cross(n, t);
        const float s = rng.range(0.4f, 1.0f);
        Mesh e;
        uint32_t vi[3];
        for (int q = 0; q < 3; ++q) {
            const float a = (2.0f * kPi / 3.0f) * (float)q;
            const V3 p = c + (t * ptm::cosf_(a) + bt * ptm::sinf_(a)) * s;
            vi[q] = e.vertex(p, n, q == 1 ? 1.0f : 0.0f, q == 2 ? 1.0f : 0.0f, t, 1.0f);
        }
        e.tri(vi[0], vi[1], vi[2]);
        rc = e.add_to(w, mi);
    }
    if (!rc) rc = atlas.add_to(w);
    if (!rc) rc = ptw_build(w);
    if (!rc && P.skybox_width > 0 && P.skybox_height > 0) {
        rc = ptw_set_procedural_skybox(w, P.skybox_width, P.skybox_height);
        if (!rc) rc = ptw_edit_skybox_average_luminance(w, P.skybox_luminance);
    }
    if (!rc) {
        // elevated camera looking down the terrain
        const float pos[3] = {0.0f, 14.0f, 20.0f};
        const float yaw = 0.0f, pitch = -0.45f, fov = 1.2f;
        rc = ptw_edit_camera(w, pos, &yaw, &pitch, &fov);
    }
    if (rc) {
        ptw_destroy(w);
        return rc;
    }
    *out = w;
    return PT_OK;
} catch (...) {
    return pt_abi_current_status(nullptr);
}

}  // extern "C"
