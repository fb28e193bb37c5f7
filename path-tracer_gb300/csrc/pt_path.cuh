// pt_path.cuh - traversal and per-bounce shading of one path, restating the
// body of compute_main (trace.slang:721-1297) in pieces that both the plain
// kernel (one thread runs a whole path) and the wavefront kernels (one
// kernel per stage) call.
#pragma once

#include "pt_device.cuh"

namespace ptd {

struct Node {
    float bmin[3];
    uint32_t left_first;
    float bmax[3];
    uint32_t tri_count;
};

PTD Node load_node(const World& w, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(w.nodes + i);
    const float4 a = __ldg(p), b = __ldg(p + 1);
    Node n;
    n.bmin[0] = a.x;
    n.bmin[1] = a.y;
    n.bmin[2] = a.z;
    n.left_first = __float_as_uint(a.w);
    n.bmax[0] = b.x;
    n.bmax[1] = b.y;
    n.bmax[2] = b.z;
    n.tri_count = __float_as_uint(b.w);
    return n;
}

// closest-hit traversal, trace.slang:764-884 (64-entry deferred stack,
// nearer child first, ties to the right child)
template <bool kRec>
PTD void closest_hit(const World& w, f3 o, f3 d, f3 rcp, Rng<kRec>& rng, Counters* c, float& hit_t, int32_t& hit,
                     float& hv, float& hw) {
    Rec<kRec> rec{};
    if constexpr (kRec) {
        rec.c = c;
        c->extend_rays += 1;
    }
    const Shear s = make_shear(d, rcp);
    const f3 nod = -o * rcp;
    uint32_t stack[64];
    uint32_t node_index = 0u, sp = 0u;
    for (;;) {
        rec.visit(node_index);
        const Node n = load_node(w, node_index);
        if (n.tri_count > 0u) {
            rec.leaf();
            for (uint32_t i = 0; i < n.tri_count; ++i) {
                const uint32_t tri = n.left_first + i;
                rec.tri();
                float t, v, wb;
                if (!triangle_test(load_tri(w, tri), o, s, &t, &v, &wb)) continue;
                if (t > 0.0f && t < hit_t) {
                    if (w.any_alpha && passes_through(w, tri, v, wb, rng)) continue;
                    hit_t = t;
                    hit = (int32_t)tri;
                    hv = v;
                    hw = wb;
                }
            }
        } else {
            rec.interior();
            const uint32_t li = n.left_first, ri = n.left_first + 1u;
            const Node l = load_node(w, li), r = load_node(w, ri);
            const float dl = intersect_aabb(l.bmin, l.bmax, nod, rcp, hit_t);
            const float dr = intersect_aabb(r.bmin, r.bmax, nod, rcp, hit_t);
            const bool hl = dl >= 0.0f, hr = dr >= 0.0f;
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
}

// any-hit traversal, trace.slang:614-717
template <bool kRec>
PTD bool occluded(const World& w, f3 o, f3 d, float hit_t, int32_t light_tri, Rng<kRec>& rng, Counters* c) {
    Rec<kRec> rec{};
    if constexpr (kRec) {
        rec.c = c;
        rec.shadow = true;
        c->shadow_rays += 1;
    }
    const f3 rcp = 1.0f / d;
    const Shear s = make_shear(d, rcp);
    const f3 nod = -o * rcp;
    uint32_t stack[64];
    uint32_t node_index = 0u, sp = 0u;
    for (;;) {
        rec.visit(node_index);
        const Node n = load_node(w, node_index);
        if (n.tri_count > 0u) {
            rec.leaf();
            for (uint32_t i = 0; i < n.tri_count; ++i) {
                const uint32_t tri = n.left_first + i;
                if ((int32_t)tri == light_tri) continue;
                rec.tri();
                float t, v, wb;
                if (!triangle_test(load_tri(w, tri), o, s, &t, &v, &wb)) continue;
                if (t > 0.0f && t < hit_t && !(w.any_alpha && passes_through(w, tri, v, wb, rng))) return true;
            }
        } else {
            rec.interior();
            const uint32_t li = n.left_first, ri = n.left_first + 1u;
            const Node l = load_node(w, li), r = load_node(w, ri);
            const float dl = intersect_aabb(l.bmin, l.bmax, nod, rcp, hit_t);
            const float dr = intersect_aabb(r.bmin, r.bmax, nod, rcp, hit_t);
            const bool hl = dl >= 0.0f, hr = dr >= 0.0f;
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

// per-path state carried between bounces
struct PathState {
    f3 o, d;
    f3 throughput;
    f3 color;
    float prev_pdf;
};

// camera ray, trace.slang:736-748; returns the RNG state after the jitter draws
template <bool kRec>
PTD void camera_ray(const pt_camera& cam, uint32_t px, uint32_t py, uint32_t img_w, uint32_t img_h,
                    Rng<kRec>& rng, PathState& ps) {
    const float jx = rng();
    const float jy = rng();
    const f2 puv = {((float)px + jx) / (float)img_w, ((float)py + jy) / (float)img_h};
    ps.o = mk(cam.position[0], cam.position[1], cam.position[2]);
    const f3 llc = mk(cam.lower_left_corner_minus_position[0], cam.lower_left_corner_minus_position[1],
                      cam.lower_left_corner_minus_position[2]);
    const f3 hor = mk(cam.horizontal[0], cam.horizontal[1], cam.horizontal[2]);
    const f3 ver = mk(cam.vertical[0], cam.vertical[1], cam.vertical[2]);
    ps.d = normalize(llc + puv.x * hor + puv.y * ver);
    ps.throughput = mk(1.0f, 1.0f, 1.0f);
    ps.color = mk(0.0f, 0.0f, 0.0f);
    ps.prev_pdf = 0.0f;
}

template <bool kRec>
PTD void camera_ray(const World& w, uint32_t px, uint32_t py, uint32_t img_w, uint32_t img_h, Rng<kRec>& rng,
                    PathState& ps) {
    camera_ray(w.camera, px, py, img_w, img_h, rng, ps);
}

// escaped ray, trace.slang:887-927
PTD void shade_miss(const World& w, uint32_t bounce, PathState& ps) {
    float mis = 1.0f;
    if (bounce > 0u) mis = power_heuristic(ps.prev_pdf, skybox_light_pdf(w, ps.d, w.scene.light_probabilities[1]));
    ps.color = ps.color + ps.throughput * evaluate_skybox(w, ps.d) * mis;
}

// a shadow ray produced by next-event estimation
struct ShadowRay {
    f3 o, d;
    float dist;
    int32_t light_tri;
    f3 contribution;  // added to the path's colour if the ray is unoccluded
    bool valid;
};

// Everything after a closest hit (trace.slang:929-1296): emission with MIS,
// shading frame, OpenPBR setup, next-event estimation, BSDF sampling,
// throughput, Russian roulette.  With kInlineShadow the shadow ray is traced
// here (required when some material is not opaque: its any-hit test draws
// random numbers before the BSDF sample does); otherwise it is returned in
// *shadow for a later shadow kernel.  Returns true if the path continues
// with ps.o / ps.d set to the next ray.
template <bool kRec, bool kInlineShadow>
PTD bool shade_hit(const World& w, uint32_t bounce, uint32_t max_bounces, PathState& ps, float hit_t, uint32_t h,
                   float hv, float hw, Rng<kRec>& rng, Counters* c, ShadowRay* shadow) {
    const float hu = 1.0f - hv - hw;
    const f2 iuv = interp_uv(w, h, hu, hv, hw);
    const pt_material& m = w.mat[attr_material(w, h)];
    f3 base_color = mk(m.base_color[0], m.base_color[1], m.base_color[2]);
    const float base_weight = m.base_weight;
    float base_metalness = m.base_metalness;
    float base_diffuse_roughness = m.base_diffuse_roughness;
    f3 specular_color = mk(m.specular_color_and_weight[0], m.specular_color_and_weight[1], m.specular_color_and_weight[2]);
    float specular_weight = m.specular_color_and_weight[3];
    if (m.base_color_tex_layer >= 0) {
        const float4 t = atlas(w, true, m.base_color_tex_layer, atlas_uv(iuv, m.base_color_uv));
        base_color = base_color * mk(t.x, t.y, t.z);
    }
    if (m.metallic_roughness_tex_layer >= 0) {
        const float4 t = atlas(w, false, m.metallic_roughness_tex_layer, atlas_uv(iuv, m.metallic_roughness_uv));
        base_metalness *= t.z;
        base_diffuse_roughness *= t.y;
    }
    if (m.specular_color_tex_layer >= 0) {
        const float4 t = atlas(w, true, m.specular_color_tex_layer, atlas_uv(iuv, m.specular_color_uv));
        specular_color = specular_color * mk(t.x, t.y, t.z);
    }
    if (m.specular_weight_tex_layer >= 0) {
        const float4 t = atlas(w, false, m.specular_weight_tex_layer, atlas_uv(iuv, m.specular_weight_uv));
        specular_weight *= t.w;
    }
    // emission with MIS, trace.slang:984-991
    const f3 emission = evaluate_emission(w, m, iuv);
    float emission_mis = 1.0f;
    if (bounce > 0u && w.scene.light_probabilities[0] > 0.0f && any_positive(emission)) {
        const float lpdf = triangle_light_pdf(w, h, ps.d, hit_t * hit_t,
                                              w.scene.light_probabilities[0] * triangle_selection_probability(w, h));
        emission_mis = power_heuristic(ps.prev_pdf, lpdf);
    }
    ps.color = ps.color + ps.throughput * emission * emission_mis;

    // shading frame, trace.slang:993-1091
    const f3 hit_point = ps.d * hit_t + ps.o;
    const f3 V = -ps.d;
    const Tri tri = load_hit_tri(w, h);
    const f3 flat_raw = normalize(cross(tri.v1 - tri.v0, tri.v2 - tri.v0));
    const float bfm = dot(V, flat_raw) > 0.0f ? 1.0f : -1.0f;
    const f3 flat_n = flat_raw * bfm;
    f3 n0, n1, n2;
    attr_normals(w, h, n0, n1, n2);
    f3 N = normalize(hu * n0 + hv * n1 + hw * n2) * bfm;
    f3 t0, t1, t2;
    float t0w;
    attr_tangents(w, h, t0, t1, t2, t0w);
    f3 Tn = orthonormal_tangent(hu * t0 + hv * t1 + hw * t2, N) * bfm;
    f3 Bn = cross(N, Tn) * t0w * bfm;
    bool n_changed = false;
    if (m.normal_tex_layer >= 0) {
        const float4 t = atlas(w, false, m.normal_tex_layer, atlas_uv(iuv, m.normal_uv));
        f3 ln = mk(t.x * 2.0f - 1.0f, t.y * 2.0f - 1.0f, t.z * 2.0f - 1.0f);
        ln = normalize(mk(ln.x * m.normal_scale, ln.y * m.normal_scale, ln.z));
        N = normalize(ln.x * Tn + ln.y * Bn + ln.z * N);
        n_changed = true;
    }
    const float flat_ndotv = dot(flat_n, V);
    const float threshold = 0.5f * flat_ndotv;
    float ndotv = dot(N, V);
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
    const f3 wo = mk(dot(Tn, V), dot(Bn, V), ndotv);
    b.opl = 1.0f + ggx_lambda(wo, b.alpha);
    const float r = base_diffuse_roughness;
    const float z = wo.z;
    b.la = 1.0f + r * (0.303392f + (-0.518982f + 0.111709f * z) * z + (-0.276266f + 0.335918f * z) * r);
    b.lb = r * (-1.16407f + 1.15859f * z + (0.150815f - 0.150105f * z) * r) / (z * z * z - 1.43545f);
    b.lc = 1.0f + r * (0.20013f + (-0.506373f + 0.261777f * z) * z);
    b.ld = r * (0.540852f + (-1.01625f + 0.475392f * z) * z) / (-1.0743f + (0.0725628f + z) * z);
    const float ls = wo.x * wo.x + wo.y * wo.y;
    f3 bx = mk(1.0f, 0.0f, 0.0f);
    if (ls > 0.0f) bx = mk(wo.x, wo.y, 0.0f) * rsqrt_(ls);
    b.bx = bx;
    b.by = mk(-bx.y, bx.x, 0.0f);
    b.e_dielectric = estimate_e_dielectric(wo, b.opl, b.alpha, b.ior_m, specular_color, rng);
    const f3 luma = mk(0.2126f, 0.7152f, 0.0722f);
    const float albedo_gloss = dot(b.e_dielectric, luma);
    const float albedo_diffuse = (1.0f - albedo_gloss) * base_weight * dot(base_color, luma);
    const f3 fsm = b.f0 + (1.0f - b.f0) * fifth_power(1.0f - wo.z);
    const float albedo_metal = dot(fsm, luma);
    const float w_ggx = mix(albedo_gloss, albedo_metal, base_metalness);
    const float w_diffuse = (1.0f - base_metalness) * albedo_diffuse;
    b.p_ggx = clampf(w_ggx / fmaxf(w_ggx + w_diffuse, 1e-7f), 0.1f, 0.9f);
    b.p_diffuse = 1.0f - b.p_ggx;
    b.p_u = ptm::powf_(r, 0.1f) * (0.162925f + (-0.372058f + (0.538233f - 0.290822f * z) * z) * z);
    b.p_c = 1.0f - b.p_u;
    b.base_color = base_color;
    b.base_weight = base_weight;
    b.base_metalness = base_metalness;
    b.base_diffuse_roughness = base_diffuse_roughness;
    b.specular_color = specular_color;
    b.specular_weight = specular_weight;

    // next-event estimation, trace.slang:1187-1206
    const f3 next_origin = hit_point + flat_n * fmaxf(1e-4f, 1e-4f * length(hit_point));
    const LightSample light = sample_light(w, next_origin, rng, c);
    const f3 lwi = mk(dot(Tn, light.direction), dot(Bn, light.direction), dot(N, light.direction));
    if constexpr (!kInlineShadow) shadow->valid = false;
#if PT_LOBE_TERMS
    const LobeTerms lt = lobe_terms(wo, b);
#endif
    if (light.pdf > 0.0f && lwi.z > 0.0f && any_positive(light.emission)) {
#if PT_LOBE_TERMS
        const Lobes lobes = evaluate_lobes_t(wo, lwi, b, lt);
#else
        const Lobes lobes = evaluate_lobes(wo, lwi, b);
#endif
        const float weight = bounce < max_bounces ? power_heuristic(light.pdf, lobes.pdf) : 1.0f;
        const f3 contribution = ps.throughput * lobes.f * lwi.z * light.emission * (weight / light.pdf);
        if constexpr (kInlineShadow) {
            if (!occluded(w, next_origin, light.direction, light.distance, light.triangle_index, rng, c))
                ps.color = ps.color + contribution;
        } else {
            shadow->o = next_origin;
            shadow->d = light.direction;
            shadow->dist = light.distance;
            shadow->light_tri = light.triangle_index;
            shadow->contribution = contribution;
            shadow->valid = true;
        }
    }
    if (bounce == max_bounces) return false;

    // BSDF sampling, trace.slang:1212-1260
    const float two_pi_r = kTwoPi * rng();
    const float r1 = rng();
    float sin_2pr, cos_2pr;  // every branch below uses both
#if PT_SHARED_SINCOS
    ptm::sincosf_(two_pi_r, &sin_2pr, &cos_2pr);
#else
    sin_2pr = ptm::sinf_(two_pi_r);
    cos_2pr = ptm::cosf_(two_pi_r);
#endif
    f3 wi;
    if (rng() < b.p_ggx) {
        wi = reflect(-wo, sample_vndf_sc(wo, b.alpha, r1, sin_2pr, cos_2pr));
    } else if (r1 < b.p_u) {
        const float u1 = r1 / b.p_u;
        const float sin_theta = sqrtf(1.0f - u1 * u1);
        wi = mk(sin_theta * cos_2pr, sin_theta * sin_2pr, u1);
    } else {
        const float u1 = (r1 - b.p_u) / b.p_c;
        const float R = sqrtf(u1);
        const float y = R * sin_2pr;
        const float s = fma_(0.5f, rsqrt_(fma_(b.ld, b.ld, 1.0f)), 0.5f);
        const float x = -mix(sqrtf(fma_(-y, y, 1.0f)), R * cos_2pr, s);
        const f3 wh = mk(x, y, sqrtf(fmaxf(1.0f - (x * x + y * y), 0.0f)));
        const f3 wu = mk(b.la * wh.x + b.lb * wh.z, b.lc * wh.y, b.ld * wh.x + wh.z);
        wi = normalize(wu.x * b.bx + wu.y * b.by + wu.z * mk(0.0f, 0.0f, 1.0f));
    }
    if (wi.z <= 0.0f) return false;
#if PT_LOBE_TERMS
    const Lobes lobes = evaluate_lobes_t(wo, wi, b, lt);
#else
    const Lobes lobes = evaluate_lobes(wo, wi, b);
#endif
    if (lobes.pdf <= 0.0f) return false;
    ps.throughput = ps.throughput * (lobes.f * wi.z / lobes.pdf);
    ps.prev_pdf = lobes.pdf;
    if (bounce > 3u) {
        const float p_survive = clampf(fmaxf(ps.throughput.x, fmaxf(ps.throughput.y, ps.throughput.z)), 0.05f, 0.95f);
        if (rng() > p_survive) return false;
        ps.throughput = ps.throughput / p_survive;
    }
    ps.o = next_origin;
    ps.d = wi.x * Tn + wi.y * Bn + wi.z * N;
    return true;
}

}  // namespace ptd
