// pt_api.cu - the C ABI of include/pt.h: context, world upload, tile state,
// dispatch, readback.
//
// Host-side mirror of the reference's PathTracer (src/render/path_tracer.rs)
// and WorldResources (src/render/world_resources.rs).  Every upload is
// validated before it reaches the device (index ranges, an acyclic BVH no
// deeper than the 64-entry traversal stack, consistent light tables), so a
// malformed world is rejected with an error instead of faulting the GPU.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/pt.h"
#include "../../include/pt_precision.h"
#include "pt_abi_guard.h"
#include "pt_kernels.h"
#include "pt_wavefront.h"

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

constexpr uint32_t kMaxTileDim = 16384;

struct Timing {
    int cls;
    cudaEvent_t start, stop;
};

}  // namespace

struct pt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string error;

    // world (bind group 1)
    DevBuf geo, attr, mat, nodes, srgb, linear, sky, sky_alias, scene_alias, srgb_lut;
    DevBuf stage_geo, stage_attr, stage_mat, stage_nodes, stage_srgb, stage_linear;  // next scene upload
    uint64_t tri_count = 0, mat_count = 0, node_count = 0, sky_alias_count = 0, scene_alias_live = 0;
    uint32_t srgb_count = 0, linear_count = 0;
    pt_camera camera{};
    pt_scene_uniforms scene{};
    pt_skybox_uniforms sky_u{};
    std::vector<uint32_t> alpha_modes;
    bool world_ready = false;

    // tile (bind group 0)
    DevBuf accum, image, display, records, totals;
    DevBuf comp;  // Kahan compensation (PT_PRECISION_KAHAN)
    DevBuf fp64;  // FP64 reference render sums (pt_render_fp64)
    uint32_t tile_w = 0, tile_h = 0;
    pt_trace_parameters params{};
    int kernel = PT_KERNEL_WAVEFRONT;
    uint32_t precision = PT_PRECISION_FP32;         // requested form
    uint32_t precision_active = PT_PRECISION_FP32;  // form of the last trace
    ptw::Wavefront* wavefront = nullptr;

    // instrumentation
    bool profiling = false;
    std::vector<Timing> pending;
    std::vector<cudaEvent_t> event_pool;
    uint64_t class_launches[PT_KERNEL_CLASS_COUNT] = {0};
    double class_ms[PT_KERNEL_CLASS_COUNT] = {0};
    uint64_t launch_count = 0;

    int fail(int code, const std::string& msg) {
        error = msg;
        return code;
    }
    int cuda(cudaError_t e, const char* what) {
        if (e == cudaSuccess) return PT_OK;
        error = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA;
    }

    ptd::World view() const {
        ptd::World w;
        w.geo = geo.as<const pt_triangle_geometry>();
        w.attr = attr.as<const pt_triangle_attribute>();
        w.mat = mat.as<const pt_material>();
        w.nodes = nodes.as<const pt_bvh_node>();
        w.srgb = srgb.as<const uint8_t>();
        w.linear = linear.as<const uint8_t>();
        w.srgb_count = srgb_count;
        w.linear_count = linear_count;
        w.sky = sky.as<const float4>();
        w.sky_alias = sky_alias.as<const pt_skybox_alias_entry>();
        w.scene_alias = scene_alias.as<const pt_scene_alias_entry>();
        w.sky_u = sky_u;
        w.scene = scene;
        w.camera = camera;
        w.srgb_lut = srgb_lut.as<const float>();
        w.attr16 = 1;  // a device allocation
        int any = 0;
        for (uint32_t m : alpha_modes) any |= (m != PT_ALPHA_MODE_OPAQUE);
        w.any_alpha = any;
        return w;
    }

    cudaEvent_t take_event() {
        if (!event_pool.empty()) {
            cudaEvent_t e = event_pool.back();
            event_pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    // bracket one kernel launch (queued on stream s) with events when profiling
    template <class F>
    cudaError_t timed(int cls, cudaStream_t s, F&& launch) {
        launch_count += 1;
        if (!profiling) return launch();
        Timing t{cls, take_event(), take_event()};
        cudaEventRecord(t.start, s);
        cudaError_t e = launch();
        cudaEventRecord(t.stop, s);
        pending.push_back(t);
        return e;
    }
    template <class F>
    cudaError_t timed(int cls, F&& launch) {
        return timed(cls, stream, launch);
    }
    // Work queued on the context stream other than wavefront groups: the next
    // pt_trace's groups then wait for the stream instead of starting beside the
    // previous call's groups (ctx_ops counts such work).
    uint64_t ctx_ops = 0, ops_at_trace = ~0ull;
    void touched() { ctx_ops += 1; }
    void harvest() {
        for (Timing& t : pending) {
            cudaEventSynchronize(t.stop);
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, t.start, t.stop) == cudaSuccess) {
                class_launches[t.cls] += 1;
                class_ms[t.cls] += ms;
            }
            event_pool.push_back(t.start);
            event_pool.push_back(t.stop);
        }
        pending.clear();
    }
};

namespace {

int copy_to(pt_ctx* c, DevBuf& buf, const void* src, size_t bytes, const char* what) {
    int rc = c->cuda(buf.reserve(bytes), what);
    if (rc) return rc;
    if (bytes) rc = c->cuda(cudaMemcpyAsync(buf.p, src, bytes, cudaMemcpyHostToDevice, c->stream), what);
    return rc;
}

// the BVH must be a tree reachable from node 0 whose traversal never needs
// more than 64 deferred entries (trace.slang:632,786).  Returns PT_OK or an
// error code with *msg set; touches no context, so it may run on a helper
// thread.
int check_bvh(const pt_bvh_node* nodes, uint64_t count, uint64_t tris, const char** msg) {
    if (count == 0) {
        *msg = "BVH has no nodes";
        return PT_ERR_INVALID_ARG;
    }
    // one forward pass when every child follows its parent (the reference
    // builder allocates children after their parent, world.rs:1578-1583): then
    // the graph is acyclic, and at most one parent per node makes it a tree.
    // reached[i]: 0 = no parent seen, else 1 + the node's depth
    {
        std::vector<uint8_t> reached(count, 0);
        reached[0] = 1;
        bool ordered = true;
        for (uint64_t i = 0; i < count && ordered; ++i) {
            const uint8_t r = reached[i];
            if (r == 0) continue;  // unreachable from the root: ignored, as by the traversal
            const pt_bvh_node& n = nodes[i];
            if (n.tri_count > 0) {
                if ((uint64_t)n.left_first + n.tri_count > tris) {
                    *msg = "BVH leaf triangle range outside the triangle buffer";
                    return PT_ERR_INVALID_ARG;
                }
                continue;
            }
            const uint64_t l = n.left_first;
            if (l <= i || l + 1 >= count) {
                ordered = false;  // out of order or out of range: the general walk below decides
                break;
            }
            if (r > 64) {
                *msg = "BVH deeper than the 64-entry traversal stack";
                return PT_ERR_OUT_OF_LIMITS;
            }
            if (reached[l] | reached[l + 1]) {
                *msg = "BVH node reached twice (not a tree)";
                return PT_ERR_INVALID_ARG;
            }
            reached[l] = reached[l + 1] = (uint8_t)(r + 1);
        }
        if (ordered) return PT_OK;
    }
    std::vector<uint8_t> seen(count, 0);
    std::vector<std::pair<uint64_t, uint32_t>> st{{0, 0}};
    while (!st.empty()) {
        auto [i, depth] = st.back();
        st.pop_back();
        if (seen[i]) {
            *msg = "BVH node reached twice (not a tree)";
            return PT_ERR_INVALID_ARG;
        }
        seen[i] = 1;
        const pt_bvh_node& n = nodes[i];
        if (n.tri_count > 0) {
            if ((uint64_t)n.left_first + n.tri_count > tris) {
                *msg = "BVH leaf triangle range outside the triangle buffer";
                return PT_ERR_INVALID_ARG;
            }
        } else {
            if (depth >= 64) {
                *msg = "BVH deeper than the 64-entry traversal stack";
                return PT_ERR_OUT_OF_LIMITS;
            }
            if ((uint64_t)n.left_first + 1 >= count || n.left_first == 0) {
                *msg = "BVH child index outside the node buffer";
                return PT_ERR_INVALID_ARG;
            }
            st.push_back({n.left_first, depth + 1});
            st.push_back({(uint64_t)n.left_first + 1, depth + 1});
        }
    }
    return PT_OK;
}

// every skybox alias entry points inside the table
bool sky_aliases_in_range(const pt_skybox_alias_entry* a, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i)
        if (a[i].alias_index >= n) return false;
    return true;
}

// every triangle's material index below material_count; large scenes are
// scanned by several host threads
bool materials_in_range(const pt_triangle_attribute* attrs, uint64_t n, uint64_t materials) {
    const auto scan = [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i)
            if (attrs[i].material_index >= materials) return false;
        return true;
    };
    const unsigned hw = std::thread::hardware_concurrency();
    const unsigned threads = n < (1u << 18) || hw < 2 ? 1u : (hw < 16 ? hw : 16u);
    if (threads == 1) return scan(0, n);
    std::vector<std::thread> pool;
    std::vector<char> ok(threads, 1);
    unsigned started = 1;  // range 0 runs on the calling thread, with any range a refused thread leaves
    for (; started < threads; ++started) {
        try {
            pool.emplace_back([&, t = started] { ok[t] = scan(n * t / threads, n * (t + 1) / threads); });
        } catch (const std::system_error&) {
            break;
        }
    }
    ok[0] = scan(0, n / threads) && scan(n * started / threads, n);
    for (auto& th : pool) th.join();
    for (char v : ok)
        if (!v) return false;
    return true;
}

int validate_lights(pt_ctx* c, const pt_scene_uniforms& s, uint64_t scene_alias_live, uint64_t sky_alias_count,
                    const pt_skybox_uniforms& sky) {
    const float p0 = s.light_probabilities[0], p1 = s.light_probabilities[1];
    if (!(std::isfinite(p0) && std::isfinite(p1) && p0 >= 0.0f && p1 >= 0.0f))
        return c->fail(PT_ERR_INVALID_ARG, "light probabilities must be finite and non-negative");
    if (s.emissive_triangles_count > scene_alias_live)
        return c->fail(PT_ERR_INVALID_ARG, "emissive_triangles_count exceeds the scene alias table");
    // sample_light and skybox_light_pdf index these tables whenever the
    // matching probability allows it (trace.slang:482-489, 531-592)
    if (p0 > 0.0f && s.emissive_triangles_count == 0)
        return c->fail(PT_ERR_INVALID_ARG, "triangle lights have probability > 0 but no emissive triangles");
    const bool sky_sampled = p1 > 0.0f || (p0 + p1 > 0.0f && p0 < 1.0f);
    if (sky_sampled && (sky_alias_count == 0 || sky_alias_count != (uint64_t)sky.width * sky.height))
        return c->fail(PT_ERR_INVALID_ARG, "skybox can be sampled but its alias table is missing");
    return PT_OK;
}

}  // namespace

namespace {

int apply(pt_ctx* c, const pt_world_updates* u, bool initial) {
    c->touched();
    if (!u) return c->fail(PT_ERR_INVALID_ARG, "updates is NULL");
    if (initial) {
        if (!u->scene) return c->fail(PT_ERR_INVALID_ARG, "initial scene upload missing");
        if (!u->skybox) return c->fail(PT_ERR_INVALID_ARG, "initial skybox upload missing");
        if (!u->camera) return c->fail(PT_ERR_INVALID_ARG, "initial camera upload missing");
        if (!u->scene_alias_table) return c->fail(PT_ERR_INVALID_ARG, "initial scene aliases missing");
        if (!u->scene_uniforms) return c->fail(PT_ERR_INVALID_ARG, "initial scene uniforms missing");
        if (!u->skybox_uniforms) return c->fail(PT_ERR_INVALID_ARG, "initial skybox uniforms missing");
    }
    // ---- the scene's buffers start copying into staging buffers while the
    // host validates the update; they replace the live buffers only if every
    // check passes, so a rejected update leaves the device state untouched
    bool staged = false;
    if (const pt_scene_upload* s = u->scene) {
        if (s->geometries && s->attributes && s->materials && s->bvh_nodes && s->triangle_count &&
            !((s->srgb_atlas_count && !s->srgb_texture_atlases) || (s->linear_atlas_count && !s->linear_texture_atlases))) {
            const size_t layer = (size_t)PT_ATLAS_SIZE * PT_ATLAS_SIZE * 4;
            int rc = copy_to(c, c->stage_geo, s->geometries, s->triangle_count * sizeof(pt_triangle_geometry), "geometries");
            if (!rc) rc = copy_to(c, c->stage_attr, s->attributes, s->triangle_count * sizeof(pt_triangle_attribute), "attributes");
            if (!rc) rc = copy_to(c, c->stage_mat, s->materials, s->material_count * sizeof(pt_material), "materials");
            if (!rc) rc = copy_to(c, c->stage_nodes, s->bvh_nodes, s->node_count * sizeof(pt_bvh_node), "BVH");
            if (!rc) rc = copy_to(c, c->stage_srgb, s->srgb_texture_atlases, s->srgb_atlas_count * layer, "sRGB atlases");
            if (!rc) rc = copy_to(c, c->stage_linear, s->linear_texture_atlases, s->linear_atlas_count * layer, "linear atlases");
            if (rc) {
                cudaStreamSynchronize(c->stream);  // copies already issued still read the caller's memory
                return rc;
            }
            staged = true;
        }
    }
    // ---- validate everything before touching the live device state
    uint64_t tri = c->tri_count, mats = c->mat_count;
    pt_skybox_uniforms sky = u->skybox_uniforms ? *u->skybox_uniforms : c->sky_u;
    uint64_t sky_alias_count = c->sky_alias_count;
    uint64_t live = u->scene ? 0 : c->scene_alias_live;
    bool sky_checked = false, sky_aliases_ok = true;  // the skybox alias scan, when it ran beside the BVH walk
    const auto validate = [&]() -> int {
        if (const pt_scene_upload* s = u->scene) {
            if (!s->geometries || !s->attributes || !s->materials || !s->bvh_nodes)
                return c->fail(PT_ERR_INVALID_ARG, "scene upload has a NULL buffer");
            if (s->triangle_count == 0) return c->fail(PT_ERR_INVALID_ARG, "scene has no triangles");
            if (s->triangle_count > 0x7fffffffull) return c->fail(PT_ERR_OUT_OF_LIMITS, "too many triangles");
            if (s->material_count == 0) return c->fail(PT_ERR_INVALID_ARG, "scene has no materials");
            if ((s->srgb_atlas_count && !s->srgb_texture_atlases) || (s->linear_atlas_count && !s->linear_texture_atlases))
                return c->fail(PT_ERR_INVALID_ARG, "atlas count without atlas data");
            // the BVH walk (and the skybox alias scan) run on a helper thread
            // while this one scans the triangles' material indices
            const pt_skybox_upload* k = u->skybox;
            const bool scan_sky = k && k->rgba && k->alias_count && k->alias_table;
            const char* bvh_msg = nullptr;
            int bvh_rc = PT_OK;
            bool sky_ok = true;
            const auto helper = [&] {
                bvh_rc = check_bvh(s->bvh_nodes, s->node_count, s->triangle_count, &bvh_msg);
                if (scan_sky) sky_ok = sky_aliases_in_range(k->alias_table, k->alias_count);
            };
            std::thread worker;
            try {
                worker = std::thread(helper);
            } catch (const std::system_error&) {
                helper();  // no thread to be had: the same work on this one
            }
            const bool mats_ok = materials_in_range(s->attributes, s->triangle_count, s->material_count);
            if (worker.joinable()) worker.join();
            sky_checked = scan_sky;
            sky_aliases_ok = sky_ok;
            if (!mats_ok) return c->fail(PT_ERR_INVALID_ARG, "triangle material index outside the material buffer");
            if (bvh_rc) return c->fail(bvh_rc, bvh_msg);
            tri = s->triangle_count;
            mats = s->material_count;
        }
        for (uint64_t i = 0; i < u->material_update_count; ++i)
            if (!u->materials || u->materials[i].index >= mats)
                return c->fail(PT_ERR_INVALID_ARG, "material update index outside the material buffer");
        if (const pt_skybox_upload* k = u->skybox) {
            if (!k->rgba) return c->fail(PT_ERR_INVALID_ARG, "skybox upload has no pixels");
            if (k->uniforms.width == 0 || k->uniforms.height == 0 || (uint64_t)k->uniforms.width * k->uniforms.height > 0xffffffffull)
                return c->fail(PT_ERR_OUT_OF_LIMITS, "skybox dimensions out of range");
            if (k->alias_count && k->alias_count != (uint64_t)k->uniforms.width * k->uniforms.height)
                return c->fail(PT_ERR_INVALID_ARG, "skybox alias table size does not match the skybox");
            if (k->alias_count && !k->alias_table) return c->fail(PT_ERR_INVALID_ARG, "skybox alias table is NULL");
            if (!u->skybox_uniforms) sky = k->uniforms;
            sky_alias_count = k->alias_count;
            if (!(sky_checked ? sky_aliases_ok : sky_aliases_in_range(k->alias_table, k->alias_count)))
                return c->fail(PT_ERR_INVALID_ARG, "skybox alias index out of range");
        }
        if (u->skybox_uniforms && !u->skybox && (u->skybox_uniforms->width != c->sky_u.width || u->skybox_uniforms->height != c->sky_u.height))
            return c->fail(PT_ERR_INVALID_ARG, "skybox uniforms change the size of the uploaded skybox");
        if (u->scene_alias_table) {
            if (u->scene_alias_count > tri)
                return c->fail(PT_ERR_OUT_OF_LIMITS, "scene alias table larger than the triangle count");
            for (uint64_t i = 0; i < u->scene_alias_count; ++i) {
                const pt_scene_alias_entry& e = u->scene_alias_table[i];
                if (e.triangle_index >= tri || e.alias_index >= u->scene_alias_count)
                    return c->fail(PT_ERR_INVALID_ARG, "scene alias entry out of range");
            }
            live = u->scene_alias_count;
        }
        const pt_scene_uniforms scene = u->scene_uniforms ? *u->scene_uniforms : c->scene;
        return validate_lights(c, scene, live, sky_alias_count, sky);
    };
    int rc = validate();
    if (rc) {
        if (staged) cudaStreamSynchronize(c->stream);
        return rc;
    }

    // ---- upload
    if (const pt_scene_upload* s = u->scene) {
        // the validated staging buffers become the live ones (stream order keeps
        // earlier traces on the previous buffers)
        std::swap(c->geo, c->stage_geo);
        std::swap(c->attr, c->stage_attr);
        std::swap(c->mat, c->stage_mat);
        std::swap(c->nodes, c->stage_nodes);
        std::swap(c->srgb, c->stage_srgb);
        std::swap(c->linear, c->stage_linear);
        // the alias buffer holds every triangle (world_resources.rs:158-165)
        if ((rc = c->cuda(c->scene_alias.reserve(s->triangle_count * sizeof(pt_scene_alias_entry)), "scene aliases"))) return rc;
        c->tri_count = s->triangle_count;
        c->mat_count = s->material_count;
        c->node_count = s->node_count;
        c->srgb_count = s->srgb_atlas_count;
        c->linear_count = s->linear_atlas_count;
        c->alpha_modes.resize(s->material_count);
        for (uint64_t i = 0; i < s->material_count; ++i) c->alpha_modes[i] = s->materials[i].alpha_mode;
        c->scene_alias_live = 0;
        if (c->wavefront) ptw::world_changed(c->wavefront);
    }
    if (const pt_skybox_upload* k = u->skybox) {
        const size_t px = (size_t)k->uniforms.width * k->uniforms.height;
        if ((rc = copy_to(c, c->sky, k->rgba, px * 16, "skybox"))) return rc;
        if ((rc = copy_to(c, c->sky_alias, k->alias_table, k->alias_count * sizeof(pt_skybox_alias_entry), "skybox aliases"))) return rc;
        c->sky_alias_count = k->alias_count;
        c->sky_u = k->uniforms;
        if (c->wavefront) ptw::sky_changed(c->wavefront);
    }
    if (u->camera) c->camera = *u->camera;
    for (uint64_t i = 0; i < u->material_update_count; ++i) {
        const pt_material_update& m = u->materials[i];
        rc = c->cuda(cudaMemcpyAsync(c->mat.as<pt_material>() + m.index, &m.material, sizeof(pt_material),
                                     cudaMemcpyHostToDevice, c->stream), "material update");
        if (rc) return rc;
        c->alpha_modes[m.index] = m.material.alpha_mode;
    }
    if (u->scene_uniforms) c->scene = *u->scene_uniforms;
    if (u->scene_alias_table) {
        if (u->scene_alias_count)
            rc = c->cuda(cudaMemcpyAsync(c->scene_alias.p, u->scene_alias_table, u->scene_alias_count * sizeof(pt_scene_alias_entry),
                                         cudaMemcpyHostToDevice, c->stream), "scene aliases");
        if (rc) return rc;
        c->scene_alias_live = u->scene_alias_count;
    }
    if (u->skybox_uniforms) c->sky_u = *u->skybox_uniforms;
    if (u->reset_accumulation) c->params.sample_count = 0;
    // host pointers are borrowed for this call only
    rc = c->cuda(cudaStreamSynchronize(c->stream), "world upload");
    if (rc) return rc;
    c->world_ready = true;
    return PT_OK;
}

int alloc_tile(pt_ctx* c, uint32_t w, uint32_t h) {
    c->touched();
    if (w == 0 || h == 0 || w > kMaxTileDim || h > kMaxTileDim) {
        char msg[160];
        snprintf(msg, sizeof msg, "tile size %ux%u must be positive and at most %u pixels in each dimension", w, h, kMaxTileDim);
        return c->fail(PT_ERR_OUT_OF_LIMITS, msg);
    }
    const size_t bytes = (size_t)w * h * 16;
    int rc = c->cuda(c->accum.reserve(bytes), "accumulation buffer");
    if (!rc) rc = c->cuda(c->image.reserve(bytes), "storage texture");
    if (!rc) rc = c->cuda(cudaMemsetAsync(c->accum.p, 0, bytes, c->stream), "clear tile");
    if (!rc) rc = c->cuda(cudaMemsetAsync(c->image.p, 0, bytes, c->stream), "clear tile");
    if (!rc && (c->precision & PT_PRECISION_KAHAN)) {
        rc = c->cuda(c->comp.reserve(bytes), "Kahan compensation");
        if (!rc) rc = c->cuda(cudaMemsetAsync(c->comp.p, 0, bytes, c->stream), "clear tile");
    }
    if (rc) return rc;
    c->tile_w = w;
    c->tile_h = h;
    return PT_OK;
}

ptk::Tile tile_of(const pt_ctx* c) {
    ptk::Tile t;
    t.image_w = c->params.image_size[0];
    t.image_h = c->params.image_size[1];
    t.origin_x = c->params.tile_origin[0];
    t.origin_y = c->params.tile_origin[1];
    t.tile_w = c->tile_w;
    t.tile_h = c->tile_h;
    t.max_bounces = c->params.max_bounces;
    t.accum = c->accum.as<float4>();
    t.image = c->image.as<float4>();
    t.comp = (c->precision & PT_PRECISION_KAHAN) ? c->comp.as<float4>() : nullptr;
    return t;
}

int trace_impl(pt_ctx* c, uint32_t samples, uint32_t* traced, pt_path_record* host_records, uint64_t* host_totals) {
    if (!c->world_ready) return c->fail(PT_ERR_STATE, "no world uploaded");
    const uint32_t n = samples < PT_MAX_SAMPLES_PER_TRACE ? samples : PT_MAX_SAMPLES_PER_TRACE;
    if (traced) *traced = 0;
    if (n == 0) return PT_OK;
    const ptd::World w = c->view();
    const ptk::Tile t = tile_of(c);
    const size_t tile_px = (size_t)c->tile_w * c->tile_h;
    pt_path_record* rec = nullptr;
    int rc = PT_OK;
    if (host_records || host_totals || c->kernel == PT_KERNEL_PLAIN) c->touched();  // work on the context stream
    if (host_records) {
        if ((rc = c->cuda(c->records.reserve(tile_px * n * sizeof(pt_path_record)), "records"))) return rc;
        if ((rc = c->cuda(cudaMemsetAsync(c->records.p, 0, tile_px * n * sizeof(pt_path_record), c->stream), "records"))) return rc;
        rec = c->records.as<pt_path_record>();
    }
    unsigned long long* tot = nullptr;
    if (host_totals) {
        if ((rc = c->cuda(c->totals.reserve(PT_COUNT_FIELDS * 8), "totals"))) return rc;
        if ((rc = c->cuda(cudaMemsetAsync(c->totals.p, 0, PT_COUNT_FIELDS * 8, c->stream), "totals"))) return rc;
        tot = c->totals.as<unsigned long long>();
    }
    const uint32_t first = c->params.sample_count + 1u;
    if (c->kernel == PT_KERNEL_PLAIN) {
        for (uint32_t s = 0; s < n; ++s) {
            const uint32_t sample = first + s;
            const ptk::Sinks sinks{rec ? rec + tile_px * s : nullptr, tot};
            rc = c->cuda(c->timed(PT_KC_PLAIN, [&] { return ptk::launch_plain(w, t, sample, sinks, c->stream); }),
                         "plain trace launch");
            if (rc) return rc;
        }
    } else {
        if (!c->wavefront) {
            const int ce = ptw::create(&c->wavefront);
            if (ce) return c->cuda((cudaError_t)ce, "wavefront streams");
        }
        const bool record = rec != nullptr || tot != nullptr;
        const uint32_t form = ptw::effective_precision(w, c->precision, record);
        bool queued = false;
        if ((rc = c->cuda(ptw::prepare(c->wavefront, w, c->node_count, c->tri_count, form, c->stream, &queued),
                          "wavefront layouts")))
            return rc;
        if (queued) c->touched();
        const bool overlap = !record && c->ctx_ops == c->ops_at_trace;
        const ptw::Timer timer = [c](int cls, cudaStream_t s, const std::function<cudaError_t()>& f) {
            return c->timed(cls, s, f);
        };
        rc = c->cuda(ptw::trace(c->wavefront, w, t, first, n, ptk::Sinks{rec, tot}, c->stream, timer, form, overlap,
                                c->profiling),
                     "wavefront trace");
        if (rc) return rc;
        c->precision_active = form;
        if (!record) c->ops_at_trace = c->ctx_ops;
    }
    c->params.sample_count += n;
    if (traced) *traced = n;
    if (host_records) {
        rc = c->cuda(cudaMemcpyAsync(host_records, rec, tile_px * n * sizeof(pt_path_record), cudaMemcpyDeviceToHost, c->stream),
                     "records readback");
        if (!rc) rc = c->cuda(cudaStreamSynchronize(c->stream), "records readback");
    }
    if (host_totals && !rc) {
        unsigned long long t[PT_COUNT_FIELDS];
        rc = c->cuda(cudaMemcpyAsync(t, tot, sizeof t, cudaMemcpyDeviceToHost, c->stream), "totals readback");
        if (!rc) rc = c->cuda(cudaStreamSynchronize(c->stream), "totals readback");
        if (!rc)
            for (int i = 0; i < PT_COUNT_FIELDS; ++i) host_totals[i] += t[i];
    }
    return rc;
}

}  // namespace

extern "C" {

int pt_create(int device, const pt_world_updates* updates, uint32_t tile_width, uint32_t tile_height, pt_ctx** out) try {
    if (!out) return PT_ERR_INVALID_ARG;
    *out = nullptr;
    pt_ctx* c = new pt_ctx();
    c->device = device;
    int rc = c->cuda(cudaSetDevice(device), "cudaSetDevice");
    if (!rc) rc = c->cuda(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!rc) {
        float lut[256];
        for (int i = 0; i < 256; ++i) {
            const double v = (double)i / 255.0;
            lut[i] = (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
        }
        rc = copy_to(c, c->srgb_lut, lut, sizeof lut, "sRGB table");
    }
    if (!rc) rc = alloc_tile(c, tile_width, tile_height);
    if (!rc) rc = apply(c, updates, true);
    if (rc) {
        // keep the message on stderr: the caller gets no context to ask
        fprintf(stderr, "pt_create: %s\n", c->error.c_str());
        pt_destroy(c);
        return rc;
    }
    c->params.image_size[0] = tile_width;
    c->params.image_size[1] = tile_height;
    c->params.tile_origin[0] = 0;
    c->params.tile_origin[1] = 0;
    c->params.max_bounces = PT_DEFAULT_MAX_BOUNCES;
    c->params.sample_count = 0;
    *out = c;
    return PT_OK;
} catch (...) {
    return pt_abi_current_status(nullptr);
}

void pt_destroy(pt_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->harvest();
    for (cudaEvent_t e : c->event_pool) cudaEventDestroy(e);
    if (c->wavefront) ptw::destroy(c->wavefront);
    for (DevBuf* b : {&c->geo, &c->attr, &c->mat, &c->nodes, &c->srgb, &c->linear, &c->sky, &c->sky_alias,
                      &c->scene_alias, &c->srgb_lut, &c->accum, &c->image, &c->comp, &c->fp64, &c->display, &c->records, &c->totals,
                      &c->stage_geo, &c->stage_attr, &c->stage_mat, &c->stage_nodes, &c->stage_srgb, &c->stage_linear})
        b->release();
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int pt_apply_updates(pt_ctx* c, const pt_world_updates* u) try {
    if (!c) return PT_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    return apply(c, u, false);
} catch (...) {
    return pt_abi_status(c);
}

int pt_set_tile(pt_ctx* c, const uint32_t image_size[2], const uint32_t origin[2], const uint32_t size[2]) try {
    if (!c || !image_size || !origin || !size) return PT_ERR_INVALID_ARG;
    if (!(origin[0] < image_size[0] && origin[1] < image_size[1]))
        return c->fail(PT_ERR_INVALID_ARG, "tile origin must be within the image");
    cudaSetDevice(c->device);
    if (size[0] != c->tile_w || size[1] != c->tile_h) {
        const int rc = alloc_tile(c, size[0], size[1]);
        if (rc) return rc;
    }
    c->params.image_size[0] = image_size[0];
    c->params.image_size[1] = image_size[1];
    c->params.tile_origin[0] = origin[0];
    c->params.tile_origin[1] = origin[1];
    c->params.sample_count = 0;
    return PT_OK;
} catch (...) {
    return pt_abi_status(c);
}

int pt_set_max_bounces(pt_ctx* c, uint32_t max_bounces) try {
    if (!c) return PT_ERR_INVALID_ARG;
    if (max_bounces > PT_MAX_BOUNCES_LIMIT) return c->fail(PT_ERR_INVALID_ARG, "max bounces must be at most 16");
    if (c->params.max_bounces != max_bounces) {
        c->params.max_bounces = max_bounces;
        c->params.sample_count = 0;
    }
    return PT_OK;
} catch (...) {
    return pt_abi_status(c);
}

uint32_t pt_max_bounces(const pt_ctx* c) { return c ? c->params.max_bounces : 0; }
uint32_t pt_sample_count(const pt_ctx* c) { return c ? c->params.sample_count : 0; }

int pt_trace(pt_ctx* c, uint32_t samples, uint32_t* traced) try {
    if (!c) return PT_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    return trace_impl(c, samples, traced, nullptr, nullptr);
} catch (...) {
    return pt_abi_status(c);
}

int pt_trace_counted(pt_ctx* c, uint32_t samples, uint32_t* traced, uint64_t totals[PT_COUNT_FIELDS]) try {
    if (!c || !totals) return PT_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    return trace_impl(c, samples, traced, nullptr, totals);
} catch (...) {
    return pt_abi_status(c);
}

int pt_trace_recorded(pt_ctx* c, uint32_t samples, uint32_t* traced, pt_path_record* host_records) try {
    if (!c || !host_records) return PT_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    return trace_impl(c, samples, traced, host_records, nullptr);
} catch (...) {
    return pt_abi_status(c);
}

int pt_read_tile(pt_ctx* c, int which, float* host_rgba) try {
    if (!c || !host_rgba || (which != PT_TILE_IMAGE && which != PT_TILE_ACCUMULATION && which != PT_TILE_COMPENSATION))
        return PT_ERR_INVALID_ARG;
    c->touched();
    cudaSetDevice(c->device);
    if (which == PT_TILE_COMPENSATION && !(c->precision & PT_PRECISION_KAHAN)) {
        std::memset(host_rgba, 0, (size_t)c->tile_w * c->tile_h * 16);
        return PT_OK;
    }
    const DevBuf& b = which == PT_TILE_IMAGE ? c->image : (which == PT_TILE_ACCUMULATION ? c->accum : c->comp);
    int rc = c->cuda(cudaMemcpyAsync(host_rgba, b.p, (size_t)c->tile_w * c->tile_h * 16, cudaMemcpyDeviceToHost, c->stream),
                     "tile readback");
    if (!rc) rc = c->cuda(cudaStreamSynchronize(c->stream), "tile readback");
    return rc;
} catch (...) {
    return pt_abi_status(c);
}

int pt_display_tile(pt_ctx* c, uint8_t* host_rgba8) try {
    if (!c || !host_rgba8) return PT_ERR_INVALID_ARG;
    c->touched();
    cudaSetDevice(c->device);
    const size_t px = (size_t)c->tile_w * c->tile_h;
    int rc = c->cuda(c->display.reserve(px * 4), "display buffer");
    if (!rc) rc = c->cuda(c->timed(PT_KC_ACCUMULATE, [&] {
        return ptk::launch_display(c->image.as<const float4>(), (uint32_t)px, c->display.as<uchar4>(), c->stream);
    }), "display launch");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(host_rgba8, c->display.p, px * 4, cudaMemcpyDeviceToHost, c->stream), "display readback");
    if (!rc) rc = c->cuda(cudaStreamSynchronize(c->stream), "display readback");
    return rc;
} catch (...) {
    return pt_abi_status(c);
}

int pt_synchronize(pt_ctx* c, uint32_t timeout_ms) try {
    if (!c) return PT_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    if (timeout_ms == 0) return c->cuda(cudaStreamSynchronize(c->stream), "synchronize");
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
    for (;;) {
        const cudaError_t e = cudaStreamQuery(c->stream);
        if (e == cudaSuccess) return PT_OK;
        if (e != cudaErrorNotReady) return c->cuda(e, "synchronize");
        if (std::chrono::steady_clock::now() >= deadline) return c->fail(PT_ERR_TIMEOUT, "queued work did not finish in time");
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
} catch (...) {
    return pt_abi_status(c);
}

const char* pt_last_error(const pt_ctx* c) { return c ? c->error.c_str() : "null context"; }

int pt_set_kernel(pt_ctx* c, int kernel) try {
    if (!c) return PT_ERR_INVALID_ARG;
    if (kernel != PT_KERNEL_WAVEFRONT && kernel != PT_KERNEL_PLAIN) return c->fail(PT_ERR_INVALID_ARG, "unknown kernel");
    if (kernel == PT_KERNEL_PLAIN && c->precision != PT_PRECISION_FP32)
        return c->fail(PT_ERR_STATE, "the precision form runs on the wavefront kernels");
    c->kernel = kernel;
    return PT_OK;
} catch (...) {
    return pt_abi_status(c);
}

int pt_set_precision(pt_ctx* c, uint32_t flags) try {
    if (!c) return PT_ERR_INVALID_ARG;
    c->touched();
    if (flags & ~PT_PRECISION_COMPRESSED) return c->fail(PT_ERR_INVALID_ARG, "unknown precision bits");
    if (flags != PT_PRECISION_FP32 && c->kernel != PT_KERNEL_WAVEFRONT)
        return c->fail(PT_ERR_STATE, "the precision form runs on the wavefront kernels");
    cudaSetDevice(c->device);
    c->precision = flags;
    if ((flags & PT_PRECISION_KAHAN) && c->tile_w) {
        const size_t bytes = (size_t)c->tile_w * c->tile_h * 16;
        int rc = c->cuda(c->comp.reserve(bytes), "Kahan compensation");
        if (!rc) rc = c->cuda(cudaMemsetAsync(c->comp.p, 0, bytes, c->stream), "clear tile");
        if (rc) return rc;
    }
    c->params.sample_count = 0;
    return PT_OK;
} catch (...) {
    return pt_abi_status(c);
}

uint32_t pt_precision(const pt_ctx* c) { return c ? c->precision : 0u; }
uint32_t pt_precision_active(const pt_ctx* c) { return c ? c->precision_active : 0u; }

int pt_get_stream(pt_ctx* c, void** stream) try {
    if (!c || !stream) return PT_ERR_INVALID_ARG;
    c->touched();
    *stream = (void*)c->stream;
    return PT_OK;
} catch (...) {
    return pt_abi_status(c);
}

int pt_set_profiling(pt_ctx* c, int enabled) try {
    if (!c) return PT_ERR_INVALID_ARG;
    c->profiling = enabled != 0;
    return PT_OK;
} catch (...) {
    return pt_abi_status(c);
}

int pt_get_kernel_times(pt_ctx* c, uint64_t launches[PT_KERNEL_CLASS_COUNT], double ms[PT_KERNEL_CLASS_COUNT]) try {
    if (!c || !launches || !ms) return PT_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    c->harvest();
    for (int i = 0; i < PT_KERNEL_CLASS_COUNT; ++i) {
        launches[i] = c->class_launches[i];
        ms[i] = c->class_ms[i];
    }
    return PT_OK;
} catch (...) {
    return pt_abi_status(c);
}

int pt_reset_kernel_times(pt_ctx* c) try {
    if (!c) return PT_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    c->harvest();
    for (int i = 0; i < PT_KERNEL_CLASS_COUNT; ++i) {
        c->class_launches[i] = 0;
        c->class_ms[i] = 0.0;
    }
    return PT_OK;
} catch (...) {
    return pt_abi_status(c);
}

uint64_t pt_launch_count(const pt_ctx* c) { return c ? c->launch_count : 0; }

int pt_render_fp64(pt_ctx* c, uint32_t sample_first, uint32_t sample_count, double* host_rgb_sums) try {
    if (!c || !host_rgb_sums) return PT_ERR_INVALID_ARG;
    c->touched();
    if (sample_first == 0 || sample_count == 0 || sample_count - 1u > 0xffffffffu - sample_first)
        return c->fail(PT_ERR_INVALID_ARG, "FP64 render needs a non-empty range of 1-based sample indices");
    if (!c->world_ready) return c->fail(PT_ERR_STATE, "no world uploaded");
    cudaSetDevice(c->device);
    const size_t bytes = (size_t)c->tile_w * c->tile_h * 3 * sizeof(double);
    int rc = c->cuda(c->fp64.reserve(bytes), "FP64 sums");
    if (!rc) rc = c->cuda(cudaMemsetAsync(c->fp64.p, 0, bytes, c->stream), "FP64 sums");
    const ptd::World w = c->view();
    const ptk::Tile t = tile_of(c);
    for (uint32_t s = 0; !rc && s < sample_count; ++s)
        rc = c->cuda(ptk::launch_fp64(w, t, sample_first + s, c->fp64.as<double>(), c->stream), "FP64 render launch");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(host_rgb_sums, c->fp64.p, bytes, cudaMemcpyDeviceToHost, c->stream), "FP64 readback");
    if (!rc) rc = c->cuda(cudaStreamSynchronize(c->stream), "FP64 render");
    return rc;
} catch (...) {
    return pt_abi_status(c);
}

int pt_debug_intersect(pt_ctx* c, uint64_t n, const float* origins, const float* directions, const float* t_max,
                       int32_t* hit, float* hit_t, pt_path_record* records) try {
    if (!c || !origins || !directions || !t_max || !hit || !hit_t) return PT_ERR_INVALID_ARG;
    c->touched();
    if (!c->world_ready) return c->fail(PT_ERR_STATE, "no world uploaded");
    if (n == 0) return PT_OK;
    cudaSetDevice(c->device);
    DevBuf o, d, tm, h, ht, rec;
    int rc = copy_to(c, o, origins, n * 12, "rays");
    if (!rc) rc = copy_to(c, d, directions, n * 12, "rays");
    if (!rc) rc = copy_to(c, tm, t_max, n * 4, "rays");
    if (!rc) rc = c->cuda(h.reserve(n * 4), "hits");
    if (!rc) rc = c->cuda(ht.reserve(n * 4), "hits");
    if (!rc && records) rc = c->cuda(rec.reserve(n * sizeof(pt_path_record)), "records");
    const ptd::World w = c->view();
    const bool wide = (ptw::effective_precision(w, c->precision, records != nullptr) & PT_PRECISION_WIDE_BVH) != 0;
    if (!rc && wide) {
        if (!c->wavefront) rc = c->cuda((cudaError_t)ptw::create(&c->wavefront), "wavefront streams");
        if (!rc) rc = c->cuda(ptw::prepare(c->wavefront, w, c->node_count, c->tri_count, PT_PRECISION_WIDE_BVH, c->stream),
                     "wide BVH");
    }
    if (!rc)
        rc = c->cuda(c->timed(PT_KC_EXTEND, [&] {
            if (wide)
                return ptw::debug_intersect_wide(c->wavefront, w, n, o.as<float>(), d.as<float>(), tm.as<float>(),
                                                 h.as<int32_t>(), ht.as<float>(), c->stream);
            return ptk::launch_debug_intersect(w, n, o.as<float>(), d.as<float>(), tm.as<float>(), h.as<int32_t>(),
                                               ht.as<float>(), records ? rec.as<pt_path_record>() : nullptr, c->stream);
        }), "debug intersect");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(hit, h.p, n * 4, cudaMemcpyDeviceToHost, c->stream), "hits");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(hit_t, ht.p, n * 4, cudaMemcpyDeviceToHost, c->stream), "hits");
    if (!rc && records)
        rc = c->cuda(cudaMemcpyAsync(records, rec.p, n * sizeof(pt_path_record), cudaMemcpyDeviceToHost, c->stream), "records");
    if (!rc) rc = c->cuda(cudaStreamSynchronize(c->stream), "debug intersect");
    for (DevBuf* b : {&o, &d, &tm, &h, &ht, &rec}) b->release();
    return rc;
} catch (...) {
    return pt_abi_status(c);
}

}  // extern "C"
