// pt_render_main.cpp - `pt-render render ...`: the reference's headless
// renderer (src/render/headless.rs) on top of the C ABI.
//
// Flags, defaults and validation follow RenderOptions (headless.rs:15-127);
// the world is loaded, the skybox luminance and camera overrides applied
// (headless.rs:180-204), the image traced tile by tile in row-major order with
// at most 16 samples per trace call (headless.rs:207-285), each finished tile
// tone mapped (display.wgsl) and the RGB8 image saved.
//
// Scenes: a glTF 2.0 file (.glb or .gltf, PNG/JPEG textures; the
// reference's default is its box.glb asset), "cornell" (36-triangle Cornell
// box) or "procedural[:SEED]" (the ~2.1M-triangle procedural scene).
// Skyboxes: "black", "procedural" (gradient + sun), or a Radiance .hdr,
// OpenEXR .exr, PNG or JPEG file (WebP skyboxes are not decoded).  Output: .png, .jpg / .jpeg, .webp (lossless) or .ppm.
#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pt.h"
#include "../../include/pt_world.h"

namespace {

struct Options {
    std::string scene = "cornell";
    std::string skybox = "black";
    float skybox_luminance = PTW_DEFAULT_SKYBOX_LUMINANCE;
    std::string output = "render.png";
    uint32_t width = 1920, height = 1080, samples = 256, max_bounces = PT_DEFAULT_MAX_BOUNCES, tile_size = 512;
    bool has_position = false, has_yaw = false, has_pitch = false, has_fov = false;
    float position[3] = {0, 0, 0};
    float yaw = 0, pitch = 0, fov = 0;
    int device = 0;
};

[[noreturn]] void usage_error(const std::string& msg) {
    fprintf(stderr, "error: %s\n\nusage: pt-render render [--scene S] [--skybox S] [--skybox-luminance NITS]\n"
                    "  [--output FILE.{png,jpg,webp}] [--width N] [--height N] [--samples N] [--max-bounces 0..16]\n"
                    "  [--tile-size N] [--camera-position X,Y,Z] [--camera-yaw DEG] [--camera-pitch DEG]\n"
                    "  [--camera-fov DEG] [--device N]\n",
            msg.c_str());
    exit(2);
}

// parse_finite, headless.rs:67-74
float parse_finite(const std::string& flag, const char* s) {
    char* end = nullptr;
    errno = 0;
    const float v = strtof(s, &end);
    if (end == s || *end != '\0' || errno == ERANGE) usage_error("invalid value for " + flag + ": " + s);
    if (!std::isfinite(v)) usage_error("invalid value for " + flag + ": must be finite");
    return v;
}

uint32_t parse_u32(const std::string& flag, const char* s, uint32_t lo, uint32_t hi) {
    char* end = nullptr;
    errno = 0;
    const unsigned long long v = strtoull(s, &end, 10);
    if (end == s || *end != '\0' || errno == ERANGE || s[0] == '-' || v < lo || v > hi)
        usage_error("invalid value for " + flag + ": " + s + " (range " + std::to_string(lo) + ".." + std::to_string(hi) + ")");
    return (uint32_t)v;
}

Options parse(int argc, char** argv) {
    Options o;
    if (argc < 2 || std::string(argv[1]) != "render") usage_error("expected the `render` command");
    for (int i = 2; i < argc; ++i) {
        const std::string f = argv[i];
        if (i + 1 >= argc) usage_error("missing value for " + f);
        const char* v = argv[++i];
        if (f == "--scene") o.scene = v;
        else if (f == "--skybox") o.skybox = v;
        else if (f == "--skybox-luminance") {
            o.skybox_luminance = parse_finite(f, v);
            if (o.skybox_luminance < 0) usage_error("--skybox-luminance must be nonnegative");
        } else if (f == "--output") {
            o.output = v;
            const auto dot = o.output.rfind('.');
            const std::string ext = dot == std::string::npos ? "" : o.output.substr(dot + 1);
            std::string lower = ext;
            for (char& c : lower) c = (char)tolower((unsigned char)c);
            // parse_output, headless.rs:118-126 (.ppm accepted as well)
            if (lower != "png" && lower != "jpg" && lower != "jpeg" && lower != "webp" && lower != "ppm")
                usage_error("--output must have a .png, .jpg, .jpeg, or .webp extension");
        } else if (f == "--width") o.width = parse_u32(f, v, 1, 0xffffffffu);
        else if (f == "--height") o.height = parse_u32(f, v, 1, 0xffffffffu);
        else if (f == "--samples") o.samples = parse_u32(f, v, 1, 0xffffffffu);
        else if (f == "--max-bounces") o.max_bounces = parse_u32(f, v, 0, PT_MAX_BOUNCES_LIMIT);
        else if (f == "--tile-size") o.tile_size = parse_u32(f, v, 1, 0xffffffffu);
        else if (f == "--camera-position") {
            // parse_position, headless.rs:107-116
            std::string s = v;
            std::vector<std::string> parts;
            size_t start = 0;
            for (size_t k = 0; k <= s.size(); ++k)
                if (k == s.size() || s[k] == ',') {
                    std::string p = s.substr(start, k - start);
                    while (!p.empty() && p.front() == ' ') p.erase(p.begin());
                    while (!p.empty() && p.back() == ' ') p.pop_back();
                    parts.push_back(p);
                    start = k + 1;
                }
            if (parts.size() != 3) usage_error("--camera-position must be three comma-separated coordinates");
            for (int k = 0; k < 3; ++k) o.position[k] = parse_finite(f, parts[k].c_str());
            o.has_position = true;
        } else if (f == "--camera-yaw") {
            o.yaw = parse_finite(f, v);
            o.has_yaw = true;
        } else if (f == "--camera-pitch") {
            o.pitch = parse_finite(f, v);
            if (o.pitch < -90.0f || o.pitch > 90.0f) usage_error("--camera-pitch must be from -90 to 90");
            o.has_pitch = true;
        } else if (f == "--camera-fov") {
            o.fov = parse_finite(f, v);
            if (!(o.fov > 0.0f && o.fov < 180.0f)) usage_error("--camera-fov must be strictly between 0 and 180");
            o.has_fov = true;
        } else if (f == "--device") o.device = (int)parse_u32(f, v, 0, 1024);
        else usage_error("unknown flag " + f);
    }
    return o;
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int fail(const char* what, const std::string& msg) {
    fprintf(stderr, "error: %s: %s\n", what, msg.c_str());
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    const Options opt = parse(argc, argv);
    const double started = now_s();
    fprintf(stderr, "Rendering %s\n", opt.scene.c_str());

    // load_world, headless.rs:180-204
    ptw_world* world = nullptr;
    int rc;
    if (opt.scene == "cornell") {
        rc = ptw_scene_cornell_box(&world);
    } else if (opt.scene.rfind("procedural", 0) == 0) {
        ptw_procedural_params p;
        ptw_procedural_defaults(&p);
        if (opt.scene.size() > 11 && opt.scene[10] == ':') p.seed = strtoull(opt.scene.c_str() + 11, nullptr, 10);
        p.skybox_width = p.skybox_height = 0;  // the --skybox flag decides the sky
        rc = ptw_scene_procedural(&p, &world);
    } else {
        char err[512] = {0};
        rc = ptw_create(&world);
        if (!rc) rc = ptw_load_gltf(world, opt.scene.c_str(), err, sizeof err);
        if (rc) return fail("scene", "cannot read scene " + opt.scene + ": " + err);
        rc = ptw_build(world);
    }
    if (rc) return fail("scene", "scene construction failed");
    if (opt.skybox == "procedural") {
        rc = ptw_set_procedural_skybox(world, 1024, 512);
    } else if (opt.skybox != "black") {
        // .hdr or .exr, decoded by the library
        uint32_t w = 0, h = 0;
        char err[512] = {0};
        if (ptw_read_image_rgba(opt.skybox.c_str(), nullptr, 0, &w, &h, err, sizeof err))
            return fail("skybox", "cannot read skybox " + opt.skybox + ": " + err);
        std::vector<float> px((size_t)w * h * 4);
        if (ptw_read_image_rgba(opt.skybox.c_str(), px.data(), px.size(), &w, &h, err, sizeof err))
            return fail("skybox", "cannot read skybox " + opt.skybox + ": " + err);
        if (w / 2 != h) fprintf(stderr, "Skybox image should usually have 2:1 aspect ratio, but is %ux%u\n", w, h);
        rc = ptw_set_skybox_rgba(world, px.data(), w, h);
    }
    if (rc) return fail("skybox", ptw_last_error(world));
    ptw_set_aspect_ratio(world, (float)opt.width / (float)opt.height);
    ptw_edit_skybox_average_luminance(world, opt.skybox_luminance);
    const float deg = 3.14159265358979323846f / 180.0f;
    const float yaw = opt.yaw * deg, pitch = opt.pitch * deg, fov = opt.fov * deg;
    if (opt.has_position || opt.has_yaw || opt.has_pitch || opt.has_fov)
        ptw_edit_camera(world, opt.has_position ? opt.position : nullptr, opt.has_yaw ? &yaw : nullptr,
                        opt.has_pitch ? &pitch : nullptr, opt.has_fov ? &fov : nullptr);
    pt_world_updates updates;
    if ((rc = ptw_take_updates(world, &updates))) return fail("world", ptw_last_error(world));

    const uint32_t tile[2] = {std::min(opt.tile_size, opt.width), std::min(opt.tile_size, opt.height)};
    pt_ctx* ctx = nullptr;
    if ((rc = pt_create(opt.device, &updates, tile[0], tile[1], &ctx))) return fail("path tracer", "pt_create failed");
    pt_set_max_bounces(ctx, opt.max_bounces);
    ptw_destroy(world);  // the GPU has its own copy of the world

    // render_tiles, headless.rs:207-285
    const uint32_t image[2] = {opt.width, opt.height};
    std::vector<uint8_t> rgb((size_t)opt.width * opt.height * 3, 0);
    std::vector<uint8_t> rgba((size_t)tile[0] * tile[1] * 4);
    const double t0 = now_s();
    double last_log = t0;
    const double total = (double)opt.width * opt.height * opt.samples;
    double traced_samples = 0;
    for (uint32_t y = 0; y < opt.height; y += tile[1]) {
        for (uint32_t x = 0; x < opt.width; x += tile[0]) {
            const uint32_t origin[2] = {x, y};
            const uint32_t vis[2] = {std::min(tile[0], opt.width - x), std::min(tile[1], opt.height - y)};
            if ((rc = pt_set_tile(ctx, image, origin, tile))) return fail("set_tile", pt_last_error(ctx));
            uint32_t remaining = opt.samples;
            while (remaining > 0) {
                uint32_t traced = 0;
                if ((rc = pt_trace(ctx, remaining, &traced))) return fail("trace", pt_last_error(ctx));
                if ((rc = pt_synchronize(ctx, 0))) return fail("trace", pt_last_error(ctx));
                remaining -= traced;
                traced_samples += (double)vis[0] * vis[1] * traced;
                if (now_s() - last_log >= 1.0) {
                    last_log = now_s();
                    const double fraction = traced_samples / total, elapsed = last_log - t0;
                    fprintf(stderr, "Progress %.1f%%; elapsed %.1fs; remaining approximately %.1fs\n", fraction * 100.0,
                            elapsed, elapsed * (1.0 - fraction) / fraction);
                }
            }
            if ((rc = pt_display_tile(ctx, rgba.data()))) return fail("readback", pt_last_error(ctx));
            for (uint32_t row = 0; row < vis[1]; ++row)
                for (uint32_t col = 0; col < vis[0]; ++col)
                    for (int c = 0; c < 3; ++c)
                        rgb[((size_t)(y + row) * opt.width + x + col) * 3 + c] = rgba[((size_t)row * tile[0] + col) * 4 + c];
        }
    }
    pt_destroy(ctx);
    char werr[512] = {0};
    if (ptw_write_image(opt.output.c_str(), rgb.data(), opt.width, opt.height, werr, sizeof werr))
        return fail("output", werr);
    fprintf(stderr, "Saved %s in %.1fs\n", opt.output.c_str(), now_s() - started);
    return 0;
}
