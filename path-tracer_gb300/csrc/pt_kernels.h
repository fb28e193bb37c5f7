// pt_kernels.h - host-callable launchers of the CUDA kernels (one definition
// per .cu file, so the translation units compile in parallel).
#pragma once

#include <cuda_runtime.h>

#include "pt_device.cuh"

namespace ptk {

// one tile of the image: bind group 0 of the reference (path_tracer.rs:88-126)
struct Tile {
    uint32_t image_w, image_h;
    uint32_t origin_x, origin_y;
    uint32_t tile_w, tile_h;
    uint32_t max_bounces;
    float4* accum;  // tile_w * tile_h running sums (w = 1)
    float4* image;  // tile_w * tile_h EXPOSURE * sum / n (alpha 1)
    float4* comp = nullptr;  // Kahan compensation of accum (precision form); null: plain sums
};

// plain kernel: one thread per tile pixel, one launch per sample
// (path_tracer.rs:342-349); `sample_count` is the 1-based sample index n
// instrumentation sinks of the counting kernel variants: per-path records
// and/or device totals (PT_COUNT_FIELDS uint64); both NULL = plain variant
struct Sinks {
    pt_path_record* records;
    unsigned long long* totals;
    bool any() const { return records != nullptr || totals != nullptr; }
};

cudaError_t launch_plain(const ptd::World& w, const Tile& t, uint32_t sample_count, Sinks sinks, cudaStream_t stream);

// debug: closest-hit traversal of given opaque rays
cudaError_t launch_debug_intersect(const ptd::World& w, uint64_t n, const float* origins, const float* directions,
                                   const float* t_max, int32_t* hit, float* hit_t, pt_path_record* records,
                                   cudaStream_t stream);

// FP64 reference render: one launch per sample (1-based index `sample`),
// adds each visible tile pixel's radiance to sums[3 * (y * tile_w + x) ..]
cudaError_t launch_fp64(const ptd::World& w, const Tile& t, uint32_t sample, double* sums, cudaStream_t stream);

// display.wgsl:19-46 on the storage texture -> RGBA8
cudaError_t launch_display(const float4* image, uint32_t count, uchar4* out, cudaStream_t stream);

}  // namespace ptk
