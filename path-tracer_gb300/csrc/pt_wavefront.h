// pt_wavefront.h - the wavefront organisation of the trace pass.
//
// One pt_trace call turns (tile pixels x samples) into paths and advances all
// of them one bounce at a time through stage kernels:
//   raygen      camera rays, seeds (trace.slang:736-748)
//   extend      closest-hit traversal of every queued ray (trace.slang:764-884)
//   shade       emission, OpenPBR setup, light sample, BSDF sample
//               (trace.slang:887-1296); appends continuing rays to the next
//               queue and NEE shadow rays to the shadow queue
//   shadow      any-hit traversal (trace.slang:614-717); adds unoccluded
//               light contributions
//   accumulate  per pixel, samples in order (trace.slang:1299-1308)
// Queue lengths live on the device; the host never waits between stages.
#pragma once

#include <functional>

#include "pt_kernels.h"

namespace ptw {

struct Wavefront;

int create(Wavefront** out);
void destroy(Wavefront* wf);
// the world buffers changed: derived layouts are rebuilt on the next trace
void world_changed(Wavefront* wf);

// wraps each kernel launch (class id from PT_KC_*, the stream it is queued
// on) so the caller can time it
using Timer = std::function<cudaError_t(int cls, cudaStream_t stream, const std::function<cudaError_t()>& launch)>;

// the skybox texels changed (its BF16 copy is rebuilt on the next trace)
void sky_changed(Wavefront* wf);

// (re)build the derived layouts after world_changed: the child-pair BVH and
// padded triangles always; for the precision form (PT_PRECISION_* bits of
// include/pt_precision.h) the 8-wide BVH (collapsed on the host from the
// device's binary nodes) and the FP16 attributes / BF16 skybox.
// *queued (if given): whether work was queued on `stream`.
cudaError_t prepare(Wavefront* wf, const ptd::World& w, uint64_t nodes, uint64_t tris, uint32_t precision,
                    cudaStream_t stream, bool* queued = nullptr);

// the precision bits a trace with these arguments runs: the wide BVH only for
// opaque worlds and not for the recording variants (their records describe
// the binary traversal)
uint32_t effective_precision(const ptd::World& w, uint32_t precision, bool record);

// Traces samples first_sample.. of the tile in groups of at most 2^25 paths.
// Each group runs on one of two internal streams with its own queues, so
// consecutive groups overlap (the next group's first bounces beside the last
// bounces of the previous one); its accumulation is queued on `stream`, so
// any later work there sees the finished samples in order.  `overlap`: no
// work was queued on `stream` since the previous call's groups began, so this
// call's groups may start where those did (otherwise they wait for `stream`).
// Within a group, a bounce's shadow rays are traced on a second stream beside
// the next bounce's extend stage.  `serial`: no overlap at all (each group
// starts after the previous one's accumulation, each stage after the one
// before), so that the timer sees every kernel alone.
cudaError_t trace(Wavefront* wf, const ptd::World& w, const ptk::Tile& tile, uint32_t first_sample,
                  uint32_t samples, ptk::Sinks sinks, cudaStream_t stream, const Timer& timer, uint32_t precision,
                  bool overlap, bool serial);

// the narrow copies of the precision form, on `stream`: FP32 attributes ->
// pt_half_attribute records (8 uint2 each), RGBA32F texels -> BF16 RGBA
cudaError_t convert_half_attributes(const pt_triangle_attribute* in, uint64_t n, uint2* out, cudaStream_t stream);
cudaError_t convert_bf16_sky(const float4* in, uint64_t n, uint2* out, cudaStream_t stream);

// closest hit of given rays through the 8-wide BVH (prepare with
// PT_PRECISION_WIDE_BVH first); device arrays
cudaError_t debug_intersect_wide(Wavefront* wf, const ptd::World& w, uint64_t n, const float* origins,
                                 const float* directions, const float* t_max, int32_t* hit, float* hit_t,
                                 cudaStream_t stream);

}  // namespace ptw
