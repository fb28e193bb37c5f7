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

// wraps each kernel launch (class id from PT_KC_*) so the caller can time it
using Timer = std::function<cudaError_t(int cls, const std::function<cudaError_t()>& launch)>;

// (re)build the derived BVH / triangle layouts after world_changed
cudaError_t prepare(Wavefront* wf, const ptd::World& w, uint64_t nodes, uint64_t tris, cudaStream_t stream);

cudaError_t trace(Wavefront* wf, const ptd::World& w, const ptk::Tile& tile, uint32_t first_sample,
                  uint32_t samples, ptk::Sinks sinks, cudaStream_t stream, const Timer& timer);

}  // namespace ptw
