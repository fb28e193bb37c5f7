// display.cu - display.wgsl:19-46 as a CUDA kernel: ACES-fit tone map and the
// sRGB OETF of the storage texture, written as RGBA8 (the Rgba8Unorm target of
// headless.rs:11).  pow goes through the deterministic pt_fmath.h power.
#include "pt_kernels.h"

namespace ptd {

// aces_film, display.wgsl:19-30
PTD float aces(float c) {
    const float a = 2.51f, b = 0.03f, c2 = 2.43f, d = 0.59f, e = 0.14f;
    return saturate((c * (a * c + b)) / (c * (c2 * c + d) + e));
}

// linear -> sRGB, display.wgsl:38-42, then UNORM8 rounding
PTD unsigned char encode(float linear) {
    const float m = aces(linear);
    const float s = m > 0.0031308f ? ptm::powf_(m, 1.0f / 2.4f) * 1.055f - 0.055f : m * 12.92f;
    return (unsigned char)floorf(saturate(s) * 255.0f + 0.5f);
}

__global__ void display_kernel(const float4* image, uint32_t count, uchar4* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float4 c = image[i];
    out[i] = make_uchar4(encode(c.x), encode(c.y), encode(c.z), (unsigned char)floorf(saturate(c.w) * 255.0f + 0.5f));
}

}  // namespace ptd

namespace ptk {

cudaError_t launch_display(const float4* image, uint32_t count, uchar4* out, cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    ptd::display_kernel<<<(count + 255u) / 256u, 256u, 0, stream>>>(image, count, out);
    return cudaGetLastError();
}

}  // namespace ptk
