// pt_fmath.h - FP32 elementary functions with identical bits on the host and
// on the GPU.
//
// The reference shader (src/render/trace.slang) calls sin, cos, acos, atan2
// and pow, whose accuracy WGSL leaves to the implementation.  To make the CUDA
// kernels and the CPU oracle agree bit for bit, both evaluate these functions
// with the code below, which uses only operations that IEEE 754 defines
// exactly (+ - * /, fma, sqrt, floor, comparisons and bit casts).  Callers must
// compile device code with -fmad=false -prec-div=true -prec-sqrt=true
// -ftz=false and host code with -ffp-contract=off.
//
// Methods (no vendor library code is reproduced):
//  - sin/cos: Cody-Waite reduction by pi/2 with a three-part constant
//    (C1 = fl(pi/2), C2 = fl(pi/2 - C1), C3 = fl(pi/2 - C1 - C2)), then the
//    Taylor series of sin and cos on [-pi/4, pi/4] (truncation < 2e-9).
//  - asin/acos: Taylor series of asin on [-1/2, 1/2]; for |x| > 1/2 the
//    identity acos(x) = 2 asin(sqrt((1 - x) / 2)).
//  - atan2: octant reduction to atan(z), z in [0, 1]; for z > 2 - sqrt(3)
//    the identity atan(z) = pi/6 + atan((sqrt(3) z - 1) / (sqrt(3) + z));
//    then the Taylor series of atan on [-0.268, 0.268].
//  - pow(x, y), x >= 0: exp2(y * log2(x)); log2 through
//    ln(m) = 2 atanh((m - 1) / (m + 1)), m in [sqrt(1/2), sqrt(2)); exp2
//    through 2^k * e^(f ln 2), f in [-1/2, 1/2], Taylor series of e^g.
// All coefficients are the exact Taylor coefficients rounded to nearest
// float; accuracy against double-precision libm is checked by the tests
// (a few ulp).
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define PT_HD __host__ __device__ __forceinline__
#else
#define PT_HD inline
#endif

namespace ptm {

PT_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

PT_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

// IEEE operations spelled out so both compilers emit the correctly rounded form.
PT_HD float fma_(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return __builtin_fmaf(a, b, c);
#endif
}
PT_HD float sqrt_(float x) {
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return __builtin_sqrtf(x);
#endif
}
PT_HD float div_(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
PT_HD float floor_(float x) {
#if defined(__CUDA_ARCH__)
    return floorf(x);
#else
    return __builtin_floorf(x);
#endif
}
PT_HD float abs_(float x) { return u2f(f2u(x) & 0x7fffffffu); }
PT_HD float copysign_(float mag, float sgn) {
    return u2f((f2u(mag) & 0x7fffffffu) | (f2u(sgn) & 0x80000000u));
}
// min/max that return the other operand when one is NaN (IEEE minNum/maxNum,
// the semantics of C fminf/fmaxf and of PTX min.f32/max.f32).
PT_HD float min_(float a, float b) {
#if defined(__CUDA_ARCH__)
    return fminf(a, b);
#else
    return __builtin_fminf(a, b);
#endif
}
PT_HD float max_(float a, float b) {
#if defined(__CUDA_ARCH__)
    return fmaxf(a, b);
#else
    return __builtin_fmaxf(a, b);
#endif
}

// pi/2 = C1 + C2 + C3
constexpr float kPio2C1 = 0x1.921fb6p+0f;
constexpr float kPio2C2 = -0x1.777a5cp-25f;
constexpr float kPio2C3 = -0x1.ee59dap-50f;
constexpr float kTwoOverPi = 0x1.45f306p-1f;
constexpr float kPi = 0x1.921fb6p+1f;
constexpr float kPiLo = 2.0f * kPio2C2;  // pi - kPi (to float precision)
constexpr float kSqrt3 = 0x1.bb67aep+0f;
constexpr float kPi6 = 0x1.0c1524p-1f;
constexpr float kPi6Lo = -0x1.f4a326p-27f;
constexpr float kLn2 = 0x1.62e430p-1f;
constexpr float kLog2e = 0x1.715476p+0f;
constexpr float kSqrt2 = 0x1.6a09e6p+0f;

// sin(r) and cos(r) for |r| <= pi/4 (Taylor to r^13 / r^14)
PT_HD float sin_kernel(float r) {
    const float r2 = r * r;
    float p = 0x1.612462p-33f;
    p = fma_(p, r2, -0x1.ae6456p-26f);
    p = fma_(p, r2, 0x1.71de3ap-19f);
    p = fma_(p, r2, -0x1.a01a02p-13f);
    p = fma_(p, r2, 0x1.111112p-7f);
    p = fma_(p, r2, -0x1.555556p-3f);
    return fma_(r * r2, p, r);
}
PT_HD float cos_kernel(float r) {
    const float r2 = r * r;
    float p = -0x1.93974ap-37f;
    p = fma_(p, r2, 0x1.1eed8ep-29f);
    p = fma_(p, r2, -0x1.27e4fcp-22f);
    p = fma_(p, r2, 0x1.a01a02p-16f);
    p = fma_(p, r2, -0x1.6c16c2p-10f);
    p = fma_(p, r2, 0x1.555556p-5f);
    const float t = 1.0f - 0.5f * r2;
    return fma_(r2 * r2, p, t);
}

// x = k * pi/2 + r, |r| <= pi/4 (|x| < 2^14 keeps the reduction accurate)
PT_HD float reduce_pio2(float x, int* quadrant) {
    const float k = floor_(fma_(x, kTwoOverPi, 0.5f));
    float r = fma_(-k, kPio2C1, x);
    r = fma_(-k, kPio2C2, r);
    r = fma_(-k, kPio2C3, r);
    *quadrant = ((int)k) & 3;
    return r;
}

PT_HD float sinf_(float x) {
    int q;
    const float r = reduce_pio2(x, &q);
    const float s = sin_kernel(r), c = cos_kernel(r);
    switch (q) {
        case 0: return s;
        case 1: return c;
        case 2: return -s;
        default: return -c;
    }
}
PT_HD float cosf_(float x) {
    int q;
    const float r = reduce_pio2(x, &q);
    const float s = sin_kernel(r), c = cos_kernel(r);
    switch (q) {
        case 0: return c;
        case 1: return -s;
        case 2: return -c;
        default: return s;
    }
}

// sin and cos of one argument with one reduction: bitwise sinf_(x), cosf_(x)
PT_HD void sincosf_(float x, float* sn, float* cs) {
    int q;
    const float r = reduce_pio2(x, &q);
    const float s = sin_kernel(r), c = cos_kernel(r);
    switch (q) {
        case 0: *sn = s; *cs = c; break;
        case 1: *sn = c; *cs = -s; break;
        case 2: *sn = -s; *cs = -c; break;
        default: *sn = -c; *cs = s; break;
    }
}

// asin(z) for |z| <= 1/2 (Taylor to z^25)
PT_HD float asin_kernel(float z) {
    const float z2 = z * z;
    float p = 0x1.a6863ep-8f;
    p = fma_(p, z2, 0x1.df3bd4p-8f);
    p = fma_(p, z2, 0x1.12ef3cp-7f);
    p = fma_(p, z2, 0x1.3fde50p-7f);
    p = fma_(p, z2, 0x1.7a8788p-7f);
    p = fma_(p, z2, 0x1.c9999ap-7f);
    p = fma_(p, z2, 0x1.1c4ec4p-6f);
    p = fma_(p, z2, 0x1.6e8ba2p-6f);
    p = fma_(p, z2, 0x1.f1c71cp-6f);
    p = fma_(p, z2, 0x1.6db6dcp-5f);
    p = fma_(p, z2, 0x1.333334p-4f);
    p = fma_(p, z2, 0x1.555556p-3f);
    return fma_(z * z2, p, z);
}

PT_HD float acosf_(float x) {
    const float ax = abs_(x);
    if (!(ax <= 1.0f)) return u2f(0x7fc00000u);  // NaN for |x| > 1 or NaN
    if (ax <= 0.5f) {
        // pi/2 - asin(x), with the low part of pi/2 added back
        return (kPio2C1 - asin_kernel(x)) + kPio2C2;
    }
    const float s = sqrt_((1.0f - ax) * 0.5f);
    const float r = 2.0f * asin_kernel(s);
    if (x < 0.0f) return (kPi - r) + kPiLo;
    return r;
}

// atan(z) for |z| <= 2 - sqrt(3) (Taylor to z^17)
PT_HD float atan_kernel(float z) {
    const float z2 = z * z;
    float p = 0x1.e1e1e2p-5f;
    p = fma_(p, z2, -0x1.111112p-4f);
    p = fma_(p, z2, 0x1.3b13b2p-4f);
    p = fma_(p, z2, -0x1.745d18p-4f);
    p = fma_(p, z2, 0x1.c71c72p-4f);
    p = fma_(p, z2, -0x1.24924ap-3f);
    p = fma_(p, z2, 0x1.99999ap-3f);
    p = fma_(p, z2, -0x1.555556p-2f);
    return fma_(z * z2, p, z);
}

// atan(z) for 0 <= z <= 1
PT_HD float atan01(float z) {
    if (z <= 0.26794919f) return atan_kernel(z);
    const float t = div_(fma_(z, kSqrt3, -1.0f), kSqrt3 + z);
    return kPi6 + (atan_kernel(t) + kPi6Lo);
}

// atan2 with the C99 conventions for signed zeros; NaN in, NaN out.
PT_HD float atan2f_(float y, float x) {
    if (y != y || x != x) return u2f(0x7fc00000u);
    const float ax = abs_(x), ay = abs_(y);
    const bool x_neg = (f2u(x) >> 31) != 0;
    float a;
    if (ay == 0.0f) {
        a = x_neg ? kPi : 0.0f;
    } else if (ax == 0.0f) {
        a = kPio2C1;
    } else if (ax == ay) {
        // both finite or both infinite: +-pi/4 or +-3pi/4
        a = x_neg ? 3.0f * 0.5f * kPio2C1 : 0.5f * kPio2C1;
    } else if (ay > ax) {
        // angle from the y axis
        const float z = div_(ax, ay);
        a = (kPio2C1 - atan01(z)) + kPio2C2;
        if (x_neg) a = (kPi - a) + kPiLo;
    } else {
        const float z = div_(ay, ax);
        a = atan01(z);
        if (x_neg) a = (kPi - a) + kPiLo;
    }
    return copysign_(a, y);
}

// log2(x) for finite x > 0
PT_HD float log2f_(float x) {
    int e_adj = 0;
    if (x < 0x1p-126f) {
        x = x * 0x1p23f;
        e_adj = -23;
    }
    const uint32_t u = f2u(x);
    int e = (int)((u >> 23) & 0xffu) - 127 + e_adj;
    float m = u2f((u & 0x007fffffu) | 0x3f800000u);  // [1, 2)
    if (m > kSqrt2) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = div_(m - 1.0f, m + 1.0f);  // |s| <= 0.1716
    const float s2 = s * s;
    float p = 0x1.3b13b2p-4f;                  // 1/13
    p = fma_(p, s2, 0x1.745d18p-4f);           // 1/11
    p = fma_(p, s2, 0x1.c71c72p-4f);           // 1/9
    p = fma_(p, s2, 0x1.24924ap-3f);           // 1/7
    p = fma_(p, s2, 0x1.99999ap-3f);           // 1/5
    p = fma_(p, s2, 0x1.555556p-2f);           // 1/3
    const float two_s = 2.0f * s;
    const float ln_m = fma_(two_s * s2, p, two_s);
    return fma_(ln_m, kLog2e, (float)e);
}

// 2^t
PT_HD float exp2f_(float t) {
    if (t != t) return t;
    if (t >= 128.0f) return u2f(0x7f800000u);
    if (t < -151.0f) return 0.0f;
    const float k = floor_(t + 0.5f);
    const float f = t - k;  // exact, |f| <= 1/2
    const float g = f * kLn2;
    float p = 0x1.27e4fcp-22f;  // 1/10!
    p = fma_(p, g, 0x1.71de3ap-19f);
    p = fma_(p, g, 0x1.a01a02p-16f);
    p = fma_(p, g, 0x1.a01a02p-13f);
    p = fma_(p, g, 0x1.6c16c2p-10f);
    p = fma_(p, g, 0x1.111112p-7f);
    p = fma_(p, g, 0x1.555556p-5f);
    p = fma_(p, g, 0x1.555556p-3f);
    p = fma_(p, g, 0.5f);
    p = fma_(p, g, 1.0f);
    const float em = fma_(p, g, 1.0f);
    int ki = (int)k;
    if (ki >= -126) return em * u2f((uint32_t)(ki + 127) << 23);
    // subnormal result: scale in two steps
    return (em * 0x1p-126f) * u2f((uint32_t)(ki + 126 + 127) << 23);
}

// pow(x, y) for x >= 0 (the only case the shader uses), WGSL's definition
// exp2(y * log2(x)) with pow(0, y > 0) = 0.
PT_HD float powf_(float x, float y) {
    if (x != x || y != y) return u2f(0x7fc00000u);
    if (x < 0.0f) return u2f(0x7fc00000u);
    if (x == 0.0f) return y > 0.0f ? 0.0f : (y == 0.0f ? 1.0f : u2f(0x7f800000u));
    if (x == 1.0f || y == 0.0f) return 1.0f;
    if (x == u2f(0x7f800000u)) return y > 0.0f ? x : 0.0f;
    return exp2f_(y * log2f_(x));
}

}  // namespace ptm
