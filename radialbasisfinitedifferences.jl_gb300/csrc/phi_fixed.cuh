// |p_i - p_j|^3 of two stencil nodes without FP64 arithmetic.
//
// On GB300 every FP64 warp instruction holds the SM sub-partition for ~64 cycles whatever else
// is in flight, so the pairwise PHS block phi(r) = r^3 (435 pairs for a 30-node stencil) is
// evaluated here on the integer and FP32 pipes instead:
//
//   * coordinates become 61-bit fixed point (exact for |x| >= 2^-9; |x| < 2 required),
//   * dx^2 + dy^2 is formed exactly in 128-bit integers after a common normalising shift,
//   * M = the top 64 bits of r^2 (scaled by an even power of two into [2^62, 2^64)),
//   * sqrt(M) = (S1 + c1) 2^-16: an FP32 reciprocal-square-root seed, one Newton step with an
//     exact integer residual M - S0^2 (S1 in 16-bit fixed point), and the last correction
//     c1 = (M 2^32 - S1^2) / (2 S1) folded into the product M sqrt(M) as a small FP32 term,
//   * M^1.5 is rounded to 53 bits and its double is assembled from the exponent bookkeeping.
//
// The result is within one unit in the last place of the exact r^3 of the fixed-point
// coordinates (CPU check against exact rational arithmetic in the test suite).  The reference
// evaluates the same quantity as r = norm(x_i - x_j); r^3 in FP64 (src/rbfblock.jl:1-23 with
// src/rbfbasis.jl:9-30), i.e. with several roundings, so both agree to a few ulps.
//
// The header compiles as plain C++ as well (no CUDA types), which is how the CPU test drives
// it; that build takes its square-root seed from 1/sqrtf, perturbed by up to 2^-20 relative so
// that the test covers the hardware approximation's error with margin.
#pragma once

#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define RBFFD_FX_HD __host__ __device__ __forceinline__
#else
#define RBFFD_FX_HD inline
#endif

namespace rbffd_fx {

RBFFD_FX_HD uint64_t umulhi(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// Leading zeros of a nonzero 64-bit value.
RBFFD_FX_HD int clz64(uint64_t x)
{
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

RBFFD_FX_HD float bits_f32(uint32_t b)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float f;
    memcpy(&f, &b, 4);
    return f;
#endif
}

RBFFD_FX_HD uint32_t f32_bits(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t b;
    memcpy(&b, &f, 4);
    return b;
#endif
}

RBFFD_FX_HD double bits_f64(uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double d;
    memcpy(&d, &b, 8);
    return d;
#endif
}

RBFFD_FX_HD uint64_t f64_bits(double d)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t b;
    memcpy(&b, &d, 8);
    return b;
#endif
}

// float(v) truncated, for v in [2^30, 2^32): the mantissa's leading one carries into the
// exponent field.
RBFFD_FX_HD float u32_to_f32_trunc(uint32_t v)
{
    const uint32_t lz = (v >> 31) ^ 1u;
    return bits_f32(((157u - lz) << 23) + ((v << lz) >> 8));
}

// ~1/sqrt(f) with relative error below 2^-20.
RBFFD_FX_HD float rsqrt_seed(float f)
{
#if defined(__CUDA_ARCH__)
    return rsqrtf(f);
#else
    const uint32_t h = f32_bits(f) * 0x9E3779B1u;
    const float jitter = ((float)(h >> 8) * 0x1p-24f - 0.5f) * 0x1p-19f;  // [-2^-20, 2^-20)
    return (1.0f / sqrtf(f)) * (1.0f + jitter);
#endif
}

RBFFD_FX_HD float i64_to_f32(int64_t v)
{
#if defined(__CUDA_ARCH__)
    return __ll2float_rn((long long)v);
#else
    return (float)v;
#endif
}

RBFFD_FX_HD int64_t f32_to_i64(float f)
{
#if defined(__CUDA_ARCH__)
    return (int64_t)__float2ll_rn(f);
#else
    return (int64_t)llrintf(f);
#endif
}

// round(f) clamped to [0, 2^32 - 1].
RBFFD_FX_HD uint32_t f32_to_u32_sat(float f)
{
#if defined(__CUDA_ARCH__)
    return __float2uint_rn(f);  // float-to-integer conversions clamp to the destination range
#else
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)llrintf(f);
#endif
}

// 61-bit fixed point of a double with |x| < 2 (exact for |x| >= 2^-9, truncated toward zero
// below; |error| < 2^-61).
RBFFD_FX_HD int64_t to_fixed61(double x)
{
    const uint64_t b = f64_bits(x);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e == 0) return 0;
    const uint64_t m = (b & 0xfffffffffffffull) | (1ull << 52);  // |x| = m 2^(e - 1075)
    const int sh = e - 1014;                                     // |X| = m 2^sh, sh <= 9
    const uint64_t mag = sh >= 0 ? (m << sh) : (sh > -64 ? (m >> -sh) : 0ull);
    return (b >> 63) ? -(int64_t)mag : (int64_t)mag;
}

// |x| < 2 (the precondition of to_fixed61), by the exponent field.
RBFFD_FX_HD bool fixed61_ok(double x) { return (f64_bits(x) & 0x7ff0000000000000ull) < 0x4000000000000000ull; }

// Round a 64-bit value v > 0 to 53 bits and return v 2^e2 as a double (normal range).
RBFFD_FX_HD double u64_scaled_to_f64(uint64_t v, int e2)
{
    const int lz = clz64(v);
    const uint64_t vn = v << lz;                               // [2^63, 2^64)
    const uint64_t mant = (vn >> 11) + ((vn >> 10) & 1ull);    // [2^52, 2^53]
    const int E = 52 + 11 - lz + e2;                           // value = mant 2^(E - 52)
    return bits_f64(((uint64_t)(E + 1023) << 52) + (mant - (1ull << 52)));
}

// r^3 (and r^2 when r2 != nullptr) of two nodes in 61-bit fixed point.
RBFFD_FX_HD double r3_fixed(int64_t xi, int64_t yi, int64_t xj, int64_t yj, double *r2)
{
    const int64_t dx = xi - xj, dy = yi - yj;  // |d| < 2^63
    uint64_t ax = dx < 0 ? 0ull - (uint64_t)dx : (uint64_t)dx;
    uint64_t ay = dy < 0 ? 0ull - (uint64_t)dy : (uint64_t)dy;
    const uint64_t mx = ax > ay ? ax : ay;
    if (mx == 0ull) {
        if (r2) *r2 = 0.0;
        return 0.0;
    }
    const int sh = clz64(mx) - 1;  // max(ax, ay) 2^sh in [2^62, 2^63)
    ax <<= sh;
    ay <<= sh;
    // R = ax^2 + ay^2 in [2^124, 2^127), as (hi, lo)
    uint64_t lo = ax * ax, hi = umulhi(ax, ax);
    const uint64_t lo2 = ay * ay;
    hi += umulhi(ay, ay);
    lo += lo2;
    hi += lo < lo2 ? 1ull : 0ull;
    // M = R 2^(s2 - 64) in [2^62, 2^64) with s2 even: r^2 = M 2^(-58 - s2 - 2 sh)
    const int s2 = clz64(hi) & ~1;
    const uint64_t M = s2 ? (hi << 2) | (lo >> 62) : hi;
    if (r2) *r2 = u64_scaled_to_f64(M, -58 - s2 - 2 * sh);
    // sqrt(M) = S: seed S0 (uint32), then S1 = S0 2^16 + c0 2^16 with c0 = (M - S0^2) / (2 S0)
    const float f = u32_to_f32_trunc((uint32_t)(M >> 32));
    const float y = rsqrt_seed(f);  // ~ 2^16 / S
    const uint32_t S0 = f32_to_u32_sat(f * y * 65536.0f);
    const int64_t D0 = (int64_t)(M - (uint64_t)S0 * S0);  // |D0| < 2^46
    const float h = y * 0x1p-17f;                         // ~ 1 / (2 S)
    const int64_t S1 = (int64_t)((uint64_t)S0 << 16) + f32_to_i64(i64_to_f32(D0) * h * 65536.0f);
    // S 2^16 = S1 + D1 h 2^-16 with D1 = M 2^32 - S1^2 (exact: |D1| < 2^60)
    const int64_t D1 = (int64_t)((M << 32) - (uint64_t)S1 * (uint64_t)S1);
    // M^1.5 2^-35 = (M S1) 2^-51 + M D1 h 2^-67
    const uint64_t Plo = M * (uint64_t)S1, Phi = umulhi(M, (uint64_t)S1);
    const float t = (i64_to_f32(D1) * h) * 0x1p-67f * (f * 0x1p32f);
    const uint64_t Q = ((Phi << 13) | (Plo >> 51)) + (uint64_t)f32_to_i64(t);
    // r^3 = M^1.5 2^(-87 - 3 s2 / 2 - 3 sh) = Q 2^(-52 - 3 s2 / 2 - 3 sh)
    return u64_scaled_to_f64(Q, -52 - 3 * (s2 >> 1) - 3 * sh);
}

}  // namespace rbffd_fx
