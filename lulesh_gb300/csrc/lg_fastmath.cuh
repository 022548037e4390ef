// lg_fastmath.cuh -- arithmetic helpers of the mixed-precision path.
//
// On GB300 the FP64 pipe issues at 1/74 of the FP32 rate, so the mixed path
// keeps FP64 only where its accuracy is needed and moves everything exact or
// approximate-enough elsewhere:
//   * FP64 <-> FP32 conversions on the integer pipe (bit re-packing);
//   * FP64 reciprocal and square root by Newton-Raphson refinement of the
//     hardware approximations (PTX rcp.approx.ftz.f64 / rsqrt.approx.ftz.f64):
//     each step r <- r + r(1 - a r) squares the relative error, so two steps
//     from the ~2^-20 seed leave the last bit or two of the double;
//   * comparisons of doubles on the integer pipe through the order-preserving
//     key of IEEE bit patterns (sign-magnitude -> two's complement order).
// None of these is used by the FP64 paths.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace lg {
namespace fast {

// double -> float, rounded to nearest (ties to even), on the integer pipe in
// 32-bit operations: the high word re-biased from the double to the float
// exponent and joined with the top 3 bits of the low word gives the
// truncated float; its 29 dropped bits plus its lowest kept bit plus half an
// ulp less one carry into bit 29 exactly when the value rounds up (ties to
// even), and that carry steps the mantissa, the exponent on overflow, and
// the largest finite float to infinity.  Values below the float normal range
// become zero, values above it infinity.
__device__ __forceinline__ float to_f32(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned mag = hi & 0x7fffffffu, ed = mag >> 20;
    unsigned r = ((mag - (896u << 20)) << 3) | (lo >> 29);
    r += ((lo & 0x1fffffffu) + (r & 1u) + 0x0fffffffu) >> 29;
    r = ed <= 896u ? 0u : (ed >= 1151u ? 0x7f800000u : r);
    return __uint_as_float((hi & 0x80000000u) | r);
}

// float -> double, exact for normal values (float subnormals become zero).
__device__ __forceinline__ double to_f64(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned sign = u & 0x80000000u;
    const unsigned ex = (u >> 23) & 0xffu;
    unsigned hi, lo;
    if (ex == 0) {
        hi = sign;
        lo = 0;
    } else {
        const unsigned e64 = (ex == 255u) ? 0x7ffu : ex - 127u + 1023u;
        hi = sign | (e64 << 20) | ((u & 0x7fffffu) >> 3);
        lo = u << 29;
    }
    return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ double rcp_nr(double a)
{
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(a));
    double e = fma(-a, r, 1.0);
    r = fma(r, e, r);
    e = fma(-a, r, 1.0);
    return fma(r, e, r);
}

// sqrt(a) for a > 0: s = a * rsqrt(a), then two corrections
// s <- s + (a - s^2) * (rsqrt(a) / 2)
__device__ __forceinline__ double sqrt_nr(double a)
{
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(a));
    double s = a * y;
    const double h = 0.5 * y;
    double r = fma(-s, s, a);
    s = fma(r, h, s);
    r = fma(-s, s, a);
    return fma(r, h, s);
}

// order-preserving integer key of a double (NaN excluded; -0 sorts just
// below +0, the one difference from IEEE ordering)
__device__ __forceinline__ unsigned long long order_key(double v)
{
    const long long b = __double_as_longlong(v);
    const unsigned long long mask = (unsigned long long)(b >> 63) | 0x8000000000000000ull;
    return (unsigned long long)b ^ mask;
}

// FP64 EOS operations of the mixed path (same interface as IeeeOps)
struct FastOps {
    static __device__ __forceinline__ double div(double a, double b) { return a * rcp_nr(b); }
    static __device__ __forceinline__ double sqrt_(double a) { return sqrt_nr(a); }
    static __device__ __forceinline__ bool lt(double a, double b) { return order_key(a) < order_key(b); }
    static __device__ __forceinline__ bool le(double a, double b) { return order_key(a) <= order_key(b); }
    // |a| < b for b >= 0: magnitude bits compare like the values
    static __device__ __forceinline__ bool abs_lt(double a, double b)
    {
        return ((unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull) <
               (unsigned long long)__double_as_longlong(b);
    }
    // the sound-speed numerator pbvc e + v^2 bvc p with its roundings fixed,
    // so every kernel that evaluates it (the fused per-element path and the
    // shared-item path) gets the same bits whatever the compiler contracts
    static __device__ __forceinline__ double ss_num(double pbvc, double e, double v, double bvc,
                                                    double p)
    {
        return __fma_rn(pbvc, e, __dmul_rn(__dmul_rn(__dmul_rn(v, v), bvc), p));
    }
};

}  // namespace fast
}  // namespace lg
