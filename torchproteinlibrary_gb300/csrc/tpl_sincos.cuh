// FP32 sin and cos in registers for the kernels' angle inputs (shared by the
// Angles2Backbone and Angles2Coords kernels).
#pragma once
#include <cuda_runtime.h>

namespace tpl {

// sin and cos without tables or special-function units: Cody-Waite reduction by
// pi/2 (two-term split of pi/2, exact products in the FMA) to |r| <= pi/4, then the
// Taylor series of sin to r^9 and of cos to r^10 (truncation below 2e-9 on that
// range), and the quadrant's swap and signs.  Valid for |a| <= 1e4; NaN and
// infinities give NaN.  Callers send larger arguments to sincosf.
__device__ __forceinline__ void sincos_fast(float a, float *s, float *c) {
    constexpr float kTwoOverPi = 0.636619772367581343f;
    constexpr float kPio2Hi = 1.57079637050628662f;      // float(pi / 2)
    constexpr float kPio2Lo = -4.37113900018624283e-8f;  // pi / 2 - kPio2Hi
    const float k = rintf(a * kTwoOverPi);
    float r = fmaf(-k, kPio2Hi, a);
    r = fmaf(-k, kPio2Lo, r);
    const float r2 = r * r;
    // 1/n! coefficients
    float ps = fmaf(r2, 2.7557319223985891e-6f, -1.9841269841269841e-4f);
    ps = fmaf(ps, r2, 8.3333333333333333e-3f);
    ps = fmaf(ps, r2, -1.6666666666666667e-1f);
    const float sr = fmaf(ps * r2, r, r);
    float pc = fmaf(r2, -2.7557319223985891e-7f, 2.4801587301587302e-5f);
    pc = fmaf(pc, r2, -1.3888888888888889e-3f);
    pc = fmaf(pc, r2, 4.1666666666666667e-2f);
    pc = fmaf(pc, r2, -0.5f);
    const float cr = fmaf(pc, r2, 1.0f);
    const int q = ((int)k) & 3;  // a = r + q pi/2 (mod 2 pi)
    float ss = (q & 1) ? cr : sr;
    float cc = (q & 1) ? sr : cr;
    if (q & 2) ss = -ss;
    if ((q + 1) & 2) cc = -cc;
    *s = ss;
    *c = cc;
}

// Two angles at once with the paired FP32 instructions of sm_100+ (FFMA2 / FMUL2:
// two lanes of arithmetic per issue).  Same method as sincos_fast, except that the
// reduction rounds with the 1.5 * 2^23 shift: t = a * 2/pi + 1.5 * 2^23 rounds to an
// integer in the FMA, k = t - 1.5 * 2^23 exactly, and the low bits of t's pattern
// are k mod 4, so no float-to-integer conversion is needed.  Valid for |a| <= 1e4.
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }

// sin and cos of a = r + q pi/2 (mod 2 pi) from sin r, cos r and the low bits of q: odd q
// swaps them; bit 1 of q is the sign of sin, bit 1 of q + 1 the sign of cos.
__device__ __forceinline__ void quadrant(float sr, float cr, int t_bits, float *s, float *c) {
    const unsigned u = (unsigned)t_bits;
    const bool odd = (u & 1u) != 0u;
    const unsigned ssign = (u << 30) & 0x80000000u;
    const unsigned csign = ((u + 1u) << 30) & 0x80000000u;
    *s = __uint_as_float(__float_as_uint(odd ? cr : sr) ^ ssign);
    *c = __uint_as_float(__float_as_uint(odd ? sr : cr) ^ csign);
}

__device__ __forceinline__ void sincos_fast2(float a0, float a1, float *s0, float *c0, float *s1, float *c1) {
    constexpr float kShift = 12582912.0f;  // 1.5 * 2^23
    const float2 a = make_float2(a0, a1);
    const float2 t = __ffma2_rn(a, f2(0.636619772367581343f), f2(kShift));
    const float2 k = __fadd2_rn(t, f2(-kShift));
    float2 r = __ffma2_rn(k, f2(-1.57079637050628662f), a);
    r = __ffma2_rn(k, f2(4.37113900018624283e-8f), r);
    const float2 r2 = __fmul2_rn(r, r);
    float2 ps = __ffma2_rn(r2, f2(2.7557319223985891e-6f), f2(-1.9841269841269841e-4f));
    ps = __ffma2_rn(ps, r2, f2(8.3333333333333333e-3f));
    ps = __ffma2_rn(ps, r2, f2(-1.6666666666666667e-1f));
    const float2 sr = __ffma2_rn(__fmul2_rn(ps, r2), r, r);
    float2 pc = __ffma2_rn(r2, f2(-2.7557319223985891e-7f), f2(2.4801587301587302e-5f));
    pc = __ffma2_rn(pc, r2, f2(-1.3888888888888889e-3f));
    pc = __ffma2_rn(pc, r2, f2(4.1666666666666667e-2f));
    pc = __ffma2_rn(pc, r2, f2(-0.5f));
    const float2 cr = __ffma2_rn(pc, r2, f2(1.0f));
    quadrant(sr.x, cr.x, __float_as_int(t.x), s0, c0);
    quadrant(sr.y, cr.y, __float_as_int(t.y), s1, c1);
}

__device__ __forceinline__ void sincos_poly(float a, float *s, float *c) {
    if (fabsf(a) > 1.0e4f) {
        sincosf(a, s, c);
        return;
    }
    sincos_fast(a, s, c);
}

}  // namespace tpl
