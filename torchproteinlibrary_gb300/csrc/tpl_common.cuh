// Shared device code for the chain-kinematics kernels (sm_103a).
//
// A "frame" is a rigid transform (3x3 rotation R, row-major, and translation p).
// One bond joint of TorchProteinLibrary's kinematic chain is
//     B(alpha, beta, d) = Ry(beta) * Tx(d) * Rx(alpha)
// (Math/cMatrix44.cpp:47-52, Layers/FullAtomModel/cConformation.cpp:7-13), and a
// chain frame advances as A_i = A_{i-1} * B_i
// (Layers/ReducedModel/cBackboneProteinCPUKernels.cpp:42-58).
//
// Instead of forming B as a 4x4 and multiplying, the kernels apply it to the
// frame's columns in factored form: R <- R*Ry(beta) touches columns 0 and 2,
// p <- p + d*(R*Ry)[:,0], then R <- R*Rx(alpha) touches columns 1 and 2.
// That is 27 FMA per joint, and the only rounded constants are cos/sin of
// beta and alpha.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tpl {

constexpr int kWarp = 32;

template <typename T>
struct Frame {
    T r[9];  // row-major rotation
    T p[3];  // translation (the joint's atom position)
};

template <typename T>
__device__ __forceinline__ void frame_identity(Frame<T> &f) {
#pragma unroll
    for (int i = 0; i < 9; i++) f.r[i] = (i % 4 == 0) ? T(1) : T(0);
    f.p[0] = f.p[1] = f.p[2] = T(0);
}

// c = a o b  (apply b first, then a):  R = Ra Rb,  p = Ra pb + pa
template <typename T>
__device__ __forceinline__ Frame<T> compose(const Frame<T> &a, const Frame<T> &b) {
    Frame<T> c;
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int j = 0; j < 3; j++)
            c.r[3 * i + j] = fma(a.r[3 * i], b.r[j], fma(a.r[3 * i + 1], b.r[3 + j], a.r[3 * i + 2] * b.r[6 + j]));
        c.p[i] = fma(a.r[3 * i], b.p[0], fma(a.r[3 * i + 1], b.p[1], fma(a.r[3 * i + 2], b.p[2], a.p[i])));
    }
    return c;
}

// Right-multiply the frame by one joint Ry(beta) Tx(d) Rx(alpha), given
// (cb, sb) = (cos, sin) beta and (ca, sa) = (cos, sin) alpha.
template <typename T>
__device__ __forceinline__ void apply_joint(Frame<T> &f, T cb, T sb, T d, T ca, T sa) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
        T c0 = f.r[3 * i], c1 = f.r[3 * i + 1], c2 = f.r[3 * i + 2];
        T n0 = fma(c0, cb, -c2 * sb);
        T n2 = fma(c0, sb, c2 * cb);
        f.p[i] = fma(d, n0, f.p[i]);
        f.r[3 * i] = n0;
        f.r[3 * i + 1] = fma(c1, ca, n2 * sa);
        f.r[3 * i + 2] = fma(n2, ca, -c1 * sa);
    }
}

// Right-multiply by Rx(alpha) only (a joint with beta = 0 and d = 0).
template <typename T>
__device__ __forceinline__ void apply_rx(Frame<T> &f, T ca, T sa) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
        T c1 = f.r[3 * i + 1], c2 = f.r[3 * i + 2];
        f.r[3 * i + 1] = fma(c1, ca, c2 * sa);
        f.r[3 * i + 2] = fma(c2, ca, -c1 * sa);
    }
}

// World position of a point given in the frame's local coordinates.
template <typename T>
__device__ __forceinline__ void frame_point(const Frame<T> &f, T x, T y, T z, T *out) {
#pragma unroll
    for (int i = 0; i < 3; i++) out[i] = fma(f.r[3 * i], x, fma(f.r[3 * i + 1], y, fma(f.r[3 * i + 2], z, f.p[i])));
}

// One Newton-Schulz step towards the nearest rotation: R <- R (3I - R^T R) / 2.
// FP32 frames drift in scale because every rounded (cos, sin) pair has a norm
// slightly off 1; the drift is coherent along a chain, so the kernels pull
// scan aggregates back onto SO(3).
template <typename T>
__device__ __forceinline__ void renormalize(Frame<T> &f) {
    T g[6];  // symmetric R^T R: (00, 01, 02, 11, 12, 22)
    const T *r = f.r;
    g[0] = fma(r[0], r[0], fma(r[3], r[3], r[6] * r[6]));
    g[1] = fma(r[0], r[1], fma(r[3], r[4], r[6] * r[7]));
    g[2] = fma(r[0], r[2], fma(r[3], r[5], r[6] * r[8]));
    g[3] = fma(r[1], r[1], fma(r[4], r[4], r[7] * r[7]));
    g[4] = fma(r[1], r[2], fma(r[4], r[5], r[7] * r[8]));
    g[5] = fma(r[2], r[2], fma(r[5], r[5], r[8] * r[8]));
    // H = (3I - G)/2
    T h00 = T(1.5) - T(0.5) * g[0], h11 = T(1.5) - T(0.5) * g[3], h22 = T(1.5) - T(0.5) * g[5];
    T h01 = T(-0.5) * g[1], h02 = T(-0.5) * g[2], h12 = T(-0.5) * g[4];
    T n[9];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        T a = r[3 * i], b = r[3 * i + 1], c = r[3 * i + 2];
        n[3 * i] = fma(a, h00, fma(b, h01, c * h02));
        n[3 * i + 1] = fma(a, h01, fma(b, h11, c * h12));
        n[3 * i + 2] = fma(a, h02, fma(b, h12, c * h22));
    }
#pragma unroll
    for (int i = 0; i < 9; i++) f.r[i] = n[i];
}

template <typename T>
__device__ __forceinline__ Frame<T> shfl_up_frame(const Frame<T> &f, int delta) {
    Frame<T> o;
#pragma unroll
    for (int i = 0; i < 9; i++) o.r[i] = __shfl_up_sync(0xffffffffu, f.r[i], delta);
#pragma unroll
    for (int i = 0; i < 3; i++) o.p[i] = __shfl_up_sync(0xffffffffu, f.p[i], delta);
    return o;
}

// Inclusive warp scan of frames in lane order (lane 0 applied first):
// out_l = f_0 o f_1 o ... o f_l.   Kogge-Stone over shuffles.
template <typename T>
__device__ __forceinline__ Frame<T> warp_scan_frames(Frame<T> f, int lane) {
#pragma unroll
    for (int off = 1; off < kWarp; off <<= 1) {
        Frame<T> o = shfl_up_frame(f, off);
        if (lane >= off) f = compose(o, f);
    }
    return f;
}

template <typename D, typename S>
__device__ __forceinline__ Frame<D> frame_cast(const Frame<S> &s) {
    Frame<D> d;
#pragma unroll
    for (int i = 0; i < 9; i++) d.r[i] = D(s.r[i]);
#pragma unroll
    for (int i = 0; i < 3; i++) d.p[i] = D(s.p[i]);
    return d;
}

template <typename T>
__device__ __forceinline__ void frame_store(T *dst, const Frame<T> &f) {
#pragma unroll
    for (int i = 0; i < 9; i++) dst[i] = f.r[i];
#pragma unroll
    for (int i = 0; i < 3; i++) dst[9 + i] = f.p[i];
}
template <typename T, typename S>
__device__ __forceinline__ void frame_load(Frame<T> &f, const S *src) {
#pragma unroll
    for (int i = 0; i < 9; i++) f.r[i] = T(src[i]);
#pragma unroll
    for (int i = 0; i < 3; i++) f.p[i] = T(src[9 + i]);
}

__device__ __forceinline__ void sincos_t(float a, float *s, float *c) { sincosf(a, s, c); }
__device__ __forceinline__ void sincos_t(double a, double *s, double *c) { sincos(a, s, c); }

__device__ __forceinline__ void cross3(const float *a, const float *b, float *o) {
    o[0] = fmaf(a[1], b[2], -a[2] * b[1]);
    o[1] = fmaf(a[2], b[0], -a[0] * b[2]);
    o[2] = fmaf(a[0], b[1], -a[1] * b[0]);
}
__device__ __forceinline__ void cross3(const double *a, const double *b, double *o) {
    o[0] = fma(a[1], b[2], -a[2] * b[1]);
    o[1] = fma(a[2], b[0], -a[0] * b[2]);
    o[2] = fma(a[0], b[1], -a[1] * b[0]);
}

// ------------------------------------------------------------ flags / waits
// Tile records are published with a release store of a flag word
// (epoch << 2 | state) after the payload, and read after an acquire load.
enum : unsigned { kFlagNone = 0u, kFlagAgg = 1u, kFlagInc = 2u };

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

}  // namespace tpl

namespace tpl {

// ---------------------------------------------------------------- sincos
// Table-driven sin/cos for |a| <= pi (Tang's method of tabulated breakpoints
// plus a short Taylor correction): a = k*h + r with h = pi/32, |r| <= pi/64,
//   sin a = S_k + (S_k (cos r - 1) + C_k sin r),  cos a = C_k + (C_k (cos r - 1) - S_k sin r),
// where (S_k, C_k) = (sin, cos)(k h) are tabulated as hi + lo float pairs, so the
// result is within about one rounding of the FP32 sin/cos.  sin r and cos r - 1
// are Taylor polynomials (terms below r^7/5040 ~ 1e-13 dropped).  Arguments
// outside [-pi, pi] take sincosf.
struct SinCosTable {
    float4 e[65];  // (S_hi, C_hi, S_lo, C_lo) for k = -32..32
};

// Built at compile time by make_sincos_table() in tpl_topology.cuh (FP64 trig).
__device__ __forceinline__ void sincos_tab(const float4 *tab, float a, float *s, float *c) {
    if (fabsf(a) > 3.14159274f) {
        sincosf(a, s, c);
        return;
    }
    constexpr float kInvH = 10.185916357881302f;       // 32 / pi
    constexpr float kHhi = 0.09817477315664291f;        // float(pi / 32)
    constexpr float kHlo = -2.7319618e-09f;             // pi/32 - kHhi (rounded)
    const float k = rintf(a * kInvH);
    float r = fmaf(-k, kHhi, a);
    r = fmaf(-k, kHlo, r);
    const float r2 = r * r;
    const float sr = fmaf(r * r2, fmaf(r2, 1.0f / 120.0f, -1.0f / 6.0f), r);
    const float cm1 = r2 * fmaf(r2, 1.0f / 24.0f, -0.5f);
    const float4 e = tab[(int)k + 32];
    *s = e.x + fmaf(e.x, cm1, fmaf(e.y, sr, e.z));
    *c = e.y + fmaf(e.y, cm1, fmaf(-e.x, sr, e.w));
}

}  // namespace tpl
