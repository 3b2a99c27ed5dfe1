// Frames with rows 0 and 1 in paired FP32 (FFMA2 / FMUL2 on sm_100+), their warp
// scan, and the named-barrier handoff of the four-warps-per-chain kernels; shared by
// the Angles2Backbone and Angles2Coords kernels.
#pragma once
#include <cuda_runtime.h>

#include "tpl_common.cuh"
#include "tpl_sincos.cuh"

namespace tpl {

// A frame with rows 0 and 1 held as pairs (one paired-FP32 instruction updates both
// rows) and row 2 as scalars: c[j] = (R[0][j], R[1][j]), r2[j] = R[2][j].
struct PairFrame {
    float2 c[3];
    float r2[3];
    float2 p;
    float p2;
};

__device__ __forceinline__ PairFrame to_pair(const Frame<float> &f) {
    PairFrame g;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        g.c[j] = make_float2(f.r[j], f.r[3 + j]);
        g.r2[j] = f.r[6 + j];
    }
    g.p = make_float2(f.p[0], f.p[1]);
    g.p2 = f.p[2];
    return g;
}
__device__ __forceinline__ void from_pair(const PairFrame &g, Frame<float> &f) {
#pragma unroll
    for (int j = 0; j < 3; j++) {
        f.r[j] = g.c[j].x;
        f.r[3 + j] = g.c[j].y;
        f.r[6 + j] = g.r2[j];
    }
    f.p[0] = g.p.x;
    f.p[1] = g.p.y;
    f.p[2] = g.p2;
}

__device__ __forceinline__ PairFrame pair_identity() {
    PairFrame g;
    g.c[0] = make_float2(1.f, 0.f);
    g.c[1] = make_float2(0.f, 1.f);
    g.c[2] = make_float2(0.f, 0.f);
    g.r2[0] = 0.f;
    g.r2[1] = 0.f;
    g.r2[2] = 1.f;
    g.p = make_float2(0.f, 0.f);
    g.p2 = 0.f;
    return g;
}

// compose (tpl_common.cuh) on PairFrames, c = a o b: 12 paired and 12 scalar
// operations, with the same rounding as the scalar form (each output is the same
// chain of fused multiply-adds).
__device__ __forceinline__ PairFrame compose_pair(const PairFrame &a, const PairFrame &b) {
    PairFrame c;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const float b0 = b.c[j].x, b1 = b.c[j].y, b2 = b.r2[j];  // column j of b's rotation
        c.c[j] = __ffma2_rn(a.c[0], f2(b0), __ffma2_rn(a.c[1], f2(b1), __fmul2_rn(a.c[2], f2(b2))));
        c.r2[j] = fmaf(a.r2[0], b0, fmaf(a.r2[1], b1, a.r2[2] * b2));
    }
    c.p = __ffma2_rn(a.c[0], f2(b.p.x), __ffma2_rn(a.c[1], f2(b.p.y), __ffma2_rn(a.c[2], f2(b.p2), a.p)));
    c.p2 = fmaf(a.r2[0], b.p.x, fmaf(a.r2[1], b.p.y, fmaf(a.r2[2], b.p2, a.p2)));
    return c;
}

__device__ __forceinline__ PairFrame shfl_up_pair(const PairFrame &f, int delta) {
    PairFrame o;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        o.c[j].x = __shfl_up_sync(0xffffffffu, f.c[j].x, delta);
        o.c[j].y = __shfl_up_sync(0xffffffffu, f.c[j].y, delta);
        o.r2[j] = __shfl_up_sync(0xffffffffu, f.r2[j], delta);
    }
    o.p.x = __shfl_up_sync(0xffffffffu, f.p.x, delta);
    o.p.y = __shfl_up_sync(0xffffffffu, f.p.y, delta);
    o.p2 = __shfl_up_sync(0xffffffffu, f.p2, delta);
    return o;
}

__device__ __forceinline__ PairFrame shfl_idx_pair(const PairFrame &f, int src) {
    PairFrame o;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        o.c[j].x = __shfl_sync(0xffffffffu, f.c[j].x, src);
        o.c[j].y = __shfl_sync(0xffffffffu, f.c[j].y, src);
        o.r2[j] = __shfl_sync(0xffffffffu, f.r2[j], src);
    }
    o.p.x = __shfl_sync(0xffffffffu, f.p.x, src);
    o.p.y = __shfl_sync(0xffffffffu, f.p.y, src);
    o.p2 = __shfl_sync(0xffffffffu, f.p2, src);
    return o;
}

__device__ __forceinline__ void renormalize_pair(PairFrame &g) {
    Frame<float> f;
    from_pair(g, f);
    renormalize(f);
    g = to_pair(f);
}

// warp_exclusive_total on PairFrames: the exclusive prefix of the lane transforms in
// lane order (Kogge-Stone over shuffles), and the warp total.
__device__ __forceinline__ PairFrame warp_exclusive_total_pair(PairFrame t, int lane, bool renorm,
                                                               PairFrame &total) {
    if (renorm) renormalize_pair(t);
#pragma unroll
    for (int off = 1; off < kWarp; off <<= 1) {
        const PairFrame o = shfl_up_pair(t, off);
        if (lane >= off) t = compose_pair(o, t);
    }
    total = shfl_idx_pair(t, 31);
    PairFrame exc = shfl_up_pair(t, 1);
    if (lane == 0) exc = pair_identity();
    return exc;
}

__device__ __forceinline__ void pair_store(float *dst, const PairFrame &g) {
    Frame<float> f;
    from_pair(g, f);
    frame_store(dst, f);
}

template <typename S>  // float, or double rounded to FP32
__device__ __forceinline__ PairFrame pair_load(const S *src) {
    Frame<float> f;
    frame_load(f, src);
    return to_pair(f);
}

// apply_joint (tpl_common.cuh) on a PairFrame: 9 paired and 9 scalar operations.
__device__ __forceinline__ void apply_joint_pair(PairFrame &f, float cb, float sb, float d, float ca, float sa) {
    const float2 c0 = f.c[0], c1 = f.c[1], c2 = f.c[2];
    const float2 n0 = __ffma2_rn(c0, f2(cb), __fmul2_rn(c2, f2(-sb)));
    const float2 n2 = __ffma2_rn(c0, f2(sb), __fmul2_rn(c2, f2(cb)));
    f.p = __ffma2_rn(f2(d), n0, f.p);
    f.c[0] = n0;
    f.c[1] = __ffma2_rn(c1, f2(ca), __fmul2_rn(n2, f2(sa)));
    f.c[2] = __ffma2_rn(n2, f2(ca), __fmul2_rn(c1, f2(-sa)));
    const float e0 = f.r2[0], e1 = f.r2[1], e2 = f.r2[2];
    const float m0 = fmaf(e0, cb, -e2 * sb);
    const float m2 = fmaf(e0, sb, e2 * cb);
    f.p2 = fmaf(d, m0, f.p2);
    f.r2[0] = m0;
    f.r2[1] = fmaf(e1, ca, m2 * sa);
    f.r2[2] = fmaf(m2, ca, -e1 * sa);
}

// Handoff between the warps of a CTA that share one chain (chunk k on one warp,
// chunk k + 1 on the next): the carry into chunk k passes through shared-memory slot
// k % NW under named barrier 1 + k % NW with 64 threads, the producer warp arriving
// and the consumer warp syncing.  Literal barrier ids, so that only barriers 1..NW
// (NW = 4 or 8) are reserved for the CTA.
template <int NW = 4>
__device__ __forceinline__ void ring_signal(int k) {
    static_assert(NW == 4 || NW == 8, "four or eight warps per chain");
    __syncwarp();
    __threadfence_block();
    switch (k & (NW - 1)) {
        case 0: asm volatile("bar.arrive 1, 64;" ::: "memory"); break;
        case 1: asm volatile("bar.arrive 2, 64;" ::: "memory"); break;
        case 2: asm volatile("bar.arrive 3, 64;" ::: "memory"); break;
        case 3: asm volatile("bar.arrive 4, 64;" ::: "memory"); break;
        case 4: asm volatile("bar.arrive 5, 64;" ::: "memory"); break;
        case 5: asm volatile("bar.arrive 6, 64;" ::: "memory"); break;
        case 6: asm volatile("bar.arrive 7, 64;" ::: "memory"); break;
        default: asm volatile("bar.arrive 8, 64;" ::: "memory"); break;
    }
}
template <int NW = 4>
__device__ __forceinline__ void ring_wait(int k) {
    static_assert(NW == 4 || NW == 8, "four or eight warps per chain");
    switch (k & (NW - 1)) {
        case 0: asm volatile("bar.sync 1, 64;" ::: "memory"); break;
        case 1: asm volatile("bar.sync 2, 64;" ::: "memory"); break;
        case 2: asm volatile("bar.sync 3, 64;" ::: "memory"); break;
        case 3: asm volatile("bar.sync 4, 64;" ::: "memory"); break;
        case 4: asm volatile("bar.sync 5, 64;" ::: "memory"); break;
        case 5: asm volatile("bar.sync 6, 64;" ::: "memory"); break;
        case 6: asm volatile("bar.sync 7, 64;" ::: "memory"); break;
        default: asm volatile("bar.sync 8, 64;" ::: "memory"); break;
    }
}

}  // namespace tpl
