// Angles2Backbone FP32, one warp per chain (threads_per_cta = 32), sm_103a.
//
// The tile kernels of tpl_a2b.cu split long chains over CTAs and join the pieces
// by decoupled look-back.  When the batch alone fills the GPU (a few hundred
// chains or more) that machinery is pure overhead, so here one warp owns one
// chain and walks it chunk after chunk, holding the chain frame at the chunk start
// in registers.  A chunk is 32 C residues, C = 4 or 8 contiguous residues per
// lane, so every global access is a coalesced row piece of the chunk.
//
// Forward, per chunk k with chain frame F_k at its start:
//   1. each lane composes the 3C joints of its residues from identity (the joint
//      algebra of Layers/ReducedModel/cBackboneProteinCPUKernels.cpp:42-58, in the
//      factored form of tpl_common.cuh) and stages the lane-local N, CA, C
//      positions in a per-warp shared buffer;
//   2. a Kogge-Stone warp scan of the lane transforms gives each lane's exclusive
//      prefix E_l, and its world frame is P_l = F_k o E_l;
//   3. lanes map their staged positions through P_l in place and the warp stores
//      the chunk's 9 * 32C coordinates as coalesced float4 rows (zeros past the
//      chain length);
//   4. F_{k+1} = F_k o (chunk total).  The world frame at every 128-residue
//      boundary is recorded in the workspace for the backward.
// Backward (reference: cBackboneProteinCUDAKernels.cu:84-163), chunks last to
// first, starting each chunk from the frame the forward recorded:
//   1. the same walk and scan; the chunk's dL/dx is staged by a coalesced load and
//      rotated into each lane's local frame;
//   2. lane sums G = sum g, S = sum x x g are moved to the chunk frame, suffix-
//      scanned over the warp and completed by the running sums of later chunks;
//   3. each lane walks its residues backwards, accumulating (G, S), and evaluates
//      dL/dtheta_m = u_m . (S_m - x_m x G_m) for its 3C joints.
// No CTA-wide barrier, no atomics and no FP64 on this path.
#include "tpl_common.cuh"
#include "tpl_internal.h"
#include "tpl_pair.cuh"
#include "tpl_sincos.cuh"

namespace tpl {
namespace {

constexpr int kWarpsPerCta = 4;
constexpr int kRecordStride = 128;  // residues between recorded chain frames

// One recorded chain frame (rotation row-major, translation), laid over the
// workspace's record array.
struct ChainRecord {
    float f[12];
};

struct ChainArgs {
    const float *angles;
    const int *lengths;
    float *coords;
    float *grad_angles;
    const float *grad_coords;
    WsHeader *hdr;
    ChainRecord *rec;
    int B, L, nrec;
    int renorm;
    int vec;  // rows are 16-byte aligned (L % 4 == 0, aligned bases): float4 accesses
    int fp64_min;  // four-warp forward: chains at least this long hand the chain frame on in FP64 (0 = never)
    BondConsts bc;
};

__device__ __forceinline__ void record_error(WsHeader *h, int code) { atomicCAS(&h->status, 0u, (unsigned)code); }

__device__ __forceinline__ Frame<float> shfl_idx_frame(const Frame<float> &f, int src) {
    Frame<float> o;
#pragma unroll
    for (int i = 0; i < 9; i++) o.r[i] = __shfl_sync(0xffffffffu, f.r[i], src);
#pragma unroll
    for (int i = 0; i < 3; i++) o.p[i] = __shfl_sync(0xffffffffu, f.p[i], src);
    return o;
}

// Exclusive prefix of the lane transforms in lane order, and the warp total.
__device__ __forceinline__ Frame<float> warp_exclusive_total(Frame<float> t, int lane, bool renorm,
                                                             Frame<float> &total) {
    if (renorm) renormalize(t);
    const Frame<float> inc = warp_scan_frames(t, lane);
    total = shfl_idx_frame(inc, 31);
    Frame<float> exc = shfl_up_frame(inc, 1);
    if (lane == 0) frame_identity(exc);
    return exc;
}

// Sum over lanes > lane (exclusive suffix) of v, and the warp total.
__device__ __forceinline__ float warp_suffix_excl(float v, int lane, float &total) {
    float inc = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const float o = __shfl_down_sync(0xffffffffu, inc, off);
        if (lane + off < 32) inc += o;
    }
    total = __shfl_sync(0xffffffffu, inc, 0);
    return inc - v;
}

// Angles of one row for residues j..j+3, zero from len on.
__device__ __forceinline__ void load4(const float *row, int j, int len, bool vec, float (&v)[4]) {
    if (vec) {
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
        if (j < len) x = __ldg(reinterpret_cast<const float4 *>(row + j));
        v[0] = x.x;
        v[1] = j + 1 < len ? x.y : 0.f;
        v[2] = j + 2 < len ? x.z : 0.f;
        v[3] = j + 3 < len ? x.w : 0.f;
    } else {
#pragma unroll
        for (int i = 0; i < 4; i++) v[i] = j + i < len ? __ldg(row + j + i) : 0.f;
    }
}

// Four residues of a lane's walk: composes their 12 joints onto f and writes the
// lane-local N, CA, C positions (36 floats, 9 float4s) to seg.  FAST: every angle
// is known to be within the range of sincos_fast.
template <bool FAST>
__device__ __forceinline__ void walk4(const BondConsts &bc, Frame<float> &f, const float (&a0)[4],
                                      const float (&a1)[4], const float (&a2)[4], float *seg) {
    float buf[36];
    if constexpr (FAST) {
        float so[4], co[4];  // omega pairs (residues 0-1, 2-3)
        sincos_fast2(a2[0], a2[1], &so[0], &co[0], &so[1], &co[1]);
        sincos_fast2(a2[2], a2[3], &so[2], &co[2], &so[3], &co[3]);
        PairFrame g = to_pair(f);
#pragma unroll
        for (int r = 0; r < 4; r++) {
            float s0, c0, s1, c1;
            sincos_fast2(a0[r], a1[r], &s0, &c0, &s1, &c1);
            buf[9 * r] = g.p.x; buf[9 * r + 1] = g.p.y; buf[9 * r + 2] = g.p2;
            apply_joint_pair(g, bc.cb[0], bc.sb[0], bc.d[0], c0, s0);
            buf[9 * r + 3] = g.p.x; buf[9 * r + 4] = g.p.y; buf[9 * r + 5] = g.p2;
            apply_joint_pair(g, bc.cb[1], bc.sb[1], bc.d[1], c1, s1);
            buf[9 * r + 6] = g.p.x; buf[9 * r + 7] = g.p.y; buf[9 * r + 8] = g.p2;
            apply_joint_pair(g, bc.cb[2], bc.sb[2], bc.d[2], co[r], so[r]);
#pragma unroll
            for (int q = 0; q < 9; q++)  // flush the float4s this residue completed
                if (4 * q + 3 <= 9 * r + 8 && 4 * q + 3 > 9 * r - 1)
                    *reinterpret_cast<float4 *>(seg + 4 * q) =
                        make_float4(buf[4 * q], buf[4 * q + 1], buf[4 * q + 2], buf[4 * q + 3]);
        }
        from_pair(g, f);
    } else {
#pragma unroll
        for (int r = 0; r < 4; r++) {
            float s0, c0, s1, c1, s2, c2;
            sincos_poly(a0[r], &s0, &c0);
            sincos_poly(a1[r], &s1, &c1);
            sincos_poly(a2[r], &s2, &c2);
            buf[9 * r] = f.p[0]; buf[9 * r + 1] = f.p[1]; buf[9 * r + 2] = f.p[2];
            apply_joint(f, bc.cb[0], bc.sb[0], bc.d[0], c0, s0);
            buf[9 * r + 3] = f.p[0]; buf[9 * r + 4] = f.p[1]; buf[9 * r + 5] = f.p[2];
            apply_joint(f, bc.cb[1], bc.sb[1], bc.d[1], c1, s1);
            buf[9 * r + 6] = f.p[0]; buf[9 * r + 7] = f.p[1]; buf[9 * r + 8] = f.p[2];
            apply_joint(f, bc.cb[2], bc.sb[2], bc.d[2], c2, s2);
#pragma unroll
            for (int q = 0; q < 9; q++)  // flush the float4s this residue completed
                if (4 * q + 3 <= 9 * r + 8 && 4 * q + 3 > 9 * r - 1)
                    *reinterpret_cast<float4 *>(seg + 4 * q) =
                        make_float4(buf[4 * q], buf[4 * q + 1], buf[4 * q + 2], buf[4 * q + 3]);
        }
    }
}

// Walk of one lane's C residues (j0..j0+C-1) from identity, in groups of four;
// positions (9C floats) go to seg.  Returns the lane transform.  Angles at and
// past the chain end (and omega of its last residue) are taken as 0, so padding
// values, NaN included, never enter a transform.
// Rare path of walk_chunk: a group with an angle beyond the range of sincos_fast.
__device__ __noinline__ void walk4_any(const BondConsts &bc, Frame<float> &f, const float (&a0)[4],
                                       const float (&a1)[4], const float (&a2)[4], float *seg) {
    walk4<false>(bc, f, a0, a1, a2, seg);
}

// The rare path inline (INL) or as a call.  Inline is faster wherever the registers
// allow it (GB300, 4096 x 1000: a2b_fwd_chain_kernel<8> 59.3 -> 52.8 us, the ring
// forwards 3-7 % faster); a2b_fwd_chain_kernel<4> spills with it inline, so it keeps
// the call.
template <bool INL>
__device__ __forceinline__ void walk4_rare(const BondConsts &bc, Frame<float> &f, const float (&a0)[4],
                                           const float (&a1)[4], const float (&a2)[4], float *seg) {
    if constexpr (INL) walk4<false>(bc, f, a0, a1, a2, seg);
    else walk4_any(bc, f, a0, a1, a2, seg);
}

template <int C, bool INL>
__device__ __forceinline__ Frame<float> walk_chunk(const BondConsts &bc, const float *ang, int L, int j0, int len,
                                                   bool vec, float *seg) {
    Frame<float> f;
    frame_identity(f);
#pragma unroll 1
    for (int g = 0; g < C / 4; g++) {
        const int j = j0 + 4 * g;
        float v0[4], v1[4], v2[4];
        if (vec && j + 4 < len) {  // whole group inside the chain, omega included
            const float4 x0 = __ldg(reinterpret_cast<const float4 *>(ang + j));
            const float4 x1 = __ldg(reinterpret_cast<const float4 *>(ang + L + j));
            const float4 x2 = __ldg(reinterpret_cast<const float4 *>(ang + 2 * L + j));
            v0[0] = x0.x; v0[1] = x0.y; v0[2] = x0.z; v0[3] = x0.w;
            v1[0] = x1.x; v1[1] = x1.y; v1[2] = x1.z; v1[3] = x1.w;
            v2[0] = x2.x; v2[1] = x2.y; v2[2] = x2.z; v2[3] = x2.w;
        } else {
            load4(ang, j, len, vec, v0);
            load4(ang + L, j, len, vec, v1);
            load4(ang + 2 * L, j, len - 1, vec, v2);  // omega of the last residue moves nothing: 0
        }
        // one range check per group (NaN passes: sincos_fast returns NaN for it)
        float m = 0.f;
#pragma unroll
        for (int i = 0; i < 4; i++) m = fmaxf(m, fmaxf(fabsf(v0[i]), fmaxf(fabsf(v1[i]), fabsf(v2[i]))));
        if (m <= 1.0e4f) walk4<true>(bc, f, v0, v1, v2, seg + 36 * g);
        else walk4_rare<INL>(bc, f, v0, v1, v2, seg + 36 * g);
    }
    return f;
}

// Angles of a chunk prefetched into shared memory with cp.async while the warp works
// on the previous chunk (C = 4 only: the double buffer costs 3 KB per warp, which
// still lets seven CTAs of four warps share an SM; at C = 8 it would cost a CTA).
// Lane l copies, and later reads, only its own float4s of the three rows, so no
// barrier is needed between lanes; a buffer is refilled one chunk after its walk read
// it, by which time those values have been consumed.  GB300, 4096 x 1000:
// a2b_fwd_chain_kernel<4> 57.4 -> 55.7 us.
template <int C>
struct AngBuf {
    static constexpr bool ON = C == 4;
    static constexpr int FLOATS = ON ? 2 * 3 * 32 * C : 0;  // per warp: two chunks of three rows
};
__device__ __forceinline__ void cp_async16(float *dst, const float *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Copy the lane's float4s of the chunk starting at s0 (rows phi, psi, omega) into buf
// (three rows of 32 C floats).  Requires L % 4 == 0 and 16-byte aligned rows.
template <int C>
__device__ __forceinline__ void prefetch_angles(float *buf, const float *ang, int L, int s0, int lane) {
    constexpr int CH = 32 * C;
#pragma unroll
    for (int g = 0; g < C / 4; g++) {
        const int o = C * lane + 4 * g, j = s0 + o;
        if (j < L) {
#pragma unroll
            for (int r = 0; r < 3; r++) cp_async16(buf + r * CH + o, ang + (size_t)r * L + j);
        }
    }
}

// walk_chunk with the angles read from the prefetch buffer (masked as load4 does).
template <int C, bool INL>
__device__ __forceinline__ Frame<float> walk_chunk_smem(const BondConsts &bc, const float *buf, int lane, int j0,
                                                        int len, float *seg) {
    constexpr int CH = 32 * C;
    Frame<float> f;
    frame_identity(f);
#pragma unroll 1
    for (int g = 0; g < C / 4; g++) {
        const int j = j0 + 4 * g, o = C * lane + 4 * g;
        const float4 x0 = *reinterpret_cast<const float4 *>(buf + o);
        const float4 x1 = *reinterpret_cast<const float4 *>(buf + CH + o);
        const float4 x2 = *reinterpret_cast<const float4 *>(buf + 2 * CH + o);
        float v0[4] = {x0.x, x0.y, x0.z, x0.w}, v1[4] = {x1.x, x1.y, x1.z, x1.w}, v2[4] = {x2.x, x2.y, x2.z, x2.w};
        if (!(j + 4 < len)) {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                v0[i] = j + i < len ? v0[i] : 0.f;
                v1[i] = j + i < len ? v1[i] : 0.f;
                v2[i] = j + i < len - 1 ? v2[i] : 0.f;
            }
        }
        float m = 0.f;
#pragma unroll
        for (int i = 0; i < 4; i++) m = fmaxf(m, fmaxf(fabsf(v0[i]), fmaxf(fabsf(v1[i]), fabsf(v2[i]))));
        if (m <= 1.0e4f) walk4<true>(bc, f, v0, v1, v2, seg + 36 * g);
        else walk4_rare<INL>(bc, f, v0, v1, v2, seg + 36 * g);
    }
    return f;
}

// Map the 3C staged points of a lane through P in place; zeros for residues at or
// past len.
template <int C, bool MASK>
__device__ __forceinline__ void map_points(float *seg, const Frame<float> &P, int nvalid) {
#pragma unroll
    for (int g = 0; g < 3 * C / 4; g++) {
        float4 *q = reinterpret_cast<float4 *>(seg + 12 * g);
        const float4 v0 = q[0], v1 = q[1], v2 = q[2];
        const float x[12] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w, v2.x, v2.y, v2.z, v2.w};
        float y[12];
#pragma unroll
        for (int pt = 0; pt < 4; pt++) {
            frame_point(P, x[3 * pt], x[3 * pt + 1], x[3 * pt + 2], &y[3 * pt]);
            if (MASK && (4 * g + pt) / 3 >= nvalid) y[3 * pt] = y[3 * pt + 1] = y[3 * pt + 2] = 0.f;
        }
        q[0] = make_float4(y[0], y[1], y[2], y[3]);
        q[1] = make_float4(y[4], y[5], y[6], y[7]);
        q[2] = make_float4(y[8], y[9], y[10], y[11]);
    }
}

template <int C>
__device__ __forceinline__ void map_positions(float *seg, const Frame<float> &P, int j0, int len) {
    if (j0 + C <= len) map_points<C, false>(seg, P, C);
    else map_points<C, true>(seg, P, len - j0);
}

// The map stays scalar: paired arithmetic there makes the forwards spill registers.
template <int C>
__device__ __forceinline__ void map_positions(float *seg, const PairFrame &P, int j0, int len) {
    Frame<float> Pf;
    from_pair(P, Pf);
    map_positions<C>(seg, Pf, j0, len);
}

// Stage floats [0, 32 SEG) of a chunk: src[f] for f < nvalid, 0 after.  Lane l's
// segment (floats l SEG .. l SEG + SEG - 1) lands at stage + l SP.
template <int SEG, int SP>
__device__ __forceinline__ void stage_chunk(float *stage, const float *src, int nvalid, int lane, bool vec) {
    if (vec) {
#pragma unroll 2
        for (int q = lane; q < 8 * SEG; q += 32) {
            const int f = 4 * q, sl = f / SEG;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (f < nvalid) {
                v = __ldcs(reinterpret_cast<const float4 *>(src) + q);
                if (f + 1 >= nvalid) v.y = 0.f;
                if (f + 2 >= nvalid) v.z = 0.f;
                if (f + 3 >= nvalid) v.w = 0.f;
            }
            *reinterpret_cast<float4 *>(stage + sl * SP + f - sl * SEG) = v;
        }
    } else {
        for (int f = lane; f < 32 * SEG; f += 32) {
            const int sl = f / SEG;
            stage[sl * SP + f - sl * SEG] = f < nvalid ? src[f] : 0.f;
        }
    }
}

// Store staged floats [0, n) of a chunk to dst (coalesced).
template <int SEG, int SP>
__device__ __forceinline__ void store_chunk(float *dst, const float *stage, int n, int lane, bool vec) {
    if (vec) {
        // float4 q = lane + 32 i lives in lane segment sl at offset off: both are
        // advanced by the constant step of 128 floats instead of divided out
        constexpr int kStepSeg = 128 / SEG, kStepOff = 128 - kStepSeg * SEG;
        int sl = (4 * lane) / SEG, off = 4 * lane - sl * SEG;
#pragma unroll 2
        for (int q = lane; 4 * q < n; q += 32) {
            __stcs(reinterpret_cast<float4 *>(dst) + q, *reinterpret_cast<const float4 *>(stage + sl * SP + off));
            sl += kStepSeg;
            off += kStepOff;
            if (off >= SEG) {
                off -= SEG;
                sl += 1;
            }
        }
    } else {
        for (int f = lane; f < n; f += 32) {
            const int sl = f / SEG;
            dst[f] = stage[sl * SP + f - sl * SEG];
        }
    }
}

// Staging layout of the forwards: lane l's 9C floats start at l SEG + GAP (l / 4).
// With an odd number of float4s per lane (C = 4) the plain layout is already free of
// bank conflicts; with an even number (C = 8) a 4-float gap after every four lanes
// puts the 8 lanes of each 128-bit shared-memory phase on 8 different bank groups,
// both for lane-local accesses and for the row-order reads of the store, at 32
// floats of padding per warp.
template <int C>
struct FwdStage {
    static constexpr int SEG = 9 * C;
    static constexpr int GAP = ((SEG / 4) % 2 == 0) ? 4 : 0;
    static constexpr int FLOATS = 32 * SEG + 8 * GAP;  // per warp
    __device__ static __forceinline__ int lane_offset(int l) { return l * SEG + GAP * (l >> 2); }
};

// store_chunk for the FwdStage layout: float4 q of the chunk (floats 4q..4q+3, in lane
// segment floor(4q / SEG)) is staged at float 4q + GAP floor(q / SEG).
__device__ __forceinline__ void st_evict_last(float4 *p, float4 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w), "l"(pol)
                 : "memory");
}

// The coordinates are stored with an L2 evict-last hint: the layer's backward reads
// them back (chains last to first, so the rows written last come first), and the rows
// still in L2 save their DRAM reads (GB300, 4096 x 1000: backward 0.0601 -> 0.0580 ms
// in the step; evict-first stores kept fewer of them).
template <int C>
__device__ __forceinline__ void store_chunk_fwd(float *dst, const float *stage, int n, int lane, bool vec) {
    using S = FwdStage<C>;
    constexpr int SEG = S::SEG;
    if (vec) {
        uint64_t pol;
        asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
#pragma unroll 2
        for (int q = lane; 4 * q < n; q += 32)
            st_evict_last(reinterpret_cast<float4 *>(dst) + q,
                          *reinterpret_cast<const float4 *>(stage + 4 * q + S::GAP * (q / SEG)), pol);
    } else {
        for (int f = lane; f < n; f += 32) {
            const int sl = f / SEG;
            dst[f] = stage[S::lane_offset(sl) + f - sl * SEG];
        }
    }
}

__device__ __forceinline__ void zero_floats(float *dst, int n, int lane, bool vec) {
    if (vec) {
        for (int q = lane; 4 * q < n; q += 32) __stcs(reinterpret_cast<float4 *>(dst) + q, make_float4(0.f, 0.f, 0.f, 0.f));
    } else {
        for (int f = lane; f < n; f += 32) dst[f] = 0.f;
    }
}

__device__ __forceinline__ int checked_length(const ChainArgs &a, int b, int lane) {
    int len = a.lengths[b];
    if (len < 0 || len > a.L) {
        if (lane == 0) record_error(a.hdr, TPL_ERR_LENGTH);
        len = max(0, min(len, a.L));
    }
    return len;
}

constexpr int fwd_min_blocks(int C) { return C >= 8 ? 5 : 7; }
constexpr int bwd_min_blocks(int C) { return C >= 8 ? 2 : 4; }

template <int C>
__global__ void __launch_bounds__(32 * kWarpsPerCta, fwd_min_blocks(C)) a2b_fwd_chain_kernel(ChainArgs a) {
    constexpr int CH = 32 * C;
    extern __shared__ __align__(16) float s_dyn[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int b = blockIdx.x * kWarpsPerCta + w;
    if (b >= a.B) return;  // warps are independent: no CTA-wide barrier follows
    float *stage = s_dyn + w * FwdStage<C>::FLOATS;
    float *seg = stage + FwdStage<C>::lane_offset(lane);
    const int len = checked_length(a, b, lane);
    const float *ang = a.angles + (size_t)b * 3 * a.L;
    float *out = a.coords + (size_t)b * 9 * a.L;
    ChainRecord *rec = a.rec + (size_t)b * a.nrec;
    const bool vec = a.vec != 0;

    PairFrame F = pair_identity();  // chain frame at the chunk start (world)
    constexpr bool PF = AngBuf<C>::ON;
    float *abuf = s_dyn + kWarpsPerCta * FwdStage<C>::FLOATS + w * AngBuf<C>::FLOATS;
    const bool pf = PF && vec;
    if (pf) {
        if (len > 0) prefetch_angles<C>(abuf, ang, a.L, 0, lane);
        cp_async_commit();
    }
    int it = 0;
    for (int s0 = 0; s0 < a.L; s0 += CH, it ^= 1) {
        const int nout = min(CH, a.L - s0);
        float *dst = out + (size_t)9 * s0;
        if (s0 >= len) {
            zero_floats(dst, 9 * nout, lane, vec);
            continue;
        }
        const int j0 = s0 + C * lane;
        PairFrame tot;
        Frame<float> T;
        if (pf) {
            if (s0 + CH < len) prefetch_angles<C>(abuf + (it ^ 1) * 3 * CH, ang, a.L, s0 + CH, lane);
            cp_async_commit();
            cp_async_wait1();  // this chunk's copies (all groups but the newest) have landed
            T = walk_chunk_smem<C, C != 4>(a.bc, abuf + it * 3 * CH, lane, j0, len, seg);
        } else {
            T = walk_chunk<C, C != 4>(a.bc, ang, a.L, j0, len, vec, seg);
        }
        // lane transforms compose 3C joints: no renormalisation before the scan (the
        // chain frame carried from chunk to chunk is renormalised)
        const PairFrame E = warp_exclusive_total_pair(to_pair(T), lane, false, tot);
        // E composes at most 31 renormalised lane transforms: P needs no renormalisation
        const PairFrame P = compose_pair(F, E);
        if ((C * lane) % kRecordStride == 0 && j0 < len) pair_store(rec[j0 / kRecordStride].f, P);
        F = compose_pair(F, tot);
        if (a.renorm) renormalize_pair(F);
        map_positions<C>(seg, P, j0, len);
        __syncwarp();
        store_chunk_fwd<C>(dst, stage, 9 * nout, lane, vec);
        __syncwarp();  // the next chunk's walk rewrites the staging buffer
    }
}

template <int C>
__global__ void __launch_bounds__(32 * kWarpsPerCta, bwd_min_blocks(C)) a2b_bwd_chain_kernel(ChainArgs a) {
    constexpr int CH = 32 * C, SEG = 9 * C, SP = SEG + 4;
    extern __shared__ __align__(16) float s_dyn[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int b = blockIdx.x * kWarpsPerCta + w;
    if (b >= a.B) return;
    float *sx = s_dyn + w * 64 * SP;  // lane-local positions
    float *sg = sx + 32 * SP;         // dL/dx, rotated in place into lane-local frames
    float *xs = sx + lane * SP, *gs = sg + lane * SP;
    const int len = checked_length(a, b, lane);
    const float *ang = a.angles + (size_t)b * 3 * a.L;
    const float *gin = a.grad_coords + (size_t)b * 9 * a.L;
    float *gout = a.grad_angles + (size_t)b * 3 * a.L;
    const ChainRecord *rec = a.rec + (size_t)b * a.nrec;
    const bool vec = a.vec != 0;
    const float inv_d0 = 1.f / a.bc.d[0], inv_d1 = 1.f / a.bc.d[1], inv_d2 = 1.f / a.bc.d[2];

    // gradient rows past the last chunk that holds residues are zero
    const int nchunk = (len + CH - 1) / CH;
    const int s_end = min(a.L, nchunk * CH);
    for (int k = 0; k < 3; k++) zero_floats(gout + (size_t)k * a.L + s_end, a.L - s_end, lane, vec && (s_end % 4 == 0));

    // sums over all atoms after the current chunk: G, and S about origin oc
    float Gc[3] = {0.f, 0.f, 0.f}, Sc[3] = {0.f, 0.f, 0.f}, oc[3] = {0.f, 0.f, 0.f};
    for (int k = nchunk - 1; k >= 0; k--) {
        const int s0 = k * CH;
        const int nreal = min(CH, len - s0);
        const int j0 = s0 + C * lane;
        Frame<float> F;
        frame_load(F, rec[s0 / kRecordStride].f);
        {  // move the carried sums to this chunk's origin: S_o = S_oc + (oc - o) x G
            const float d[3] = {oc[0] - F.p[0], oc[1] - F.p[1], oc[2] - F.p[2]};
            float dx[3];
            cross3(d, Gc, dx);
#pragma unroll
            for (int i = 0; i < 3; i++) {
                Sc[i] += dx[i];
                oc[i] = F.p[i];
            }
        }
        stage_chunk<SEG, SP>(sg, gin + (size_t)9 * s0, 9 * nreal, lane, vec);
        const Frame<float> t = walk_chunk<C, true>(a.bc, ang, a.L, j0, len, vec, xs);
        Frame<float> tot;
        const Frame<float> E = warp_exclusive_total(t, lane, false, tot);  // as the forward's scan
        F.p[0] = F.p[1] = F.p[2] = 0.f;  // lane frames relative to the chunk origin
        Frame<float> P = compose(F, E);
        if (a.renorm) renormalize(P);
        __syncwarp();  // staged dL/dx complete

        // rotate the lane's dL/dx into its frame; lane sums about the lane origin
        float Gl[3] = {0.f, 0.f, 0.f}, Sl[3] = {0.f, 0.f, 0.f};
#pragma unroll 1
        for (int g = 0; g < 3 * C / 4; g++) {
            float4 *gq = reinterpret_cast<float4 *>(gs + 12 * g);
            const float4 *xq = reinterpret_cast<const float4 *>(xs + 12 * g);
            const float4 g0 = gq[0], g1 = gq[1], g2 = gq[2];
            const float4 x0 = xq[0], x1 = xq[1], x2 = xq[2];
            const float gw[12] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w, g2.x, g2.y, g2.z, g2.w};
            const float xv[12] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w, x2.x, x2.y, x2.z, x2.w};
            float gl[12];
#pragma unroll
            for (int pt = 0; pt < 4; pt++) {
                const float *v = gw + 3 * pt;
                float *o = gl + 3 * pt;
                o[0] = fmaf(P.r[0], v[0], fmaf(P.r[3], v[1], P.r[6] * v[2]));
                o[1] = fmaf(P.r[1], v[0], fmaf(P.r[4], v[1], P.r[7] * v[2]));
                o[2] = fmaf(P.r[2], v[0], fmaf(P.r[5], v[1], P.r[8] * v[2]));
                float xg[3];
                cross3(xv + 3 * pt, o, xg);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    Gl[c] += o[c];
                    Sl[c] += xg[c];
                }
            }
            gq[0] = make_float4(gl[0], gl[1], gl[2], gl[3]);
            gq[1] = make_float4(gl[4], gl[5], gl[6], gl[7]);
            gq[2] = make_float4(gl[8], gl[9], gl[10], gl[11]);
        }
        // lane sums in the chunk frame: G = R Gl, S = R Sl + p x G
        float v6[6];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            v6[i] = fmaf(P.r[3 * i], Gl[0], fmaf(P.r[3 * i + 1], Gl[1], P.r[3 * i + 2] * Gl[2]));
            v6[3 + i] = fmaf(P.r[3 * i], Sl[0], fmaf(P.r[3 * i + 1], Sl[1], P.r[3 * i + 2] * Sl[2]));
        }
        {
            float pg[3];
            cross3(P.p, v6, pg);
#pragma unroll
            for (int i = 0; i < 3; i++) v6[3 + i] += pg[i];
        }
        float Gin[3], Sin[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            float tg, ts;
            Gin[i] = warp_suffix_excl(v6[i], lane, tg) + Gc[i];
            Sin[i] = warp_suffix_excl(v6[3 + i], lane, ts) + Sc[i];
            Gc[i] += tg;
            Sc[i] += ts;
        }
        // incoming sums in the lane frame: G' = R^T G, S' = R^T (S - p x G)
        float G[3], S[3];
        {
            float pg[3], Sm[3];
            cross3(P.p, Gin, pg);
#pragma unroll
            for (int i = 0; i < 3; i++) Sm[i] = Sin[i] - pg[i];
#pragma unroll
            for (int i = 0; i < 3; i++) {
                G[i] = fmaf(P.r[i], Gin[0], fmaf(P.r[3 + i], Gin[1], P.r[6 + i] * Gin[2]));
                S[i] = fmaf(P.r[i], Sm[0], fmaf(P.r[3 + i], Sm[1], P.r[6 + i] * Sm[2]));
            }
        }
        // backwards over the lane's residues, four at a time (9 float4s of positions
        // and of gradients per group)
        float nxt[3] = {t.p[0], t.p[1], t.p[2]};  // N of the residue after the lane's last
#pragma unroll 1
        for (int gi = C / 4 - 1; gi >= 0; gi--) {
            const float4 *xq = reinterpret_cast<const float4 *>(xs + 36 * gi);
            const float4 *gq = reinterpret_cast<const float4 *>(gs + 36 * gi);
            float xb[36], gb[36];  // read as float4s when first needed
            float gph[4], gps[4], gom[4];
#pragma unroll
            for (int r = 3; r >= 0; r--) {
#pragma unroll
                for (int q = (9 * r) / 4; q <= (9 * r + 8) / 4; q++)
                    if (r == 3 || q < (9 * (r + 1)) / 4) {  // not read for residue r + 1
                        const float4 xv = xq[q], gv = gq[q];
                        xb[4 * q] = xv.x; xb[4 * q + 1] = xv.y; xb[4 * q + 2] = xv.z; xb[4 * q + 3] = xv.w;
                        gb[4 * q] = gv.x; gb[4 * q + 1] = gv.y; gb[4 * q + 2] = gv.z; gb[4 * q + 3] = gv.w;
                    }
                float xN[3], xA[3], xC[3], gN[3], gA[3], gC[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    xN[c] = xb[9 * r + c]; xA[c] = xb[9 * r + 3 + c]; xC[c] = xb[9 * r + 6 + c];
                    gN[c] = gb[9 * r + c]; gA[c] = gb[9 * r + 3 + c]; gC[c] = gb[9 * r + 6 + c];
                }
                float u[3], tmp[3], cr[3];
                // omega_j: axis C -> N_{j+1}, through N_{j+1}; moves the atoms after C_j
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (nxt[c] - xC[c]) * inv_d2;
                cross3(nxt, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                gom[r] = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                // psi_j: axis CA -> C, through C; same atoms
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (xC[c] - xA[c]) * inv_d1;
                cross3(xC, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                gps[r] = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                cross3(xC, gC, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    G[c] += gC[c];
                    S[c] += cr[c];
                }
                // phi_j: axis N -> CA, through CA; moves C_j and everything after
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (xA[c] - xN[c]) * inv_d0;
                cross3(xA, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                gph[r] = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                cross3(xA, gA, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    G[c] += gA[c];
                    S[c] += cr[c];
                }
                cross3(xN, gN, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    G[c] += gN[c];
                    S[c] += cr[c];
                    nxt[c] = xN[c];
                }
            }
            // zeros at and past len; psi and omega of the last residue move nothing
            const int jg = j0 + 4 * gi;
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int j = jg + r;
                const bool ok = j < len, last = j == len - 1;
                gph[r] = ok ? gph[r] : 0.f;
                gps[r] = ok && !last ? gps[r] : 0.f;
                gom[r] = ok && !last ? gom[r] : 0.f;
            }
            if (vec) {
                if (jg < a.L) {
                    __stcs(reinterpret_cast<float4 *>(gout + jg), make_float4(gph[0], gph[1], gph[2], gph[3]));
                    __stcs(reinterpret_cast<float4 *>(gout + a.L + jg), make_float4(gps[0], gps[1], gps[2], gps[3]));
                    __stcs(reinterpret_cast<float4 *>(gout + 2 * a.L + jg),
                           make_float4(gom[0], gom[1], gom[2], gom[3]));
                }
            } else {
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    const int j = jg + r;
                    if (j < a.L) {
                        gout[j] = gph[r];
                        gout[a.L + j] = gps[r];
                        gout[2 * a.L + j] = gom[r];
                    }
                }
            }
        }
        __syncwarp();  // the next chunk rewrites both staging buffers
    }
}

// ------------------------------------------------- backward from the coordinates
// The forward's output already holds every atom position, so this backward reads
// them instead of re-walking the chain: per chunk (last to first) a warp stages
// the chunk's coordinates and dL/dx (two bulk copies into shared memory when the
// rows are 16-byte aligned), and evaluates
//     dL/dtheta_m = u_m . (S_m - x_m x G_m),  G_m = sum_{i>m} g_i,  S_m = sum_{i>m} x_i x g_i,
// with u_m the unit bond vector into the rotated joint, as a lane pass (lane
// sums), a warp suffix scan and a reverse pass over each lane's residues.
// Positions are taken relative to the chunk's first N atom to keep the sums small.

constexpr unsigned kWaitPolls = 1u << 22;  // bounded mbarrier wait (~0.5 s with back-off)

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void bulk_load_pair(float *dx, const float *sx, float *dg, const float *sg, unsigned bytes,
                                               uint64_t *bar) {
    // the buffers were last read through the generic proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(2 * bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dx)),
                 "l"(sx), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dg)),
                 "l"(sg), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// Wait for the phase with the given parity to complete; false after kWaitPolls polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    for (unsigned i = 0; i < kWaitPolls; i++) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (i >= 8) __nanosleep(100);
    }
    return false;
}

// The float4s 4q..4q+3 of a lane's staged segment that residue r needs, each
// fetched once when residues are visited in descending (DESC) or ascending order:
// a float4 shared with the residue visited before is already in buf.
template <bool DESC>
__device__ __forceinline__ void fetch_residue(const float *seg, float *buf, int r, bool first) {
#pragma unroll
    for (int q = (9 * r) / 4; q <= (9 * r + 8) / 4; q++)
        if (first || (DESC ? q < (9 * (r + 1)) / 4 : q > (9 * r - 1) / 4)) {
            const float4 v = reinterpret_cast<const float4 *>(seg)[q];
            buf[4 * q] = v.x; buf[4 * q + 1] = v.y; buf[4 * q + 2] = v.z; buf[4 * q + 3] = v.w;
        }
}

constexpr int coords_min_blocks(int C, int NB) { return C * NB >= 16 ? 1 : (C * NB >= 8 ? 3 : 5); }

// NB = 1: each chunk's copies are issued and waited for in turn.  NB = 2: two
// buffer pairs; the copies of the next chunk are in flight while a chunk is
// evaluated.
template <int C, int NB>
__global__ void __launch_bounds__(32 * kWarpsPerCta, coords_min_blocks(C, NB)) a2b_bwd_coords_kernel(ChainArgs a) {
    constexpr int CH = 32 * C, SEG = 9 * C;
    extern __shared__ __align__(16) float s_dyn[];
    __shared__ __align__(8) uint64_t s_bar[kWarpsPerCta][NB];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int idx = blockIdx.x * kWarpsPerCta + w;
    if (idx >= a.B) return;  // warps are independent
    const int b = a.B - 1 - idx;  // chains last to first, as in a2b_bwd_coords_ring_kernel
    // per buffer: coordinates of a chunk (contiguous as in the row), then its dL/dx
    float *sbase = s_dyn + (size_t)w * NB * 64 * SEG;
    uint64_t *bars = s_bar[w];
    const bool vec = a.vec != 0;
    if (vec && lane == 0)
        for (int i = 0; i < NB; i++) mbar_init(&bars[i]);
    __syncwarp();
    const int len = checked_length(a, b, lane);
    const float *xin = a.coords + (size_t)b * 9 * a.L;
    const float *gin = a.grad_coords + (size_t)b * 9 * a.L;
    float *gout = a.grad_angles + (size_t)b * 3 * a.L;
    const float inv_d0 = 1.f / a.bc.d[0], inv_d1 = 1.f / a.bc.d[1], inv_d2 = 1.f / a.bc.d[2];

    const int nchunk = (len + CH - 1) / CH;
    const int s_end = min(a.L, nchunk * CH);
    for (int k = 0; k < 3; k++) zero_floats(gout + (size_t)k * a.L + s_end, a.L - s_end, lane, vec && (s_end % 4 == 0));

    float Gc[3] = {0.f, 0.f, 0.f}, Sc[3] = {0.f, 0.f, 0.f}, oc[3] = {0.f, 0.f, 0.f};  // sums after the chunk
    float nN[3] = {0.f, 0.f, 0.f};  // N of the first residue after the chunk (world)
    // chunk kk into buffer q: whole residues up to a multiple of 4 (inside the row
    // since L % 4 == 0), by lane 0
    auto issue = [&](int kk, int q) {
        if (lane == 0) {
            const int n4 = (min(CH, len - kk * CH) + 3) & ~3;
            float *bx = sbase + (size_t)q * 64 * SEG;
            bulk_load_pair(bx, xin + (size_t)9 * kk * CH, bx + 32 * SEG, gin + (size_t)9 * kk * CH, 36u * (unsigned)n4,
                           &bars[q]);
        }
    };
    unsigned parity = 0;  // bit q: parity of buffer q's pending phase
    if (vec && NB == 2 && nchunk > 0) issue(nchunk - 1, 0);
    for (int k = nchunk - 1, it = 0; k >= 0; k--, it++) {
        const int s0 = k * CH;
        const int nreal = min(CH, len - s0);
        const int q = NB == 2 ? (it & 1) : 0;
        float *sx = sbase + (size_t)q * 64 * SEG;
        float *sg = sx + 32 * SEG;
        const float *xs = sx + lane * SEG, *gs = sg + lane * SEG;
        __syncwarp();  // the previous chunk's reads of its buffers are done
        if (vec) {
            if (NB == 1) issue(k, 0);
            else if (k > 0) issue(k - 1, q ^ 1);  // prefetch: the other buffer held the previous chunk
            const bool ok = mbar_wait(&bars[q], (parity >> q) & 1u);
            parity ^= 1u << q;
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) record_error(a.hdr, TPL_ERR_LOOKBACK_TIMEOUT);
                // bounded: let the copies in flight land before exiting
                (void)mbar_wait(&bars[q], ((parity >> q) & 1u) ^ 1u);
                if (NB == 2 && k > 0) (void)mbar_wait(&bars[q ^ 1], (parity >> (q ^ 1)) & 1u);
                return;
            }
        } else {
            stage_chunk<SEG, SEG>(sx, xin + (size_t)9 * s0, 9 * nreal, lane, false);
            stage_chunk<SEG, SEG>(sg, gin + (size_t)9 * s0, 9 * nreal, lane, false);
            __syncwarp();
        }
        const int j0 = s0 + C * lane;
        const float o[3] = {sx[0], sx[1], sx[2]};  // chunk origin: its first N atom
        {
            const float d[3] = {oc[0] - o[0], oc[1] - o[1], oc[2] - o[2]};
            float dx[3];
            cross3(d, Gc, dx);
#pragma unroll
            for (int i = 0; i < 3; i++) {
                Sc[i] += dx[i];
                oc[i] = o[i];
            }
        }
        // lane sums about o over the lane's residues below len
        float Gl[3] = {0.f, 0.f, 0.f}, Sl[3] = {0.f, 0.f, 0.f};
        {
            float xb[9 * C], gb[9 * C];
#pragma unroll
            for (int r = 0; r < C; r++) {
#pragma unroll
                for (int q = (9 * r) / 4; q <= (9 * r + 8) / 4; q++)
                    if (r == 0 || q > (9 * r - 1) / 4) {  // not fetched for residue r - 1
                        const float4 xv = reinterpret_cast<const float4 *>(xs)[q];
                        const float4 gv = reinterpret_cast<const float4 *>(gs)[q];
                        xb[4 * q] = xv.x; xb[4 * q + 1] = xv.y; xb[4 * q + 2] = xv.z; xb[4 * q + 3] = xv.w;
                        gb[4 * q] = gv.x; gb[4 * q + 1] = gv.y; gb[4 * q + 2] = gv.z; gb[4 * q + 3] = gv.w;
                    }
                if (j0 + r < len) {
#pragma unroll
                    for (int at = 0; at < 3; at++) {
                        const float *x = xb + 9 * r + 3 * at, *g = gb + 9 * r + 3 * at;
                        const float xr[3] = {x[0] - o[0], x[1] - o[1], x[2] - o[2]};
                        float xg[3];
                        cross3(xr, g, xg);
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            Gl[c] += g[c];
                            Sl[c] += xg[c];
                        }
                    }
                }
            }
        }
        float G[3], S[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            float tg, ts;
            G[i] = warp_suffix_excl(Gl[i], lane, tg) + Gc[i];
            S[i] = warp_suffix_excl(Sl[i], lane, ts) + Sc[i];
            Gc[i] += tg;
            Sc[i] += ts;
        }
        // N after the lane's last residue: the next lane's first N, or the next chunk's
        float nxt[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float mine = xs[c];
            const float nb = __shfl_down_sync(0xffffffffu, mine, 1);
            const float first = __shfl_sync(0xffffffffu, mine, 0);
            nxt[c] = (lane == 31 ? nN[c] : nb) - o[c];
            nN[c] = first;
        }
        // backwards over the lane's residues, positions relative to o
        float gph[C], gps[C], gom[C];
        {
            float xb[9 * C], gb[9 * C];
#pragma unroll
            for (int r = C - 1; r >= 0; r--) {
#pragma unroll
                for (int q = (9 * r) / 4; q <= (9 * r + 8) / 4; q++)
                    if (r == C - 1 || q < (9 * (r + 1)) / 4) {  // not fetched for residue r + 1
                        const float4 xv = reinterpret_cast<const float4 *>(xs)[q];
                        const float4 gv = reinterpret_cast<const float4 *>(gs)[q];
                        xb[4 * q] = xv.x; xb[4 * q + 1] = xv.y; xb[4 * q + 2] = xv.z; xb[4 * q + 3] = xv.w;
                        gb[4 * q] = gv.x; gb[4 * q + 1] = gv.y; gb[4 * q + 2] = gv.z; gb[4 * q + 3] = gv.w;
                    }
                const int j = j0 + r;
                float xN[3], xA[3], xC[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    xN[c] = xb[9 * r + c] - o[c];
                    xA[c] = xb[9 * r + 3 + c] - o[c];
                    xC[c] = xb[9 * r + 6 + c] - o[c];
                }
                const float *gN = gb + 9 * r, *gA = gb + 9 * r + 3, *gC = gb + 9 * r + 6;
                float u[3], tmp[3], cr[3];
                // omega_j: axis C -> N_{j+1}, through N_{j+1}; moves the atoms after C_j
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (nxt[c] - xC[c]) * inv_d2;
                cross3(nxt, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                gom[r] = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                // psi_j: axis CA -> C, through C; same atoms
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (xC[c] - xA[c]) * inv_d1;
                cross3(xC, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                gps[r] = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                const bool in = j < len;
                if (in) {
                    cross3(xC, gC, cr);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        G[c] += gC[c];
                        S[c] += cr[c];
                    }
                }
                // phi_j: axis N -> CA, through CA; moves C_j and everything after
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (xA[c] - xN[c]) * inv_d0;
                cross3(xA, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                gph[r] = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                if (in) {
                    cross3(xA, gA, cr);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        G[c] += gA[c];
                        S[c] += cr[c];
                    }
                    cross3(xN, gN, cr);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        G[c] += gN[c];
                        S[c] += cr[c];
                    }
                }
#pragma unroll
                for (int c = 0; c < 3; c++) nxt[c] = xN[c];
            }
        }
        // zeros at and past len (stale or padding positions are never stored);
        // psi and omega of the last residue move nothing
#pragma unroll
        for (int r = 0; r < C; r++) {
            const int j = j0 + r;
            const bool ok = j < len, last = j == len - 1;
            gph[r] = ok ? gph[r] : 0.f;
            gps[r] = ok && !last ? gps[r] : 0.f;
            gom[r] = ok && !last ? gom[r] : 0.f;
        }
        if (vec) {
#pragma unroll
            for (int i = 0; i < C / 4; i++) {
                const int j = j0 + 4 * i;
                if (j < a.L) {
                    __stcs(reinterpret_cast<float4 *>(gout + j),
                           make_float4(gph[4 * i], gph[4 * i + 1], gph[4 * i + 2], gph[4 * i + 3]));
                    __stcs(reinterpret_cast<float4 *>(gout + a.L + j),
                           make_float4(gps[4 * i], gps[4 * i + 1], gps[4 * i + 2], gps[4 * i + 3]));
                    __stcs(reinterpret_cast<float4 *>(gout + 2 * a.L + j),
                           make_float4(gom[4 * i], gom[4 * i + 1], gom[4 * i + 2], gom[4 * i + 3]));
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < C; r++) {
                const int j = j0 + r;
                if (j < a.L) {
                    gout[j] = gph[r];
                    gout[a.L + j] = gps[r];
                    gout[2 * a.L + j] = gom[r];
                }
            }
        }
    }
}

// ------------------------------------------------- four warps per chain ("ring")
// One CTA of kRingWarps warps owns one chain; chunk k belongs to warp k % 4 in the
// forward and to warp (nchunk - 1 - k) % 4 in the backward, so a chain is split
// into chunk-sized work items and a batch of equal chains no longer leaves most of
// the GPU idle in a last partial wave of whole chains.  Each warp does the
// expensive part of its chunk (walk and scan, or the staged sums) on its own; only
// a 12-float carry passes between the warps of neighbouring chunks:
//   forward:  the chain frame at the start of chunk k, from the warp of chunk k-1;
//   backward: G and S of every atom after chunk k (S about the first N atom of
//             chunk k+1) and that atom, from the warp of chunk k+1.
// The carry goes through shared-memory slot k % 4 under named barrier 1 + k % 4
// (64 threads: the producer warp arrives, the consumer warp syncs).  A slot and
// its barrier are reused for the handoff into chunk k +- 4 only after the handoff
// into chunk k completed, since the producer of the later handoff has itself
// received the three handoffs in between.  Every warp runs every handoff of its
// chunks whatever happens in them (chunks past the chain, a failed copy), so the
// arrivals always match the syncs.

constexpr int kRingWarps = 4;

// FP64 carry of the four-warp forward: the chain frame at the start of chunk k + 1 is
// F_k o T_k with F_k the FP64 frame of slot `in` (identity when null) and T_k the
// FP32 chunk total.  Lanes 0..11 each compute one entry (rotation row-major, then
// the translation) with three FP64 fused multiply-adds and write it to slot `out`.
__device__ __forceinline__ void carry_f64(const double *in, const PairFrame &tot, double *out, int lane) {
    if (lane < 12) {
        Frame<float> t;
        from_pair(tot, t);
        const int r = lane < 9 ? lane / 3 : lane - 9;  // output row
        double f[4];                                    // row r of F: rotation, translation
#pragma unroll
        for (int j = 0; j < 3; j++) f[j] = in ? in[3 * r + j] : (j == r ? 1.0 : 0.0);
        f[3] = in ? in[9 + r] : 0.0;
        double v;
        if (lane < 9) {
            const int c = lane % 3;
            v = fma(f[0], (double)t.r[c], fma(f[1], (double)t.r[3 + c], f[2] * (double)t.r[6 + c]));
        } else {
            v = fma(f[0], (double)t.p[0], fma(f[1], (double)t.p[1], fma(f[2], (double)t.p[2], f[3])));
        }
        out[lane] = v;
    }
}
// Six CTAs of four warps with 9.3 KB of staging per warp (C = 8), or seven with 4.5 KB
// of staging plus the 3 KB angle buffer per warp (C = 4), fit an SM's shared memory
constexpr int ring_fwd_min_blocks(int C) { return C >= 8 ? 6 : 7; }

template <int C>
__global__ void __launch_bounds__(32 * kRingWarps, ring_fwd_min_blocks(C)) a2b_fwd_ring_kernel(ChainArgs a) {
    constexpr int CH = 32 * C;
    extern __shared__ __align__(16) float s_dyn[];
    __shared__ __align__(16) float s_ring[kRingWarps][12];
    // FP64 carries, after the staging buffers: the launch adds their 384 bytes only
    // when fp64_min is set, so that the FP32 default keeps six CTAs per SM
    double(*s_ring64)[12] =
        reinterpret_cast<double(*)[12]>(s_dyn + kRingWarps * (FwdStage<C>::FLOATS + AngBuf<C>::FLOATS));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int b = blockIdx.x;  // one CTA per chain: the grid is the batch
    float *stage = s_dyn + w * FwdStage<C>::FLOATS;
    float *seg = stage + FwdStage<C>::lane_offset(lane);
    const int len = checked_length(a, b, lane);
    const float *ang = a.angles + (size_t)b * 3 * a.L;
    float *out = a.coords + (size_t)b * 9 * a.L;
    ChainRecord *rec = a.rec + (size_t)b * a.nrec;
    const bool vec = a.vec != 0;
    const int nchunk = (a.L + CH - 1) / CH;
    // chains at least fp64_min long hand the chain frame on in FP64 (the same for the
    // whole CTA, so every warp takes the same branch at every handoff)
    const bool carry64 = a.fp64_min > 0 && len >= a.fp64_min;

    constexpr bool PF = AngBuf<C>::ON;
    float *abuf = s_dyn + kRingWarps * FwdStage<C>::FLOATS + w * AngBuf<C>::FLOATS;
    const bool pf = PF && vec;
    if (pf) {
        if (w * CH < len) prefetch_angles<C>(abuf, ang, a.L, w * CH, lane);
        cp_async_commit();
    }
    int it = 0;
#pragma unroll 1
    for (int k = w; k < nchunk; k += kRingWarps, it ^= 1) {
        const int s0 = k * CH;
        const int nout = min(CH, a.L - s0);
        const bool live = s0 < len;
        const int j0 = s0 + C * lane;
        PairFrame E = pair_identity(), tot = pair_identity();
        if (live) {  // no renormalisation of the lane transforms (3C joints each), as in a2b_fwd_chain_kernel
            Frame<float> T;
            if (pf) {
                const int sn = s0 + kRingWarps * CH;
                if (sn < len) prefetch_angles<C>(abuf + (it ^ 1) * 3 * CH, ang, a.L, sn, lane);
                cp_async_commit();
                cp_async_wait1();
                T = walk_chunk_smem<C, true>(a.bc, abuf + it * 3 * CH, lane, j0, len, seg);
            } else {
                T = walk_chunk<C, true>(a.bc, ang, a.L, j0, len, vec, seg);
            }
            E = warp_exclusive_total_pair(to_pair(T), lane, false, tot);
        }
        PairFrame F = pair_identity();  // chain frame at the chunk start
        if (k > 0) {
            ring_wait(k);
            F = carry64 ? pair_load(s_ring64[k & 3]) : pair_load(s_ring[k & 3]);
        }
        if (k + 1 < nchunk) {
            if (carry64) {
                // the chunk total composes 96C unrenormalised joints: pull it back onto SO(3)
                // first, or the FP64 product of the totals drifts in scale chunk by chunk
                // (the FP32 carry below renormalises the carried frame instead)
                PairFrame t = tot;
                if (a.renorm) renormalize_pair(t);
                carry_f64(k > 0 ? s_ring64[k & 3] : nullptr, t, s_ring64[(k + 1) & 3], lane);
            } else {
                PairFrame Fn = compose_pair(F, tot);
                if (a.renorm) renormalize_pair(Fn);
                if (lane == 0) pair_store(s_ring[(k + 1) & 3], Fn);
            }
            ring_signal(k + 1);
        }
        float *dst = out + (size_t)9 * s0;
        if (!live) {
            zero_floats(dst, 9 * nout, lane, vec);
            continue;
        }
        const PairFrame P = compose_pair(F, E);
        if ((C * lane) % kRecordStride == 0 && j0 < len) pair_store(rec[j0 / kRecordStride].f, P);
        map_positions<C>(seg, P, j0, len);
        __syncwarp();
        store_chunk_fwd<C>(dst, stage, 9 * nout, lane, vec);
        __syncwarp();  // the warp's next chunk rewrites the staging buffer
    }
}

// Backward from the coordinates with the ring split of a2b_bwd_coords_kernel: the
// same per-chunk evaluation, with the carried sums received from the warp of the
// next chunk instead of kept in registers.
template <int C, int NB>
__global__ void __launch_bounds__(32 * kRingWarps, coords_min_blocks(C, NB)) a2b_bwd_coords_ring_kernel(ChainArgs a) {
    constexpr int CH = 32 * C, SEG = 9 * C;
    extern __shared__ __align__(16) float s_dyn[];
    __shared__ __align__(8) uint64_t s_bar[kRingWarps][NB];
    __shared__ __align__(16) float s_ring[kRingWarps][12];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // chains last to first: CTAs are dispatched in index order, so the first ones
    // read the rows the forward wrote last, which may still be in L2
    const int b = a.B - 1 - (int)blockIdx.x;
    float *sbase = s_dyn + (size_t)w * NB * 64 * SEG;
    uint64_t *bars = s_bar[w];
    const bool vec = a.vec != 0;
    if (vec && lane == 0)
        for (int i = 0; i < NB; i++) mbar_init(&bars[i]);
    __syncwarp();
    const int len = checked_length(a, b, lane);
    const float *xin = a.coords + (size_t)b * 9 * a.L;
    const float *gin = a.grad_coords + (size_t)b * 9 * a.L;
    float *gout = a.grad_angles + (size_t)b * 3 * a.L;
    const float inv_d0 = 1.f / a.bc.d[0], inv_d1 = 1.f / a.bc.d[1], inv_d2 = 1.f / a.bc.d[2];

    const int nchunk = (len + CH - 1) / CH;
    if (w == kRingWarps - 1) {  // gradient rows past the last chunk that holds residues are zero
        const int s_end = min(a.L, nchunk * CH);
        for (int k = 0; k < 3; k++)
            zero_floats(gout + (size_t)k * a.L + s_end, a.L - s_end, lane, vec && (s_end % 4 == 0));
    }
    auto issue = [&](int kk, int q) {
        if (lane == 0) {
            const int n4 = (min(CH, len - kk * CH) + 3) & ~3;
            float *bx = sbase + (size_t)q * 64 * SEG;
            bulk_load_pair(bx, xin + (size_t)9 * kk * CH, bx + 32 * SEG, gin + (size_t)9 * kk * CH, 36u * (unsigned)n4,
                           &bars[q]);
        }
    };
    unsigned parity = 0;  // bit q: parity of buffer q's pending phase
    bool failed = false;  // a bulk copy timed out: the remaining chunks only pass the carry on
    const int first = nchunk - 1 - w;
    if (vec && NB == 2 && first >= 0) issue(first, 0);
#pragma unroll 1
    for (int k = first, it = 0; k >= 0; k -= kRingWarps, it++) {
        const int s0 = k * CH;
        const int nreal = min(CH, len - s0);
        const int q = NB == 2 ? (it & 1) : 0;
        float *sx = sbase + (size_t)q * 64 * SEG;
        float *sg = sx + 32 * SEG;
        const float *xs = sx + lane * SEG, *gs = sg + lane * SEG;
        __syncwarp();  // the previous chunk's reads of its buffers are done
        if (vec && !failed) {
            if (NB == 1) issue(k, 0);
            else if (k - kRingWarps >= 0) issue(k - kRingWarps, q ^ 1);
            const bool ok = mbar_wait(&bars[q], (parity >> q) & 1u);
            parity ^= 1u << q;
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) record_error(a.hdr, TPL_ERR_LOOKBACK_TIMEOUT);
                // bounded: let the copies in flight land before the buffers go unused
                (void)mbar_wait(&bars[q], ((parity >> q) & 1u) ^ 1u);
                if (NB == 2 && k - kRingWarps >= 0) (void)mbar_wait(&bars[q ^ 1], (parity >> (q ^ 1)) & 1u);
                failed = true;
            }
        } else if (!vec) {
            stage_chunk<SEG, SEG>(sx, xin + (size_t)9 * s0, 9 * nreal, lane, false);
            stage_chunk<SEG, SEG>(sg, gin + (size_t)9 * s0, 9 * nreal, lane, false);
            __syncwarp();
        }
        const int j0 = s0 + C * lane;
        float o[3] = {0.f, 0.f, 0.f};  // chunk origin: its first N atom
        float Gl[3] = {0.f, 0.f, 0.f}, Sl[3] = {0.f, 0.f, 0.f};
        if (!failed) {
#pragma unroll
            for (int c = 0; c < 3; c++) o[c] = sx[c];
            float xb[9 * C], gb[9 * C];
#pragma unroll
            for (int r = 0; r < C; r++) {
                fetch_residue<false>(xs, xb, r, r == 0);
                fetch_residue<false>(gs, gb, r, r == 0);
                if (j0 + r < len) {
#pragma unroll
                    for (int at = 0; at < 3; at++) {
                        const float *x = xb + 9 * r + 3 * at, *g = gb + 9 * r + 3 * at;
                        const float xr[3] = {x[0] - o[0], x[1] - o[1], x[2] - o[2]};
                        float xg[3];
                        cross3(xr, g, xg);
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            Gl[c] += g[c];
                            Sl[c] += xg[c];
                        }
                    }
                }
            }
        }
        float G[3], S[3], tg[3], ts[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            G[i] = warp_suffix_excl(Gl[i], lane, tg[i]);
            S[i] = warp_suffix_excl(Sl[i], lane, ts[i]);
        }
        // the carry from chunk k + 1, moved to this chunk's origin: S_o = S_oc + (oc - o) x Gc
        float Gc[3] = {0.f, 0.f, 0.f}, Sc[3] = {0.f, 0.f, 0.f}, nN[3] = {0.f, 0.f, 0.f};
        if (k + 1 < nchunk) {
            ring_wait(k);
            const float *cin = s_ring[k & 3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                Gc[c] = cin[c];
                Sc[c] = cin[3 + c];
                nN[c] = cin[6 + c];
            }
            const float d[3] = {nN[0] - o[0], nN[1] - o[1], nN[2] - o[2]};
            float dx[3];
            cross3(d, Gc, dx);
#pragma unroll
            for (int c = 0; c < 3; c++) Sc[c] += dx[c];
        }
        if (k > 0) {
            if (lane == 0) {
                float *cout = s_ring[(k - 1) & 3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    cout[c] = Gc[c] + tg[c];
                    cout[3 + c] = Sc[c] + ts[c];
                    cout[6 + c] = o[c];
                }
            }
            ring_signal(k - 1);
        }
        if (failed) continue;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            G[i] += Gc[i];
            S[i] += Sc[i];
        }
        // N after the lane's last residue: the next lane's first N, or the next chunk's
        float nxt[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float nb = __shfl_down_sync(0xffffffffu, xs[c], 1);
            nxt[c] = (lane == 31 ? nN[c] : nb) - o[c];
        }
        float gph[C], gps[C], gom[C];
        {
            float xb[9 * C], gb[9 * C];
#pragma unroll
            for (int r = C - 1; r >= 0; r--) {
                fetch_residue<true>(xs, xb, r, r == C - 1);
                fetch_residue<true>(gs, gb, r, r == C - 1);
                const int j = j0 + r;
                float xN[3], xA[3], xC[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    xN[c] = xb[9 * r + c] - o[c];
                    xA[c] = xb[9 * r + 3 + c] - o[c];
                    xC[c] = xb[9 * r + 6 + c] - o[c];
                }
                const float *gN = gb + 9 * r, *gA = gb + 9 * r + 3, *gC = gb + 9 * r + 6;
                float u[3], tmp[3], cr[3];
                // omega_j: axis C -> N_{j+1}, through N_{j+1}
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (nxt[c] - xC[c]) * inv_d2;
                cross3(nxt, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                gom[r] = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                // psi_j: axis CA -> C, through C
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (xC[c] - xA[c]) * inv_d1;
                cross3(xC, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                gps[r] = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                const bool in = j < len;
                if (in) {
                    cross3(xC, gC, cr);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        G[c] += gC[c];
                        S[c] += cr[c];
                    }
                }
                // phi_j: axis N -> CA, through CA
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (xA[c] - xN[c]) * inv_d0;
                cross3(xA, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                gph[r] = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                if (in) {
                    cross3(xA, gA, cr);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        G[c] += gA[c];
                        S[c] += cr[c];
                    }
                    cross3(xN, gN, cr);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        G[c] += gN[c];
                        S[c] += cr[c];
                    }
                }
#pragma unroll
                for (int c = 0; c < 3; c++) nxt[c] = xN[c];
            }
        }
        // zeros at and past len; psi and omega of the last residue move nothing
#pragma unroll
        for (int r = 0; r < C; r++) {
            const int j = j0 + r;
            const bool ok = j < len, last = j == len - 1;
            gph[r] = ok ? gph[r] : 0.f;
            gps[r] = ok && !last ? gps[r] : 0.f;
            gom[r] = ok && !last ? gom[r] : 0.f;
        }
        if (vec) {
#pragma unroll
            for (int i = 0; i < C / 4; i++) {
                const int j = j0 + 4 * i;
                if (j < a.L) {
                    __stcs(reinterpret_cast<float4 *>(gout + j),
                           make_float4(gph[4 * i], gph[4 * i + 1], gph[4 * i + 2], gph[4 * i + 3]));
                    __stcs(reinterpret_cast<float4 *>(gout + a.L + j),
                           make_float4(gps[4 * i], gps[4 * i + 1], gps[4 * i + 2], gps[4 * i + 3]));
                    __stcs(reinterpret_cast<float4 *>(gout + 2 * a.L + j),
                           make_float4(gom[4 * i], gom[4 * i + 1], gom[4 * i + 2], gom[4 * i + 3]));
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < C; r++) {
                const int j = j0 + r;
                if (j < a.L) {
                    gout[j] = gph[r];
                    gout[a.L + j] = gps[r];
                    gout[2 * a.L + j] = gom[r];
                }
            }
        }
    }
}

// Sincos check kernel for the tests: s[i], c[i] = sincos_poly(a[i]).
// Even elements through the paired form (the kernels' fast path), odd elements
// through sincos_poly; |a| > 1e4 always through sincos_poly.
__global__ void sincos_poly_kernel(const float *a, float *s, float *c, int n) {
    const int i = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    const float x0 = a[i], x1 = i + 1 < n ? a[i + 1] : 0.f;
    if (fabsf(x0) <= 1.0e4f && fabsf(x1) <= 1.0e4f) {
        float s1, c1;
        sincos_fast2(x0, x1, s + i, c + i, &s1, &c1);
        if (i + 1 < n) {
            sincos_poly(x1, s + i + 1, c + i + 1);
        }
    } else {
        sincos_poly(x0, s + i, c + i);
        if (i + 1 < n) sincos_poly(x1, s + i + 1, c + i + 1);
    }
}

template <int C>
constexpr int fwd_smem() {
    return kWarpsPerCta * (FwdStage<C>::FLOATS + AngBuf<C>::FLOATS) * (int)sizeof(float);
}
template <int C>
constexpr int bwd_smem() {  // positions and dL/dx of every lane, padded lane stride 9C + 4
    return kWarpsPerCta * 64 * (9 * C + 4) * (int)sizeof(float);
}

ChainArgs chain_args(const float *angles, const int32_t *lengths, void *ws, int B, int L, const tpl_options &opt) {
    ChainArgs a{};
    a.angles = angles;
    a.lengths = lengths;
    a.hdr = reinterpret_cast<WsHeader *>(ws);
    a.rec = reinterpret_cast<ChainRecord *>(reinterpret_cast<char *>(ws) + sizeof(WsHeader));
    a.B = B;
    a.L = L;
    a.nrec = (L + kRecordStride - 1) / kRecordStride;
    a.renorm = opt.renormalize >= 0 ? 1 : 0;
    a.fp64_min = opt.fp64_carry_min_len > 0 ? opt.fp64_carry_min_len : 0;
    a.bc = bond_constants();
    return a;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

template <typename K>
int launch_chain(K kernel, int smem, int B, const ChainArgs &a, cudaStream_t st) {
    if (!set_max_dynamic_smem(reinterpret_cast<const void *>(kernel), smem))
        return TPL_ERR_LAUNCH;
    const int grid = (B + kWarpsPerCta - 1) / kWarpsPerCta;
    kernel<<<grid, 32 * kWarpsPerCta, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

template <typename K>
int launch_ring(K kernel, int smem, int B, const ChainArgs &a, cudaStream_t st) {
    if (!set_max_dynamic_smem(reinterpret_cast<const void *>(kernel), smem))
        return TPL_ERR_LAUNCH;
    kernel<<<B, 32 * kRingWarps, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

}  // namespace

int a2b_chain_record_stride() { return kRecordStride; }

int a2b_forward_chain(const float *angles, const int32_t *lengths, float *coords, void *ws, int B, int L,
                      const tpl_options &opt, cudaStream_t st) {
    if (B == 0 || L == 0) return TPL_OK;
    ChainArgs a = chain_args(angles, lengths, ws, B, L, opt);
    a.coords = coords;
    a.vec = (L % 4 == 0) && aligned16(angles) && aligned16(coords);
    const int C = opt.residues_per_thread > 0 ? opt.residues_per_thread : 8;
    const bool ring = opt.threads_per_cta == kRingWarps;
    const int carry_bytes = a.fp64_min > 0 ? kRingWarps * 12 * (int)sizeof(double) : 0;  // FP64 carry slots
    switch (C) {
        case 4:
            return ring ? launch_ring(a2b_fwd_ring_kernel<4>, fwd_smem<4>() + carry_bytes, B, a, st)
                        : launch_chain(a2b_fwd_chain_kernel<4>, fwd_smem<4>(), B, a, st);
        case 8:
            return ring ? launch_ring(a2b_fwd_ring_kernel<8>, fwd_smem<8>() + carry_bytes, B, a, st)
                        : launch_chain(a2b_fwd_chain_kernel<8>, fwd_smem<8>(), B, a, st);
    }
    return TPL_ERR_UNSUPPORTED;
}

int a2b_backward_chain(float *grad_angles, const float *grad_coords, const float *angles, const int32_t *lengths,
                       void *ws, int B, int L, const tpl_options &opt, cudaStream_t st) {
    if (B == 0 || L == 0) return TPL_OK;
    ChainArgs a = chain_args(angles, lengths, ws, B, L, opt);
    a.grad_angles = grad_angles;
    a.grad_coords = grad_coords;
    a.vec = (L % 4 == 0) && aligned16(angles) && aligned16(grad_angles) && aligned16(grad_coords);
    const int C = opt.residues_per_thread > 0 ? opt.residues_per_thread : 8;
    switch (C) {
        case 4: return launch_chain(a2b_bwd_chain_kernel<4>, bwd_smem<4>(), B, a, st);
        case 8: return launch_chain(a2b_bwd_chain_kernel<8>, bwd_smem<8>(), B, a, st);
    }
    return TPL_ERR_UNSUPPORTED;
}

int a2b_backward_coords(float *grad_angles, const float *grad_coords, const float *coords, const int32_t *lengths,
                        void *ws, int B, int L, const tpl_options &opt, cudaStream_t st) {
    if (B == 0 || L == 0) return TPL_OK;
    ChainArgs a = chain_args(nullptr, lengths, ws, B, L, opt);
    a.coords = const_cast<float *>(coords);  // read only
    a.grad_angles = grad_angles;
    a.grad_coords = grad_coords;
    a.vec = (L % 4 == 0) && aligned16(coords) && aligned16(grad_angles) && aligned16(grad_coords);
    const int C = opt.residues_per_thread > 0 ? opt.residues_per_thread : 4;
    const int NB = opt.copy_buffers > 0 ? opt.copy_buffers : 1;
    constexpr int smem4 = kWarpsPerCta * 64 * 36 * (int)sizeof(float);
    constexpr int smem8 = kWarpsPerCta * 64 * 72 * (int)sizeof(float);
    // automatic: four warps per chain from 384 residues (three or more 128-residue
    // chunks), one warp per chain for shorter chains (measured on GB300)
    if (opt.threads_per_cta == kRingWarps || (opt.threads_per_cta == 0 && L >= 384)) {
        if (C == 4 && NB == 1) return launch_ring(a2b_bwd_coords_ring_kernel<4, 1>, smem4, B, a, st);
        if (C == 4 && NB == 2) return launch_ring(a2b_bwd_coords_ring_kernel<4, 2>, 2 * smem4, B, a, st);
        if (C == 8 && NB == 1) return launch_ring(a2b_bwd_coords_ring_kernel<8, 1>, smem8, B, a, st);
        return TPL_ERR_UNSUPPORTED;
    }
    if (C == 4 && NB == 1) return launch_chain(a2b_bwd_coords_kernel<4, 1>, smem4, B, a, st);
    if (C == 4 && NB == 2) return launch_chain(a2b_bwd_coords_kernel<4, 2>, 2 * smem4, B, a, st);
    if (C == 8 && NB == 1) return launch_chain(a2b_bwd_coords_kernel<8, 1>, smem8, B, a, st);
    return TPL_ERR_UNSUPPORTED;
}

int sincos_poly_f32(const float *a, float *s, float *c, int n, cudaStream_t st) {
    if (n <= 0) return TPL_OK;
    sincos_poly_kernel<<<((n + 1) / 2 + 255) / 256, 256, 0, st>>>(a, s, c, n);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

}  // namespace tpl
