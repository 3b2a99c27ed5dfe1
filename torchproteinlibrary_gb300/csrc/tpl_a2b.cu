// Angles2Backbone kernels for sm_103a.
//
// Forward (reference: Layers/ReducedModel/cBackboneProteinCUDAKernels.cu:6-41 runs
// one thread per chain over 3L serial 4x4 products).  Here the chain of bond
// transforms is a parallel scan:
//   * work item = (chain, tile of R*NT residues), handed out by an atomic ticket
//     counter to a persistent grid, tiles of a chain in order;
//   * each thread composes the 3R joints of its R residues from identity (walk 1),
//     warps scan the per-thread transforms with shuffles, warp totals are scanned
//     in shared memory;
//   * chains longer than a tile get the carry from earlier tiles by decoupled
//     look-back on per-tile records (aggregate / inclusive prefix), composed in
//     FP64 for chains of at least fp64_carry_min_len residues;
//   * each thread re-walks its residues from its world prefix (walk 2) and the
//     tile's N, CA, C positions are staged in shared memory and written with
//     coalesced float4 stores, zeros past the chain length.
//
// Backward (reference: computeGradientsOptimizedBackbone + backwardFromCoordinates-
// Backbone, cBackboneProteinCUDAKernels.cu:84-163, which materialise dR/dangle of
// size 27 L^2 per chain).  Here the adjoint is a reverse suffix scan: with u_m the
// rotation axis of joint m (x-axis of frame m) and x_m its origin,
//     dL/dtheta_m = u_m . sum_{i>m} (x_i - x_m) x g_i = u_m . (S_m - x_m x G_m),
// G_m = sum_{i>m} g_i, S_m = sum_{i>m} x_i x g_i.  The kernel recomputes the
// forward positions (angles are 3x smaller than coordinates), scans (G, S)
// backwards over threads, warps and tiles (tiles handed out last-first), and
// evaluates the three joint gradients of each residue.
#include <algorithm>
#include <cstdio>

#include "tpl_common.cuh"
#include "tpl_internal.h"
#include "tpl_topology.cuh"

namespace tpl {

constexpr unsigned kSpinLimit = 1u << 22;  // ~0.5 s of 100 ns sleeps

struct A2bArgs {
    const float *angles;
    const int *lengths;
    float *coords;
    float *grad_angles;
    const float *grad_coords;
    WsHeader *hdr;
    TileRecord *rec;
    int L, ntiles, total;
    int fp64_min_len;
    int renorm;
    BondConsts bc;
};

__device__ __forceinline__ void record_error(WsHeader *h, int code) {
    atomicCAS(&h->status, 0u, (unsigned)code);
}

// Write n_total floats to global dst: src[i] (shared) for i < n_valid, 0 after.
// 16-byte aligned body as float4, scalar head/tail.
template <int NT>
__device__ __forceinline__ void store_floats(float *dst, const float *src, int n_valid, int n_total) {
    const int tid = threadIdx.x;
    int head = (int)(((16u - ((unsigned)(uintptr_t)dst & 15u)) & 15u) >> 2);
    head = min(head, n_total);
    for (int i = tid; i < head; i += NT) dst[i] = i < n_valid ? src[i] : 0.f;
    const int nvec = (n_total - head) >> 2;
    float4 *d4 = reinterpret_cast<float4 *>(dst + head);
    for (int v = tid; v < nvec; v += NT) {
        const int i = head + 4 * v;
        float4 x;
        x.x = i < n_valid ? src[i] : 0.f;
        x.y = i + 1 < n_valid ? src[i + 1] : 0.f;
        x.z = i + 2 < n_valid ? src[i + 2] : 0.f;
        x.w = i + 3 < n_valid ? src[i + 3] : 0.f;  // src is only read below n_valid
        d4[v] = x;
    }
    for (int i = head + 4 * nvec + tid; i < n_total; i += NT) dst[i] = i < n_valid ? src[i] : 0.f;
}

// Load n floats from global src into shared dst (coalesced).
template <int NT>
__device__ __forceinline__ void load_floats(float *dst, const float *src, int n) {
    const int tid = threadIdx.x;
    int head = (int)(((16u - ((unsigned)(uintptr_t)src & 15u)) & 15u) >> 2);
    head = min(head, n);
    for (int i = tid; i < head; i += NT) dst[i] = __ldg(src + i);
    const int nvec = (n - head) >> 2;
    const float4 *s4 = reinterpret_cast<const float4 *>(src + head);
    for (int v = tid; v < nvec; v += NT) {
        float4 x = __ldg(s4 + v);
        const int i = head + 4 * v;
        dst[i] = x.x; dst[i + 1] = x.y; dst[i + 2] = x.z; dst[i + 3] = x.w;
    }
    for (int i = head + 4 * nvec + tid; i < n; i += NT) dst[i] = __ldg(src + i);
}

__device__ __forceinline__ void round_to_float(Frame<double> &f) {
#pragma unroll
    for (int i = 0; i < 9; i++) f.r[i] = (double)(float)f.r[i];
#pragma unroll
    for (int i = 0; i < 3; i++) f.p[i] = (double)(float)f.p[i];
}

__device__ __forceinline__ void store_frame_d(double *dst, const Frame<double> &f) { frame_store(dst, f); }

// Spin (bounded) until the record flag carries this launch's epoch and a state.
__device__ __forceinline__ unsigned wait_flag(const unsigned *flag, unsigned epoch_bits, WsHeader *h, bool &ok) {
    unsigned f = 0;
    for (unsigned spins = 0;; spins++) {
        f = ld_acquire(flag);
        if ((f & ~3u) == epoch_bits && (f & 3u)) return f;
        if (spins >= kSpinLimit) {
            record_error(h, TPL_ERR_LOOKBACK_TIMEOUT);
            ok = false;
            return 0;
        }
        __nanosleep(100);
    }
}

__device__ const SinCosTableC g_sincos_tab = make_sincos_table();

template <int NT>
__device__ __forceinline__ void load_sincos_table(float4 *s_tab) {
    const float4 *src = reinterpret_cast<const float4 *>(&g_sincos_tab);
    for (int i = threadIdx.x; i < 65; i += NT) s_tab[i] = src[i];
}

// Walk 1 of a tile: each thread composes the joints of its R residues from
// identity, recording the thread-local positions of N, CA and C in shared memory
// (s_loc[(9 r + c) * NT + tid], conflict-free).  Returns the thread's aggregate
// transform.  omega of the chain's last residue moves nothing and is skipped.
template <int R, int NT>
__device__ __forceinline__ Frame<float> walk_local(const A2bArgs &a, const float4 *s_tab, const float *ang0,
                                                   const float *ang1, const float *ang2, int j0, int nreal,
                                                   bool chain_end, float *s_loc) {
    Frame<float> agg;
    frame_identity(agg);
    float *l = s_loc + threadIdx.x;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int j = j0 + r;
        if (j < nreal) {
            float s, c;
            l[(9 * r + 0) * NT] = agg.p[0]; l[(9 * r + 1) * NT] = agg.p[1]; l[(9 * r + 2) * NT] = agg.p[2];
            sincos_tab(s_tab, ang0[j], &s, &c);
            apply_joint(agg, a.bc.cb[0], a.bc.sb[0], a.bc.d[0], c, s);
            l[(9 * r + 3) * NT] = agg.p[0]; l[(9 * r + 4) * NT] = agg.p[1]; l[(9 * r + 5) * NT] = agg.p[2];
            sincos_tab(s_tab, ang1[j], &s, &c);
            apply_joint(agg, a.bc.cb[1], a.bc.sb[1], a.bc.d[1], c, s);
            l[(9 * r + 6) * NT] = agg.p[0]; l[(9 * r + 7) * NT] = agg.p[1]; l[(9 * r + 8) * NT] = agg.p[2];
            if (!(chain_end && j == nreal - 1)) {
                sincos_tab(s_tab, ang2[j], &s, &c);
                apply_joint(agg, a.bc.cb[2], a.bc.sb[2], a.bc.d[2], c, s);
            }
        }
    }
    return agg;
}

// Warp scan of the thread aggregates; returns the exclusive prefix inside the
// warp and leaves the warp totals in s_wtot.
__device__ __forceinline__ Frame<float> warp_exclusive(Frame<float> agg, bool renorm, Frame<float> *s_wtot) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (renorm) renormalize(agg);
    Frame<float> inc = warp_scan_frames(agg, lane);
    Frame<float> exc = shfl_up_frame(inc, 1);
    if (lane == 0) frame_identity(exc);
    if (lane == 31) s_wtot[w] = inc;
    return exc;
}

// Warp 0: exclusive scan of the NW warp totals across lanes 0..NW-1 (log2 NW
// shuffle steps).  Lane l < NW gets the prefix of warps < l; every lane gets the
// tile aggregate.
template <int NW>
__device__ __forceinline__ Frame<float> warp_totals_scan(const Frame<float> *s_wtot, bool renorm, Frame<float> &tile) {
    const int lane = threadIdx.x & 31;
    Frame<float> f;
    if (lane < NW) f = s_wtot[lane];
    else frame_identity(f);
#pragma unroll
    for (int off = 1; off < NW; off <<= 1) {
        Frame<float> o = shfl_up_frame(f, off);
        if (lane >= off) f = compose(o, f);
    }
    if (renorm) renormalize(f);
    Frame<float> exc = shfl_up_frame(f, 1);
    if (lane == 0) frame_identity(exc);
#pragma unroll
    for (int i = 0; i < 9; i++) tile.r[i] = __shfl_sync(0xffffffffu, f.r[i], NW - 1);
#pragma unroll
    for (int i = 0; i < 3; i++) tile.p[i] = __shfl_sync(0xffffffffu, f.p[i], NW - 1);
    return exc;
}

// FP64 frame arithmetic on 12-double arrays (rotation row-major, translation),
// used by the single look-back thread; kept out of line and in memory so that
// the kernels' register budget is set by their parallel parts.
__device__ __noinline__ void compose_d(double *c, const double *a, const double *b) {
#pragma unroll 1
    for (int i = 0; i < 3; i++) {
        const double a0 = a[3 * i], a1 = a[3 * i + 1], a2 = a[3 * i + 2];
        c[3 * i] = fma(a0, b[0], fma(a1, b[3], a2 * b[6]));
        c[3 * i + 1] = fma(a0, b[1], fma(a1, b[4], a2 * b[7]));
        c[3 * i + 2] = fma(a0, b[2], fma(a1, b[5], a2 * b[8]));
        c[9 + i] = fma(a0, b[9], fma(a1, b[10], fma(a2, b[11], a[9 + i])));
    }
}
__device__ __noinline__ void renormalize_d(double *f) {
    Frame<double> x;
    frame_load(x, f);
    renormalize(x);
    frame_store(f, x);
}
__device__ __noinline__ void round_to_float_d(double *f) {
#pragma unroll 1
    for (int i = 0; i < 12; i++) f[i] = (double)(float)f[i];
}
__device__ __forceinline__ void identity_d(double *f) {
#pragma unroll 1
    for (int i = 0; i < 12; i++) f[i] = (i < 9 && i % 4 == 0) ? 1.0 : 0.0;
}
__device__ __forceinline__ void copy_d(double *d, const double *s) {
#pragma unroll 1
    for (int i = 0; i < 12; i++) d[i] = s[i];
}

// Element e of the composition A o B of two 12-double frames (e < 9: rotation
// entry (e / 3, e % 3); e >= 9: translation entry e - 9).
__device__ __forceinline__ double compose_elem(const double *A, const double *B, int e) {
    if (e < 9) {
        const int i = e / 3, j = e % 3;
        return fma(A[3 * i], B[j], fma(A[3 * i + 1], B[3 + j], A[3 * i + 2] * B[6 + j]));
    }
    const int i = e - 9;
    return fma(A[3 * i], B[9], fma(A[3 * i + 1], B[10], fma(A[3 * i + 2], B[11], A[9 + i])));
}

__device__ __forceinline__ float frame_elem(const Frame<float> &f, int e) {
    float v = 0.f;
#pragma unroll
    for (int k = 0; k < 12; k++) v = (e == k) ? (k < 9 ? f.r[k] : f.p[k - 9]) : v;
    return v;
}

// Forward inter-tile carry by decoupled look-back, executed by one full warp.
// FP64 is slow on GB300 and a one-lane FP64 instruction costs a full pipe slot,
// so every FP64 frame product is spread over 12 lanes (one entry each, 3 FMA).
// Lane i polls the flag of predecessor tile t-1-i; the published frames are then
// folded from the nearest inclusive prefix.  `carry` (12 doubles, shared) receives
// the chain frame at the start of tile t; `scr` holds 36 doubles of shared memory.
__device__ __noinline__ void fwd_carry_warp(const A2bArgs &a, int b, int t, bool more, const Frame<float> &tile_agg,
                                            unsigned epoch_bits, bool use64, double *carry, double *scr) {
    const int lane = threadIdx.x & 31;
    const bool el = lane < 12;
    TileRecord *base = a.rec + (size_t)b * a.ntiles;
    double *acc = scr, *agg = scr + 24;
    if (el) {
        agg[lane] = (double)frame_elem(tile_agg, lane);
        acc[lane] = (lane < 9 && lane % 4 == 0) ? 1.0 : 0.0;
    }
    __syncwarp();
    if (t > 0 && more) {
        if (el) base[t].fagg[lane] = agg[lane];
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(&base[t].fflag, epoch_bits | kFlagAgg);
    }
    bool ok = true;
    for (int tt0 = t - 1; tt0 >= 0; tt0 -= 32) {
        const int tt = tt0 - lane;
        bool lane_ok = true;
        unsigned f = 0;
        if (tt >= 0) f = wait_flag(&base[tt].fflag, epoch_bits, a.hdr, lane_ok);
        if (__ballot_sync(0xffffffffu, !lane_ok)) {
            ok = false;
            break;
        }
        const unsigned incm = __ballot_sync(0xffffffffu, tt >= 0 && (f & 3u) == kFlagInc);
        const int stop = incm ? __ffs(incm) - 1 : min(31, tt0);
        for (int i = 0; i <= stop; i++) {
            const TileRecord *q = base + (tt0 - i);
            double v = 0.0;
            if (el) {
                (void)ld_acquire(&q->fflag);
                v = compose_elem((incm && i == stop) ? q->finc : q->fagg, acc, lane);
            }
            __syncwarp();
            if (el) acc[lane] = use64 ? v : (double)(float)v;
            __syncwarp();
        }
        if (incm) break;
    }
    if (!ok && el) acc[lane] = (lane < 9 && lane % 4 == 0) ? 1.0 : 0.0;
    __syncwarp();
    if (el) {
        carry[lane] = acc[lane];
        if (t > 0) base[t].fexc[lane] = acc[lane];
    }
    // test hook: the first tile of chain 0 stays unpublished when the workspace asks
    // for it, so that its successor's bounded wait runs out
    const bool skip = (t == 0 && b == 0 && a.hdr->test_skip_publish);
    if (more && !skip) {
        if (el) {
            const double v = compose_elem(acc, agg, lane);
            base[t].finc[lane] = use64 ? v : (double)(float)v;
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(&base[t].fflag, epoch_bits | kFlagInc);
    }
    __syncwarp();
}

// Backward suffix look-back over the later tiles of a chain, executed by one full
// warp; lanes 0..5 own one component of (G, S) each (S about the world origin,
// FP64).  own: this tile's sums (shared); carry: the sums over all later tiles.
__device__ __noinline__ void bwd_carry_warp(const A2bArgs &a, int b, int t, int t_last, const double *own,
                                            unsigned epoch_bits, double *carry) {
    const int lane = threadIdx.x & 31;
    const bool el = lane < 6;
    TileRecord *base = a.rec + (size_t)b * a.ntiles;
    double c = 0.0;
    if (t > 0 && t < t_last) {
        if (el) base[t].bagg[lane] = own[lane];
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(&base[t].bflag, epoch_bits | kFlagAgg);
    }
    bool ok = true;
    for (int tt0 = t + 1; tt0 <= t_last; tt0 += 32) {
        const int tt = tt0 + lane;
        bool lane_ok = true;
        unsigned f = 0;
        if (tt <= t_last) f = wait_flag(&base[tt].bflag, epoch_bits, a.hdr, lane_ok);
        if (__ballot_sync(0xffffffffu, !lane_ok)) {
            ok = false;
            break;
        }
        const unsigned incm = __ballot_sync(0xffffffffu, tt <= t_last && (f & 3u) == kFlagInc);
        const int stop = incm ? __ffs(incm) - 1 : min(31, t_last - tt0);
        if (el)
            for (int i = 0; i <= stop; i++) {
                const TileRecord *q = base + tt0 + i;
                (void)ld_acquire(&q->bflag);
                c += (incm && i == stop) ? q->binc[lane] : q->bagg[lane];
            }
        if (incm) break;
    }
    if (!ok) c = 0.0;
    if (el) carry[lane] = c;
    if (t > 0) {
        if (el) base[t].binc[lane] = own[lane] + c;
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(&base[t].bflag, epoch_bits | kFlagInc);
    }
    __syncwarp();
}

// Lanes 0..5 of a warp: own[k] = tile sums (G, S) moved from the tile origin o to
// the world origin (S + o x G), from the FP32 totals present in every lane.
__device__ __forceinline__ void own_sums_world(const float *tot, const float *o, double *own) {
    const int k = threadIdx.x & 31;
    if (k < 3) {
        own[k] = (double)tot[k];
    } else if (k < 6) {
        const int i = k - 3, i1 = (i + 1) % 3, i2 = (i + 2) % 3;
        own[k] = (double)tot[3 + i] + fma((double)o[i1], (double)tot[i2], -(double)o[i2] * (double)tot[i1]);
    }
    __syncwarp();
}

// Every lane: the carry from later tiles moved to the tile origin o,
// S_o = S_world - o x G, in FP32.
__device__ __forceinline__ void carry_to_origin(const double *cw, const float *o, float *g, float *sv) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
        g[i] = (float)cw[i];
        sv[i] = (float)(cw[3 + i] - ((double)o[i1] * cw[i2] - (double)o[i2] * cw[i1]));
    }
}

__device__ __forceinline__ void finish_launch(unsigned *ticket, unsigned *done, unsigned *epoch) {
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned prev = atomicAdd(done, 1u);
        if (prev == gridDim.x - 1) {
            atomicExch(ticket, 0u);
            atomicExch(done, 0u);
            __threadfence();
            atomicAdd(epoch, 1u);
        }
    }
}

template <int R, int NT>
__global__ void __launch_bounds__(NT, 5) a2b_fwd_f32_kernel(A2bArgs a) {
    constexpr int TILE = R * NT;
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) float s_dyn[];
    float(*s_ang)[TILE] = reinterpret_cast<float(*)[TILE]>(s_dyn);  // [3][TILE]
    float *s_loc = s_dyn + 3 * TILE;                                 // [9 * TILE]
    __shared__ float4 s_tab[65];
    __shared__ Frame<float> s_wtot[NW];
    __shared__ Frame<float> s_wpre[NW];
    __shared__ Frame<float> s_carry;
    __shared__ double s_fcarry[12], s_fscratch[36];
    __shared__ float s_org[3];
    __shared__ int s_item;
    __shared__ unsigned s_epoch;

    const int tid = threadIdx.x, w = tid >> 5;
    if (tid == 0) s_epoch = (*(volatile unsigned *)&a.hdr->fwd_epoch & 0x3fffffffu) << 2;
    load_sincos_table<NT>(s_tab);

    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(&a.hdr->fwd_ticket, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= a.total) break;
        const int b = item / a.ntiles, t = item - b * a.ntiles;
        int len = a.lengths[b];
        if (len < 0 || len > a.L) {
            if (tid == 0) record_error(a.hdr, TPL_ERR_LENGTH);
            len = max(0, min(len, a.L));
        }
        const int s0 = t * TILE;
        const int ntile = min(TILE, a.L - s0);
        const int nreal = max(0, min(ntile, len - s0));
        float *out = a.coords + (size_t)b * 9 * a.L + (size_t)9 * s0;
        if (nreal < ntile) store_floats<NT>(out + 9 * nreal, nullptr, 0, 9 * (ntile - nreal));
        if (nreal == 0) {
            __syncthreads();
            continue;
        }
        const float *ang = a.angles + (size_t)b * 3 * a.L + s0;
        load_floats<NT>(s_ang[0], ang, nreal);
        load_floats<NT>(s_ang[1], ang + a.L, nreal);
        load_floats<NT>(s_ang[2], ang + 2 * a.L, nreal);
        __syncthreads();

        const bool chain_end = (s0 + nreal == len);
        const int j0 = tid * R;
        Frame<float> agg = walk_local<R, NT>(a, s_tab, s_ang[0], s_ang[1], s_ang[2], j0, nreal, chain_end, s_loc);
        Frame<float> exc = warp_exclusive(agg, a.renorm, s_wtot);
        __syncthreads();

        if (w == 0) {
            Frame<float> tile;
            Frame<float> wexc = warp_totals_scan<NW>(s_wtot, a.renorm, tile);
            const bool more = s0 + TILE < len;
            const bool use64 = a.fp64_min_len >= 0 && len >= a.fp64_min_len;
            fwd_carry_warp(a, b, t, more, tile, s_epoch, use64, s_fcarry, s_fscratch);
            Frame<float> c32;
            frame_load(c32, s_fcarry);
            if (tid == 0) {
                s_org[0] = c32.p[0]; s_org[1] = c32.p[1]; s_org[2] = c32.p[2];
            }
            c32.p[0] = c32.p[1] = c32.p[2] = 0.f;  // positions relative to the tile origin
            if (a.renorm) renormalize(c32);
            if (tid < NW) s_wpre[tid] = compose(c32, wexc);
        }
        __syncthreads();

        // walk 2: world position = P (x) local position, written straight to HBM
        Frame<float> P = compose(s_wpre[w], exc);
        if (a.renorm) renormalize(P);
        const float t0 = P.p[0] + s_org[0], t1 = P.p[1] + s_org[1], t2 = P.p[2] + s_org[2];
        float *dst = out + (size_t)9 * j0;
        const bool vec = (R % 4 == 0) && (j0 + R <= nreal) && ((((uintptr_t)dst) & 15u) == 0);
        const float *l = s_loc + tid;
        auto world = [&](int e) {  // element e = 9 r + 3 q + c of this thread's output
            const int r = e / 9, q = (e % 9) / 3, c = e % 3;
            const float x = l[(9 * r + 3 * q) * NT], y = l[(9 * r + 3 * q + 1) * NT], z = l[(9 * r + 3 * q + 2) * NT];
            const float tc = c == 0 ? t0 : (c == 1 ? t1 : t2);
            return fmaf(P.r[3 * c], x, fmaf(P.r[3 * c + 1], y, fmaf(P.r[3 * c + 2], z, tc)));
        };
        if (vec) {
            float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll
            for (int i = 0; i < 9 * R / 4; i++)
                d4[i] = make_float4(world(4 * i), world(4 * i + 1), world(4 * i + 2), world(4 * i + 3));
        } else {
#pragma unroll
            for (int e = 0; e < 9 * R; e++)
                if (j0 + e / 9 < nreal) dst[e] = world(e);
        }
        __syncthreads();
    }
    finish_launch(&a.hdr->fwd_ticket, &a.hdr->fwd_done, &a.hdr->fwd_epoch);
}

// ------------------------------------------------------------------ backward
__device__ __forceinline__ float warp_suffix_exclusive(float v, int lane, float &total) {
    // inclusive suffix sum: sum over lanes >= lane
    float inc = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        float o = __shfl_down_sync(0xffffffffu, inc, off);
        if (lane + off < 32) inc += o;
    }
    total = __shfl_sync(0xffffffffu, inc, 0);
    return inc - v;
}

// Rotate a vector by R^T (into a frame's local coordinates) and by R.
__device__ __forceinline__ void rot_t(const Frame<float> &f, const float *v, float *o) {
    o[0] = fmaf(f.r[0], v[0], fmaf(f.r[3], v[1], f.r[6] * v[2]));
    o[1] = fmaf(f.r[1], v[0], fmaf(f.r[4], v[1], f.r[7] * v[2]));
    o[2] = fmaf(f.r[2], v[0], fmaf(f.r[5], v[1], f.r[8] * v[2]));
}
__device__ __forceinline__ void rot(const Frame<float> &f, const float *v, float *o) {
    o[0] = fmaf(f.r[0], v[0], fmaf(f.r[1], v[1], f.r[2] * v[2]));
    o[1] = fmaf(f.r[3], v[0], fmaf(f.r[4], v[1], f.r[5] * v[2]));
    o[2] = fmaf(f.r[6], v[0], fmaf(f.r[7], v[1], f.r[8] * v[2]));
}

// The adjoint is evaluated in each thread's local frame (the frame its walk
// started from): for a rigid motion (R, p), u . sum (x_i - x_m) x g_i is
// unchanged when u and x are replaced by their local coordinates and g by
// R^T g.  Each thread therefore only rotates its upstream gradients (27 FMA per
// residue); joint axes are its local bond directions.
template <int R, int NT>
__global__ void __launch_bounds__(NT, 5) a2b_bwd_f32_kernel(A2bArgs a) {
    constexpr int TILE = R * NT;
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) float s_dyn[];
    float(*s_ang)[TILE] = reinterpret_cast<float(*)[TILE]>(s_dyn);  // [3][TILE]
    float *s_g = s_dyn + 3 * TILE;                                   // [9 * TILE]
    float *s_loc = s_dyn + 12 * TILE;                                // [9 * TILE]
    __shared__ float4 s_tab[65];
    __shared__ Frame<float> s_wtot[NW];
    __shared__ Frame<float> s_wpre[NW];
    __shared__ float s_wsum[NW][6];
    __shared__ float s_wsuf[NW][6];
    __shared__ double s_bown[6], s_bcarry[6];
    __shared__ float s_org[3];
    __shared__ int s_item;
    __shared__ unsigned s_epoch;

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) s_epoch = (*(volatile unsigned *)&a.hdr->bwd_epoch & 0x3fffffffu) << 2;
    load_sincos_table<NT>(s_tab);
    const float inv_d0 = 1.f / a.bc.d[0], inv_d1 = 1.f / a.bc.d[1], inv_d2 = 1.f / a.bc.d[2];

    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(&a.hdr->bwd_ticket, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= a.total) break;
        const int b = item / a.ntiles, t = a.ntiles - 1 - (item - b * a.ntiles);
        int len = a.lengths[b];
        if (len < 0 || len > a.L) {
            if (tid == 0) record_error(a.hdr, TPL_ERR_LENGTH);
            len = max(0, min(len, a.L));
        }
        const int s0 = t * TILE;
        const int ntile = min(TILE, a.L - s0);
        const int nreal = max(0, min(ntile, len - s0));
        float *gout = a.grad_angles + (size_t)b * 3 * a.L + s0;
        if (nreal == 0) {
            for (int k = 0; k < 3; k++) store_floats<NT>(gout + (size_t)k * a.L, nullptr, 0, ntile);
            __syncthreads();
            continue;
        }
        const float *ang = a.angles + (size_t)b * 3 * a.L + s0;
        load_floats<NT>(s_ang[0], ang, nreal);
        load_floats<NT>(s_ang[1], ang + a.L, nreal);
        load_floats<NT>(s_ang[2], ang + 2 * a.L, nreal);
        load_floats<NT>(s_g, a.grad_coords + (size_t)b * 9 * a.L + (size_t)9 * s0, 9 * nreal);
        __syncthreads();

        const bool chain_end = (s0 + nreal == len);
        const int j0 = tid * R;
        Frame<float> agg = walk_local<R, NT>(a, s_tab, s_ang[0], s_ang[1], s_ang[2], j0, nreal, chain_end, s_loc);
        const float nx = agg.p[0], ny = agg.p[1], nz = agg.p[2];  // N after the thread's last residue
        Frame<float> exc = warp_exclusive(agg, a.renorm, s_wtot);
        __syncthreads();

        if (w == 0) {
            Frame<float> tile;
            Frame<float> wexc = warp_totals_scan<NW>(s_wtot, a.renorm, tile);
            Frame<float> c32;
            if (t == 0) frame_identity(c32);
            else frame_load(c32, a.rec[(size_t)b * a.ntiles + t].fexc);
            if (tid == 0) {
                s_org[0] = c32.p[0]; s_org[1] = c32.p[1]; s_org[2] = c32.p[2];
            }
            c32.p[0] = c32.p[1] = c32.p[2] = 0.f;
            if (tid < NW) s_wpre[tid] = compose(c32, wexc);
        }
        __syncthreads();

        Frame<float> P = compose(s_wpre[w], exc);
        if (a.renorm) renormalize(P);
        // rotate this thread's upstream gradients into its local frame (in place)
        // and sum G' = sum g', S' = sum x_local x g'
        float Gl[3] = {0.f, 0.f, 0.f}, Sl[3] = {0.f, 0.f, 0.f};
        const float *lp = s_loc + tid;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int j = j0 + r;
            if (j < nreal) {
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    float *gp = s_g + 9 * j + 3 * q;
                    float gw[3] = {gp[0], gp[1], gp[2]}, gl[3], xg[3];
                    rot_t(P, gw, gl);
                    gp[0] = gl[0]; gp[1] = gl[1]; gp[2] = gl[2];
                    const float xq[3] = {lp[(9 * r + 3 * q) * NT], lp[(9 * r + 3 * q + 1) * NT],
                                         lp[(9 * r + 3 * q + 2) * NT]};
                    cross3(xq, gl, xg);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        Gl[c] += gl[c];
                        Sl[c] += xg[c];
                    }
                }
            }
        }
        // thread totals in the tile frame: G = R G', S = R S' + p x G
        float Gt[3], St[3], pxg[3];
        rot(P, Gl, Gt);
        rot(P, Sl, St);
        cross3(P.p, Gt, pxg);
#pragma unroll
        for (int c = 0; c < 3; c++) St[c] += pxg[c];
        float suf[6], wt[6];
        const float v6[6] = {Gt[0], Gt[1], Gt[2], St[0], St[1], St[2]};
#pragma unroll
        for (int i = 0; i < 6; i++) suf[i] = warp_suffix_exclusive(v6[i], lane, wt[i]);
        if (lane == 0)
#pragma unroll
            for (int i = 0; i < 6; i++) s_wsum[w][i] = wt[i];
        __syncthreads();
        if (w == 0) {
            float tot6[6];
#pragma unroll
            for (int i = 0; i < 6; i++) {
                float v = 0.f;
                for (int ww = 0; ww < NW; ww++) v += s_wsum[ww][i];
                tot6[i] = v;
            }
            const float o3[3] = {s_org[0], s_org[1], s_org[2]};
            own_sums_world(tot6, o3, s_bown);
            const int t_last = (len - 1) / TILE;
            bwd_carry_warp(a, b, t, t_last, s_bown, s_epoch, s_bcarry);
            float cg[3], cs[3];
            carry_to_origin(s_bcarry, o3, cg, cs);
            if (tid == 0) {
                float run[6] = {cg[0], cg[1], cg[2], cs[0], cs[1], cs[2]};
                for (int ww = NW - 1; ww >= 0; ww--)
                    for (int i = 0; i < 6; i++) {
                        s_wsuf[ww][i] = run[i];
                        run[i] += s_wsum[ww][i];
                    }
            }
        }
        __syncthreads();
        // incoming suffix (atoms after this thread) in the thread's local frame:
        // G' = R^T G, S' = R^T (S - p x G)
        float Gw[3], Sw[3], G[3], S[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            Gw[c] = suf[c] + s_wsuf[w][c];
            Sw[c] = suf[3 + c] + s_wsuf[w][3 + c];
        }
        cross3(P.p, Gw, pxg);
#pragma unroll
        for (int c = 0; c < 3; c++) Sw[c] -= pxg[c];
        rot_t(P, Gw, G);
        rot_t(P, Sw, S);

        float(*s_gr)[TILE] = s_ang;  // angles are no longer needed: stage gradients there
        float nxt[3] = {nx, ny, nz};
#pragma unroll
        for (int r = R - 1; r >= 0; r--) {
            const int j = j0 + r;
            float xN[3], xA[3], xC[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                xN[c] = lp[(9 * r + c) * NT];
                xA[c] = lp[(9 * r + 3 + c) * NT];
                xC[c] = lp[(9 * r + 6 + c) * NT];
            }
            if (j < nreal) {
                const float *g = s_g + 9 * j;
                float u[3], tmp[3], cr[3];
                // omega_j: axis C -> N_{j+1}, origin N_{j+1}; subtree = atoms from N_{j+1} on
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (nxt[c] - xC[c]) * inv_d2;
                cross3(nxt, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                const float gom = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                // psi_j: axis CA -> C, origin C; same subtree
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (xC[c] - xA[c]) * inv_d1;
                cross3(xC, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                const float gps = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                // C_j joins the subtree of phi_j
                cross3(xC, g + 6, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    G[c] += g[6 + c];
                    S[c] += cr[c];
                }
                // phi_j: axis N -> CA, origin CA
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (xA[c] - xN[c]) * inv_d0;
                cross3(xA, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                const float gph = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                // CA_j and N_j join the suffix of residue j-1
                cross3(xA, g + 3, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    G[c] += g[3 + c];
                    S[c] += cr[c];
                }
                cross3(xN, g, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    G[c] += g[c];
                    S[c] += cr[c];
                }
                const bool last = chain_end && (j == nreal - 1);
                s_gr[0][j] = gph;
                s_gr[1][j] = last ? 0.f : gps;
                s_gr[2][j] = last ? 0.f : gom;
            }
#pragma unroll
            for (int c = 0; c < 3; c++) nxt[c] = xN[c];
        }
        __syncthreads();
        for (int k = 0; k < 3; k++) store_floats<NT>(gout + (size_t)k * a.L, s_gr[k], nreal, ntile);
        __syncthreads();
    }
    finish_launch(&a.hdr->bwd_ticket, &a.hdr->bwd_done, &a.hdr->bwd_epoch);
}

// ----------------------------------------------- warp-granular tiles (default)
// Each warp takes its own ticket for a tile of 32 R residues, so no CTA-wide
// barrier sits on the path: angles are loaded straight into registers, the scan
// is a warp shuffle scan, and the inter-tile carry is a warp-wide decoupled
// look-back (every lane polls one predecessor's flag; lane 0 composes the
// published frames in FP64).  The backward mirrors it with tiles handed out
// last-first and a look-back over successors' (G, S) sums.

template <int R>
__device__ __forceinline__ void load_row(const float *row, int j0, int nreal, float (&v)[R]) {
    if (R % 4 == 0 && j0 + R <= nreal && ((((uintptr_t)(row + j0)) & 15u) == 0)) {
#pragma unroll
        for (int i = 0; i < R / 4; i++) {
            const float4 x = __ldg(reinterpret_cast<const float4 *>(row + j0) + i);
            v[4 * i] = x.x; v[4 * i + 1] = x.y; v[4 * i + 2] = x.z; v[4 * i + 3] = x.w;
        }
    } else {
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = (j0 + r < nreal) ? __ldg(row + j0 + r) : 0.f;
    }
}

// Walk 1 with the thread-local N, CA, C positions kept in registers.
template <int R>
__device__ __forceinline__ Frame<float> walk_regs(const A2bArgs &a, const float4 *s_tab, const float (&phi)[R],
                                                  const float (&psi)[R], const float (&om)[R], int j0, int nreal,
                                                  bool chain_end, float (&loc)[R][9]) {
    Frame<float> agg;
    frame_identity(agg);
#pragma unroll
    for (int r = 0; r < R; r++) {
#pragma unroll
        for (int c = 0; c < 9; c++) loc[r][c] = 0.f;
        if (j0 + r < nreal) {
            float s, c;
            loc[r][0] = agg.p[0]; loc[r][1] = agg.p[1]; loc[r][2] = agg.p[2];
            sincos_tab(s_tab, phi[r], &s, &c);
            apply_joint(agg, a.bc.cb[0], a.bc.sb[0], a.bc.d[0], c, s);
            loc[r][3] = agg.p[0]; loc[r][4] = agg.p[1]; loc[r][5] = agg.p[2];
            sincos_tab(s_tab, psi[r], &s, &c);
            apply_joint(agg, a.bc.cb[1], a.bc.sb[1], a.bc.d[1], c, s);
            loc[r][6] = agg.p[0]; loc[r][7] = agg.p[1]; loc[r][8] = agg.p[2];
            if (!(chain_end && j0 + r == nreal - 1)) {
                sincos_tab(s_tab, om[r], &s, &c);
                apply_joint(agg, a.bc.cb[2], a.bc.sb[2], a.bc.d[2], c, s);
            }
        }
    }
    return agg;
}

__device__ __forceinline__ Frame<float> shfl_frame(const Frame<float> &f, int src) {
    Frame<float> o;
#pragma unroll
    for (int i = 0; i < 9; i++) o.r[i] = __shfl_sync(0xffffffffu, f.r[i], src);
#pragma unroll
    for (int i = 0; i < 3; i++) o.p[i] = __shfl_sync(0xffffffffu, f.p[i], src);
    return o;
}

// Resident CTAs of 128 threads per SM the register budget is sized for.
constexpr int warp_tile_min_blocks(int R) { return R <= 2 ? 5 : (R == 4 ? 4 : 3); }

template <int R>
__global__ void __launch_bounds__(128, warp_tile_min_blocks(R)) a2b_fwd_w_kernel(A2bArgs a) {
    constexpr int TILE = 32 * R;
    constexpr int NW = 4;
    __shared__ float4 s_tab[65];
    __shared__ double s_carry[NW][12], s_scratch[NW][36];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    load_sincos_table<128>(s_tab);
    __syncthreads();
    const unsigned epoch_bits = (*(volatile unsigned *)&a.hdr->fwd_epoch & 0x3fffffffu) << 2;

    for (;;) {
        int item = 0;
        if (lane == 0) item = (int)atomicAdd(&a.hdr->fwd_ticket, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= a.total) break;
        const int b = item / a.ntiles, t = item - b * a.ntiles;
        int len = a.lengths[b];
        if (len < 0 || len > a.L) {
            if (lane == 0) record_error(a.hdr, TPL_ERR_LENGTH);
            len = max(0, min(len, a.L));
        }
        const int s0 = t * TILE;
        const int ntile = min(TILE, a.L - s0);
        const int nreal = max(0, min(ntile, len - s0));
        float *out = a.coords + (size_t)b * 9 * a.L + (size_t)9 * s0;
        for (int i = 9 * nreal + lane; i < 9 * ntile; i += 32) out[i] = 0.f;
        if (nreal == 0) continue;

        const int j0 = lane * R;
        const float *ang = a.angles + (size_t)b * 3 * a.L + s0;
        float phi[R], psi[R], om[R];
        load_row<R>(ang, j0, nreal, phi);
        load_row<R>(ang + a.L, j0, nreal, psi);
        load_row<R>(ang + 2 * a.L, j0, nreal, om);
        const bool chain_end = (s0 + nreal == len);
        float loc[R][9];
        Frame<float> agg = walk_regs<R>(a, s_tab, phi, psi, om, j0, nreal, chain_end, loc);
        if (a.renorm) renormalize(agg);
        Frame<float> inc = warp_scan_frames(agg, lane);
        Frame<float> exc = shfl_up_frame(inc, 1);
        if (lane == 0) frame_identity(exc);
        Frame<float> tile = shfl_frame(inc, 31);
        if (a.renorm) renormalize(tile);

        const bool more = s0 + TILE < len;
        const bool use64 = a.fp64_min_len >= 0 && len >= a.fp64_min_len;
        fwd_carry_warp(a, b, t, more, tile, epoch_bits, use64, s_carry[w], s_scratch[w]);
        Frame<float> c32;
        frame_load(c32, s_carry[w]);
        const float o0 = c32.p[0], o1 = c32.p[1], o2 = c32.p[2];
        c32.p[0] = c32.p[1] = c32.p[2] = 0.f;  // positions relative to the tile origin
        if (a.renorm) renormalize(c32);
        Frame<float> P = compose(c32, exc);
        if (a.renorm) renormalize(P);
        const float t0 = P.p[0] + o0, t1 = P.p[1] + o1, t2 = P.p[2] + o2;
        float *dst = out + (size_t)9 * j0;
        auto world = [&](int e) {
            const int r = e / 9, q = (e % 9) / 3, c = e % 3;
            const float x = loc[r][3 * q], y = loc[r][3 * q + 1], z = loc[r][3 * q + 2];
            const float tc = c == 0 ? t0 : (c == 1 ? t1 : t2);
            return fmaf(P.r[3 * c], x, fmaf(P.r[3 * c + 1], y, fmaf(P.r[3 * c + 2], z, tc)));
        };
        if ((R % 4 == 0) && (j0 + R <= nreal) && ((((uintptr_t)dst) & 15u) == 0)) {
            float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll
            for (int i = 0; i < 9 * R / 4; i++)
                __stcs(d4 + i, make_float4(world(4 * i), world(4 * i + 1), world(4 * i + 2), world(4 * i + 3)));
        } else {
#pragma unroll
            for (int e = 0; e < 9 * R; e++)
                if (j0 + e / 9 < nreal) dst[e] = world(e);
        }
    }
    __syncthreads();
    finish_launch(&a.hdr->fwd_ticket, &a.hdr->fwd_done, &a.hdr->fwd_epoch);
}

template <int R>
__global__ void __launch_bounds__(128, warp_tile_min_blocks(R)) a2b_bwd_w_kernel(A2bArgs a) {
    constexpr int TILE = 32 * R;
    constexpr int NW = 4;
    __shared__ float4 s_tab[65];
    __shared__ float s_g[NW][9 * R][32];  // this lane's upstream gradients, rotated to its local frame
    __shared__ double s_own[NW][6], s_carry[NW][6];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    load_sincos_table<128>(s_tab);
    __syncthreads();
    const unsigned epoch_bits = (*(volatile unsigned *)&a.hdr->bwd_epoch & 0x3fffffffu) << 2;
    const float inv_d0 = 1.f / a.bc.d[0], inv_d1 = 1.f / a.bc.d[1], inv_d2 = 1.f / a.bc.d[2];

    for (;;) {
        int item = 0;
        if (lane == 0) item = (int)atomicAdd(&a.hdr->bwd_ticket, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= a.total) break;
        const int b = item / a.ntiles, t = a.ntiles - 1 - (item - b * a.ntiles);
        int len = a.lengths[b];
        if (len < 0 || len > a.L) {
            if (lane == 0) record_error(a.hdr, TPL_ERR_LENGTH);
            len = max(0, min(len, a.L));
        }
        const int s0 = t * TILE;
        const int ntile = min(TILE, a.L - s0);
        const int nreal = max(0, min(ntile, len - s0));
        float *gout = a.grad_angles + (size_t)b * 3 * a.L + s0;
        for (int k = 0; k < 3; k++)
            for (int i = nreal + lane; i < ntile; i += 32) gout[(size_t)k * a.L + i] = 0.f;
        if (nreal == 0) continue;

        const int j0 = lane * R;
        const float *ang = a.angles + (size_t)b * 3 * a.L + s0;
        float phi[R], psi[R], om[R];
        load_row<R>(ang, j0, nreal, phi);
        load_row<R>(ang + a.L, j0, nreal, psi);
        load_row<R>(ang + 2 * a.L, j0, nreal, om);
        const bool chain_end = (s0 + nreal == len);
        float loc[R][9];
        Frame<float> agg = walk_regs<R>(a, s_tab, phi, psi, om, j0, nreal, chain_end, loc);
        float nxt[3] = {agg.p[0], agg.p[1], agg.p[2]};  // N after this lane's last residue
        if (a.renorm) renormalize(agg);
        Frame<float> inc = warp_scan_frames(agg, lane);
        Frame<float> exc = shfl_up_frame(inc, 1);
        if (lane == 0) frame_identity(exc);

        Frame<float> c32;
        if (t == 0) frame_identity(c32);
        else frame_load(c32, a.rec[(size_t)b * a.ntiles + t].fexc);
        const float org[3] = {c32.p[0], c32.p[1], c32.p[2]};
        c32.p[0] = c32.p[1] = c32.p[2] = 0.f;
        if (a.renorm) renormalize(c32);
        Frame<float> P = compose(c32, exc);
        if (a.renorm) renormalize(P);

        // upstream gradients of this lane's atoms, rotated into its local frame
        const float *gin = a.grad_coords + (size_t)b * 9 * a.L + (size_t)9 * (s0 + j0);
        float Gl[3] = {0.f, 0.f, 0.f}, Sl[3] = {0.f, 0.f, 0.f};
        const bool gvec = (R % 4 == 0) && (j0 + R <= nreal) && ((((uintptr_t)gin) & 15u) == 0);
#pragma unroll
        for (int r = 0; r < R; r++) {
            float gw[9];
            if (gvec) {
                // 9 floats per residue; residues r..r+3 span 9 float4
#pragma unroll
                for (int c = 0; c < 9; c++) gw[c] = __ldcs(gin + 9 * r + c);
            } else {
#pragma unroll
                for (int c = 0; c < 9; c++) gw[c] = (j0 + r < nreal) ? __ldcs(gin + 9 * r + c) : 0.f;
            }
#pragma unroll
            for (int q = 0; q < 3; q++) {
                float gl[3], xg[3];
                rot_t(P, gw + 3 * q, gl);
#pragma unroll
                for (int c = 0; c < 3; c++) s_g[w][9 * r + 3 * q + c][lane] = gl[c];
                cross3(&loc[r][3 * q], gl, xg);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    Gl[c] += gl[c];
                    Sl[c] += xg[c];
                }
            }
        }
        // lane totals in the tile frame, exclusive suffix over lanes, tile total
        float Gt[3], St[3], pxg[3];
        rot(P, Gl, Gt);
        rot(P, Sl, St);
        cross3(P.p, Gt, pxg);
#pragma unroll
        for (int c = 0; c < 3; c++) St[c] += pxg[c];
        float suf[6], tot[6];
        const float v6[6] = {Gt[0], Gt[1], Gt[2], St[0], St[1], St[2]};
#pragma unroll
        for (int i = 0; i < 6; i++) suf[i] = warp_suffix_exclusive(v6[i], lane, tot[i]);
        own_sums_world(tot, org, s_own[w]);
        const int t_last = (len - 1) / TILE;
        bwd_carry_warp(a, b, t, t_last, s_own[w], epoch_bits, s_carry[w]);
        // carry from later tiles, moved to this tile's origin: S_o = S_w - o x G
        float cg[3], cs[3];
        carry_to_origin(s_carry[w], org, cg, cs);
        // incoming suffix of this lane, in its local frame: G' = R^T G, S' = R^T (S - p x G)
        float Gw[3], Sw[3], G[3], S[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            Gw[c] = suf[c] + cg[c];
            Sw[c] = suf[3 + c] + cs[c];
        }
        cross3(P.p, Gw, pxg);
#pragma unroll
        for (int c = 0; c < 3; c++) Sw[c] -= pxg[c];
        rot_t(P, Gw, G);
        rot_t(P, Sw, S);

        float gr[3][R];
#pragma unroll
        for (int r = R - 1; r >= 0; r--) {
            gr[0][r] = gr[1][r] = gr[2][r] = 0.f;
            const float *xN = &loc[r][0], *xA = &loc[r][3], *xC = &loc[r][6];
            if (j0 + r < nreal) {
                float g[9];
#pragma unroll
                for (int c = 0; c < 9; c++) g[c] = s_g[w][9 * r + c][lane];
                float u[3], tmp[3], cr[3];
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (nxt[c] - xC[c]) * inv_d2;
                cross3(nxt, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                const float gom = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (xC[c] - xA[c]) * inv_d1;
                cross3(xC, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                const float gps = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                cross3(xC, g + 6, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    G[c] += g[6 + c];
                    S[c] += cr[c];
                }
#pragma unroll
                for (int c = 0; c < 3; c++) u[c] = (xA[c] - xN[c]) * inv_d0;
                cross3(xA, G, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) tmp[c] = S[c] - cr[c];
                const float gph = u[0] * tmp[0] + u[1] * tmp[1] + u[2] * tmp[2];
                cross3(xA, g + 3, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    G[c] += g[3 + c];
                    S[c] += cr[c];
                }
                cross3(xN, g, cr);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    G[c] += g[c];
                    S[c] += cr[c];
                }
                const bool last = chain_end && (j0 + r == nreal - 1);
                gr[0][r] = gph;
                gr[1][r] = last ? 0.f : gps;
                gr[2][r] = last ? 0.f : gom;
            }
#pragma unroll
            for (int c = 0; c < 3; c++) nxt[c] = xN[c];
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            float *dst = gout + (size_t)k * a.L + j0;
            if ((R % 4 == 0) && (j0 + R <= nreal) && ((((uintptr_t)dst) & 15u) == 0)) {
#pragma unroll
                for (int i = 0; i < R / 4; i++)
                    __stcs(reinterpret_cast<float4 *>(dst) + i,
                           make_float4(gr[k][4 * i], gr[k][4 * i + 1], gr[k][4 * i + 2], gr[k][4 * i + 3]));
            } else {
#pragma unroll
                for (int r = 0; r < R; r++)
                    if (j0 + r < nreal) dst[r] = gr[k][r];
            }
        }
    }
    __syncthreads();
    finish_launch(&a.hdr->bwd_ticket, &a.hdr->bwd_done, &a.hdr->bwd_epoch);
}

// ----------------------------------------------------------- plain FP64 form
// One chain per CTA, one residue per thread per chunk, Hillis-Steele block scan
// of residue transforms in shared memory, carry between chunks in registers.
constexpr int kPlainThreads = 256;

struct PlainArgs {
    const double *angles;
    const int *lengths;
    double *coords;
    double *grad_angles;
    const double *grad_coords;
    WsHeader *hdr;
    TileRecord *rec;
    int L, nchunks;
    BondConsts bc;
};

__device__ __forceinline__ Frame<double> plain_residue(const PlainArgs &a, const double *ang, int j, int len,
                                                       double cs[3], double sn[3]) {
    Frame<double> T;
    frame_identity(T);
    for (int k = 0; k < 3; k++) {
        cs[k] = 1.0;
        sn[k] = 0.0;
    }
    if (j < len) {
        for (int k = 0; k < 3; k++) {
            if (k == 2 && j == len - 1) break;
            sincos(ang[(size_t)k * a.L + j], &sn[k], &cs[k]);
            apply_joint(T, a.bc.cbd[k], a.bc.sbd[k], a.bc.dd[k], cs[k], sn[k]);
        }
    }
    return T;
}

// Inclusive block scan of frames (Hillis-Steele); returns the exclusive prefix.
__device__ __forceinline__ Frame<double> plain_block_scan(Frame<double> T, Frame<double> *s, Frame<double> &total) {
    const int tid = threadIdx.x;
    s[tid] = T;
    __syncthreads();
    for (int off = 1; off < kPlainThreads; off <<= 1) {
        Frame<double> o;
        if (tid >= off) o = s[tid - off];
        __syncthreads();
        if (tid >= off) {
            T = compose(o, T);
            s[tid] = T;
        }
        __syncthreads();
    }
    Frame<double> exc;
    if (tid == 0) frame_identity(exc);
    else exc = s[tid - 1];
    total = s[kPlainThreads - 1];
    __syncthreads();
    return exc;
}

__global__ void __launch_bounds__(kPlainThreads) a2b_fwd_f64_plain_kernel(PlainArgs a) {
    __shared__ Frame<double> s_scan[kPlainThreads];
    const int b = blockIdx.x, tid = threadIdx.x;
    int len = a.lengths[b];
    if (len < 0 || len > a.L) {
        if (tid == 0 && a.hdr) record_error(a.hdr, TPL_ERR_LENGTH);
        len = max(0, min(len, a.L));
    }
    const double *ang = a.angles + (size_t)b * 3 * a.L;
    double *out = a.coords + (size_t)b * 9 * a.L;
    Frame<double> carry;
    frame_identity(carry);
    for (int s0 = 0; s0 < a.L; s0 += kPlainThreads) {
        const int j = s0 + tid;
        double cs[3], sn[3];
        Frame<double> T = plain_residue(a, ang, j, len, cs, sn);
        Frame<double> total;
        Frame<double> exc = plain_block_scan(T, s_scan, total);
        Frame<double> P = compose(carry, exc);
        if (j < len) {
            double *o = out + (size_t)9 * j;
            for (int q = 0; q < 3; q++) {
                o[3 * q] = P.p[0]; o[3 * q + 1] = P.p[1]; o[3 * q + 2] = P.p[2];
                apply_joint(P, a.bc.cbd[q], a.bc.sbd[q], a.bc.dd[q], cs[q], sn[q]);
            }
        } else if (j < a.L) {
            double *o = out + (size_t)9 * j;
            for (int q = 0; q < 9; q++) o[q] = 0.0;
        }
        carry = compose(carry, total);
    }
}

__global__ void __launch_bounds__(kPlainThreads) a2b_bwd_f64_plain_kernel(PlainArgs a) {
    __shared__ Frame<double> s_scan[kPlainThreads];
    __shared__ double s_sum[kPlainThreads][6];
    const int b = blockIdx.x, tid = threadIdx.x;
    int len = a.lengths[b];
    if (len < 0 || len > a.L) {
        if (tid == 0 && a.hdr) record_error(a.hdr, TPL_ERR_LENGTH);
        len = max(0, min(len, a.L));
    }
    const double *ang = a.angles + (size_t)b * 3 * a.L;
    const double *gc = a.grad_coords + (size_t)b * 9 * a.L;
    double *gout = a.grad_angles + (size_t)b * 3 * a.L;
    TileRecord *rec = a.rec + (size_t)b * a.nchunks;
    // pass 1: chunk carries
    Frame<double> carry;
    frame_identity(carry);
    for (int c = 0; c < a.nchunks; c++) {
        if (tid == 0) frame_store(rec[c].fexc, carry);
        const int j = c * kPlainThreads + tid;
        double cs[3], sn[3];
        Frame<double> T = plain_residue(a, ang, j, len, cs, sn);
        Frame<double> total;
        plain_block_scan(T, s_scan, total);
        carry = compose(carry, total);
    }
    __syncthreads();
    // pass 2: chunks last-first with the running suffix (G, S) about the world origin
    double Gc[3] = {0, 0, 0}, Sc[3] = {0, 0, 0};
    for (int c = a.nchunks - 1; c >= 0; c--) {
        const int j = c * kPlainThreads + tid;
        double cs[3], sn[3];
        Frame<double> T = plain_residue(a, ang, j, len, cs, sn);
        Frame<double> total, start;
        Frame<double> exc = plain_block_scan(T, s_scan, total);
        frame_load(start, rec[c].fexc);
        Frame<double> P = compose(start, exc);
        double x[3][3], u[3][3], xn[3];
        double G[3] = {0, 0, 0}, S[3] = {0, 0, 0};
        if (j < len) {
            for (int q = 0; q < 3; q++) {
                for (int k = 0; k < 3; k++) x[q][k] = P.p[k];
                apply_joint(P, a.bc.cbd[q], a.bc.sbd[q], a.bc.dd[q], cs[q], sn[q]);
                for (int k = 0; k < 3; k++) u[q][k] = P.r[3 * k];
            }
            for (int k = 0; k < 3; k++) xn[k] = P.p[k];
            for (int q = 0; q < 3; q++) {
                const double *g = gc + (size_t)9 * j + 3 * q;
                double xg[3];
                cross3(x[q], g, xg);
                for (int k = 0; k < 3; k++) {
                    G[k] += g[k];
                    S[k] += xg[k];
                }
            }
        }
        // exclusive suffix over threads (Hillis-Steele on sums, reversed)
        double v[6] = {G[0], G[1], G[2], S[0], S[1], S[2]};
        for (int i = 0; i < 6; i++) s_sum[tid][i] = v[i];
        __syncthreads();
        for (int off = 1; off < kPlainThreads; off <<= 1) {
            double o[6];
            const bool has = tid + off < kPlainThreads;
            if (has)
                for (int i = 0; i < 6; i++) o[i] = s_sum[tid + off][i];
            __syncthreads();
            if (has)
                for (int i = 0; i < 6; i++) {
                    v[i] += o[i];
                    s_sum[tid][i] = v[i];
                }
            __syncthreads();
        }
        double Gr[3], Sr[3], chunk_tot[6];
        for (int i = 0; i < 6; i++) chunk_tot[i] = s_sum[0][i];
        for (int k = 0; k < 3; k++) {
            const double nxt_g = tid + 1 < kPlainThreads ? s_sum[tid + 1][k] : 0.0;
            const double nxt_s = tid + 1 < kPlainThreads ? s_sum[tid + 1][3 + k] : 0.0;
            Gr[k] = nxt_g + Gc[k];
            Sr[k] = nxt_s + Sc[k];
        }
        __syncthreads();
        if (j < len) {
            double tmp[3], cr[3];
            cross3(xn, Gr, cr);
            for (int k = 0; k < 3; k++) tmp[k] = Sr[k] - cr[k];
            const double gom = u[2][0] * tmp[0] + u[2][1] * tmp[1] + u[2][2] * tmp[2];
            cross3(x[2], Gr, cr);
            for (int k = 0; k < 3; k++) tmp[k] = Sr[k] - cr[k];
            const double gps = u[1][0] * tmp[0] + u[1][1] * tmp[1] + u[1][2] * tmp[2];
            const double *g = gc + (size_t)9 * j + 6;
            cross3(x[2], g, cr);
            for (int k = 0; k < 3; k++) {
                Gr[k] += g[k];
                Sr[k] += cr[k];
            }
            cross3(x[1], Gr, cr);
            for (int k = 0; k < 3; k++) tmp[k] = Sr[k] - cr[k];
            const double gph = u[0][0] * tmp[0] + u[0][1] * tmp[1] + u[0][2] * tmp[2];
            const bool last = (j == len - 1);
            gout[j] = gph;
            gout[(size_t)a.L + j] = last ? 0.0 : gps;
            gout[(size_t)2 * a.L + j] = last ? 0.0 : gom;
        } else if (j < a.L) {
            gout[j] = gout[(size_t)a.L + j] = gout[(size_t)2 * a.L + j] = 0.0;
        }
        for (int i = 0; i < 3; i++) {
            Gc[i] += chunk_tot[i];
            Sc[i] += chunk_tot[3 + i];
        }
    }
}

// ------------------------------------------------------------------- host side
template <typename K>
static int persistent_grid(K kernel, int threads, int items, int max_ctas, int dyn_smem = 0) {
    const int num_sms = device_sm_count();
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, dyn_smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    int grid = num_sms * per_sm;
    if (max_ctas > 0 && grid > max_ctas) grid = max_ctas;
    if (grid > items) grid = items;
    return grid < 1 ? 1 : grid;
}

struct A2bShape {
    int R, NT;
    bool warp;  // warp-granular tiles (default) or CTA tiles of NT threads
};

// threads_per_cta = 1 (or 0 when the automatic choice is not one warp per chain):
// warp-granular tiles of 32 R residues.  threads_per_cta = 128: CTA tiles of 128 R
// residues with block-wide scans.
static A2bShape a2b_shape(const tpl_options &opt, bool backward) {
    (void)backward;
    A2bShape s;
    s.R = opt.residues_per_thread > 0 ? opt.residues_per_thread : 4;
    s.warp = opt.threads_per_cta != 128;
    s.NT = s.warp ? 32 : 128;
    return s;
}

static int num_sms() { return device_sm_count(); }

// threads_per_cta = 0 picks, from the shape, the scheme that measured fastest on
// GB300 (4-residue-per-lane and 8-residue-per-lane chunks, one warp or one CTA of
// four warps per chain, warp tiles; batches of 32 to 16384 chains of 64 to 1000
// residues):
//   * max_len >= 384: one CTA of four warps per chain (the chunks of a chain run on
//     four warps at once), 8 residues per lane from max_len 768 and 4 below;
//   * shorter chains: one warp per chain with 4 residues per lane when the batch
//     gives every SM two chains, else one CTA of four warps per chain;
//   * fewer than two chains per SM and chains over 4096 residues: warp tiles, whose
//     look-back spreads one chain over many warps.
// An explicit residues_per_thread of 4 or 8 is kept; 1 or 2 selects warp tiles.
// The forward and the backward of one shape make the same choice.
static bool use_chain_scheme(const tpl_options &opt, int B, int L) {
    if (opt.threads_per_cta == 32 || opt.threads_per_cta == 4) return true;
    if (opt.threads_per_cta != 0) return false;
    const int r = opt.residues_per_thread;
    if (!(r == 0 || r == 4 || r == 8)) return false;
    return !(B < 2 * num_sms() && L > 4096);
}

static tpl_options chain_options(const tpl_options &opt, int B, int L) {
    tpl_options o = opt;
    if (o.threads_per_cta == 0) {
        const bool ring = L >= 384 || B < 2 * num_sms();
        o.threads_per_cta = ring ? 4 : 32;
        if (o.residues_per_thread == 0) o.residues_per_thread = (ring && L >= 768) ? 8 : 4;
    }
    if (o.residues_per_thread == 0) o.residues_per_thread = 8;
    return o;
}

int a2b_tile_for(const tpl_options &opt) {
    if (opt.threads_per_cta == 32 || opt.threads_per_cta == 4)
        return a2b_chain_record_stride();  // one warp or one CTA per chain: frame records
    A2bShape f = a2b_shape(opt, false);
    const int tile = f.R * f.NT;
    if (opt.threads_per_cta == 0) return std::min(tile, a2b_chain_record_stride());  // either scheme fits
    return tile;
}

static A2bArgs make_args(const float *angles, const int32_t *lengths, void *ws, int B, int L, int tile,
                         const tpl_options &opt) {
    A2bArgs a;
    a.angles = angles;
    a.lengths = lengths;
    a.coords = nullptr;
    a.grad_angles = nullptr;
    a.grad_coords = nullptr;
    a.hdr = reinterpret_cast<WsHeader *>(ws);
    a.rec = reinterpret_cast<TileRecord *>(reinterpret_cast<char *>(ws) + sizeof(WsHeader));
    a.L = L;
    a.ntiles = (L + tile - 1) / tile;
    a.total = B * a.ntiles;
    a.fp64_min_len = opt.fp64_carry_min_len == 0 ? 0 : opt.fp64_carry_min_len;
    a.renorm = opt.renormalize >= 0 ? 1 : 0;
    a.bc = bond_constants();
    return a;
}

template <int R>
static int launch_fwd_w(A2bArgs &a, int max_ctas, cudaStream_t st) {
    auto k = a2b_fwd_w_kernel<R>;
    int grid = persistent_grid(k, 128, (a.total + 3) / 4, max_ctas);
    k<<<grid, 128, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}
template <int R>
static int launch_bwd_w(A2bArgs &a, int max_ctas, cudaStream_t st) {
    auto k = a2b_bwd_w_kernel<R>;
    int grid = persistent_grid(k, 128, (a.total + 3) / 4, max_ctas);
    k<<<grid, 128, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

template <int R>
static int launch_fwd(A2bArgs &a, int max_ctas, cudaStream_t st) {
    auto k = a2b_fwd_f32_kernel<R, 128>;
    const int smem = 12 * R * 128 * (int)sizeof(float);
    if (!set_max_dynamic_smem(reinterpret_cast<const void *>(k), smem))
        return TPL_ERR_LAUNCH;
    int grid = persistent_grid(k, 128, a.total, max_ctas, smem);
    k<<<grid, 128, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}
template <int R, int NT>
static int launch_bwd(A2bArgs &a, int max_ctas, cudaStream_t st) {
    auto k = a2b_bwd_f32_kernel<R, NT>;
    const int smem = 21 * R * NT * (int)sizeof(float);
    if (!set_max_dynamic_smem(reinterpret_cast<const void *>(k), smem))
        return TPL_ERR_LAUNCH;
    int grid = persistent_grid(k, NT, a.total, max_ctas, smem);
    k<<<grid, NT, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

int a2b_forward_f32(const float *angles, const int32_t *lengths, float *coords, void *ws, int B, int L,
                    const tpl_options &opt, cudaStream_t st) {
    if (B == 0 || L == 0) return TPL_OK;
    if (use_chain_scheme(opt, B, L))
        return a2b_forward_chain(angles, lengths, coords, ws, B, L, chain_options(opt, B, L), st);
    A2bShape s = a2b_shape(opt, false);
    A2bArgs a = make_args(angles, lengths, ws, B, L, s.R * s.NT, opt);
    a.coords = coords;
    if (s.warp) {
        switch (s.R) {
            case 1: return launch_fwd_w<1>(a, opt.max_ctas, st);
            case 2: return launch_fwd_w<2>(a, opt.max_ctas, st);
            case 4: return launch_fwd_w<4>(a, opt.max_ctas, st);
            case 8: return launch_fwd_w<8>(a, opt.max_ctas, st);
        }
        return TPL_ERR_UNSUPPORTED;
    }
    switch (s.R) {
        case 1: return launch_fwd<1>(a, opt.max_ctas, st);
        case 2: return launch_fwd<2>(a, opt.max_ctas, st);
        case 4: return launch_fwd<4>(a, opt.max_ctas, st);
        case 8: return launch_fwd<8>(a, opt.max_ctas, st);
    }
    return TPL_ERR_UNSUPPORTED;
}

int a2b_backward_f32(float *grad_angles, const float *grad_coords, const float *angles, const int32_t *lengths,
                     void *ws, int B, int L, const tpl_options &opt, cudaStream_t st) {
    if (B == 0 || L == 0) return TPL_OK;
    if (use_chain_scheme(opt, B, L))
        return a2b_backward_chain(grad_angles, grad_coords, angles, lengths, ws, B, L, chain_options(opt, B, L), st);
    A2bShape s = a2b_shape(opt, true);
    A2bArgs a = make_args(angles, lengths, ws, B, L, s.R * s.NT, opt);
    a.grad_angles = grad_angles;
    a.grad_coords = grad_coords;
    if (s.warp) {
        switch (s.R) {
            case 1: return launch_bwd_w<1>(a, opt.max_ctas, st);
            case 2: return launch_bwd_w<2>(a, opt.max_ctas, st);
            case 4: return launch_bwd_w<4>(a, opt.max_ctas, st);
            case 8: return launch_bwd_w<8>(a, opt.max_ctas, st);
        }
        return TPL_ERR_UNSUPPORTED;
    }
    switch (s.R) {
        case 1: return launch_bwd<1, 128>(a, opt.max_ctas, st);
        case 2: return launch_bwd<2, 128>(a, opt.max_ctas, st);
        case 4: return launch_bwd<4, 128>(a, opt.max_ctas, st);
        case 8: return launch_bwd<8, 128>(a, opt.max_ctas, st);
    }
    return TPL_ERR_UNSUPPORTED;
}

int a2b_forward_f64_plain(const double *angles, const int32_t *lengths, double *coords, int B, int L,
                          cudaStream_t st) {
    if (B == 0 || L == 0) return TPL_OK;
    PlainArgs a{};
    a.angles = angles;
    a.lengths = lengths;
    a.coords = coords;
    a.hdr = nullptr;
    a.rec = nullptr;
    a.L = L;
    a.nchunks = (L + kPlainThreads - 1) / kPlainThreads;
    a.bc = bond_constants();
    a2b_fwd_f64_plain_kernel<<<B, kPlainThreads, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

int a2b_backward_f64_plain(double *grad_angles, const double *grad_coords, const double *angles,
                           const int32_t *lengths, void *ws, int B, int L, cudaStream_t st) {
    if (B == 0 || L == 0) return TPL_OK;
    PlainArgs a{};
    a.angles = angles;
    a.lengths = lengths;
    a.grad_angles = grad_angles;
    a.grad_coords = grad_coords;
    a.hdr = reinterpret_cast<WsHeader *>(ws);
    a.rec = reinterpret_cast<TileRecord *>(reinterpret_cast<char *>(ws) + sizeof(WsHeader));
    a.L = L;
    a.nchunks = (L + kPlainThreads - 1) / kPlainThreads;
    a.bc = bond_constants();
    a2b_bwd_f64_plain_kernel<<<B, kPlainThreads, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

}  // namespace tpl
