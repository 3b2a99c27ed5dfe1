// Angles2Coords kernels for sm_103a (the reference has no GPU path here: it
// builds one heap-allocated node graph per chain on the CPU,
// Layers/FullAtomModel/cConformation.cpp:30-211, OpenMP over chains in
// Angles2Coords/angles2coords_interface.cpp:27,92).
//
// float32 runs the chunked kernels further down by default (a2c_fwd_ring_kernel,
// a2c_bwd_coords_ring_kernel: four or eight warps per chain on chunks of 32
// residues, the carry handed between warps).  The CTA kernels described here serve
// float64, the tree-rebuilding backward and the threads_per_cta options 128, 256
// and 512.
//
// One CTA per chain, looping over tiles of R*NT residues with the carry (frame
// and atom offset) kept in shared memory.  Inside a tile the backbone is the
// same parallel scan as Angles2Backbone (per-thread joint products, warp
// shuffles, shared-memory warp totals); the atom offsets of the residues are an
// integer scan of per-residue atom counts carried alongside.  Each thread then
// walks its residues from its world frame and places every atom of each residue
// (backbone, Pro ring, side-chain joints below the dummy transform, carbonyl),
// stages them in shared memory and the tile's contiguous atom range is written
// with coalesced stores.
//
// The backward is the adjoint of the same tree: for a joint with axis u and
// origin o, dL/dalpha = u . sum over its subtree of (x - o) x g.  Subtrees of the
// backbone joints are "everything after" in atom order (plus the residue's own
// side chain for phi), so the kernel scans (G, S) = (sum g, sum x x g) backwards
// over tiles, threads and residues; side-chain joints use prefix sums over the
// side-chain path of their residue.  Complexity O(atoms) per chain instead of
// the reference's O(nodes x subtree).
#include <cstddef>
#include <cstdio>

#include "tpl_common.cuh"
#include "tpl_internal.h"
#include "tpl_pair.cuh"
#include "tpl_sincos.cuh"
#include "tpl_topology.cuh"

namespace tpl {

__device__ const Topology<float> g_topo_f32 = make_topology<float>();
__device__ const Topology<double> g_topo_f64 = make_topology<double>();

template <typename T>
__device__ __forceinline__ const Topology<T> &topo_global();
template <>
__device__ __forceinline__ const Topology<float> &topo_global<float>() { return g_topo_f32; }
template <>
__device__ __forceinline__ const Topology<double> &topo_global<double>() { return g_topo_f64; }

template <typename T>
struct A2cArgs {
    const unsigned char *seq;
    int seq_stride;
    const T *angles;
    T *coords;
    uint32_t *res_names;
    uint32_t *atom_names;
    T *grad_angles;
    const T *grad_coords;
    WsHeader *hdr;
    int L, maxA;
};

__device__ __forceinline__ void a2c_error(WsHeader *h, int code) {
    if (h) atomicCAS(&h->status, 0u, (unsigned)code);
}

template <typename T>
__device__ __forceinline__ void sc(T a, T *s, T *c) { sincos_t(a, s, c); }
// float angles: the register polynomial of the Angles2Backbone kernels (about one
// ulp, no special-function unit; sincosf beyond |a| = 1e4)
template <>
__device__ __forceinline__ void sc<float>(float a, float *s, float *c) { sincos_poly(a, s, c); }

template <typename T>
__device__ __forceinline__ void renorm_if(Frame<T> &f, bool on) {
    if (on) renormalize(f);
}

// Shared-memory layout of the tile buffers (dynamic).
template <typename T, int TILE>
struct A2cSmem {
    Topology<T> topo;
    T ang[8][TILE];
    T xyz[TILE * kMaxResAtoms * 3];
    signed char type[TILE];
    signed char lut[256];
};

// The forward also stages the tile's residue and atom names, so that they leave
// with the coordinates' coalesced store instead of per-residue scattered writes.
template <typename T, int TILE>
struct A2cSmemFwd {
    A2cSmem<T, TILE> f;
    uint32_t res_name[TILE * kMaxResAtoms];
    uint32_t atom_name[TILE * kMaxResAtoms];
};

template <typename T, int TILE>
struct A2cSmemBwd {
    A2cSmem<T, TILE> f;
    T g[TILE * kMaxResAtoms * 3];
};

// Copy the topology to shared memory and build the letter -> type table.
template <typename T, int NT>
__device__ __forceinline__ void load_topology(Topology<T> &dst, signed char *lut) {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(&topo_global<T>());
    uint32_t *d = reinterpret_cast<uint32_t *>(&dst);
    constexpr int n = sizeof(Topology<T>) / 4;
    static_assert(sizeof(Topology<T>) % 4 == 0, "topology size");
    for (int i = threadIdx.x; i < n; i += NT) d[i] = src[i];
    for (int i = threadIdx.x; i < 256; i += NT) lut[i] = (signed char)residue_type((unsigned char)i);
}

// Chain length = index of the first NUL of the sequence row (at most the row
// stride); every letter before it must be one of the 20 residues.
template <int NT>
__device__ __forceinline__ int chain_length(const unsigned char *row, int stride, const signed char *lut, int *s_len,
                                            int *s_bad) {
    if (threadIdx.x == 0) {
        *s_len = stride;
        *s_bad = 0;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < stride; j += NT)
        if (row[j] == 0) atomicMin(s_len, j);
    __syncthreads();
    const int len = *s_len;
    for (int j = threadIdx.x; j < len; j += NT)
        if (lut[row[j]] < 0) *s_bad = 1;
    __syncthreads();
    return len;
}

// Per-thread scan state for one tile: backbone aggregate of the thread's
// residues, its exclusive prefix inside the warp, atom counts.
template <typename T, int R, int NT>
struct TileScan {
    T cs[R][3], sn[R][3];
    Frame<T> exc;     // exclusive prefix inside the warp
    int cnt_exc;      // atoms before this thread inside the warp
    int cnt_own;      // atoms of this thread
};

template <typename T, int R, int NT>
__device__ __forceinline__ void a2c_tile_scan(const Topology<T> &tp, const T (*ang)[R * NT],
                                              const signed char *type, int n, bool chain_end, bool renorm,
                                              TileScan<T, R, NT> &ts, Frame<T> *s_wtot, int *s_wcnt) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    Frame<T> agg;
    frame_identity(agg);
    int cnt = 0;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int j = tid * R + r;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            ts.cs[r][k] = T(1);
            ts.sn[r][k] = T(0);
        }
        if (j < n) {
            cnt += tp.natoms[type[j]];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                if (k == 2 && chain_end && j == n - 1) break;
                sc(ang[k][j], &ts.sn[r][k], &ts.cs[r][k]);
                apply_joint(agg, tp.bb_cb[k], tp.bb_sb[k], tp.bb_d[k], ts.cs[r][k], ts.sn[r][k]);
            }
        }
    }
    renorm_if(agg, renorm);
    Frame<T> inc = warp_scan_frames(agg, lane);
    ts.exc = shfl_up_frame(inc, 1);
    if (lane == 0) frame_identity(ts.exc);
    int ci = cnt;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int o = __shfl_up_sync(0xffffffffu, ci, off);
        if (lane >= off) ci += o;
    }
    ts.cnt_exc = ci - cnt;
    ts.cnt_own = cnt;
    if (lane == 31) {
        s_wtot[w] = inc;
        s_wcnt[w] = ci;
    }
}

// Thread 0: warp prefixes with the tile carry folded in (rotation only: positions
// are relative to the tile origin), the tile aggregate and the tile atom count.
template <typename T, int NW>
__device__ __forceinline__ void a2c_tile_prefix(const Frame<T> &carry, const Frame<T> *s_wtot, const int *s_wcnt,
                                                bool renorm, Frame<T> *s_wpre, int *s_wcpre, Frame<T> &tile_agg,
                                                int &tile_cnt) {
    Frame<T> run;
    frame_identity(run);
    Frame<T> c0 = carry;
    c0.p[0] = c0.p[1] = c0.p[2] = T(0);
    int cr = 0;
    for (int w = 0; w < NW; w++) {
        s_wpre[w] = compose(c0, run);
        s_wcpre[w] = cr;
        run = compose(run, s_wtot[w]);
        renorm_if(run, renorm);
        cr += s_wcnt[w];
    }
    tile_agg = run;
    tile_cnt = cr;
}

// All atoms of residue j (type ty) from the frame P at its N atom.  chi_angle(q)
// returns the residue's chi_(q+1); emit(slot, xyz) receives positions in P's
// coordinates; returns the frame at the next N.
template <typename T, typename Chi, typename Emit>
__device__ __forceinline__ void residue_atoms(const Topology<T> &tp, int ty, Frame<T> &P, const T cs[3],
                                              const T sn[3], Chi chi_angle, Emit emit) {
    emit(0, P.p);
    Frame<T> F = P;
    apply_joint(F, tp.bb_cb[0], tp.bb_sb[0], tp.bb_d[0], cs[0], sn[0]);
    emit(1, F.p);
    const int na = tp.natoms[ty];
    if (tp.pro[ty]) {
        for (int a = 0; a < 3; a++) {
            T x[3];
            frame_point(F, tp.pro_local[a][0], tp.pro_local[a][1], tp.pro_local[a][2], x);
            emit(2 + a, x);
        }
    }
    const int nj = tp.njoints[ty];
    if (nj > 0) {
        Frame<T> S = F;
        apply_rx(S, tp.dummy_c, tp.dummy_s);
        for (int k = 0; k < nj; k++) {
            const int chi = tp.jchi[ty][k];
            T c = T(1), s = T(0);
            if (chi >= 0) sc(chi_angle(chi), &s, &c);
            apply_joint(S, tp.jcb[ty][k], tp.jsb[ty][k], tp.jd[ty][k], c, s);
            const int f0 = tp.jfirst[ty][k];
            for (int a = 0; a < tp.jna[ty][k]; a++) {
                T x[3];
                frame_point(S, tp.sc[ty][f0 + a][0], tp.sc[ty][f0 + a][1], tp.sc[ty][f0 + a][2], x);
                emit(2 + f0 + a, x);
            }
        }
    }
    Frame<T> C = F;
    apply_joint(C, tp.bb_cb[1], tp.bb_sb[1], tp.bb_d[1], cs[1], sn[1]);
    emit(na - 2, C.p);
    {
        T x[3];
        frame_point(C, tp.o_local[0], tp.o_local[1], tp.o_local[2], x);
        emit(na - 1, x);
    }
    P = C;
    apply_joint(P, tp.bb_cb[2], tp.bb_sb[2], tp.bb_d[2], cs[2], sn[2]);
}

// apply_rx and frame_point (tpl_common.cuh) on a PairFrame: the same chain of fused
// multiply-adds per output, so the same rounding.
__device__ __forceinline__ void apply_rx_pair(PairFrame &f, float ca, float sa) {
    const float2 c1 = f.c[1], c2 = f.c[2];
    f.c[1] = __ffma2_rn(c1, f2(ca), __fmul2_rn(c2, f2(sa)));
    f.c[2] = __ffma2_rn(c2, f2(ca), __fmul2_rn(c1, f2(-sa)));
    const float e1 = f.r2[1], e2 = f.r2[2];
    f.r2[1] = fmaf(e1, ca, e2 * sa);
    f.r2[2] = fmaf(e2, ca, -e1 * sa);
}

__device__ __forceinline__ void pair_point(const PairFrame &P, float x, float y, float z, float *out) {
    const float2 xy = __ffma2_rn(P.c[0], f2(x), __ffma2_rn(P.c[1], f2(y), __ffma2_rn(P.c[2], f2(z), P.p)));
    out[0] = xy.x;
    out[1] = xy.y;
    out[2] = fmaf(P.r2[0], x, fmaf(P.r2[1], y, fmaf(P.r2[2], z, P.p2)));
}

// residue_atoms for float32 on paired frames, with the chi angles' cos and sin
// computed beforehand (chi_c[q], chi_s[q] for chi_(q+1)): the same atoms in the
// same slots, without the frame at the next N.
template <typename Emit>
__device__ __forceinline__ void residue_atoms_pair(const Topology<float> &tp, int ty, const PairFrame &P,
                                                   const float cs[2], const float sn[2], const float chi_c[5],
                                                   const float chi_s[5], Emit emit) {
    {
        const float x[3] = {P.p.x, P.p.y, P.p2};
        emit(0, x);
    }
    PairFrame F = P;
    apply_joint_pair(F, tp.bb_cb[0], tp.bb_sb[0], tp.bb_d[0], cs[0], sn[0]);
    {
        const float x[3] = {F.p.x, F.p.y, F.p2};
        emit(1, x);
    }
    const int na = tp.natoms[ty];
    if (tp.pro[ty]) {
        for (int a = 0; a < 3; a++) {
            float x[3];
            pair_point(F, tp.pro_local[a][0], tp.pro_local[a][1], tp.pro_local[a][2], x);
            emit(2 + a, x);
        }
    }
    const int nj = tp.njoints[ty];
    if (nj > 0) {
        PairFrame S = F;
        apply_rx_pair(S, tp.dummy_c, tp.dummy_s);
        // unrolled over the joints: joint k reads chi angle k or none (Ala's fixed
        // alpha; topology_layout_ok), so the angle is a register, not a select
#pragma unroll
        for (int k = 0; k < kMaxScJoints; k++) {
            if (k >= nj) break;
            const bool fixed = tp.jchi[ty][k] < 0;
            apply_joint_pair(S, tp.jcb[ty][k], tp.jsb[ty][k], tp.jd[ty][k], fixed ? 1.f : chi_c[k],
                             fixed ? 0.f : chi_s[k]);
            const int f0 = tp.jfirst[ty][k];
            {  // the group's first atom sits at the joint's origin
                const float x[3] = {S.p.x, S.p.y, S.p2};
                emit(2 + f0, x);
            }
            for (int a = 1; a < tp.jna[ty][k]; a++) {
                float x[3];
                pair_point(S, tp.sc[ty][f0 + a][0], tp.sc[ty][f0 + a][1], tp.sc[ty][f0 + a][2], x);
                emit(2 + f0 + a, x);
            }
        }
    }
    PairFrame C = F;
    apply_joint_pair(C, tp.bb_cb[1], tp.bb_sb[1], tp.bb_d[1], cs[1], sn[1]);
    {
        const float x[3] = {C.p.x, C.p.y, C.p2};
        emit(na - 2, x);
    }
    float x[3];
    pair_point(C, tp.o_local[0], tp.o_local[1], tp.o_local[2], x);
    emit(na - 1, x);
}

// Copy n staged values (world coordinates, xyz interleaved) to dst, coalesced.
template <typename T, int NT>
__device__ __forceinline__ void store_tile_atoms(T *dst, const T *src, int n) {
    for (int i = threadIdx.x; i < n; i += NT) dst[i] = src[i];
}

template <typename T, int R, int NT>
__global__ void __launch_bounds__(NT) a2c_fwd_kernel(A2cArgs<T> a, int renorm) {
    constexpr int TILE = R * NT, NW = NT / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    A2cSmemFwd<T, TILE> &smf = *reinterpret_cast<A2cSmemFwd<T, TILE> *>(smem_raw);
    A2cSmem<T, TILE> &sm = smf.f;
    __shared__ Frame<T> s_wtot[NW], s_wpre[NW];
    __shared__ int s_wcnt[NW], s_wcpre[NW];
    __shared__ Frame<T> s_carry;
    __shared__ T s_org[3];
    __shared__ int s_len, s_bad, s_abase, s_tcnt;

    const int b = blockIdx.x, tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    load_topology<T, NT>(sm.topo, sm.lut);
    const unsigned char *row = a.seq + (size_t)b * a.seq_stride;
    int len = chain_length<NT>(row, a.seq_stride, sm.lut, &s_len, &s_bad);
    T *out = a.coords + (size_t)b * 3 * a.maxA;
    uint32_t *rn = a.res_names ? a.res_names + (size_t)b * a.maxA : nullptr;
    uint32_t *an = a.atom_names ? a.atom_names + (size_t)b * a.maxA : nullptr;
    bool ok = true;
    if (s_bad) {
        if (tid == 0) a2c_error(a.hdr, TPL_ERR_SEQUENCE);
        ok = false;
    }
    if (len > a.L) {
        if (tid == 0) a2c_error(a.hdr, TPL_ERR_LENGTH);
        ok = false;
    }
    if (tid == 0) {
        frame_identity(s_carry);
        s_abase = 0;
    }
    __syncthreads();
    const T *ang_b = a.angles + (size_t)b * 8 * a.L;
    for (int s0 = 0; ok && s0 < len; s0 += TILE) {
        const int n = min(TILE, len - s0);
        for (int k = 0; k < 8; k++)
            for (int i = tid; i < n; i += NT) sm.ang[k][i] = ang_b[(size_t)k * a.L + s0 + i];
        for (int i = tid; i < n; i += NT) sm.type[i] = sm.lut[row[s0 + i]];
        __syncthreads();
        const bool chain_end = (s0 + n == len);
        TileScan<T, R, NT> ts;
        a2c_tile_scan<T, R, NT>(sm.topo, sm.ang, sm.type, n, chain_end, renorm, ts, s_wtot, s_wcnt);
        __syncthreads();
        if (tid == 0) {
            Frame<T> agg;
            int tcnt;
            a2c_tile_prefix<T, NW>(s_carry, s_wtot, s_wcnt, renorm, s_wpre, s_wcpre, agg, tcnt);
            s_org[0] = s_carry.p[0]; s_org[1] = s_carry.p[1]; s_org[2] = s_carry.p[2];
            s_tcnt = tcnt;
            Frame<T> nc = compose(s_carry, agg);
            renorm_if(nc, renorm);
            s_carry = nc;
        }
        __syncthreads();
        Frame<T> P = compose(s_wpre[w], ts.exc);
        renorm_if(P, renorm);
        int aoff = s_wcpre[w] + ts.cnt_exc;  // first atom of this thread inside the tile
        const int abase = s_abase;
        // positions are built relative to the tile origin and moved to it as they are
        // staged (the same FP32 addition as at store time, without a per-value modulo)
        const T org[3] = {s_org[0], s_org[1], s_org[2]};
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int j = tid * R + r;
            if (j < n) {
                const int ty = sm.type[j];
                T *dst = sm.xyz + 3 * aoff;
                residue_atoms<T>(sm.topo, ty, P, ts.cs[r], ts.sn[r], [&](int q) { return sm.ang[3 + q][j]; },
                                 [&](int slot, const T *x) {
                                     dst[3 * slot] = x[0] + org[0];
                                     dst[3 * slot + 1] = x[1] + org[1];
                                     dst[3 * slot + 2] = x[2] + org[2];
                                 });
                if (rn && an) {
                    const int na = sm.topo.natoms[ty];
                    for (int k = 0; k < na; k++) {
                        smf.res_name[aoff + k] = sm.topo.res_name[ty];
                        smf.atom_name[aoff + k] = sm.topo.atom_name[ty][k];
                    }
                }
                aoff += sm.topo.natoms[ty];
            }
        }
        __syncthreads();
        const int tcnt = s_tcnt;
        const int nstore = max(0, min(tcnt, a.maxA - abase));
        store_tile_atoms<T, NT>(out + (size_t)3 * abase, sm.xyz, 3 * nstore);
        if (rn && an)
            for (int i = tid; i < nstore; i += NT) {
                rn[abase + i] = smf.res_name[i];
                an[abase + i] = smf.atom_name[i];
            }
        __syncthreads();
        if (tid == 0) s_abase = abase + tcnt;
        __syncthreads();
    }
    int total = ok ? s_abase : 0;
    if (total > a.maxA) {
        if (tid == 0) a2c_error(a.hdr, TPL_ERR_ATOMS);
        total = a.maxA;
    }
    for (int i = 3 * total + tid; i < 3 * a.maxA; i += NT) out[i] = T(0);
    if (rn && an)
        for (int i = total + tid; i < a.maxA; i += NT) rn[i] = an[i] = 0u;
    (void)lane;
}

// ------------------------------------------ forward, four or eight warps per chain
// One CTA of NW = 4 or 8 warps per chain and chunks of 32 residues, one per lane;
// chunk k belongs to warp k % NW.  Per chunk a warp loads its residues' angles,
// composes each residue's three backbone joints (N -> CA -> C -> next N), scans the
// lane transforms and the atom counts over the warp, and places every atom of its
// residue from the lane's frame at N into a per-warp staging buffer, from which the
// chunk's contiguous atom range leaves with coalesced stores.  Only the chain frame
// at the chunk start and the chunk's first atom index pass between warps, through
// the named-barrier handoff of tpl_pair.cuh, so the chunk loop has no CTA-wide
// barrier.  Positions are built relative to the chunk's first N atom and moved to
// it as they are staged.
constexpr int kA2cChunk = 32;
constexpr int kA2cStageAtoms = kA2cChunk * kMaxResAtoms;

// The coordinate staging rows carry 4 words of slack: a chunk's values start at the
// word offset of their global destination inside its 16-byte block (0..3), so that
// whole blocks move as aligned 16-byte loads and stores (copy_span).
template <int NW>
struct A2cRingSmem {
    Topology<float> topo;
    signed char lut[256];
    alignas(16) float xyz[NW][kA2cStageAtoms * 3 + 4];
    uint32_t res_name[NW][kA2cStageAtoms];  // present when names are written
    uint32_t atom_name[NW][kA2cStageAtoms];
};

// Word offset of p inside its 16-byte block.
__device__ __forceinline__ int block_offset(const void *p) { return (int)((reinterpret_cast<uintptr_t>(p) >> 2) & 3u); }

// Copy n 4-byte words from the 16-byte-aligned staging row src (the values start at
// src + block_offset(dst)) to dst, by the warp: every 16-byte block of dst that lies
// whole inside [dst, dst + n) as one vector load and store, the ragged ends word by word.
template <typename W, typename W4>
__device__ __forceinline__ void copy_span(W *dst, const W *src, int n, int lane) {
    const int sh = block_offset(dst);
    W *base = dst - sh;  // 16-byte aligned; only words inside [dst, dst + n) are written
    const int nb = (n + sh + 3) >> 2;
    for (int b = lane; b < nb; b += 32) {
        const int lo = 4 * b - sh;
        if (lo >= 0 && lo + 4 <= n) {
            *reinterpret_cast<W4 *>(base + 4 * b) = *reinterpret_cast<const W4 *>(src + 4 * b);
        } else {
#pragma unroll
            for (int e = 0; e < 4; e++)
                if (lo + e >= 0 && lo + e < n) dst[lo + e] = src[sh + lo + e];
        }
    }
}
template <int NW>
constexpr size_t a2c_ring_smem_no_names() { return offsetof(A2cRingSmem<NW>, res_name); }

template <int NW, bool NAMES>
__global__ void __launch_bounds__(32 * NW, NW == 4 ? 6 : 3) a2c_fwd_ring_kernel(A2cArgs<float> a, int renorm, int nb) {
    constexpr int NT = 32 * NW;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    A2cRingSmem<NW> &sm = *reinterpret_cast<A2cRingSmem<NW> *>(smem_raw);
    __shared__ __align__(16) float s_ring[NW][16];  // chain frame (12) and first atom index
    __shared__ int s_len, s_bad, s_total;

    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    load_topology<float, NT>(sm.topo, sm.lut);
    const Topology<float> &tp = sm.topo;
    // persistent: the grid fills the SMs once and each CTA takes chains b, b + grid, ...,
    // so the topology loads once per CTA and no partial last wave of chains is left
    // (GB300, 4096 x 500 random residues: forward 0.155 -> 0.152 ms, with names
    // 0.203 -> 0.197 ms).  The barrier at the end of a chain orders its last reads of
    // the shared state before the next chain's writes.
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        if (tid == 0) s_total = 0;  // ordered before every chunk by the barriers of chain_length
        const unsigned char *row = a.seq + (size_t)b * a.seq_stride;
        const int len = chain_length<NT>(row, a.seq_stride, sm.lut, &s_len, &s_bad);
        const bool ok = !s_bad && len <= a.L;
        if (tid == 0) {
            if (s_bad) a2c_error(a.hdr, TPL_ERR_SEQUENCE);
            if (len > a.L) a2c_error(a.hdr, TPL_ERR_LENGTH);
        }
        float *out = a.coords + (size_t)b * 3 * a.maxA;
        uint32_t *rn = NAMES ? a.res_names + (size_t)b * a.maxA : nullptr;
        uint32_t *an = NAMES ? a.atom_names + (size_t)b * a.maxA : nullptr;
        const float *ang = a.angles + (size_t)b * 8 * a.L;
        float *stage = sm.xyz[w];
        const int nchunk = ok ? (len + kA2cChunk - 1) / kA2cChunk : 0;

#pragma unroll 1
        for (int k = w; k < nchunk; k += NW) {
            const int j = k * kA2cChunk + lane;
            const bool live = j < len;
            const int ty = live ? sm.lut[row[j]] : 0;
            const int na = live ? tp.natoms[ty] : 0;
            // backbone angles; omega of the chain's last residue moves no atom
            // cos and sin of the eight angles, in pairs and for every lane at once (the chi
            // angles' outside the divergent side-chain walk); omega of the chain's last
            // residue moves no atom
            float cs[3] = {1.f, 1.f, 1.f}, sn[3] = {0.f, 0.f, 0.f};
            float chc[5] = {1.f, 1.f, 1.f, 1.f, 1.f}, chs[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
            PairFrame t = pair_identity();
            if (live) {
                const float phi = ang[j], psi = ang[a.L + j];
                const float om = j + 1 < len ? ang[2 * a.L + j] : 0.f;
                float chi[5];
#pragma unroll
                for (int q = 0; q < 5; q++) chi[q] = ang[(size_t)(3 + q) * a.L + j];
                float m = fmaxf(fabsf(phi), fmaxf(fabsf(psi), fabsf(om)));
#pragma unroll
                for (int q = 0; q < 5; q++) m = fmaxf(m, fabsf(chi[q]));
                if (m <= 1.0e4f) {  // NaN passes: sincos_fast2 returns NaN for it
                    sincos_fast2(phi, psi, &sn[0], &cs[0], &sn[1], &cs[1]);
                    sincos_fast2(om, chi[0], &sn[2], &cs[2], &chs[0], &chc[0]);
                    sincos_fast2(chi[1], chi[2], &chs[1], &chc[1], &chs[2], &chc[2]);
                    sincos_fast2(chi[3], chi[4], &chs[3], &chc[3], &chs[4], &chc[4]);
                } else {
                    sincos_poly(phi, &sn[0], &cs[0]);
                    sincos_poly(psi, &sn[1], &cs[1]);
                    sincos_poly(om, &sn[2], &cs[2]);
#pragma unroll
                    for (int q = 0; q < 5; q++) sincos_poly(chi[q], &chs[q], &chc[q]);
                }
#pragma unroll
                for (int q = 0; q < 3; q++) apply_joint_pair(t, tp.bb_cb[q], tp.bb_sb[q], tp.bb_d[q], cs[q], sn[q]);
            }
            PairFrame tot;
            const PairFrame E = warp_exclusive_total_pair(t, lane, renorm != 0, tot);
            int ci = na;  // atoms of the lanes up to this one
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int o = __shfl_up_sync(0xffffffffu, ci, off);
                if (lane >= off) ci += o;
            }
            const int cnt = __shfl_sync(0xffffffffu, ci, 31), aoff = ci - na;

            PairFrame F = pair_identity();  // chain frame at the chunk start
            int abase = 0;                  // first atom of the chunk
            if (k > 0) {
                ring_wait<NW>(k);
                F = pair_load(s_ring[k % NW]);
                abase = __float_as_int(s_ring[k % NW][12]);
            }
            if (k + 1 < nchunk) {
                PairFrame Fn = compose_pair(F, tot);
                if (renorm) renormalize_pair(Fn);
                if (lane == 0) {
                    pair_store(s_ring[(k + 1) % NW], Fn);
                    s_ring[(k + 1) % NW][12] = __int_as_float(abase + cnt);
                }
                ring_signal<NW>(k + 1);
            } else if (lane == 0) {
                s_total = abase + cnt;
            }

            const float org[3] = {F.p.x, F.p.y, F.p2};
            PairFrame Fr = F;  // rotation only: positions relative to the chunk origin
            Fr.p = make_float2(0.f, 0.f);
            Fr.p2 = 0.f;
            float *gdst = out + (size_t)3 * abase;
            float *stg = stage + block_offset(gdst);  // the chunk's values keep their global 16-byte phase
            if (live) {
                const PairFrame P = compose_pair(Fr, E);
                float *dst = stg + 3 * aoff;
                residue_atoms_pair(tp, ty, P, cs, sn, chc, chs, [&](int slot, const float *x) {
                    dst[3 * slot] = x[0] + org[0];
                    dst[3 * slot + 1] = x[1] + org[1];
                    dst[3 * slot + 2] = x[2] + org[2];
                });
                if (NAMES)
                    for (int q = 0; q < na; q++) {
                        sm.res_name[w][aoff + q] = tp.res_name[ty];
                        sm.atom_name[w][aoff + q] = tp.atom_name[ty][q];
                    }
            }
            __syncwarp();
            const int nstore = max(0, min(cnt, a.maxA - abase));
            copy_span<float, float4>(gdst, stage, 3 * nstore, lane);
            if (NAMES)  // word stores: the names' own block phase would hold two more pointers through the walk
                for (int i = lane; i < nstore; i += 32) {
                    rn[abase + i] = sm.res_name[w][i];
                    an[abase + i] = sm.atom_name[w][i];
                }
            __syncwarp();  // the warp's next chunk rewrites the staging buffers
        }
        __syncthreads();
        int total = s_total;
        if (total > a.maxA) {
            if (tid == 0) a2c_error(a.hdr, TPL_ERR_ATOMS);
            total = a.maxA;
        }
        for (int i = 3 * total + tid; i < 3 * a.maxA; i += NT) out[i] = 0.f;
        if (NAMES)
            for (int i = total + tid; i < a.maxA; i += NT) rn[i] = an[i] = 0u;
        __syncthreads();
    }
}

// ------------------------------------------------------------------ backward
template <typename T, int R, int NT>
__global__ void __launch_bounds__(NT) a2c_bwd_kernel(A2cArgs<T> a, int renorm, int max_tiles) {
    constexpr int TILE = R * NT, NW = NT / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    A2cSmemBwd<T, TILE> &sm = *reinterpret_cast<A2cSmemBwd<T, TILE> *>(smem_raw);
    Frame<T> *s_carries = reinterpret_cast<Frame<T> *>(smem_raw + sizeof(A2cSmemBwd<T, TILE>));
    int *s_tbase = reinterpret_cast<int *>(s_carries + max_tiles);
    __shared__ Frame<T> s_wtot[NW], s_wpre[NW];
    __shared__ int s_wcnt[NW], s_wcpre[NW];
    __shared__ T s_wsum[NW][6], s_wsuf[NW][6];
    __shared__ double s_tail[6];
    __shared__ int s_len, s_bad;

    const int b = blockIdx.x, tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    load_topology<T, NT>(sm.f.topo, sm.f.lut);
    const Topology<T> &tp = sm.f.topo;
    const unsigned char *row = a.seq + (size_t)b * a.seq_stride;
    int len = chain_length<NT>(row, a.seq_stride, sm.f.lut, &s_len, &s_bad);
    T *gout = a.grad_angles + (size_t)b * 8 * a.L;
    const T *gin = a.grad_coords + (size_t)b * 3 * a.maxA;
    const T *ang_b = a.angles + (size_t)b * 8 * a.L;
    bool ok = !s_bad && len <= a.L;
    if (tid == 0) {
        if (s_bad) a2c_error(a.hdr, TPL_ERR_SEQUENCE);
        if (len > a.L) a2c_error(a.hdr, TPL_ERR_LENGTH);
    }
    const int ntiles = ok ? (len + TILE - 1) / TILE : 0;
    if (ntiles > max_tiles) {
        if (tid == 0) a2c_error(a.hdr, TPL_ERR_ARGUMENT);
        ok = false;
    }
    // sweep 1: tile carries and atom bases
    if (tid == 0) {
        frame_identity(s_carries[0]);
        s_tbase[0] = 0;
    }
    __syncthreads();
    for (int t = 0; ok && t < ntiles; t++) {
        const int s0 = t * TILE, n = min(TILE, len - s0);
        for (int k = 0; k < 3; k++)
            for (int i = tid; i < n; i += NT) sm.f.ang[k][i] = ang_b[(size_t)k * a.L + s0 + i];
        for (int i = tid; i < n; i += NT) sm.f.type[i] = sm.f.lut[row[s0 + i]];
        __syncthreads();
        TileScan<T, R, NT> ts;
        a2c_tile_scan<T, R, NT>(tp, sm.f.ang, sm.f.type, n, s0 + n == len, renorm, ts, s_wtot, s_wcnt);
        __syncthreads();
        if (tid == 0) {
            Frame<T> agg;
            int tcnt;
            a2c_tile_prefix<T, NW>(s_carries[t], s_wtot, s_wcnt, renorm, s_wpre, s_wcpre, agg, tcnt);
            if (t + 1 < max_tiles) {
                Frame<T> nc = compose(s_carries[t], agg);
                renorm_if(nc, renorm);
                s_carries[t + 1] = nc;
                s_tbase[t + 1] = s_tbase[t] + tcnt;
            }
        }
        __syncthreads();
    }
    if (tid == 0)
        for (int i = 0; i < 6; i++) s_tail[i] = 0.0;
    __syncthreads();
    // sweep 2: tiles last-first
    for (int t = ntiles - 1; ok && t >= 0; t--) {
        const int s0 = t * TILE, n = min(TILE, len - s0);
        const int abase = s_tbase[t];
        for (int k = 0; k < 8; k++)
            for (int i = tid; i < n; i += NT) sm.f.ang[k][i] = ang_b[(size_t)k * a.L + s0 + i];
        for (int i = tid; i < n; i += NT) sm.f.type[i] = sm.f.lut[row[s0 + i]];
        __syncthreads();
        TileScan<T, R, NT> ts;
        a2c_tile_scan<T, R, NT>(tp, sm.f.ang, sm.f.type, n, s0 + n == len, renorm, ts, s_wtot, s_wcnt);
        __syncthreads();
        if (tid == 0) {
            Frame<T> agg;
            int tcnt;
            a2c_tile_prefix<T, NW>(s_carries[t], s_wtot, s_wcnt, renorm, s_wpre, s_wcpre, agg, tcnt);
            s_wcnt[0] = tcnt;  // reuse: tile atom count
        }
        __syncthreads();
        const int tcnt = s_wcnt[0];
        const int nload = max(0, min(tcnt, a.maxA - abase));
        for (int i = tid; i < 3 * tcnt; i += NT) sm.g[i] = i < 3 * nload ? gin[(size_t)3 * abase + i] : T(0);
        Frame<T> P = compose(s_wpre[w], ts.exc);
        renorm_if(P, renorm);
        Frame<T> start[R];
        int roff[R];
        int aoff = s_wcpre[w] + ts.cnt_exc;
        __syncthreads();  // sm.g complete
        T G[3] = {0, 0, 0}, S[3] = {0, 0, 0};
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int j = tid * R + r;
            start[r] = P;
            roff[r] = aoff;
            if (j < n) {
                const int ty = sm.f.type[j];
                T *dst = sm.f.xyz + 3 * aoff;
                const T *gg = sm.g + 3 * aoff;
                residue_atoms<T>(tp, ty, P, ts.cs[r], ts.sn[r], [&](int q) { return sm.f.ang[3 + q][j]; },
                                 [&](int slot, const T *x) {
                    dst[3 * slot] = x[0];
                    dst[3 * slot + 1] = x[1];
                    dst[3 * slot + 2] = x[2];
                    T xg[3];
                    cross3(x, gg + 3 * slot, xg);
                    for (int c = 0; c < 3; c++) {
                        G[c] += gg[3 * slot + c];
                        S[c] += xg[c];
                    }
                });
                aoff += tp.natoms[ty];
            }
        }
        // block-exclusive suffix over threads, plus the carry from later tiles
        T suf[6];
        const T v[6] = {G[0], G[1], G[2], S[0], S[1], S[2]};
        for (int i = 0; i < 6; i++) {
            T inc = v[i];
            for (int off = 1; off < 32; off <<= 1) {
                T o = __shfl_down_sync(0xffffffffu, inc, off);
                if (lane + off < 32) inc += o;
            }
            T tot = __shfl_sync(0xffffffffu, inc, 0);
            suf[i] = inc - v[i];
            if (lane == 0) s_wsum[w][i] = tot;
        }
        __syncthreads();
        if (tid == 0) {
            // later tiles' (G, S) are kept about the world origin in FP64; move them
            // to this tile's origin o: S_o = S_world - o x G
            const double o[3] = {(double)s_carries[t].p[0], (double)s_carries[t].p[1], (double)s_carries[t].p[2]};
            double ox[3];
            cross3(o, s_tail, ox);
            double run[6];
            for (int i = 0; i < 3; i++) {
                run[i] = s_tail[i];
                run[3 + i] = s_tail[3 + i] - ox[i];
            }
            double tot[6] = {0, 0, 0, 0, 0, 0};
            for (int ww = NW - 1; ww >= 0; ww--)
                for (int i = 0; i < 6; i++) {
                    s_wsuf[ww][i] = (T)run[i];
                    run[i] += (double)s_wsum[ww][i];
                    tot[i] += (double)s_wsum[ww][i];
                }
            double ot[3];
            cross3(o, tot, ot);
            for (int i = 0; i < 3; i++) {
                s_tail[i] += tot[i];
                s_tail[3 + i] += tot[3 + i] + ot[i];
            }
        }
        __syncthreads();
        T Gn[3], Sn[3];
        for (int c = 0; c < 3; c++) {
            Gn[c] = suf[c] + s_wsuf[w][c];
            Sn[c] = suf[3 + c] + s_wsuf[w][3 + c];
        }
        T(*s_gr)[TILE] = sm.f.ang;  // angles of this tile stay in registers (ts) / are re-read below
#pragma unroll
        for (int r = R - 1; r >= 0; r--) {
            const int j = tid * R + r;
            if (j >= n) continue;
            const int ty = sm.f.type[j];
            const int na = tp.natoms[ty], nj = tp.njoints[ty];
            const T *X = sm.f.xyz + 3 * roff[r];
            const T *Gg = sm.g + 3 * roff[r];
            // per-group sums of this residue
            auto acc = [&](int lo, int hi, T *gs, T *ss) {
                for (int c = 0; c < 3; c++) gs[c] = ss[c] = T(0);
                for (int q = lo; q < hi; q++) {
                    T xg[3];
                    cross3(X + 3 * q, Gg + 3 * q, xg);
                    for (int c = 0; c < 3; c++) {
                        gs[c] += Gg[3 * q + c];
                        ss[c] += xg[c];
                    }
                }
            };
            T Gco[3], Sco[3], Gmid[3], Smid[3], Gn0[3], Sn0[3];
            acc(na - 2, na, Gco, Sco);
            acc(1, na - 2, Gmid, Smid);   // CA, Pro ring / side chain
            acc(0, 1, Gn0, Sn0);          // N
            // frames of the residue
            Frame<T> F = start[r];
            apply_joint(F, tp.bb_cb[0], tp.bb_sb[0], tp.bb_d[0], ts.cs[r][0], ts.sn[r][0]);
            Frame<T> C = F;
            apply_joint(C, tp.bb_cb[1], tp.bb_sb[1], tp.bb_d[1], ts.cs[r][1], ts.sn[r][1]);
            Frame<T> Nn = C;
            apply_joint(Nn, tp.bb_cb[2], tp.bb_sb[2], tp.bb_d[2], ts.cs[r][2], ts.sn[r][2]);
            T tmp[3], cr[3];
            auto gradient = [&](const Frame<T> &J, const T *Gs, const T *Ss) {
                cross3(J.p, Gs, cr);
                for (int c = 0; c < 3; c++) tmp[c] = Ss[c] - cr[c];
                return J.r[0] * tmp[0] + J.r[3] * tmp[1] + J.r[6] * tmp[2];
            };
            const bool last = (s0 + j == len - 1);
            const T g_om = last ? T(0) : gradient(Nn, Gn, Sn);
            T Gc[3], Sc[3];
            for (int c = 0; c < 3; c++) {
                Gc[c] = Gn[c] + Gco[c];
                Sc[c] = Sn[c] + Sco[c];
            }
            const T g_ps = gradient(C, Gc, Sc);
            for (int c = 0; c < 3; c++) {
                Gc[c] += Gmid[c];
                Sc[c] += Smid[c];
            }
            const T g_ph = gradient(F, Gc, Sc);
            // side-chain joints: subtree of joint k = its group and all later groups
            T g_chi[5] = {0, 0, 0, 0, 0};
            if (nj > 0) {
                T Gsc[3], Ssc[3];
                acc(2, na - 2, Gsc, Ssc);
                Frame<T> Sf = F;
                apply_rx(Sf, tp.dummy_c, tp.dummy_s);
                for (int k = 0; k < nj; k++) {
                    const int chi = tp.jchi[ty][k];
                    T c = T(1), s = T(0);
                    if (chi >= 0) sc(sm.f.ang[3 + chi][j], &s, &c);
                    apply_joint(Sf, tp.jcb[ty][k], tp.jsb[ty][k], tp.jd[ty][k], c, s);
                    if (chi >= 0) g_chi[chi] = gradient(Sf, Gsc, Ssc);
                    const int f0 = 2 + tp.jfirst[ty][k];
                    T Gk[3], Sk[3];
                    acc(f0, f0 + tp.jna[ty][k], Gk, Sk);
                    for (int q = 0; q < 3; q++) {
                        Gsc[q] -= Gk[q];
                        Ssc[q] -= Sk[q];
                    }
                }
            }
            // suffix for the previous residue: this residue's atoms join it
            for (int c = 0; c < 3; c++) {
                Gn[c] = Gc[c] + Gn0[c];
                Sn[c] = Sc[c] + Sn0[c];
            }
            // chi angles are read from shared memory above, so stage gradients in
            // registers until every thread has finished with the angle rows
            start[r].r[0] = g_ph; start[r].r[1] = g_ps; start[r].r[2] = g_om;
            for (int q = 0; q < 5; q++) start[r].r[3 + q] = g_chi[q];
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int j = tid * R + r;
            if (j < n)
                for (int q = 0; q < 8; q++) s_gr[q][j] = start[r].r[q];
        }
        __syncthreads();
        for (int k = 0; k < 8; k++)
            for (int i = tid; i < n; i += NT) gout[(size_t)k * a.L + s0 + i] = s_gr[k][i];
        __syncthreads();
    }
    // zeros past the chain (and everywhere when the chain was rejected)
    const int from = ok ? len : 0;
    for (int k = 0; k < 8; k++)
        for (int i = from + tid; i < a.L; i += NT) gout[(size_t)k * a.L + i] = T(0);
}

// ------------------------------------------------- backward from the coordinates
// The forward's output holds the origin of every joint: N, CA and C for the
// backbone, and for each side-chain joint the first atom of its group, which sits
// at the joint's origin (every group of the table starts at its local origin).
// Each rotation axis is a bond of known length: u = (origin - parent origin) / d,
// with CA as the parent of the first side-chain joint (the dummy joint has no
// length).  So dL/dalpha = u . (S - o x G) over the joint's subtree needs only the
// coordinates and dL/dx, and this backward never rebuilds the tree.  Each lane owns
// one residue: it sums G and S over the residue's atoms, a warp suffix scan adds the
// later residues of its chunk and a carry the later chunks, and the lane visits its
// residue's atoms last to first:
//   omega_j  subtree: every later residue        axis C_j -> N_j+1, origin N_j+1
//   psi_j    + O_j                                axis CA_j -> C_j,  origin C_j
//   chi_k    side-chain groups k.. only           axis o_k-1 -> o_k, origin o_k
//   phi_j    + side chain + C_j                   axis N_j -> CA_j,  origin CA_j
// Positions are taken relative to the chunk's first N atom to keep the sums small.
__device__ __forceinline__ float joint_grad(const float *o, const float *p_prev, float inv_d, const float *G,
                                            const float *S) {
    float cr[3];
    cross3(o, G, cr);
    return ((o[0] - p_prev[0]) * (S[0] - cr[0]) + (o[1] - p_prev[1]) * (S[1] - cr[1]) +
            (o[2] - p_prev[2]) * (S[2] - cr[2])) *
           inv_d;
}

// Sum of v over lanes above this one (exclusive suffix), and the warp total.
__device__ __forceinline__ float suffix_excl(float v, int lane, float &total) {
    float inc = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const float o = __shfl_down_sync(0xffffffffu, inc, off);
        if (lane + off < 32) inc += o;
    }
    total = __shfl_sync(0xffffffffu, inc, 0);
    return inc - v;
}

__device__ __forceinline__ void add_atom(const float *xs, const float *gs, const float *o, float *G, float *S) {
    const float xr[3] = {xs[0] - o[0], xs[1] - o[1], xs[2] - o[2]};
    float xg[3];
    cross3(xr, gs, xg);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        G[c] += gs[c];
        S[c] += xg[c];
    }
}

// The kernel: NW = 4 or 8 warps per chain on chunks of 32 residues (one per lane),
// chunk k on warp (nchunk - 1 - k) % NW, last chunk first.  The chunks' first atom indices come from
// one pass over the sequence at the start; per chunk a warp stages the chunk's atom
// range of coordinates and dL/dx with coalesced loads, sums G and S over each
// lane's residue about the chunk's first N atom, suffix-scans them over the warp
// and takes the sums over later chunks from the warp of chunk k + 1 (G, S and that
// chunk's first N atom, through the named-barrier handoff of tpl_pair.cuh).
__device__ __forceinline__ void cp_async4(float *dst_smem, const float *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(dst_smem)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

template <int NW>
struct A2cBwdRingSmem {
    Topology<float> topo;
    signed char lut[256];
    alignas(16) float x[NW][kA2cStageAtoms * 3 + 4];  // 4 floats of slack, as in A2cRingSmem
    alignas(16) float g[NW][kA2cStageAtoms * 3 + 4];
    int base[1];  // first atom of each chunk, nchunk + 1 entries (dynamic)
};

__device__ __forceinline__ void cp_async16(float *dst_smem, const float *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst_smem)),
                 "l"(src)
                 : "memory");
}

// Stage n floats of src into the 16-byte-aligned row dst, starting at
// dst + block_offset(src), by the warp: 16-byte asynchronous copies for every block
// of src that lies whole inside the span, 4-byte ones for the ragged ends.  Returns
// where the values start.
__device__ __forceinline__ float *stage_span_async(float *dst, const float *src, int n, int lane) {
    const int sh = block_offset(src);
    const float *base = src - sh;  // 16-byte aligned; only [src, src + n) is read
    const int nb = (n + sh + 3) >> 2;
    for (int b = lane; b < nb; b += 32) {
        const int lo = 4 * b - sh;
        if (lo >= 0 && lo + 4 <= n) {
            cp_async16(dst + 4 * b, base + 4 * b);
        } else {
#pragma unroll
            for (int e = 0; e < 4; e++)
                if (lo + e >= 0 && lo + e < n) cp_async4(dst + sh + lo + e, src + lo + e);
        }
    }
    return dst + sh;
}

template <int NW>
__global__ void __launch_bounds__(32 * NW) a2c_bwd_coords_ring_kernel(A2cArgs<float> a, int nb) {
    constexpr int NT = 32 * NW;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    A2cBwdRingSmem<NW> &sm = *reinterpret_cast<A2cBwdRingSmem<NW> *>(smem_raw);
    __shared__ __align__(16) float s_ring[NW][12];
    __shared__ int s_len, s_bad;

    // chains last to first: the first CTAs read the rows the forward wrote last, which may still be in L2
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    load_topology<float, NT>(sm.topo, sm.lut);
    const Topology<float> &tp = sm.topo;
    // persistent, as a2c_fwd_ring_kernel, counting down from the last chain (GB300,
    // 4096 x 500: 0.199 -> 0.189 ms)
    for (int b = nb - 1 - (int)blockIdx.x; b >= 0; b -= (int)gridDim.x) {
        const unsigned char *row = a.seq + (size_t)b * a.seq_stride;
        const int len = chain_length<NT>(row, a.seq_stride, sm.lut, &s_len, &s_bad);
        float *gout = a.grad_angles + (size_t)b * 8 * a.L;
        const float *xin = a.coords + (size_t)b * 3 * a.maxA;
        const float *gin = a.grad_coords + (size_t)b * 3 * a.maxA;
        bool ok = !s_bad && len <= a.L;
        const int nchunk = ok ? (len + kA2cChunk - 1) / kA2cChunk : 0;

        // atoms per chunk (warp w counts chunks w, w + 4, ...), then their exclusive prefix
        for (int c = w; c < nchunk; c += NW) {
            const int j = c * kA2cChunk + lane;
            int n = j < len ? tp.natoms[sm.lut[row[j]]] : 0;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) n += __shfl_xor_sync(0xffffffffu, n, off);
            if (lane == 0) sm.base[c + 1] = n;
        }
        __syncthreads();
        if (w == 0) {
            int run = 0;
            for (int c0 = 0; c0 < nchunk; c0 += 32) {
                const int c = c0 + lane;
                int v = c < nchunk ? sm.base[c + 1] : 0;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const int o = __shfl_up_sync(0xffffffffu, v, off);
                    if (lane >= off) v += o;
                }
                if (c < nchunk) sm.base[c + 1] = run + v;
                run += __shfl_sync(0xffffffffu, v, 31);
            }
            if (lane == 0) sm.base[0] = 0;
        }
        __syncthreads();
        const int total = nchunk > 0 ? sm.base[nchunk] : 0;
        if (tid == 0) {
            if (s_bad) a2c_error(a.hdr, TPL_ERR_SEQUENCE);
            if (len > a.L) a2c_error(a.hdr, TPL_ERR_LENGTH);
            if (ok && total > a.maxA) a2c_error(a.hdr, TPL_ERR_ATOMS);
        }
        const int nrun = total > a.maxA ? 0 : nchunk;  // a chain whose atoms overflow the rows gets zeros
        const float inv_dphi = 1.f / tp.bb_d[0], inv_dpsi = 1.f / tp.bb_d[1], inv_dom = 1.f / tp.bb_d[2];

#pragma unroll 1
        for (int k = nrun - 1 - w; k >= 0; k -= NW) {
            const int j = k * kA2cChunk + lane;
            const bool live = j < len;
            const int ty = live ? sm.lut[row[j]] : 0;
            const int na = live ? tp.natoms[ty] : 0;
            int inc = na;  // the residue's first atom inside the chunk: warp exclusive scan
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, inc, off);
                if (lane >= off) inc += v;
            }
            const int aoff = inc - na;
            const int abase = sm.base[k], n3 = 3 * (sm.base[k + 1] - abase);
            __syncwarp();  // the previous chunk's reads of the staging buffers are done
            // asynchronous copies: every copy of the chunk is in flight before the one wait
            const float *sx = stage_span_async(sm.x[w], xin + (size_t)3 * abase, n3, lane);
            const float *sg = stage_span_async(sm.g[w], gin + (size_t)3 * abase, n3, lane);
            cp_async_wait_all();
            __syncwarp();
            const float o[3] = {sx[0], sx[1], sx[2]};  // chunk origin: its first N atom
            // One walk over the residue's atoms, last to first, from G = S = 0.  Every
            // joint gradient u . (S - o x G) is linear in (G, S), so each joint's share of
            // its own residue is taken here and the share of the later residues is added
            // after the scan: complete for the chi joints (side-chain atoms only), and
            // the own parts of psi and phi.  The walk ends with the residue's totals.
            float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            float gr[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            float xN[3] = {0.f, 0.f, 0.f}, xA[3] = {0.f, 0.f, 0.f}, xC[3] = {0.f, 0.f, 0.f};
            if (live) {
                const float *X = sx + 3 * aoff, *Gg = sg + 3 * aoff;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    xN[c] = X[c] - o[c];
                    xA[c] = X[3 + c] - o[c];
                    xC[c] = X[3 * (na - 2) + c] - o[c];
                }
                float *G = v, *S = v + 3;
                add_atom(X + 3 * (na - 1), Gg + 3 * (na - 1), o, G, S);  // O
                gr[1] = joint_grad(xC, xA, inv_dpsi, G, S);
                add_atom(X + 3 * (na - 2), Gg + 3 * (na - 2), o, G, S);  // C
                // side chain, groups last to first; chi subtrees hold side-chain atoms only
                float Gs[3] = {0.f, 0.f, 0.f}, Ss[3] = {0.f, 0.f, 0.f};
                const int nj = tp.njoints[ty];
                if (nj == 0)
                    for (int q = 2; q < na - 2; q++) add_atom(X + 3 * q, Gg + 3 * q, o, Gs, Ss);  // Pro ring (none for Gly)
                // unrolled over the joints: joint kk reads chi angle kk or none (Ala;
                // topology_layout_ok), so its gradient goes to a register, not a select
#pragma unroll
                for (int kk = kMaxScJoints - 1; kk >= 0; kk--) {
                    if (kk >= nj) continue;
                    const int f0 = 2 + tp.jfirst[ty][kk], f1 = f0 + tp.jna[ty][kk];
                    for (int q = f1 - 1; q >= f0; q--) add_atom(X + 3 * q, Gg + 3 * q, o, Gs, Ss);
                    if (tp.jchi[ty][kk] >= 0) {
                        const float *pk = X + 3 * f0;
                        const float *pp = kk == 0 ? X + 3 : X + 3 * (2 + tp.jfirst[ty][kk - 1]);
                        const float ok_[3] = {pk[0] - o[0], pk[1] - o[1], pk[2] - o[2]};
                        const float op_[3] = {pp[0] - o[0], pp[1] - o[1], pp[2] - o[2]};
                        gr[3 + kk] = joint_grad(ok_, op_, 1.f / tp.jd[ty][kk], Gs, Ss);
                    }
                }
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    G[c] += Gs[c];
                    S[c] += Ss[c];
                }
                gr[0] = joint_grad(xA, xN, inv_dphi, G, S);
                add_atom(X + 3, Gg + 3, o, G, S);  // CA
                add_atom(X, Gg, o, G, S);          // N
            }
            float later[6], ctot[6];
#pragma unroll
            for (int i = 0; i < 6; i++) later[i] = suffix_excl(v[i], lane, ctot[i]);
            // the sums over later chunks, moved to this chunk's origin: S_o = S_on + (on - o) x G
            float Gc[3] = {0.f, 0.f, 0.f}, Sc[3] = {0.f, 0.f, 0.f}, nN[3] = {0.f, 0.f, 0.f};
            if (k + 1 < nrun) {
                ring_wait<NW>(k);
                const float *cin = s_ring[k % NW];
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
                    float *cout = s_ring[(k - 1) % NW];
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        cout[c] = Gc[c] + ctot[c];
                        cout[3 + c] = Sc[c] + ctot[3 + c];
                        cout[6 + c] = o[c];
                    }
                }
                ring_signal<NW>(k - 1);
            }
            if (live) {
                // the later residues' share: sums over every atom after this residue
                const float G[3] = {later[0] + Gc[0], later[1] + Gc[1], later[2] + Gc[2]};
                const float S[3] = {later[3] + Sc[0], later[4] + Sc[1], later[5] + Sc[2]};
                if (j + 1 < len) {  // omega_j: the next residue's N joint (the next chunk's first N after lane 31)
                    const float *X = sx + 3 * aoff;
                    float xn[3];
#pragma unroll
                    for (int c = 0; c < 3; c++) xn[c] = (lane == 31 ? nN[c] : X[3 * na + c]) - o[c];
                    gr[2] = joint_grad(xn, xC, inv_dom, G, S);
                }
                gr[1] += joint_grad(xC, xA, inv_dpsi, G, S);
                gr[0] += joint_grad(xA, xN, inv_dphi, G, S);
#pragma unroll
                for (int q = 0; q < 8; q++) gout[(size_t)q * a.L + j] = gr[q];
            }
        }
        // zeros past the chain (and everywhere when the chain was rejected)
        const int from = nrun > 0 ? len : 0;
        for (int q = 0; q < 8; q++)
            for (int i = from + tid; i < a.L; i += NT) gout[(size_t)q * a.L + i] = 0.f;
        __syncthreads();
    }
}

// ------------------------------------------------------------------ host side
template <typename T, int R, int NT>
static int launch_a2c_fwd(const A2cArgs<T> &a, int B, int renorm, cudaStream_t st) {
    constexpr int TILE = R * NT;
    const size_t smem = sizeof(A2cSmemFwd<T, TILE>);
    auto k = a2c_fwd_kernel<T, R, NT>;
    if (!set_max_dynamic_smem(reinterpret_cast<const void *>(k), (int)smem))
        return TPL_ERR_LAUNCH;
    k<<<B, NT, smem, st>>>(a, renorm);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

template <typename T, int R, int NT>
static int launch_a2c_bwd(const A2cArgs<T> &a, int B, int renorm, cudaStream_t st) {
    constexpr int TILE = R * NT;
    const int max_tiles = (a.L + TILE - 1) / TILE + 1;
    const size_t smem = sizeof(A2cSmemBwd<T, TILE>) + (sizeof(Frame<T>) + sizeof(int)) * max_tiles;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if ((int)smem > optin) return TPL_ERR_UNSUPPORTED;
    auto k = a2c_bwd_kernel<T, R, NT>;
    if (!set_max_dynamic_smem(reinterpret_cast<const void *>(k), (int)smem))
        return TPL_ERR_LAUNCH;
    k<<<B, NT, smem, st>>>(a, renorm, max_tiles);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

// Warps per chain of the float32 kernels: eight while the batch leaves SMs short of
// chains, four once every SM has several (GB300, forward without names, 0.099 against
// 0.109 ms at 1024 x 1000 residues and 0.188 against 0.170 ms at 4096 x 500; with
// names or in the backward the crossing comes at about half the batch).
static int a2c_ring_warps(int B, int chains_per_sm) { return B < chains_per_sm * device_sm_count() ? 8 : 4; }

template <int NW>
static int launch_a2c_fwd_ring(const A2cArgs<float> &a, int B, int renorm, cudaStream_t st) {
    const bool names = a.res_names && a.atom_names;
    const size_t smem = names ? sizeof(A2cRingSmem<NW>) : a2c_ring_smem_no_names<NW>();
    auto k = names ? a2c_fwd_ring_kernel<NW, true> : a2c_fwd_ring_kernel<NW, false>;
    if (!set_max_dynamic_smem(reinterpret_cast<const void *>(k), (int)smem))
        return TPL_ERR_LAUNCH;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 32 * NW, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
    const int grid = std::min(B, per_sm * device_sm_count());
    k<<<grid, 32 * NW, smem, st>>>(a, renorm, B);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

template <int NW>
static int launch_a2c_bwd_coords_ring(const A2cArgs<float> &a, int B, int L, cudaStream_t st) {
    const size_t smem = offsetof(A2cBwdRingSmem<NW>, base) + sizeof(int) * (size_t)((L + kA2cChunk - 1) / kA2cChunk + 1);
    auto k = a2c_bwd_coords_ring_kernel<NW>;
    if (!set_max_dynamic_smem(reinterpret_cast<const void *>(k), (int)smem))
        return TPL_ERR_LAUNCH;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 32 * NW, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
    const int grid = std::min(B, per_sm * device_sm_count());
    k<<<grid, 32 * NW, smem, st>>>(a, B);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

int a2c_forward(bool f64, const unsigned char *seq, int seq_stride, const void *angles, void *coords,
                uint32_t *res_names, uint32_t *atom_names, void *ws, int B, int L, int maxA,
                const tpl_options &opt, cudaStream_t st) {
    if (B == 0) return TPL_OK;
    const int renorm = opt.renormalize >= 0 ? 1 : 0;
    if (f64) {
        A2cArgs<double> a{seq, seq_stride, (const double *)angles, (double *)coords, res_names, atom_names,
                          nullptr, nullptr, (WsHeader *)ws, L, maxA};
        return launch_a2c_fwd<double, 1, 128>(a, B, renorm, st);
    }
    A2cArgs<float> a{seq, seq_stride, (const float *)angles, (float *)coords, res_names, atom_names,
                     nullptr, nullptr, (WsHeader *)ws, L, maxA};
    // threads_per_cta: 128 = 128 threads x 2 residues; 0 / 256 (default) or 512 = one
    // residue per thread
    switch (opt.threads_per_cta) {
        case 4: return launch_a2c_fwd_ring<4>(a, B, renorm, st);
        case 8: return launch_a2c_fwd_ring<8>(a, B, renorm, st);
        case 128: return launch_a2c_fwd<float, 2, 128>(a, B, renorm, st);
        case 256: return launch_a2c_fwd<float, 1, 256>(a, B, renorm, st);
        case 512: return launch_a2c_fwd<float, 1, 512>(a, B, renorm, st);
    }
    return a2c_ring_warps(B, res_names && atom_names ? 4 : 8) == 8 ? launch_a2c_fwd_ring<8>(a, B, renorm, st)
                                                                    : launch_a2c_fwd_ring<4>(a, B, renorm, st);
}

int a2c_backward(bool f64, void *grad_angles, const void *grad_coords, const unsigned char *seq, int seq_stride,
                 const void *angles, void *ws, int B, int L, int maxA, const tpl_options &opt, cudaStream_t st) {
    if (B == 0) return TPL_OK;
    const int renorm = opt.renormalize >= 0 ? 1 : 0;
    if (f64) {
        A2cArgs<double> a{seq, seq_stride, (const double *)angles, nullptr, nullptr, nullptr,
                          (double *)grad_angles, (const double *)grad_coords, (WsHeader *)ws, L, maxA};
        return launch_a2c_bwd<double, 1, 128>(a, B, renorm, st);
    }
    A2cArgs<float> a{seq, seq_stride, (const float *)angles, nullptr, nullptr, nullptr, (float *)grad_angles,
                     (const float *)grad_coords, (WsHeader *)ws, L, maxA};
    switch (opt.threads_per_cta) {
        case 128: return launch_a2c_bwd<float, 2, 128>(a, B, renorm, st);
        case 512: return launch_a2c_bwd<float, 1, 512>(a, B, renorm, st);
    }
    return launch_a2c_bwd<float, 1, 256>(a, B, renorm, st);
}

int a2c_backward_coords(float *grad_angles, const float *grad_coords, const float *coords, const unsigned char *seq,
                        int seq_stride, void *ws, int B, int L, int maxA, cudaStream_t st) {
    if (B == 0) return TPL_OK;
    A2cArgs<float> a{seq, seq_stride, nullptr, const_cast<float *>(coords), nullptr, nullptr, grad_angles, grad_coords,
                     (WsHeader *)ws, L, maxA};
    return a2c_ring_warps(B, 4) == 8 ? launch_a2c_bwd_coords_ring<8>(a, B, L, st)
                                     : launch_a2c_bwd_coords_ring<4>(a, B, L, st);
}

int num_atoms_host(const char *seq) {
    static constexpr Topology<double> tp = make_topology<double>();
    int n = 0;
    for (const char *p = seq; *p; p++) {
        int t = residue_type((unsigned char)*p);
        if (t < 0) return -1;
        n += tp.natoms[t];
    }
    return n;
}

}  // namespace tpl
