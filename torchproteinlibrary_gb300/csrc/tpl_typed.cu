// Coords2TypedCoords on the GPU (sm_103a): atoms regrouped by the 11 atom types of
// ProtUtil::get11AtomType (Math/nUtil.cpp:567-703), stable within a type.
//
// Reference: Layers/FullAtomModel/Coords2TypedCoords/coords2typedcoords_interface.cpp
// runs on the CPU, one OpenMP task per chain, with string compares per atom.  Here
// one CTA per chain classifies its atoms from the packed 4-byte name words that
// Angles2Coords writes, counts them per type, and scatters coordinates in a stable
// order: per 256-atom tile, one warp ballot per type gives each atom its rank among
// the atoms of its type before it.  The backward is the inverse gather.  Integer and
// byte work only; coordinates are copied unchanged.
#include <cstdint>

#include "tpl_internal.h"

namespace tpl {
namespace {

constexpr int kTypes = 11;
constexpr int kTypedThreads = 256;

// Name word: the bytes of a NUL-padded 4-byte name slot, little-endian.
constexpr uint32_t nm(const char *s) {
    uint32_t w = 0;
    for (int i = 0; i < 4 && s[i]; i++) w |= (uint32_t)(unsigned char)s[i] << (8 * i);
    return w;
}

struct TypedName {
    uint32_t res, atom;
    int type;
};

// Residue-specific types (0-based, as get11AtomType returns them); the
// residue-agnostic backbone names are handled first in atom_type().
constexpr TypedName kTypedNames[] = {
    // 0: sulfur / selenium
    {nm("CYS"), nm("SG"), 0}, {nm("MET"), nm("SD"), 0}, {nm("MSE"), nm("SE"), 0},
    // 1: amide N
    {nm("ASN"), nm("ND2"), 1}, {nm("GLN"), nm("NE2"), 1},
    // 2: aromatic N
    {nm("HIS"), nm("ND1"), 2}, {nm("HIS"), nm("NE2"), 2}, {nm("TRP"), nm("NE1"), 2},
    // 3: guanidine N
    {nm("ARG"), nm("NH1"), 3}, {nm("ARG"), nm("NH2"), 3}, {nm("ARG"), nm("NE"), 3},
    // 4: N with three hydrogens
    {nm("LYS"), nm("NZ"), 4},
    // 5: carbonyl / amide O
    {nm("ACE"), nm("O"), 5}, {nm("ASN"), nm("OD1"), 5}, {nm("GLN"), nm("OE1"), 5},
    // 6: hydroxyl O
    {nm("SER"), nm("OG"), 6}, {nm("THR"), nm("OG1"), 6}, {nm("TYR"), nm("OH"), 6},
    // 7: carboxyl O
    {nm("ASP"), nm("OD1"), 7}, {nm("ASP"), nm("OD2"), 7}, {nm("GLU"), nm("OE1"), 7}, {nm("GLU"), nm("OE2"), 7},
    // 8: sp2 C
    {nm("ARG"), nm("CZ"), 8}, {nm("ASP"), nm("CG"), 8}, {nm("GLU"), nm("CD"), 8}, {nm("ACE"), nm("C"), 8},
    {nm("ASN"), nm("CG"), 8}, {nm("GLN"), nm("CD"), 8},
    // 9: aromatic C
    {nm("HIS"), nm("CD2"), 9}, {nm("HIS"), nm("CE1"), 9}, {nm("HIS"), nm("CG"), 9},
    {nm("PHE"), nm("CD1"), 9}, {nm("PHE"), nm("CD2"), 9}, {nm("PHE"), nm("CE1"), 9}, {nm("PHE"), nm("CE2"), 9},
    {nm("PHE"), nm("CG"), 9}, {nm("PHE"), nm("CZ"), 9},
    {nm("TRP"), nm("CD1"), 9}, {nm("TRP"), nm("CD2"), 9}, {nm("TRP"), nm("CE2"), 9}, {nm("TRP"), nm("CE3"), 9},
    {nm("TRP"), nm("CG"), 9}, {nm("TRP"), nm("CH2"), 9}, {nm("TRP"), nm("CZ2"), 9}, {nm("TRP"), nm("CZ3"), 9},
    {nm("TYR"), nm("CD1"), 9}, {nm("TYR"), nm("CD2"), 9}, {nm("TYR"), nm("CE1"), 9}, {nm("TYR"), nm("CE2"), 9},
    {nm("TYR"), nm("CG"), 9}, {nm("TYR"), nm("CZ"), 9},
    // 10: sp3 C
    {nm("ALA"), nm("CB"), 10}, {nm("ARG"), nm("CB"), 10}, {nm("ARG"), nm("CG"), 10}, {nm("ARG"), nm("CD"), 10},
    {nm("ASN"), nm("CB"), 10}, {nm("ASP"), nm("CB"), 10}, {nm("GLN"), nm("CB"), 10}, {nm("GLN"), nm("CG"), 10},
    {nm("GLU"), nm("CB"), 10}, {nm("GLU"), nm("CG"), 10}, {nm("HIS"), nm("CB"), 10},
    {nm("ILE"), nm("CB"), 10}, {nm("ILE"), nm("CD1"), 10}, {nm("ILE"), nm("CG1"), 10}, {nm("ILE"), nm("CG2"), 10},
    {nm("LEU"), nm("CB"), 10}, {nm("LEU"), nm("CD1"), 10}, {nm("LEU"), nm("CD2"), 10}, {nm("LEU"), nm("CG"), 10},
    {nm("LYS"), nm("CB"), 10}, {nm("LYS"), nm("CD"), 10}, {nm("LYS"), nm("CG"), 10}, {nm("LYS"), nm("CE"), 10},
    {nm("MET"), nm("CB"), 10}, {nm("MET"), nm("CE"), 10}, {nm("MET"), nm("CG"), 10},
    {nm("MSE"), nm("CB"), 10}, {nm("MSE"), nm("CE"), 10}, {nm("MSE"), nm("CG"), 10}, {nm("PHE"), nm("CB"), 10},
    {nm("PRO"), nm("CB"), 10}, {nm("PRO"), nm("CG"), 10}, {nm("PRO"), nm("CD"), 10}, {nm("SER"), nm("CB"), 10},
    {nm("THR"), nm("CG2"), 10}, {nm("TRP"), nm("CB"), 10}, {nm("TYR"), nm("CB"), 10},
    {nm("VAL"), nm("CB"), 10}, {nm("VAL"), nm("CG1"), 10}, {nm("VAL"), nm("CG2"), 10},
    {nm("ACE"), nm("CH3"), 10}, {nm("THR"), nm("CB"), 10}, {nm("CYS"), nm("CB"), 10},
};
constexpr int kTypedNameCount = sizeof(kTypedNames) / sizeof(TypedName);

// The table as an open-addressing hash of 256 slots (filled at compile time; load
// factor about 0.4), so that a lookup takes one or two probes instead of a walk
// over every entry.  A residue word of 0 marks an empty slot.
constexpr int kHashSlots = 256;
struct TypedHash {
    uint32_t res[kHashSlots], atom[kHashSlots];
    int type[kHashSlots];
};
constexpr uint32_t typed_hash(uint32_t res, uint32_t atom) {
    return ((res * 0x9E3779B1u) ^ (atom * 0x85EBCA77u)) >> 24;  // top 8 bits
}
constexpr TypedHash build_typed_hash() {
    TypedHash h{};
    for (int i = 0; i < kHashSlots; i++) h.type[i] = -1;
    for (int i = 0; i < kTypedNameCount; i++) {
        uint32_t k = typed_hash(kTypedNames[i].res, kTypedNames[i].atom);
        while (h.res[k] != 0) k = (k + 1) & (kHashSlots - 1);
        h.res[k] = kTypedNames[i].res;
        h.atom[k] = kTypedNames[i].atom;
        h.type[k] = kTypedNames[i].type;
    }
    return h;
}
static_assert(kTypedNameCount < kHashSlots / 2, "hash load factor");
__device__ const TypedHash g_typed_hash = build_typed_hash();

// Drop the space bytes of a name word (the reference erases whitespace from the
// atom name before comparing) and stop at the first NUL.
__device__ __forceinline__ uint32_t squeeze(uint32_t w) {
    uint32_t out = 0;
    int k = 0;
    for (int i = 0; i < 4; i++) {
        const uint32_t c = (w >> (8 * i)) & 0xffu;
        if (c == 0) break;
        if (c == ' ' || (c >= 9 && c <= 13)) continue;
        out |= c << (8 * k++);
    }
    return out;
}

// squeeze() without the byte loop when the name has no byte below '!' before its
// first NUL (the names Angles2Coords writes): the word up to that NUL.  Per byte,
// (w - 0x01) & ~w & 0x80 flags a NUL and (w - 0x21) & ~w & 0x80 a byte below 0x21;
// borrows only make false flags above a true one, so the lowest flag is exact.
__device__ __forceinline__ uint32_t squeeze_fast(uint32_t w) {
    const uint32_t nul = (w - 0x01010101u) & ~w & 0x80808080u;
    const uint32_t valid = nul ? (((nul & (0u - nul)) >> 7) - 1u) : 0xffffffffu;  // bytes before the first NUL
    const uint32_t low = (w - 0x21212121u) & ~w & 0x80808080u;
    if ((low & valid) == 0u) return w & valid;
    return squeeze(w);
}

// The 0-based type of an atom, or -1 for a name pair the reference rejects; h is the
// name hash (global memory, or a copy in shared memory).
__device__ __forceinline__ int atom_type(uint32_t res, uint32_t atom, const TypedHash &h) {
    atom = squeeze_fast(atom);
    res = res & 0x00ffffffu;  // the residue is its 3-letter code
    if (atom == nm("O")) return 5;  // not a terminal oxygen (the reference's call passes false)
    if (atom == nm("OXT") || atom == nm("OT2")) return 7;
    if (atom == nm("N")) return 1;
    if (atom == nm("C")) return 8;
    if (atom == nm("CA")) return 10;
    uint32_t k = typed_hash(res, atom);
    for (int probe = 0; probe < kHashSlots; probe++) {
        const uint32_t r = h.res[k];
        if (r == 0u) return -1;
        if (r == res && h.atom[k] == atom) return h.type[k];
        k = (k + 1) & (kHashSlots - 1);
    }
    return -1;
}
__device__ __forceinline__ int atom_type(uint32_t res, uint32_t atom) { return atom_type(res, atom, g_typed_hash); }

// Input rows hold in_stride atoms (coordinates and names); typed rows and atom
// indexes hold out_stride slots.  One CTA per chain, for chains too long for
// typed_fwd_seg_kernel's type cache: the scatter pass looks the types up again.
template <typename T>
__global__ void __launch_bounds__(kTypedThreads) typed_fwd_kernel(const T *coords, const uint32_t *res_names,
                                                                  const uint32_t *atom_names, const int *num_atoms,
                                                                  int in_stride, int out_stride, T *out,
                                                                  int *n_of_type, int *offsets, int *atom_index,
                                                                  WsHeader *hdr) {
    constexpr int NW = kTypedThreads / 32;
    __shared__ int s_count[kTypes], s_off[kTypes], s_base[kTypes];
    __shared__ int s_wc[kTypes][NW];
    const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int n = max(0, min(num_atoms[b], min(in_stride, out_stride)));
    const size_t row = (size_t)b * in_stride, orow = (size_t)b * out_stride;
    if (tid < kTypes) {
        s_count[tid] = 0;
        s_base[tid] = 0;
    }
    __syncthreads();
    for (int j = tid; j < n; j += kTypedThreads) {
        const int t = atom_type(res_names[row + j], atom_names[row + j]);
        if (t >= 0) atomicAdd(&s_count[t], 1);
        else atomicCAS(&hdr->status, 0u, (unsigned)TPL_ERR_ATOM_TYPE);
    }
    __syncthreads();
    if (tid == 0) {
        int o = 0;
        for (int k = 0; k < kTypes; k++) {
            s_off[k] = o;
            o += s_count[k];
        }
    }
    __syncthreads();
    if (tid < kTypes) {
        n_of_type[(size_t)b * kTypes + tid] = s_count[tid];
        offsets[(size_t)b * kTypes + tid] = s_off[tid];
    }
    const int ntyped = s_off[kTypes - 1] + s_count[kTypes - 1];
    // stable scatter, one tile of kTypedThreads atoms at a time
    for (int j0 = 0; j0 < n; j0 += kTypedThreads) {
        const int j = j0 + tid;
        // the atom's coordinates, loaded before the ranking so that the load overlaps it
        T x0 = T(0), x1 = T(0), x2 = T(0);
        if (j < n) {
            const T *src = coords + 3 * (row + j);
            x0 = src[0];
            x1 = src[1];
            x2 = src[2];
        }
        const int t = j < n ? atom_type(res_names[row + j], atom_names[row + j]) : -1;
        int rank = 0;
        const unsigned below = (1u << lane) - 1u;
#pragma unroll
        for (int k = 0; k < kTypes; k++) {
            const unsigned m = __ballot_sync(0xffffffffu, t == k);
            if (t == k) rank = __popc(m & below);
            if (lane == 0) s_wc[k][w] = __popc(m);
        }
        __syncthreads();
        if (t >= 0) {
            int before = s_base[t];
            for (int v = 0; v < w; v++) before += s_wc[t][v];
            const int slot = s_off[t] + before + rank;
            T *dst = out + 3 * (orow + slot);
            dst[0] = x0;
            dst[1] = x1;
            dst[2] = x2;
            atom_index[orow + slot] = j;
        }
        __syncthreads();
        if (tid < kTypes)
            for (int v = 0; v < NW; v++) s_base[tid] += s_wc[tid][v];
        __syncthreads();
    }
    // slots past the typed atoms are zero, as in the reference's zero-filled outputs
    for (int s = ntyped + tid; s < out_stride; s += kTypedThreads) {
        T *dst = out + 3 * (orow + s);
        dst[0] = dst[1] = dst[2] = T(0);
        atom_index[orow + s] = 0;
    }
}

// The same regrouping by four warps per chain with three CTA barriers in all: each
// warp takes a quarter of the chain's 32-atom tiles.  Pass 1 types the atoms of the
// warp's tiles and counts them per type (per tile, __match_any_sync groups the lanes
// of each type and the lowest of them adds their number); after a barrier every warp
// knows where its atoms of each type start (the type's offset plus the counts of the
// earlier warps), and pass 2 scatters its tiles in order: an atom's slot is its
// type's next free slot plus its rank among the tile's atoms of that type, so the
// order within a type is the input order.  Both passes load kTypedUnroll tiles
// before working on them, so that a warp has several tiles' loads in flight.  Pass
// 1's types stay in shared memory (in_stride bytes) for pass 2, and the name hash is
// copied there too.  GB300, 4096 chains of U{50..500} residues: 0.158 -> 0.145 ms
// against typed_fwd_kernel, which keeps chains of more than kTypeCacheMax atoms.
constexpr int kTypedWarps = 4;  // warps per chain
constexpr int kTypedUnroll = 4;

template <typename T>
__global__ void __launch_bounds__(32 * kTypedWarps) typed_fwd_seg_kernel(
    const T *__restrict__ coords, const uint32_t *__restrict__ res_names, const uint32_t *__restrict__ atom_names,
    const int *__restrict__ num_atoms, int in_stride, int out_stride, T *__restrict__ out,
    int *__restrict__ n_of_type, int *__restrict__ offsets, int *__restrict__ atom_index, WsHeader *hdr) {
    extern __shared__ signed char s_ty[];
    __shared__ int s_cnt[kTypedWarps][kTypes];
    __shared__ int s_ntyped;
    __shared__ TypedHash s_hash;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, b = blockIdx.x;
    {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(&g_typed_hash);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&s_hash);
        for (int i = threadIdx.x; i < (int)(sizeof(TypedHash) / 4); i += 32 * kTypedWarps) dst[i] = src[i];
    }
    const int n = max(0, min(num_atoms[b], min(in_stride, out_stride)));
    const size_t row = (size_t)b * in_stride, orow = (size_t)b * out_stride;
    const uint32_t *rn = res_names + row, *an = atom_names + row;
    const unsigned below = (1u << lane) - 1u;
    const int ntiles = (n + 31) >> 5, per = (ntiles + kTypedWarps - 1) / kTypedWarps;
    const int t0 = min(ntiles, w * per), t1 = min(ntiles, t0 + per);

    if (lane < kTypes) s_cnt[w][lane] = 0;
    __syncthreads();  // the hash copy and the zeroed counts
    bool bad = false;
    for (int tb = t0; tb < t1; tb += kTypedUnroll) {
        uint32_t r[kTypedUnroll], a[kTypedUnroll];
#pragma unroll
        for (int u = 0; u < kTypedUnroll; u++) {
            const int j = 32 * (tb + u) + lane;
            const bool in = tb + u < t1 && j < n;
            r[u] = in ? rn[j] : 0u;
            a[u] = in ? an[j] : 0u;
        }
#pragma unroll
        for (int u = 0; u < kTypedUnroll; u++) {
            const int j = 32 * (tb + u) + lane;
            const bool in = tb + u < t1 && j < n;
            const int t = in ? atom_type(r[u], a[u], s_hash) : -2;  // -1: a name pair the reference rejects
            if (in) s_ty[j] = (signed char)t;
            bad |= t == -1;
            // the lanes of each type: the lowest of them adds their number
            const unsigned m = __match_any_sync(0xffffffffu, t);
            if (t >= 0 && (m & below) == 0u) s_cnt[w][t] += __popc(m);
            __syncwarp();
        }
    }
    if (bad) atomicCAS(&hdr->status, 0u, (unsigned)TPL_ERR_ATOM_TYPE);
    __syncthreads();
    // lane k < kTypes: the type's total, its offset, and this warp's first slot of it
    int tot = 0, before = 0;
    if (lane < kTypes)
#pragma unroll
        for (int v = 0; v < kTypedWarps; v++) {
            const int c = s_cnt[v][lane];
            tot += c;
            before += v < w ? c : 0;
        }
    int inc = tot;
#pragma unroll
    for (int off = 1; off < 16; off <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= off) inc += v;
    }
    const int type_off = inc - tot;
    if (w == 0 && lane < kTypes) {
        n_of_type[(size_t)b * kTypes + lane] = tot;
        offsets[(size_t)b * kTypes + lane] = type_off;
    }
    if (w == 0 && lane == kTypes - 1) s_ntyped = inc;
    __syncthreads();  // every warp has read the counts
    int *s_next = s_cnt[w];  // reused: this warp's next free slot of each type
    if (lane < kTypes) s_next[lane] = type_off + before;
    __syncwarp();

    for (int tb = t0; tb < t1; tb += kTypedUnroll) {
        T x[kTypedUnroll][3];
        int ty[kTypedUnroll];
#pragma unroll
        for (int u = 0; u < kTypedUnroll; u++) {
            const int j = 32 * (tb + u) + lane;
            const bool in = tb + u < t1 && j < n;
            const T *src = coords + 3 * (row + j);
#pragma unroll
            for (int c = 0; c < 3; c++) x[u][c] = in ? src[c] : T(0);
            ty[u] = in ? (int)s_ty[j] : -2;
        }
#pragma unroll
        for (int u = 0; u < kTypedUnroll; u++) {
            const int j = 32 * (tb + u) + lane, t = ty[u];
            const unsigned m = __match_any_sync(0xffffffffu, t);
            if (t >= 0) {
                const int slot = s_next[t] + __popc(m & below);
                T *dst = out + 3 * (orow + slot);
                dst[0] = x[u][0];
                dst[1] = x[u][1];
                dst[2] = x[u][2];
                atom_index[orow + slot] = j;
            }
            __syncwarp();
            if (t >= 0 && (m & below) == 0u) s_next[t] += __popc(m);
            __syncwarp();
        }
    }
    __syncthreads();
    // slots past the typed atoms are zero, as in the reference's zero-filled outputs
    const int ntyped = s_ntyped;
    T *o = out + 3 * orow;
    for (int e = 3 * ntyped + threadIdx.x; e < 3 * out_stride; e += 32 * kTypedWarps) o[e] = T(0);
    for (int q = ntyped + threadIdx.x; q < out_stride; q += 32 * kTypedWarps) atom_index[orow + q] = 0;
}

// grad_flat[atom_index[s]] = grad_typed[s] for the typed slots, zero elsewhere;
// grad_flat rows hold in_stride atoms, grad_typed rows out_stride slots.
template <typename T>
__global__ void __launch_bounds__(kTypedThreads) typed_bwd_kernel(const T *grad_typed, T *grad_flat,
                                                                  const int *n_of_type, const int *atom_index,
                                                                  int in_stride, int out_stride) {
    const int b = blockIdx.x, tid = threadIdx.x;
    const size_t row = (size_t)b * in_stride, orow = (size_t)b * out_stride;
    int ntyped = 0;
    for (int k = 0; k < kTypes; k++) ntyped += n_of_type[(size_t)b * kTypes + k];
    ntyped = max(0, min(ntyped, out_stride));
    for (int e = tid; e < 3 * in_stride; e += kTypedThreads) grad_flat[3 * row + e] = T(0);
    __syncthreads();
    for (int s = tid; s < ntyped; s += kTypedThreads) {
        const int j = atom_index[orow + s];
        if (j < 0 || j >= in_stride) continue;
        const T *src = grad_typed + 3 * (orow + s);
        T *dst = grad_flat + 3 * (row + j);
        dst[0] = src[0];
        dst[1] = src[1];
        dst[2] = src[2];
    }
}

// The same with every flat row written once, in order: the slot of each atom is
// first inverted into shared memory (in_stride ints), then grad_flat[j] is gathered
// from grad_typed[slot(j)] with coalesced stores (zero for atoms without a slot).
template <typename T>
__global__ void __launch_bounds__(kTypedThreads) typed_bwd_gather_kernel(const T *__restrict__ grad_typed,
                                                                         T *__restrict__ grad_flat,
                                                                         const int *__restrict__ n_of_type,
                                                                         const int *__restrict__ atom_index,
                                                                         int in_stride, int out_stride) {
    extern __shared__ int s_slot[];
    const int b = blockIdx.x, tid = threadIdx.x;
    const size_t row = (size_t)b * in_stride, orow = (size_t)b * out_stride;
    int ntyped = 0;
    for (int k = 0; k < kTypes; k++) ntyped += n_of_type[(size_t)b * kTypes + k];
    ntyped = max(0, min(ntyped, out_stride));
    for (int j = tid; j < in_stride; j += kTypedThreads) s_slot[j] = -1;
    __syncthreads();
    for (int s = tid; s < ntyped; s += kTypedThreads) {
        const int j = atom_index[orow + s];
        if (j >= 0 && j < in_stride) s_slot[j] = s;
    }
    __syncthreads();
    const T *src = grad_typed + 3 * orow;
    T *dst = grad_flat + 3 * row;
    // eight gathers per thread in flight before their stores (GB300, 4096 chains of
    // 2300 atoms: 0.086 / 0.074 / 0.070 / 0.075 ms with 2 / 4 / 8 / 16)
    constexpr int U = 8;
    const int ne = 3 * in_stride;
    for (int e0 = tid; e0 < ne; e0 += U * kTypedThreads) {
        T v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int e = e0 + u * kTypedThreads;
            v[u] = T(0);
            if (e < ne) {
                const int j = e / 3, c = e - 3 * j;
                const int s = s_slot[j];
                if (s >= 0) v[u] = src[3 * s + c];
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int e = e0 + u * kTypedThreads;
            if (e < ne) dst[e] = v[u];
        }
    }
}

constexpr int kGatherMaxAtoms = 16384;  // 64 KB of slots per CTA
constexpr int kTypeCacheMax = 32768;    // typed_fwd_seg_kernel's type cache: one byte per input atom

}  // namespace

int typed_forward(bool f64, const void *coords, const uint32_t *res_names, const uint32_t *atom_names,
                  const int *num_atoms, int B, int in_stride, int out_stride, void *out, int *n_of_type, int *offsets,
                  int *atom_index, void *ws, cudaStream_t st) {
    if (B == 0) return TPL_OK;
    WsHeader *hdr = reinterpret_cast<WsHeader *>(ws);
    if (in_stride <= kTypeCacheMax) {  // four warps per chain, types cached in shared memory
        const size_t smem = (size_t)in_stride;
        auto launch_s = [&](auto kernel, auto *out_t, auto *coords_t) -> int {
            if (smem > 48 * 1024 && !set_max_dynamic_smem(reinterpret_cast<const void *>(kernel), (int)smem))
                return TPL_ERR_LAUNCH;
            kernel<<<B, 32 * kTypedWarps, smem, st>>>(coords_t, res_names, atom_names, num_atoms, in_stride,
                                                       out_stride, out_t, n_of_type, offsets, atom_index, hdr);
            return cudaGetLastError() == cudaSuccess ? (int)TPL_OK : (int)TPL_ERR_LAUNCH;
        };
        if (f64)
            return launch_s(typed_fwd_seg_kernel<double>, static_cast<double *>(out),
                            static_cast<const double *>(coords));
        return launch_s(typed_fwd_seg_kernel<float>, static_cast<float *>(out), static_cast<const float *>(coords));
    }
    // longer chains: one CTA per chain, the types looked up again in the scatter pass
    if (f64)
        typed_fwd_kernel<double><<<B, kTypedThreads, 0, st>>>(
            static_cast<const double *>(coords), res_names, atom_names, num_atoms, in_stride, out_stride,
            static_cast<double *>(out), n_of_type, offsets, atom_index, hdr);
    else
        typed_fwd_kernel<float><<<B, kTypedThreads, 0, st>>>(
            static_cast<const float *>(coords), res_names, atom_names, num_atoms, in_stride, out_stride,
            static_cast<float *>(out), n_of_type, offsets, atom_index, hdr);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

int typed_backward(bool f64, const void *grad_typed, void *grad_flat, const int *n_of_type, const int *atom_index,
                   int B, int in_stride, int out_stride, cudaStream_t st) {
    if (B == 0) return TPL_OK;
    if (in_stride <= kGatherMaxAtoms) {
        const int smem = in_stride * (int)sizeof(int);
        if (f64) {
            auto k = typed_bwd_gather_kernel<double>;
            if (!set_max_dynamic_smem(reinterpret_cast<const void *>(k), smem))
                return TPL_ERR_LAUNCH;
            k<<<B, kTypedThreads, smem, st>>>(static_cast<const double *>(grad_typed), static_cast<double *>(grad_flat),
                                              n_of_type, atom_index, in_stride, out_stride);
        } else {
            auto k = typed_bwd_gather_kernel<float>;
            if (!set_max_dynamic_smem(reinterpret_cast<const void *>(k), smem))
                return TPL_ERR_LAUNCH;
            k<<<B, kTypedThreads, smem, st>>>(static_cast<const float *>(grad_typed), static_cast<float *>(grad_flat),
                                              n_of_type, atom_index, in_stride, out_stride);
        }
        return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
    }
    if (f64)
        typed_bwd_kernel<double><<<B, kTypedThreads, 0, st>>>(static_cast<const double *>(grad_typed),
                                                             static_cast<double *>(grad_flat), n_of_type, atom_index,
                                                             in_stride, out_stride);
    else
        typed_bwd_kernel<float><<<B, kTypedThreads, 0, st>>>(static_cast<const float *>(grad_typed),
                                                            static_cast<float *>(grad_flat), n_of_type, atom_index,
                                                            in_stride, out_stride);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

}  // namespace tpl
