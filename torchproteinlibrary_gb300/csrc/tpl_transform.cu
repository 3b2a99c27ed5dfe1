// CoordsTransform on the GPU (sm_103a): translate, rotate, centre and bounding box
// of batched coordinate rows [B, 3 * atoms_stride]; atoms at and past num_atoms[b]
// are written as zeros, as the reference's zero-initialised outputs leave them.
//
// Reference: Layers/FullAtomModel/TransformCUDAKernels.cu:4-107 launches one block
// per atom index with one thread per chain (<<<atoms_stride, batch_size>>>, so
// batch_size <= 1024) and sums each centroid serially in one thread; the bounding
// box runs on the CPU (Layers/FullAtomModel/CoordsTransform/
// coordsTransform_interface.cpp:175-200, Math/nUtil.cpp:27-57).  Here the
// elementwise transforms are flat, coalesced, 16-byte-vectorised passes over the
// whole batch (HBM-bound: 2 x 12 B per atom in FP32), and centroid and box are
// block reductions, one CTA per chain.
#include <cfloat>
#include <cmath>

#include "tpl_internal.h"

namespace tpl {
namespace {

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using type = float4;
    static constexpr int n = 4;
};
template <>
struct Vec16<double> {
    using type = double2;
    static constexpr int n = 2;
};

constexpr int kUnroll = 4;  // vectors in flight per thread in the elementwise passes

// 16-byte streaming load / store (data touched once).
template <typename T>
__device__ __forceinline__ void load16(const T *p, T (&v)[Vec16<T>::n]) {
    const typename Vec16<T>::type x = __ldcs(reinterpret_cast<const typename Vec16<T>::type *>(p));
    memcpy(v, &x, sizeof(x));
}
template <typename T>
__device__ __forceinline__ void store16(T *p, const T (&v)[Vec16<T>::n]) {
    typename Vec16<T>::type x;
    memcpy(&x, v, sizeof(x));
    __stcs(reinterpret_cast<typename Vec16<T>::type *>(p), x);
}

// out[b, e] = (in ? in[b, e] : 0) + (add ? add[b, e % 3] * (scale_by_count ? 1 / n_b : 1) : 0)
// for e < 3 n_b, 0 after.  Covers translate (add = T), its backward (add = null),
// and the centre's backward (in = null, add = dL/dcentre, scaled by 1 / n_b).
// Grid: y over rows (strided), x over pieces of a row, so no thread divides by the
// row length; VEC: 16-byte vectors inside a row (3 * atoms_stride a multiple of the
// vector width and 16-byte-aligned rows).
struct ShiftArgs {
    const void *in;
    void *out;
    const void *add;
    const int *num_atoms;
    int B;
    int row;  // 3 * atoms_stride
    int scale_by_count;
};

template <typename T, bool VEC>
__global__ void __launch_bounds__(256) shift_kernel(ShiftArgs a) {
    constexpr int N = VEC ? Vec16<T>::n : 1;
    const T *in = static_cast<const T *>(a.in);
    T *out = static_cast<T *>(a.out);
    const T *add = static_cast<const T *>(a.add);
    const int nv = a.row / N;  // vectors per row
    for (int b = blockIdx.y; b < a.B; b += gridDim.y) {
        const int n = max(0, min(a.num_atoms[b], a.row / 3)), n3 = 3 * n;
        T t[3] = {T(0), T(0), T(0)};
        if (add)
            for (int k = 0; k < 3; k++) {
                t[k] = add[3 * (size_t)b + k];
                if (a.scale_by_count && n > 0) t[k] = t[k] / T(n);
            }
        const size_t base = (size_t)b * a.row;
        // kUnroll independent vectors per thread and step: loads issued before use
        const int step = gridDim.x * blockDim.x;
        for (int v0 = blockIdx.x * blockDim.x + threadIdx.x; v0 < nv; v0 += kUnroll * step) {
            T x[kUnroll][Vec16<T>::n];
#pragma unroll
            for (int u = 0; u < kUnroll; u++) {
                const int v = v0 + u * step;
                if (v >= nv) continue;
                if (VEC) {
                    if (in) load16(in + base + (size_t)v * N, x[u]);
                    else
                        for (int k = 0; k < N; k++) x[u][k] = T(0);
                } else {
                    x[u][0] = in ? __ldcs(in + base + v) : T(0);
                }
            }
#pragma unroll
            for (int u = 0; u < kUnroll; u++) {
                const int v = v0 + u * step;
                if (v >= nv) continue;
#pragma unroll
                for (int k = 0; k < N; k++) {
                    const int e = v * N + k;
                    x[u][k] = e < n3 ? x[u][k] + t[e % 3] : T(0);
                }
                if (VEC) store16(out + base + (size_t)v * N, x[u]);
                else __stcs(out + base + v, x[u][0]);
            }
        }
    }
}

// out[b, atom] = R_b x (or R_b^T x) for atom < n_b, 0 after; R row-major [B, 3, 3].
// Grid: y over rows (strided), x over atoms of a row.
template <typename T>
__global__ void __launch_bounds__(256) rotate_kernel(const T *in, T *out, const T *R, const int *num_atoms, int B,
                                                     int stride, int transpose) {
    for (int b = blockIdx.y; b < B; b += gridDim.y) {
        const int n = num_atoms[b];
        T m[9];
        for (int k = 0; k < 9; k++) m[k] = R[9 * (size_t)b + (transpose ? 3 * (k % 3) + k / 3 : k)];
        const T *x = in + (size_t)b * 3 * stride;
        T *y = out + (size_t)b * 3 * stride;
        const int step = gridDim.x * blockDim.x;
        for (int i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < stride; i0 += kUnroll * step) {
            T v[kUnroll][3];
#pragma unroll
            for (int u = 0; u < kUnroll; u++) {  // loads of kUnroll atoms in flight
                const int i = i0 + u * step;
                if (i < min(n, stride))
                    for (int k = 0; k < 3; k++) v[u][k] = __ldcs(x + 3 * i + k);
            }
#pragma unroll
            for (int u = 0; u < kUnroll; u++) {
                const int i = i0 + u * step;
                if (i >= stride) continue;
                T r0 = T(0), r1 = T(0), r2 = T(0);
                if (i < n) {
                    const T x0 = v[u][0], x1 = v[u][1], x2 = v[u][2];
                    r0 = m[0] * x0 + m[1] * x1 + m[2] * x2;
                    r1 = m[3] * x0 + m[4] * x1 + m[5] * x2;
                    r2 = m[6] * x0 + m[7] * x1 + m[8] * x2;
                }
                __stcs(y + 3 * i, r0);
                __stcs(y + 3 * i + 1, r1);
                __stcs(y + 3 * i + 2, r2);
            }
        }
    }
}

constexpr int kReduceThreads = 256;

template <typename R, typename Op>
__device__ __forceinline__ R block_reduce(R v, Op op, R *s_warp) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, off));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) s_warp[w] = v;
    __syncthreads();
    R r = s_warp[0];
    for (int k = 1; k < kReduceThreads / 32; k++) r = op(r, s_warp[k]);
    __syncthreads();  // s_warp is reused by the next reduction
    return r;
}

// Centroid of the first n_b atoms of chain b = blockIdx.x (FP64 accumulation);
// 0 for an empty chain.
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) center_kernel(const T *in, T *center, const int *num_atoms,
                                                                int stride, int vec) {
    constexpr int NW = kReduceThreads / 32;
    __shared__ double s_warp[NW][3];
    const int b = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n = min(num_atoms[b], stride);  // a count past the row is clamped to it
    const T *x = in + (size_t)b * 3 * stride;
    // offsets from the chain's first atom, summed in the coordinate type per thread and
    // per warp and in FP64 across the warps: the offsets stay of the chain's own extent
    // wherever the chain sits, and GB300's FP64 rate is a small fraction of its FP32 rate
    const T p0 = n > 0 ? x[0] : T(0), p1 = n > 0 ? x[1] : T(0), p2 = n > 0 ? x[2] : T(0);
    T s[3] = {T(0), T(0), T(0)};
    int i0 = 0;  // first atom of the scalar loop
    if constexpr (sizeof(T) == 4) {
        if (vec) {  // 16-byte rows: a thread reads 4 atoms as three float4s, two groups in flight
            const float4 *x4 = reinterpret_cast<const float4 *>(x);
            const int ng = n >> 2;
#pragma unroll 2
            for (int g = threadIdx.x; g < ng; g += kReduceThreads) {
                const float4 a = x4[3 * g], b = x4[3 * g + 1], c = x4[3 * g + 2];
                s[0] += ((a.x - p0) + (a.w - p0)) + ((b.z - p0) + (c.y - p0));
                s[1] += ((a.y - p1) + (b.x - p1)) + ((b.w - p1) + (c.z - p1));
                s[2] += ((a.z - p2) + (b.y - p2)) + ((c.x - p2) + (c.w - p2));
            }
            i0 = 4 * ng;
        }
    }
    for (int i = i0 + threadIdx.x; i < n; i += kReduceThreads) {
        s[0] += x[3 * i] - p0;
        s[1] += x[3 * i + 1] - p1;
        s[2] += x[3 * i + 2] - p2;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int c = 0; c < 3; c++) s[c] += __shfl_xor_sync(0xffffffffu, s[c], off);
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < 3; c++) s_warp[w][c] = (double)s[c];
    __syncthreads();
    if (threadIdx.x < 3) {
        const int c = threadIdx.x;
        double t = 0.0;
#pragma unroll
        for (int q = 0; q < NW; q++) t += s_warp[q][c];
        const double pc = c == 0 ? (double)p0 : (c == 1 ? (double)p1 : (double)p2);
        center[3 * b + c] = n > 0 ? (T)(pc + t / n) : T(0);
    }
}

// Axis-aligned bounding box of the first n_b atoms of chain b: lo = min, hi = max
// per coordinate (+inf / -inf for an empty chain, as Math/nUtil.cpp:27-57).
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) bbox_kernel(const T *in, T *lo, T *hi, const int *num_atoms,
                                                              int stride) {
    __shared__ T s_warp[kReduceThreads / 32];
    const int b = blockIdx.x;
    const int n = min(num_atoms[b], stride);
    const T *x = in + (size_t)b * 3 * stride;
    const T inf = (T)INFINITY;
    T mn[3] = {inf, inf, inf}, mx[3] = {-inf, -inf, -inf};
    for (int i = threadIdx.x; i < n; i += kReduceThreads)
        for (int c = 0; c < 3; c++) {
            const T v = x[3 * i + c];
            mn[c] = v < mn[c] ? v : mn[c];
            mx[c] = v > mx[c] ? v : mx[c];
        }
    auto fmin_ = [](T p, T q) { return q < p ? q : p; };
    auto fmax_ = [](T p, T q) { return q > p ? q : p; };
    for (int c = 0; c < 3; c++) {
        const T a = block_reduce<T>(mn[c], fmin_, s_warp);
        const T z = block_reduce<T>(mx[c], fmax_, s_warp);
        if (threadIdx.x == 0) {
            lo[3 * b + c] = a;
            hi[3 * b + c] = z;
        }
    }
}

// Row-major 2-D grid: x covers one row's items in 256-thread blocks, y the rows
// (capped; the kernels stride over the remaining rows).
dim3 grid_rows(int B, long long items_per_row) {
    long long gx = (items_per_row + 255) / 256;
    if (gx < 1) gx = 1;
    if (gx > 65535) gx = 65535;
    int gy = B < 1 ? 1 : B;
    if (gy > 65535) gy = 65535;
    return dim3((unsigned)gx, (unsigned)gy, 1);
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace

template <typename T>
int coords_shift(const T *in, T *out, const T *add, int scale_by_count, const int *num_atoms, int B, int stride,
                 cudaStream_t st) {
    if (B == 0 || stride == 0) return TPL_OK;
    ShiftArgs a{in, out, add, num_atoms, B, 3 * stride, scale_by_count};
    // 16-byte vectors when every row starts 16-byte aligned and holds whole vectors
    const bool vec = aligned16(out) && (!in || aligned16(in)) && (a.row % Vec16<T>::n == 0) &&
                     ((a.row * sizeof(T)) % 16 == 0);
    const int n = vec ? Vec16<T>::n : 1;
    if (vec) {
        shift_kernel<T, true><<<grid_rows(B, (a.row / n + kUnroll - 1) / kUnroll), 256, 0, st>>>(a);
    } else {
        shift_kernel<T, false><<<grid_rows(B, (a.row + kUnroll - 1) / kUnroll), 256, 0, st>>>(a);
    }
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

template <typename T>
int coords_rotate(const T *in, T *out, const T *R, int transpose, const int *num_atoms, int B, int stride,
                  cudaStream_t st) {
    if (B == 0 || stride == 0) return TPL_OK;
    rotate_kernel<T><<<grid_rows(B, (stride + kUnroll - 1) / kUnroll), 256, 0, st>>>(in, out, R, num_atoms, B, stride,
                                                                                   transpose);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

template <typename T>
int coords_center(const T *in, T *center, const int *num_atoms, int B, int stride, cudaStream_t st) {
    if (B == 0) return TPL_OK;
    const int vec = stride % 4 == 0 && (reinterpret_cast<uintptr_t>(in) & 15u) == 0;
    center_kernel<T><<<B, kReduceThreads, 0, st>>>(in, center, num_atoms, stride, vec);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

template <typename T>
int coords_bbox(const T *in, T *lo, T *hi, const int *num_atoms, int B, int stride, cudaStream_t st) {
    if (B == 0) return TPL_OK;
    bbox_kernel<T><<<B, kReduceThreads, 0, st>>>(in, lo, hi, num_atoms, stride);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

template int coords_shift<float>(const float *, float *, const float *, int, const int *, int, int, cudaStream_t);
template int coords_shift<double>(const double *, double *, const double *, int, const int *, int, int, cudaStream_t);
template int coords_rotate<float>(const float *, float *, const float *, int, const int *, int, int, cudaStream_t);
template int coords_rotate<double>(const double *, double *, const double *, int, const int *, int, int, cudaStream_t);
template int coords_center<float>(const float *, float *, const int *, int, int, cudaStream_t);
template int coords_center<double>(const double *, double *, const int *, int, int, cudaStream_t);
template int coords_bbox<float>(const float *, float *, float *, const int *, int, int, cudaStream_t);
template int coords_bbox<double>(const double *, double *, double *, const int *, int, int, cudaStream_t);

}  // namespace tpl
