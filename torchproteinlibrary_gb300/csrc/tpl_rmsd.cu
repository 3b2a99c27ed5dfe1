// Coords2RMSD on the GPU: least RMSD after optimal superposition, with its
// gradient.  The reference (Layers/RMSD/Coords2RMSD/coords2rmsd_interface.cpp:52-111,
// RMSDKernels.cu:5-57) builds the 3x3 correlation on the GPU with one thread per
// matrix entry, copies the 4x4 quaternion matrix to the CPU for an eigen solve per
// chain, computes sum |x|^2 with single-thread kernels, and backpropagates with a
// Python loop of .item() calls (TorchProteinLibrary/RMSD/Coords2RMSD/Coords2RMSD.py:40-62).
//
// Here one CTA per chain does everything in one launch: optional centring, the
// correlation R_ab = sum x_a y_b and R2 = sum |x|^2 + |y|^2 (sums in the coordinate
// type per thread and per warp, in FP64 across the warps: GB300's FP64 rate is a
// small fraction of its FP32 rate), the 4x4 matrix T (same layout as the
// reference), its largest eigenpair by the characteristic-polynomial method on one
// warp (key_eigen_warp: lane-parallel coefficients, FP32 Newton polished in FP64;
// for float32 inputs the eigenvector, U and rmsd then in FP32: GB300, 256 chains of
// about 2300 atoms, 18.6 -> 15.8 us per forward), U from the unit quaternion, UT = U^T and
// rmsd = sqrt((R2 - 2 |lambda_max| + 1e-10) / N).  The backward is one launch with
// one thread per atom (chains on x, blocks of atoms on y):
// dL/dx_i = g (x_i - UT y_i) / (rmsd N) on the centred coordinates.
#include <cmath>

#include "tpl_common.cuh"
#include "tpl_internal.h"

namespace tpl {

constexpr int kRmsdThreads = 256;

template <typename T>
struct RmsdArgs {
    const T *src;
    const T *dst;
    const int *num_atoms;
    int atoms_stride;
    int center;
    T *rmsd;
    T *ut;              // [B, 9]
    double *centroids;  // [B, 6] (src, dst), may be null
    const T *grad_rmsd;
    T *grad_src;
    WsHeader *hdr;
};

constexpr int kRmsdWarps = kRmsdThreads / 32;

// Block sums of NV per-thread values: in the coordinate type within each warp, then
// in FP64 across the warps on one lane per value, so that the FP64 work is NV x
// warps additions rather than a shuffle tree per value on every thread (GB300's
// FP64 rate is a small fraction of its FP32 rate).  Every thread returns with the
// sums in s_out.
template <typename T, int NV>
__device__ __forceinline__ void block_sums(T (&v)[NV], double *s_red, double *s_out) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] += __shfl_xor_sync(0xffffffffu, v[k], off);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) s_red[w * NV + k] = (double)v[k];
    __syncthreads();
    if (threadIdx.x < NV) {
        double r = 0.0;
#pragma unroll
        for (int i = 0; i < kRmsdWarps; i++) r += s_red[i * NV + threadIdx.x];
        s_out[threadIdx.x] = r;
    }
    __syncthreads();
}

__device__ __forceinline__ double det3(double a, double b, double c, double d, double e, double f, double g, double h,
                                       double k) {
    return a * (e * k - f * h) - b * (d * k - f * g) + c * (d * h - e * g);
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Largest eigenpair of the symmetric 4x4 K by cyclic Jacobi rotations in FP64, on one
// thread: the fallback of key_eigen_warp for a near-multiple largest root (collinear
// or otherwise degenerate structures, two-atom chains), where Newton on the quartic
// converges only linearly and stalls at about the square root of the rounding error.
// Rotation (p, r) with t = sgn(theta) / (|theta| + sqrt(theta^2 + 1)),
// theta = (a_rr - a_pp) / (2 a_pr), zeroes a_pr (A' = J^T A J, V' = V J).  a and v
// are 16 doubles of shared scratch each, so that the rare path adds no registers to
// the kernel.
__device__ __forceinline__ void jacobi_top_eigenpair(const double *K, double *a, double *v, double &lam,
                                                  double (&q)[4]) {
    for (int i = 0; i < 16; i++) {
        a[i] = K[i];
        v[i] = (i % 5 == 0) ? 1.0 : 0.0;
    }
    for (int sweep = 0; sweep < 16; sweep++) {
        double off = 0.0, dg = 0.0;
        for (int i = 0; i < 4; i++) {
            dg += a[5 * i] * a[5 * i];
            for (int j = i + 1; j < 4; j++) off += a[4 * i + j] * a[4 * i + j];
        }
        if (!(off > 1e-30 * (dg + off))) break;
        for (int p = 0; p < 3; p++)
            for (int r = p + 1; r < 4; r++) {
                const double apr = a[4 * p + r];
                if (!(fabs(apr) > 1e-300)) continue;
                const double theta = (a[5 * r] - a[5 * p]) / (2.0 * apr);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < 4; k++) {  // A J
                    const double akp = a[4 * k + p], akr = a[4 * k + r];
                    a[4 * k + p] = c * akp - sn * akr;
                    a[4 * k + r] = sn * akp + c * akr;
                }
                for (int k = 0; k < 4; k++) {  // J^T (A J)
                    const double apk = a[4 * p + k], ark = a[4 * r + k];
                    a[4 * p + k] = c * apk - sn * ark;
                    a[4 * r + k] = sn * apk + c * ark;
                }
                for (int k = 0; k < 4; k++) {  // V J
                    const double vkp = v[4 * k + p], vkr = v[4 * k + r];
                    v[4 * k + p] = c * vkp - sn * vkr;
                    v[4 * k + r] = sn * vkp + c * vkr;
                }
            }
    }
    int best = 0;
    for (int i = 1; i < 4; i++)
        if (a[5 * i] > a[5 * best]) best = i;
    lam = a[5 * best];
    for (int k = 0; k < 4; k++) q[k] = v[4 * k + best];
}

// The eigenvector for lam of key_eigen_warp<true>, in FP32: the largest row of the
// cofactor matrix of K / e0 - (lam / e0) I (entries of order one), one cofactor per
// lane.  The root itself stays FP64: when the top two eigenvalues nearly meet it is
// ill-conditioned, and an all-FP32 solve moved it by up to 3e-5 relative (a 2.4e-4
// gradient error on one of 256 training-step chains), where this form matches the
// FP64 solve to 1e-5 of the largest gradient.
__device__ void eigvec_f32(const double *sK, double e0, double l, double (&q)[4]) {
    const int lane = threadIdx.x & 31;
    const float ief = e0 > 0.0 ? 1.f / (float)e0 : 0.f, sf = (float)l * ief;
    float cf = 0.f;
    if (lane < 16) {
        const int i = lane >> 2, j = lane & 3;
        float m[9];
        int t = 0;
#pragma unroll
        for (int r = 0; r < 4; r++)
            if (r != i)
#pragma unroll
                for (int c = 0; c < 4; c++)
                    if (c != j) m[t++] = (float)sK[4 * r + c] * ief - (r == c ? sf : 0.f);
        cf = fmaf(m[0], fmaf(m[4], m[8], -m[5] * m[7]),
                  fmaf(-m[1], fmaf(m[3], m[8], -m[5] * m[6]), m[2] * fmaf(m[3], m[7], -m[4] * m[6])));
        if ((i + j) & 1) cf = -cf;
    }
    float nrm = cf * cf;
    nrm += __shfl_xor_sync(0xffffffffu, nrm, 1);
    nrm += __shfl_xor_sync(0xffffffffu, nrm, 2);
    int best = 0;
    float bn = __shfl_sync(0xffffffffu, nrm, 0);
    for (int i = 1; i < 4; i++) {
        const float v = __shfl_sync(0xffffffffu, nrm, 4 * i);
        if (v > bn) {
            bn = v;
            best = i;
        }
    }
    const bool ok = bn > 1e-30f;
    const float inv = ok ? rsqrtf(bn) : 0.f;
    for (int k = 0; k < 4; k++) q[k] = (double)(__shfl_sync(0xffffffffu, cf, 4 * best + k) * inv);
    if (!ok) {
        q[0] = 1.0;
        q[1] = q[2] = q[3] = 0.0;
    }
}

// Largest eigenpair of the 4x4 key matrix K (symmetric and traceless, row-major in
// shared memory) by its characteristic polynomial, as in Theobald's
// quaternion-characteristic-polynomial method (Acta Cryst. A61, 478, 2005):
// det(K - l I) = l^4 + c2 l^2 + c1 l + c0 with, by Newton's identities for a
// traceless matrix, c2 = -tr(K^2)/2, c1 = -tr(K^3)/3, c0 = det K.
//   * tr(K^2), tr(K^3) and det K are spread over the lanes: entry (i, j) of K^2 on
//     lane 4 i + j, the cofactor expansion of det K along row 0 on lanes 16-19.
//   * Newton's method from e0 >= l_max (e0 = (sum |x|^2 + |y|^2) / 2) descends
//     monotonically to the largest root.  It runs in FP32 on s = l / e0, whose
//     coefficients are of order one, and is then polished by three FP64 Newton
//     steps whose quotient uses an FP32 reciprocal (each step gains about seven
//     digits), so that only a handful of FP64 operations remain.
//   * The eigenvector is the largest row of the cofactor matrix of K - l_max I
//     (rank one for a simple root), one cofactor per lane.
//   * F32_VEC (float32 inputs): the eigenvector in FP32 instead (eigvec_f32).
// Executed by a full warp; every lane returns lam and the unit q (q = 1, 0, 0, 0
// when every cofactor vanishes).
template <bool F32_VEC>
__device__ void key_eigen_warp(const double *sK, double e0, double &lam, double (&q)[4], double *s_jac) {
    const int lane = threadIdx.x & 31;
    double t2 = 0.0, t3 = 0.0, c0 = 0.0;
    if (lane < 16) {
        const int i = lane >> 2, j = lane & 3;
        double k2 = 0.0;  // (K^2)_ij
#pragma unroll
        for (int m = 0; m < 4; m++) k2 = fma(sK[4 * i + m], sK[4 * m + j], k2);
        const double kij = sK[4 * i + j];
        t2 = kij * kij;
        t3 = k2 * sK[4 * j + i];
    } else if (lane < 20) {
        const int j = lane - 16;
        const int ca = j == 0 ? 1 : 0, cb = j <= 1 ? 2 : 1, cc = j <= 2 ? 3 : 2;
        c0 = sK[j] * det3(sK[4 + ca], sK[4 + cb], sK[4 + cc], sK[8 + ca], sK[8 + cb], sK[8 + cc], sK[12 + ca],
                          sK[12 + cb], sK[12 + cc]);
        if (j & 1) c0 = -c0;
    }
    t2 = warp_sum_d(t2);
    t3 = warp_sum_d(t3);
    c0 = warp_sum_d(c0);
    const double c2 = -0.5 * t2, c1 = t3 * (-1.0 / 3.0);
    double l = 0.0;
    if (e0 > 0.0) {
        const double ie = 1.0 / e0, ie2 = ie * ie;
        const float ief = (float)ie;
        const float a2 = (float)(c2 * ie2), a1 = (float)(c1 * ie2 * ie), a0 = (float)(c0 * ie2 * ie2);
        float s = 1.f;
        for (int it = 0; it < 64; it++) {
            const float P = fmaf(fmaf(fmaf(s, s, a2), s, a1), s, a0);
            const float dP = fmaf(fmaf(4.f * s, s, 2.f * a2), s, a1);
            if (!(dP != 0.f)) break;
            const float d = P / dP;
            s -= d;
            if (fabsf(d) <= 1e-6f) break;
        }
        l = (double)s * e0;
        float corr = INFINITY;  // the last polish step, relative to e0
        for (int it = 0; it < 3; it++) {
            const double P = fma(fma(fma(l, l, c2), l, c1), l, c0);
            const double dP = fma(fma(4.0 * l, l, 2.0 * c2), l, c1);
            const float dPf = (float)dP;
            if (!(dPf != 0.f) || !isfinite(dPf)) {
                corr = INFINITY;
                break;
            }
            const double d = P * (double)(1.f / dPf);
            l -= d;
            corr = (float)d * ief;
        }
        // a simple root has converged by the third polish step (each gains about
        // seven digits); a near-multiple one (the top eigenvalues of K nearly or
        // exactly equal) converges only linearly: a last step above 1e-10 of e0 sends
        // the chain to the Jacobi solve (the same decision on every lane)
        if (!(fabsf(corr) <= 1e-10f)) {
            double lj = 0.0, qj[4] = {1.0, 0.0, 0.0, 0.0};
            if (lane == 0) jacobi_top_eigenpair(sK, s_jac, s_jac + 16, lj, qj);
            lam = __shfl_sync(0xffffffffu, lj, 0);
            for (int k = 0; k < 4; k++) q[k] = __shfl_sync(0xffffffffu, qj[k], 0);
            return;
        }
    }
    lam = l;
    if (F32_VEC) {
        eigvec_f32(sK, e0, l, q);
        return;
    }
    // cofactor (i, j) of M = K - l I on lane 4 i + j
    double cof = 0.0;
    if (lane < 16) {
        const int i = lane >> 2, j = lane & 3;
        double m[9];
        int t = 0;
#pragma unroll
        for (int r = 0; r < 4; r++)
            if (r != i)
#pragma unroll
                for (int c = 0; c < 4; c++)
                    if (c != j) m[t++] = sK[4 * r + c] - (r == c ? l : 0.0);
        cof = det3(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8]);
        if ((i + j) & 1) cof = -cof;
    }
    // squared norm of the row of this lane (lanes 4 i .. 4 i + 3)
    double nrm = cof * cof;
    nrm += __shfl_xor_sync(0xffffffffu, nrm, 1);
    nrm += __shfl_xor_sync(0xffffffffu, nrm, 2);
    int best = 0;
    double bn = __shfl_sync(0xffffffffu, nrm, 0);
    for (int i = 1; i < 4; i++) {
        const double v = __shfl_sync(0xffffffffu, nrm, 4 * i);
        if (v > bn) {
            bn = v;
            best = i;
        }
    }
    const double inv = bn > 1e-300 ? 1.0 / sqrt(bn) : 0.0;
    for (int k = 0; k < 4; k++) q[k] = __shfl_sync(0xffffffffu, cof, 4 * best + k) * inv;
    if (!(bn > 1e-300)) {
        q[0] = 1.0;
        q[1] = q[2] = q[3] = 0.0;
    }
}

// The end of the float32 forward on warp 0: the FP64 key-matrix eigen solve (its
// largest root is ill-conditioned in FP32 when the top two eigenvalues nearly meet),
// then UT and rmsd in FP32.
__device__ void rmsd_finish_f32(const RmsdArgs<float> &a, int b, int n, const double *s_out, double *s_K,
                                const double *s_c, double *s_jac) {
    const int tid = threadIdx.x;
    if (tid == 0) {
        const double *R = s_out;
        const double F[16] = {R[0] + R[4] + R[8], R[5] - R[7], R[6] - R[2], R[1] - R[3],
                              R[5] - R[7], R[0] - R[4] - R[8], R[1] + R[3], R[2] + R[6],
                              R[6] - R[2], R[1] + R[3], -R[0] + R[4] - R[8], R[5] + R[7],
                              R[1] - R[3], R[2] + R[6], R[5] + R[7], -R[0] - R[4] + R[8]};
        for (int k = 0; k < 16; k++) s_K[k] = F[k];
    }
    __syncwarp();
    const double r2 = s_out[9];
    double lam, qd[4];
    key_eigen_warp<true>(s_K, 0.5 * r2, lam, qd, s_jac);
    if (tid != 0) return;
    const float q[4] = {(float)qd[0], (float)qd[1], (float)qd[2], (float)qd[3]};
    float U[9];
    U[0] = q[0] * q[0] + q[1] * q[1] - q[2] * q[2] - q[3] * q[3];
    U[1] = 2.f * (q[1] * q[2] - q[0] * q[3]);
    U[2] = 2.f * (q[1] * q[3] + q[0] * q[2]);
    U[3] = 2.f * (q[1] * q[2] + q[0] * q[3]);
    U[4] = q[0] * q[0] - q[1] * q[1] + q[2] * q[2] - q[3] * q[3];
    U[5] = 2.f * (q[2] * q[3] - q[0] * q[1]);
    U[6] = 2.f * (q[1] * q[3] - q[0] * q[2]);
    U[7] = 2.f * (q[2] * q[3] + q[0] * q[1]);
    U[8] = q[0] * q[0] - q[1] * q[1] - q[2] * q[2] + q[3] * q[3];
    float *ut = a.ut + (size_t)9 * b;
    for (int j = 0; j < 3; j++)
        for (int k = 0; k < 3; k++) ut[3 * j + k] = U[3 * k + j];
    const float msd = n > 0 ? (float)(r2 - 2.0 * fabs(lam) + 1e-10) * (1.f / (float)n) : 0.f;
    a.rmsd[b] = sqrtf(msd > 0.f ? msd : 0.f);
    if (a.centroids)
        for (int k = 0; k < 6; k++) a.centroids[6 * b + k] = s_c[k];
}

template <typename T>
__global__ void __launch_bounds__(kRmsdThreads) rmsd_fwd_kernel(RmsdArgs<T> a) {
    __shared__ double s_red[kRmsdWarps * 10];
    __shared__ double s_out[10];
    __shared__ double s_K[16];
    __shared__ double s_jac[32];  // scratch of the Jacobi fallback
    __shared__ double s_c[6];  // centroids (src, dst)
    __shared__ T s_ct[6];
    const int b = blockIdx.x, tid = threadIdx.x;
    int n = a.num_atoms[b];
    if (n < 0 || n > a.atoms_stride) {
        if (tid == 0 && a.hdr) atomicCAS(&a.hdr->status, 0u, (unsigned)TPL_ERR_ATOMS);
        n = max(0, min(n, a.atoms_stride));
    }
    const T *x = a.src + (size_t)b * 3 * a.atoms_stride;
    const T *y = a.dst + (size_t)b * 3 * a.atoms_stride;
    if (a.center) {
        T sx[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll 4
        for (int i = tid; i < n; i += kRmsdThreads)
            for (int k = 0; k < 3; k++) {
                sx[k] += x[3 * i + k];
                sx[3 + k] += y[3 * i + k];
            }
        block_sums<T, 6>(sx, s_red, s_out);
        if (tid < 6) {  // one division per value, on six lanes (FP64 is slow on GB300)
            const double v = n > 0 ? (sizeof(T) == 4 ? s_out[tid] * (double)(1.f / (float)n) : s_out[tid] / n) : 0.0;
            s_c[tid] = v;
            s_ct[tid] = (T)v;
        }
    } else if (tid < 6) {
        s_c[tid] = 0.0;
        s_ct[tid] = T(0);
    }
    __syncthreads();
    T ct[6];
    for (int k = 0; k < 6; k++) ct[k] = s_ct[k];
    T acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};  // R (row-major) and R2
#pragma unroll 4
    for (int i = tid; i < n; i += kRmsdThreads) {
        T xi[3], yi[3];
        for (int k = 0; k < 3; k++) {
            xi[k] = x[3 * i + k] - ct[k];
            yi[k] = y[3 * i + k] - ct[3 + k];
        }
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++) acc[3 * p + q] = fma(xi[p], yi[q], acc[3 * p + q]);
        acc[9] += xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2] + yi[0] * yi[0] + yi[1] * yi[1] + yi[2] * yi[2];
    }
    block_sums<T, 10>(acc, s_red, s_out);
    if constexpr (sizeof(T) == 4) {
        if (tid < 32) rmsd_finish_f32(a, b, n, s_out, s_K, s_c, s_jac);
        return;
    }
    if (tid < 32) {
        const double *R = s_out;
        double tot[10];
        for (int k = 0; k < 10; k++) tot[k] = s_out[k];
        if (tid == 0) {
            // quaternion matrix, same layout as the reference (coords2rmsd_interface.cpp:146-149)
            const double F[16] = {R[0] + R[4] + R[8], R[5] - R[7], R[6] - R[2], R[1] - R[3],
                                  R[5] - R[7], R[0] - R[4] - R[8], R[1] + R[3], R[2] + R[6],
                                  R[6] - R[2], R[1] + R[3], -R[0] + R[4] - R[8], R[5] + R[7],
                                  R[1] - R[3], R[2] + R[6], R[5] + R[7], -R[0] - R[4] + R[8]};
            for (int k = 0; k < 16; k++) s_K[k] = F[k];
        }
        __syncwarp();
        double lam, q[4];
        key_eigen_warp<false>(s_K, 0.5 * tot[9], lam, q, s_jac);
        if (tid != 0) return;
        // rotation from the unit quaternion (coords2rmsd_interface.cpp:36-46)
        double U[9];
        U[0] = q[0] * q[0] + q[1] * q[1] - q[2] * q[2] - q[3] * q[3];
        U[1] = 2.0 * (q[1] * q[2] - q[0] * q[3]);
        U[2] = 2.0 * (q[1] * q[3] + q[0] * q[2]);
        U[3] = 2.0 * (q[1] * q[2] + q[0] * q[3]);
        U[4] = q[0] * q[0] - q[1] * q[1] + q[2] * q[2] - q[3] * q[3];
        U[5] = 2.0 * (q[2] * q[3] - q[0] * q[1]);
        U[6] = 2.0 * (q[1] * q[3] - q[0] * q[2]);
        U[7] = 2.0 * (q[2] * q[3] + q[0] * q[1]);
        U[8] = q[0] * q[0] - q[1] * q[1] - q[2] * q[2] + q[3] * q[3];
        T *ut = a.ut + (size_t)9 * b;
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) ut[3 * j + k] = (T)U[3 * k + j];
        const double msd = n > 0 ? (tot[9] - 2.0 * fabs(lam) + 1e-10) / (double)n : 0.0;
        a.rmsd[b] = (T)sqrt(msd > 0.0 ? msd : 0.0);
        if (a.centroids)
            for (int k = 0; k < 6; k++) a.centroids[6 * b + k] = s_c[k];
    }
}

template <typename T>
__global__ void __launch_bounds__(kRmsdThreads) rmsd_bwd_kernel(RmsdArgs<T> a) {
    const int b = blockIdx.x, tid = threadIdx.x;
    const int n = max(0, min(a.num_atoms[b], a.atoms_stride));
    const T *x = a.src + (size_t)b * 3 * a.atoms_stride;
    const T *y = a.dst + (size_t)b * 3 * a.atoms_stride;
    T *gx = a.grad_src + (size_t)b * 3 * a.atoms_stride;
    // per-chain constants once per block: converting the FP64 centroids on every
    // thread would keep GB300's slow FP64 pipe busy
    __shared__ T s_c[6], s_U[9], s_scale;
    if (tid < 6) s_c[tid] = (a.center && a.centroids) ? (T)a.centroids[6 * b + tid] : T(0);
    if (tid < 9) s_U[tid] = a.ut[(size_t)9 * b + tid];
    if (tid == 0) {
        const T r = a.rmsd[b];
        s_scale = (n > 0 && r > T(0)) ? a.grad_rmsd[b] / (r * (T)n) : T(0);
    }
    __syncthreads();
    T c[6], U[9];
    for (int k = 0; k < 6; k++) c[k] = s_c[k];
    for (int k = 0; k < 9; k++) U[k] = s_U[k];
    const T scale = s_scale;
    // one atom per thread: chains on x, blocks of atoms on y
    const int i = blockIdx.y * kRmsdThreads + tid;
    if (i < a.atoms_stride) {
        if (i < n) {
            T xi[3], yi[3];
            for (int k = 0; k < 3; k++) {
                xi[k] = x[3 * i + k] - c[k];
                yi[k] = y[3 * i + k] - c[3 + k];
            }
            for (int k = 0; k < 3; k++)
                gx[3 * i + k] = scale * (xi[k] - (U[3 * k] * yi[0] + U[3 * k + 1] * yi[1] + U[3 * k + 2] * yi[2]));
        } else {
            gx[3 * i] = gx[3 * i + 1] = gx[3 * i + 2] = T(0);
        }
    }
}

template <typename T>
static int rmsd_fwd_launch(const T *src, const T *dst, const int *num_atoms, int B, int stride, int center, T *rmsd,
                           T *ut, double *centroids, void *ws, cudaStream_t st) {
    if (B == 0) return TPL_OK;
    RmsdArgs<T> a{src, dst, num_atoms, stride, center, rmsd, ut, centroids, nullptr, nullptr, (WsHeader *)ws};
    rmsd_fwd_kernel<T><<<B, kRmsdThreads, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

template <typename T>
static int rmsd_bwd_launch(const T *grad_rmsd, const T *src, const T *dst, const int *num_atoms, const T *rmsd,
                           const T *ut, const double *centroids, int B, int stride, int center, T *grad_src,
                           cudaStream_t st) {
    if (B == 0) return TPL_OK;
    RmsdArgs<T> a{src, dst, num_atoms, stride, center, const_cast<T *>(rmsd), const_cast<T *>(ut),
                  const_cast<double *>(centroids), grad_rmsd, grad_src, nullptr};
    const int ablocks = (max(stride, 1) + kRmsdThreads - 1) / kRmsdThreads;
    if (ablocks > 65535) return TPL_ERR_UNSUPPORTED;
    rmsd_bwd_kernel<T><<<dim3((unsigned)B, (unsigned)ablocks), kRmsdThreads, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

int rmsd_forward(bool f64, const void *src, const void *dst, const int *num_atoms, int B, int stride, int center,
                 void *rmsd, void *ut, double *centroids, void *ws, cudaStream_t st) {
    if (f64)
        return rmsd_fwd_launch<double>((const double *)src, (const double *)dst, num_atoms, B, stride, center,
                                       (double *)rmsd, (double *)ut, centroids, ws, st);
    return rmsd_fwd_launch<float>((const float *)src, (const float *)dst, num_atoms, B, stride, center, (float *)rmsd,
                                  (float *)ut, centroids, ws, st);
}

int rmsd_backward(bool f64, const void *grad_rmsd, const void *src, const void *dst, const int *num_atoms,
                  const void *rmsd, const void *ut, const double *centroids, int B, int stride, int center,
                  void *grad_src, cudaStream_t st) {
    if (f64)
        return rmsd_bwd_launch<double>((const double *)grad_rmsd, (const double *)src, (const double *)dst, num_atoms,
                                       (const double *)rmsd, (const double *)ut, centroids, B, stride, center,
                                       (double *)grad_src, st);
    return rmsd_bwd_launch<float>((const float *)grad_rmsd, (const float *)src, (const float *)dst, num_atoms,
                                  (const float *)rmsd, (const float *)ut, centroids, B, stride, center,
                                  (float *)grad_src, st);
}

}  // namespace tpl
