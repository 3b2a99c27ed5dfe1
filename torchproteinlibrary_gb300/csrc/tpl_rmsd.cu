// Coords2RMSD on the GPU: least RMSD after optimal superposition, with its
// gradient.  The reference (Layers/RMSD/Coords2RMSD/coords2rmsd_interface.cpp:52-111,
// RMSDKernels.cu:5-57) builds the 3x3 correlation on the GPU with one thread per
// matrix entry, copies the 4x4 quaternion matrix to the CPU for an eigen solve per
// chain, computes sum |x|^2 with single-thread kernels, and backpropagates with a
// Python loop of .item() calls (TorchProteinLibrary/RMSD/Coords2RMSD/Coords2RMSD.py:40-62).
//
// Here one CTA per chain does everything in one launch: optional centring, the
// correlation R_ab = sum x_a y_b and R2 = sum |x|^2 + |y|^2 accumulated in FP64,
// the 4x4 matrix T (same layout as the reference), its largest eigenpair by cyclic
// Jacobi rotations in FP64 on one thread, U from the unit quaternion, UT = U^T and
// rmsd = sqrt((R2 - 2 |lambda_max| + 1e-10) / N).  The backward is one launch:
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

__device__ __forceinline__ double block_sum(double v, double *s_red) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) s_red[w] = v;
    __syncthreads();
    double r = 0.0;
    for (int i = 0; i < kRmsdThreads / 32; i++) r += s_red[i];
    return r;
}

// Largest eigenpair of a symmetric 4x4 matrix by cyclic Jacobi rotations
// (Golub & Van Loan, Matrix Computations, 8.5).  a is destroyed.
__device__ void jacobi4_max(double a[4][4], double &lam, double q[4]) {
    double v[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) v[i][j] = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 32; sweep++) {
        double off = 0.0;
        for (int p = 0; p < 4; p++)
            for (int r = p + 1; r < 4; r++) off += a[p][r] * a[p][r];
        if (off < 1e-30) break;
        for (int p = 0; p < 3; p++)
            for (int r = p + 1; r < 4; r++) {
                if (fabs(a[p][r]) < 1e-300) continue;
                const double theta = (a[r][r] - a[p][p]) / (2.0 * a[p][r]);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 4; k++) {  // columns p, r
                    const double akp = a[k][p], akr = a[k][r];
                    a[k][p] = c * akp - s * akr;
                    a[k][r] = s * akp + c * akr;
                }
                for (int k = 0; k < 4; k++) {  // rows p, r
                    const double apk = a[p][k], ark = a[r][k];
                    a[p][k] = c * apk - s * ark;
                    a[r][k] = s * apk + c * ark;
                }
                for (int k = 0; k < 4; k++) {
                    const double vkp = v[k][p], vkr = v[k][r];
                    v[k][p] = c * vkp - s * vkr;
                    v[k][r] = s * vkp + c * vkr;
                }
            }
    }
    int best = 0;
    for (int i = 1; i < 4; i++)
        if (a[i][i] > a[best][best]) best = i;
    lam = a[best][best];
    for (int k = 0; k < 4; k++) q[k] = v[k][best];
}

template <typename T>
__global__ void __launch_bounds__(kRmsdThreads) rmsd_fwd_kernel(RmsdArgs<T> a) {
    __shared__ double s_red[kRmsdThreads / 32];
    __shared__ double s_c[6];
    const int b = blockIdx.x, tid = threadIdx.x;
    int n = a.num_atoms[b];
    if (n < 0 || n > a.atoms_stride) {
        if (tid == 0 && a.hdr) atomicCAS(&a.hdr->status, 0u, (unsigned)TPL_ERR_ATOMS);
        n = max(0, min(n, a.atoms_stride));
    }
    const T *x = a.src + (size_t)b * 3 * a.atoms_stride;
    const T *y = a.dst + (size_t)b * 3 * a.atoms_stride;
    double c[6] = {0, 0, 0, 0, 0, 0};
    if (a.center) {
        double sx[6] = {0, 0, 0, 0, 0, 0};
        for (int i = tid; i < n; i += kRmsdThreads)
            for (int k = 0; k < 3; k++) {
                sx[k] += (double)x[3 * i + k];
                sx[3 + k] += (double)y[3 * i + k];
            }
        for (int k = 0; k < 6; k++) {
            const double s = block_sum(sx[k], s_red);
            if (tid == 0) s_c[k] = n > 0 ? s / n : 0.0;
        }
        __syncthreads();
        for (int k = 0; k < 6; k++) c[k] = s_c[k];
    }
    double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};  // R (row-major) and R2
    for (int i = tid; i < n; i += kRmsdThreads) {
        double xi[3], yi[3];
        for (int k = 0; k < 3; k++) {
            xi[k] = (double)x[3 * i + k] - c[k];
            yi[k] = (double)y[3 * i + k] - c[3 + k];
        }
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++) acc[3 * p + q] = fma(xi[p], yi[q], acc[3 * p + q]);
        acc[9] += xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2] + yi[0] * yi[0] + yi[1] * yi[1] + yi[2] * yi[2];
    }
    double tot[10];
    for (int k = 0; k < 10; k++) tot[k] = block_sum(acc[k], s_red);
    if (tid == 0) {
        const double *R = tot;
        // quaternion matrix, same layout as the reference (coords2rmsd_interface.cpp:146-149)
        double F[4][4] = {
            {R[0] + R[4] + R[8], R[5] - R[7], R[6] - R[2], R[1] - R[3]},
            {R[5] - R[7], R[0] - R[4] - R[8], R[1] + R[3], R[2] + R[6]},
            {R[6] - R[2], R[1] + R[3], -R[0] + R[4] - R[8], R[5] + R[7]},
            {R[1] - R[3], R[2] + R[6], R[5] + R[7], -R[0] - R[4] + R[8]}};
        double lam, q[4];
        jacobi4_max(F, lam, q);
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
            for (int k = 0; k < 6; k++) a.centroids[6 * b + k] = c[k];
    }
}

template <typename T>
__global__ void __launch_bounds__(kRmsdThreads) rmsd_bwd_kernel(RmsdArgs<T> a) {
    const int b = blockIdx.x, tid = threadIdx.x;
    const int n = max(0, min(a.num_atoms[b], a.atoms_stride));
    const T *x = a.src + (size_t)b * 3 * a.atoms_stride;
    const T *y = a.dst + (size_t)b * 3 * a.atoms_stride;
    T *gx = a.grad_src + (size_t)b * 3 * a.atoms_stride;
    double c[6] = {0, 0, 0, 0, 0, 0};
    if (a.center && a.centroids)
        for (int k = 0; k < 6; k++) c[k] = a.centroids[6 * b + k];
    const T *ut = a.ut + (size_t)9 * b;
    double U[9];
    for (int k = 0; k < 9; k++) U[k] = (double)ut[k];
    const double r = (double)a.rmsd[b];
    const double scale = (n > 0 && r > 0.0) ? (double)a.grad_rmsd[b] / (r * (double)n) : 0.0;
    for (int i = tid; i < a.atoms_stride; i += kRmsdThreads) {
        if (i < n) {
            double xi[3], yi[3];
            for (int k = 0; k < 3; k++) {
                xi[k] = (double)x[3 * i + k] - c[k];
                yi[k] = (double)y[3 * i + k] - c[3 + k];
            }
            for (int k = 0; k < 3; k++)
                gx[3 * i + k] = (T)(scale * (xi[k] - (U[3 * k] * yi[0] + U[3 * k + 1] * yi[1] + U[3 * k + 2] * yi[2])));
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
    rmsd_bwd_kernel<T><<<B, kRmsdThreads, 0, st>>>(a);
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
