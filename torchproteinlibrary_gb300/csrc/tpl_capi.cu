// extern "C" entry points of libtpl_gb300.so (declared in include/tpl_gb300.h).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>

#include "tpl_internal.h"

namespace tpl {

// Backbone bond geometry, Layers/ReducedModel/cBackboneProteinCPUKernels.cpp:6-12:
// joint phi:   N->CA, bond angle beta = pi - 1.9391, length 1.460
// joint psi:   CA->C, beta = pi - 2.061,  length 1.525
// joint omega: C->N,  beta = pi - 2.1186, length 1.330
static const double kBeta[3] = {M_PI - 1.9391, M_PI - 2.061, M_PI - 2.1186};
static const double kBond[3] = {1.460, 1.525, 1.330};

// FP32 (cos, sin) pairs of the three backbone bond angles.
//
// Rounding cos(beta) and sin(beta) to FP32 independently leaves the pair's norm
// off 1 by up to ~3e-8.  Every residue applies the same three pairs, so the
// frames of an FP32 chain shrink or grow coherently (about -2.6e-8 per residue
// for the nearest-rounded pairs) and positions drift by ~1e-3 A over 1000
// residues.  Among pairs within a few ulps of (cos, sin) beta whose angle is
// still within 4e-8 rad and whose own norm error is below 3e-8, pick the triple
// whose norm errors cancel over a residue.
static void pick_fp32_pairs(float cb[3], float sb[3]) {
    struct Cand {
        float c, s;
        double ang_err, norm_err;
    };
    Cand cand[3][64];
    int nc[3] = {0, 0, 0};
    for (int k = 0; k < 3; k++) {
        const double c0 = std::cos(kBeta[k]), s0 = std::sin(kBeta[k]);
        const float cf = (float)c0, sf = (float)s0;
        for (int i = -3; i <= 3; i++)
            for (int j = -3; j <= 3; j++) {
                float c = cf, s = sf;
                for (int q = 0; q < (i < 0 ? -i : i); q++) c = std::nextafter(c, i < 0 ? -2.f : 2.f);
                for (int q = 0; q < (j < 0 ? -j : j); q++) s = std::nextafter(s, j < 0 ? -2.f : 2.f);
                const double ae = std::atan2((double)s, (double)c) - kBeta[k];
                const double ne = std::hypot((double)c, (double)s) - 1.0;
                if (std::fabs(ae) < 4e-8 && std::fabs(ne) < 3e-8 && nc[k] < 64) cand[k][nc[k]++] = {c, s, ae, ne};
            }
        if (nc[k] == 0) cand[k][nc[k]++] = {cf, sf, 0.0, 0.0};
    }
    double best = 1e30, best_ang = 1e30;
    int bi[3] = {0, 0, 0};
    for (int a = 0; a < nc[0]; a++)
        for (int b = 0; b < nc[1]; b++)
            for (int c = 0; c < nc[2]; c++) {
                const double tot = std::fabs(cand[0][a].norm_err + cand[1][b].norm_err + cand[2][c].norm_err);
                const double ang = std::fabs(cand[0][a].ang_err) + std::fabs(cand[1][b].ang_err) +
                                   std::fabs(cand[2][c].ang_err);
                if (tot < best - 1e-15 || (std::fabs(tot - best) <= 1e-15 && ang < best_ang)) {
                    best = tot;
                    best_ang = ang;
                    bi[0] = a; bi[1] = b; bi[2] = c;
                }
            }
    for (int k = 0; k < 3; k++) {
        cb[k] = cand[k][bi[k]].c;
        sb[k] = cand[k][bi[k]].s;
    }
}

const BondConsts &bond_constants() {
    static BondConsts bc = [] {
        BondConsts c{};
        pick_fp32_pairs(c.cb, c.sb);
        for (int k = 0; k < 3; k++) {
            c.d[k] = (float)kBond[k];
            c.cbd[k] = std::cos(kBeta[k]);
            c.sbd[k] = std::sin(kBeta[k]);
            c.dd[k] = kBond[k];
        }
        return c;
    }();
    return bc;
}

bool set_max_dynamic_smem(const void *func, int bytes) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, int> done;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = done.find({func, dev});
        if (it != done.end() && it->second >= bytes) return true;
    }
    if (cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) return false;
    std::lock_guard<std::mutex> lk(mu);
    int &v = done[{func, dev}];
    v = v > bytes ? v : bytes;
    return true;
}

int device_sm_count() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    static std::mutex mu;
    static std::map<int, int> known;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = known.find(dev);
        if (it != known.end()) return it->second;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
    std::lock_guard<std::mutex> lk(mu);
    known[dev] = n;
    return n;
}

tpl_options resolve(const tpl_options *opt) {
    tpl_options o{};
    if (opt) o = *opt;
    return o;
}

bool options_ok(const tpl_options &o) {
    const int r = o.residues_per_thread;
    if (!(r == 0 || r == 1 || r == 2 || r == 4 || r == 8)) return false;
    // 0: automatic, 1: warp tiles, 128: CTA tiles, 32: one warp per chain, 4: one CTA of four warps per
    // chain (both 4 or 8 residues per lane)
    const int t = o.threads_per_cta;
    if (!(t == 0 || t == 1 || t == 128 || t == 32 || t == 4)) return false;
    if ((t == 32 || t == 4) && !(r == 0 || r == 4 || r == 8)) return false;
    if (o.max_ctas < 0) return false;
    if (o.copy_buffers < 0 || o.copy_buffers > 2) return false;
    return true;
}

size_t a2b_ws(int B, int L, const tpl_options &o) {
    const int tile = a2b_tile_for(o);
    const int plain_chunk = 256;  // the plain FP64 backward keeps one record per 256-residue chunk
    const int smallest = tile < plain_chunk ? tile : plain_chunk;
    return ws_bytes_for(B, (L + smallest - 1) / smallest);
}

}  // namespace tpl

using namespace tpl;

extern "C" {

const char *tpl_status_string(int status) {
    switch (status) {
        case TPL_OK: return "ok";
        case TPL_ERR_ARGUMENT: return "invalid argument";
        case TPL_ERR_WORKSPACE: return "workspace missing, misaligned or too small";
        case TPL_ERR_LAUNCH: return "CUDA kernel launch failed";
        case TPL_ERR_LENGTH: return "chain length outside [0, max_len]";
        case TPL_ERR_SEQUENCE: return "unknown residue letter";
        case TPL_ERR_LOOKBACK_TIMEOUT: return "a bounded device wait timed out (inter-tile look-back or bulk copy)";
        case TPL_ERR_ATOMS: return "chain has more atoms than max_atoms";
        case TPL_ERR_UNSUPPORTED: return "unsupported option combination";
        case TPL_ERR_TOO_LARGE: return "problem exceeds the fixed scratch of the no-allocation entry point";
        case TPL_ERR_ATOM_TYPE: return "a (residue, atom) name pair has no atom type";
        case TPL_ERR_IO: return "a file could not be opened";
    }
    return "unknown status";
}

int tpl_version(void) { return 100; }

int tpl_sincos_f32(const float *a, float *s, float *c, int n, void *stream) {
    if (n < 0 || (n > 0 && (!a || !s || !c))) return TPL_ERR_ARGUMENT;
    return sincos_poly_f32(a, s, c, n, (cudaStream_t)stream);
}

size_t tpl_a2b_workspace_bytes(int batch, int max_len, const tpl_options *opt) {
    if (batch < 0 || max_len < 0) return 0;
    return a2b_ws(batch, max_len, resolve(opt));
}

int tpl_workspace_init(void *workspace, size_t workspace_bytes, void *stream) {
    if (!workspace || workspace_bytes < sizeof(WsHeader)) return TPL_ERR_WORKSPACE;
    cudaError_t e = cudaMemsetAsync(workspace, 0, workspace_bytes, (cudaStream_t)stream);
    return e == cudaSuccess ? TPL_OK : TPL_ERR_LAUNCH;
}

int tpl_workspace_status(void *workspace, void *stream, int *status_out) {
    if (!workspace || !status_out) return TPL_ERR_ARGUMENT;
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return TPL_ERR_LAUNCH;
    unsigned v = 0;
    if (cudaMemcpy(&v, workspace, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return TPL_ERR_LAUNCH;
    if (v != 0 && cudaMemset(workspace, 0, sizeof(unsigned)) != cudaSuccess) return TPL_ERR_LAUNCH;
    *status_out = (int)v;
    return TPL_OK;
}

static int check_ws(const void *ws, size_t bytes, size_t need) {
    if (!ws || bytes < need || ((uintptr_t)ws & 15u)) return TPL_ERR_WORKSPACE;
    return TPL_OK;
}

int tpl_a2b_forward_f32(const float *angles, const int32_t *lengths, float *coords, void *workspace,
                        size_t workspace_bytes, int batch, int max_len, const tpl_options *opt, void *stream) {
    if (batch < 0 || max_len < 0) return TPL_ERR_ARGUMENT;
    const tpl_options o = resolve(opt);
    if (!options_ok(o)) return TPL_ERR_ARGUMENT;
    if (batch == 0 || max_len == 0) return TPL_OK;
    if (!angles || !lengths || !coords) return TPL_ERR_ARGUMENT;
    int s = check_ws(workspace, workspace_bytes, a2b_ws(batch, max_len, o));
    if (s) return s;
    return a2b_forward_f32(angles, lengths, coords, workspace, batch, max_len, o, (cudaStream_t)stream);
}

int tpl_a2b_backward_f32(float *grad_angles, const float *grad_coords, const float *angles,
                         const int32_t *lengths, void *workspace, size_t workspace_bytes, int batch, int max_len,
                         const tpl_options *opt, void *stream) {
    if (batch < 0 || max_len < 0) return TPL_ERR_ARGUMENT;
    const tpl_options o = resolve(opt);
    if (!options_ok(o)) return TPL_ERR_ARGUMENT;
    if (batch == 0 || max_len == 0) return TPL_OK;
    if (!grad_angles || !grad_coords || !angles || !lengths) return TPL_ERR_ARGUMENT;
    int s = check_ws(workspace, workspace_bytes, a2b_ws(batch, max_len, o));
    if (s) return s;
    return a2b_backward_f32(grad_angles, grad_coords, angles, lengths, workspace, batch, max_len, o,
                            (cudaStream_t)stream);
}

int tpl_a2b_backward_coords_f32(float *grad_angles, const float *grad_coords, const float *coords,
                                const int32_t *lengths, void *workspace, size_t workspace_bytes, int batch,
                                int max_len, const tpl_options *opt, void *stream) {
    if (batch < 0 || max_len < 0) return TPL_ERR_ARGUMENT;
    const tpl_options o = resolve(opt);
    if (!(o.residues_per_thread == 0 || o.residues_per_thread == 4 || o.residues_per_thread == 8))
        return TPL_ERR_ARGUMENT;
    if (o.copy_buffers < 0 || o.copy_buffers > 2 || (o.copy_buffers == 2 && o.residues_per_thread == 8))
        return TPL_ERR_ARGUMENT;
    if (!(o.threads_per_cta == 0 || o.threads_per_cta == 32 || o.threads_per_cta == 4)) return TPL_ERR_ARGUMENT;
    if (batch == 0 || max_len == 0) return TPL_OK;
    if (!grad_angles || !grad_coords || !coords || !lengths) return TPL_ERR_ARGUMENT;
    int s = check_ws(workspace, workspace_bytes, sizeof(WsHeader));
    if (s) return s;
    return a2b_backward_coords(grad_angles, grad_coords, coords, lengths, workspace, batch, max_len, o,
                               (cudaStream_t)stream);
}

int tpl_a2b_forward_f64(const double *angles, const int32_t *lengths, double *coords, int batch, int max_len,
                        void *stream) {
    if (batch < 0 || max_len < 0) return TPL_ERR_ARGUMENT;
    if (batch == 0 || max_len == 0) return TPL_OK;
    if (!angles || !lengths || !coords) return TPL_ERR_ARGUMENT;
    return a2b_forward_f64_plain(angles, lengths, coords, batch, max_len, (cudaStream_t)stream);
}

int tpl_a2b_backward_f64(double *grad_angles, const double *grad_coords, const double *angles,
                         const int32_t *lengths, void *workspace, size_t workspace_bytes, int batch, int max_len,
                         void *stream) {
    if (batch < 0 || max_len < 0) return TPL_ERR_ARGUMENT;
    if (batch == 0 || max_len == 0) return TPL_OK;
    if (!grad_angles || !grad_coords || !angles || !lengths) return TPL_ERR_ARGUMENT;
    int s = check_ws(workspace, workspace_bytes, ws_bytes_for(batch, (max_len + 255) / 256));
    if (s) return s;
    return a2b_backward_f64_plain(grad_angles, grad_coords, angles, lengths, workspace, batch, max_len,
                                  (cudaStream_t)stream);
}

int tpl_num_atoms(const char *sequence) {
    if (!sequence) return TPL_ERR_ARGUMENT;
    int n = num_atoms_host(sequence);
    return n < 0 ? TPL_ERR_SEQUENCE : n;
}

size_t tpl_a2c_workspace_bytes(int batch, int max_len, int max_atoms, const tpl_options *opt) {
    (void)batch; (void)max_len; (void)max_atoms; (void)opt;
    return sizeof(WsHeader);
}

// Angles2Coords reads only threads_per_cta (0 / 4, 128, 256 or 512) and renormalize.
static bool a2c_options_ok(const tpl_options &o) {
    return o.threads_per_cta == 0 || o.threads_per_cta == 4 || o.threads_per_cta == 8 || o.threads_per_cta == 128 ||
           o.threads_per_cta == 256 || o.threads_per_cta == 512;
}

static int a2c_fwd_common(bool f64, const uint8_t *sequences, int seq_stride, const void *angles, void *coords,
                          uint8_t *res_names, uint8_t *atom_names, void *workspace, size_t workspace_bytes,
                          int batch, int max_len, int max_atoms, const tpl_options *opt, void *stream) {
    if (batch < 0 || max_len < 0 || max_atoms < 0 || seq_stride <= 0) return TPL_ERR_ARGUMENT;
    const tpl_options o = resolve(opt);
    if (!a2c_options_ok(o)) return TPL_ERR_ARGUMENT;
    if (batch == 0) return TPL_OK;
    if (!sequences || (!angles && max_len > 0) || (!coords && max_atoms > 0)) return TPL_ERR_ARGUMENT;
    if ((res_names == nullptr) != (atom_names == nullptr)) return TPL_ERR_ARGUMENT;
    if (((uintptr_t)res_names & 3u) || ((uintptr_t)atom_names & 3u)) return TPL_ERR_ARGUMENT;
    int s = check_ws(workspace, workspace_bytes, sizeof(WsHeader));
    if (s) return s;
    return a2c_forward(f64, sequences, seq_stride, angles, coords, (uint32_t *)res_names, (uint32_t *)atom_names,
                       workspace, batch, max_len, max_atoms, o, (cudaStream_t)stream);
}

static int a2c_bwd_common(bool f64, void *grad_angles, const void *grad_coords, const uint8_t *sequences,
                          int seq_stride, const void *angles, void *workspace, size_t workspace_bytes, int batch,
                          int max_len, int max_atoms, const tpl_options *opt, void *stream) {
    if (batch < 0 || max_len < 0 || max_atoms < 0 || seq_stride <= 0) return TPL_ERR_ARGUMENT;
    const tpl_options o = resolve(opt);
    if (!a2c_options_ok(o)) return TPL_ERR_ARGUMENT;
    if (batch == 0) return TPL_OK;
    if (!sequences || ((!angles || !grad_angles) && max_len > 0) || (!grad_coords && max_atoms > 0))
        return TPL_ERR_ARGUMENT;
    int s = check_ws(workspace, workspace_bytes, sizeof(WsHeader));
    if (s) return s;
    return a2c_backward(f64, grad_angles, grad_coords, sequences, seq_stride, angles, workspace, batch, max_len,
                        max_atoms, o, (cudaStream_t)stream);
}

int tpl_a2c_forward_f32(const uint8_t *sequences, int seq_stride, const float *angles, float *coords,
                        uint8_t *res_names, uint8_t *atom_names, void *workspace, size_t workspace_bytes, int batch,
                        int max_len, int max_atoms, const tpl_options *opt, void *stream) {
    return a2c_fwd_common(false, sequences, seq_stride, angles, coords, res_names, atom_names, workspace,
                          workspace_bytes, batch, max_len, max_atoms, opt, stream);
}

int tpl_a2c_forward_f64(const uint8_t *sequences, int seq_stride, const double *angles, double *coords,
                        uint8_t *res_names, uint8_t *atom_names, void *workspace, size_t workspace_bytes, int batch,
                        int max_len, int max_atoms, const tpl_options *opt, void *stream) {
    return a2c_fwd_common(true, sequences, seq_stride, angles, coords, res_names, atom_names, workspace,
                          workspace_bytes, batch, max_len, max_atoms, opt, stream);
}

int tpl_a2c_backward_f32(float *grad_angles, const float *grad_coords, const uint8_t *sequences, int seq_stride,
                         const float *angles, void *workspace, size_t workspace_bytes, int batch, int max_len,
                         int max_atoms, const tpl_options *opt, void *stream) {
    return a2c_bwd_common(false, grad_angles, grad_coords, sequences, seq_stride, angles, workspace,
                          workspace_bytes, batch, max_len, max_atoms, opt, stream);
}

int tpl_a2c_backward_coords_f32(float *grad_angles, const float *grad_coords, const float *coords,
                                const uint8_t *sequences, int seq_stride, void *workspace, size_t workspace_bytes,
                                int batch, int max_len, int max_atoms, void *stream) {
    if (batch < 0 || max_len < 0 || max_atoms < 0 || seq_stride <= 0) return TPL_ERR_ARGUMENT;
    if (batch == 0) return TPL_OK;
    if (!sequences || (!grad_angles && max_len > 0) || ((!grad_coords || !coords) && max_atoms > 0))
        return TPL_ERR_ARGUMENT;
    int s = check_ws(workspace, workspace_bytes, sizeof(WsHeader));
    if (s) return s;
    return a2c_backward_coords(grad_angles, grad_coords, coords, sequences, seq_stride, workspace, batch, max_len,
                               max_atoms, (cudaStream_t)stream);
}

int tpl_a2c_backward_f64(double *grad_angles, const double *grad_coords, const uint8_t *sequences, int seq_stride,
                         const double *angles, void *workspace, size_t workspace_bytes, int batch, int max_len,
                         int max_atoms, const tpl_options *opt, void *stream) {
    return a2c_bwd_common(true, grad_angles, grad_coords, sequences, seq_stride, angles, workspace,
                          workspace_bytes, batch, max_len, max_atoms, opt, stream);
}

static int rmsd_fwd_common(bool f64, const void *src, const void *dst, const int32_t *num_atoms, int batch,
                           int stride, int center, void *rmsd, void *ut, double *centroids, void *ws, size_t ws_bytes,
                           void *stream) {
    if (batch < 0 || stride < 0) return TPL_ERR_ARGUMENT;
    if (batch == 0) return TPL_OK;
    if (!src || !dst || !num_atoms || !rmsd || !ut || (center && !centroids)) return TPL_ERR_ARGUMENT;
    if (ws) {
        int s = check_ws(ws, ws_bytes, sizeof(WsHeader));
        if (s) return s;
    }
    return rmsd_forward(f64, src, dst, num_atoms, batch, stride, center, rmsd, ut, centroids, ws,
                        (cudaStream_t)stream);
}

int tpl_rmsd_forward_f32(const float *src, const float *dst, const int32_t *num_atoms, int batch, int atoms_stride,
                         int center, float *rmsd, float *ut, double *centroids, void *workspace,
                         size_t workspace_bytes, void *stream) {
    return rmsd_fwd_common(false, src, dst, num_atoms, batch, atoms_stride, center, rmsd, ut, centroids, workspace,
                           workspace_bytes, stream);
}

int tpl_rmsd_forward_f64(const double *src, const double *dst, const int32_t *num_atoms, int batch, int atoms_stride,
                         int center, double *rmsd, double *ut, double *centroids, void *workspace,
                         size_t workspace_bytes, void *stream) {
    return rmsd_fwd_common(true, src, dst, num_atoms, batch, atoms_stride, center, rmsd, ut, centroids, workspace,
                           workspace_bytes, stream);
}

static int rmsd_bwd_common(bool f64, const void *grad_rmsd, const void *src, const void *dst, const int32_t *num_atoms,
                           const void *rmsd, const void *ut, const double *centroids, int batch, int stride,
                           int center, void *grad_src, void *stream) {
    if (batch < 0 || stride < 0) return TPL_ERR_ARGUMENT;
    if (batch == 0) return TPL_OK;
    if (!grad_rmsd || !src || !dst || !num_atoms || !rmsd || !ut || !grad_src || (center && !centroids))
        return TPL_ERR_ARGUMENT;
    return rmsd_backward(f64, grad_rmsd, src, dst, num_atoms, rmsd, ut, centroids, batch, stride, center, grad_src,
                         (cudaStream_t)stream);
}

int tpl_rmsd_backward_f32(const float *grad_rmsd, const float *src, const float *dst, const int32_t *num_atoms,
                          const float *rmsd, const float *ut, const double *centroids, int batch, int atoms_stride,
                          int center, float *grad_src, void *stream) {
    return rmsd_bwd_common(false, grad_rmsd, src, dst, num_atoms, rmsd, ut, centroids, batch, atoms_stride, center,
                           grad_src, stream);
}

int tpl_rmsd_backward_f64(const double *grad_rmsd, const double *src, const double *dst, const int32_t *num_atoms,
                          const double *rmsd, const double *ut, const double *centroids, int batch, int atoms_stride,
                          int center, double *grad_src, void *stream) {
    return rmsd_bwd_common(true, grad_rmsd, src, dst, num_atoms, rmsd, ut, centroids, batch, atoms_stride, center,
                           grad_src, stream);
}

// ------------------------------------------------------------- CoordsTransform
#define TPL_TRANSFORM_ENTRIES(T, SFX)                                                                              \
    int tpl_coords_translate_##SFX(const T *in, T *out, const T *translation, const int32_t *num_atoms, int batch, \
                                   int atoms_stride, void *stream) {                                               \
        if (batch < 0 || atoms_stride < 0) return TPL_ERR_ARGUMENT;                                                \
        if (batch == 0 || atoms_stride == 0) return TPL_OK;                                                        \
        if (!in || !out || !num_atoms) return TPL_ERR_ARGUMENT;                                                    \
        return coords_shift<T>(in, out, translation, 0, num_atoms, batch, atoms_stride, (cudaStream_t)stream);     \
    }                                                                                                              \
    int tpl_coords_rotate_##SFX(const T *in, T *out, const T *rotation, int transpose, const int32_t *num_atoms,   \
                                int batch, int atoms_stride, void *stream) {                                       \
        if (batch < 0 || atoms_stride < 0) return TPL_ERR_ARGUMENT;                                                \
        if (batch == 0 || atoms_stride == 0) return TPL_OK;                                                        \
        if (!in || !out || !rotation || !num_atoms) return TPL_ERR_ARGUMENT;                                       \
        return coords_rotate<T>(in, out, rotation, transpose, num_atoms, batch, atoms_stride, (cudaStream_t)stream); \
    }                                                                                                              \
    int tpl_coords_center_##SFX(const T *in, T *center, const int32_t *num_atoms, int batch, int atoms_stride,     \
                                void *stream) {                                                                    \
        if (batch < 0 || atoms_stride < 0) return TPL_ERR_ARGUMENT;                                                \
        if (batch == 0) return TPL_OK;                                                                             \
        if (!center || !num_atoms || (atoms_stride > 0 && !in)) return TPL_ERR_ARGUMENT;                           \
        return coords_center<T>(in, center, num_atoms, batch, atoms_stride, (cudaStream_t)stream);                 \
    }                                                                                                              \
    int tpl_coords_center_backward_##SFX(const T *grad_center, T *grad_in, const int32_t *num_atoms, int batch,    \
                                         int atoms_stride, void *stream) {                                         \
        if (batch < 0 || atoms_stride < 0) return TPL_ERR_ARGUMENT;                                                \
        if (batch == 0 || atoms_stride == 0) return TPL_OK;                                                        \
        if (!grad_center || !grad_in || !num_atoms) return TPL_ERR_ARGUMENT;                                       \
        return coords_shift<T>(nullptr, grad_in, grad_center, 1, num_atoms, batch, atoms_stride,                   \
                               (cudaStream_t)stream);                                                              \
    }                                                                                                              \
    int tpl_coords_bbox_##SFX(const T *in, T *lo, T *hi, const int32_t *num_atoms, int batch, int atoms_stride,    \
                              void *stream) {                                                                      \
        if (batch < 0 || atoms_stride < 0) return TPL_ERR_ARGUMENT;                                                \
        if (batch == 0) return TPL_OK;                                                                             \
        if (!lo || !hi || !num_atoms || (atoms_stride > 0 && !in)) return TPL_ERR_ARGUMENT;                        \
        return coords_bbox<T>(in, lo, hi, num_atoms, batch, atoms_stride, (cudaStream_t)stream);                   \
    }

// ---------------------------------------------------------- Coords2TypedCoords
#define TPL_TYPED_ENTRIES(T, SFX, F64)                                                                             \
    int tpl_typed_coords_forward_##SFX(const T *coords, const uint8_t *res_names, const uint8_t *atom_names,       \
                                       const int32_t *num_atoms, int batch, int in_stride, int out_stride, T *out, \
                                       int32_t *num_atoms_of_type, int32_t *offsets, int32_t *atom_indexes,        \
                                       void *workspace, size_t workspace_bytes, void *stream) {                    \
        if (batch < 0 || in_stride < 0 || out_stride < 0) return TPL_ERR_ARGUMENT;                                 \
        if (batch == 0) return TPL_OK;                                                                             \
        if (!num_atoms || !num_atoms_of_type || !offsets) return TPL_ERR_ARGUMENT;                                 \
        if ((in_stride > 0 && (!coords || !res_names || !atom_names)) || (out_stride > 0 && (!out || !atom_indexes))) \
            return TPL_ERR_ARGUMENT;                                                                               \
        if (((uintptr_t)res_names & 3u) || ((uintptr_t)atom_names & 3u)) return TPL_ERR_ARGUMENT;                 \
        int s = check_ws(workspace, workspace_bytes, sizeof(WsHeader));                                            \
        if (s) return s;                                                                                           \
        return typed_forward(F64, coords, reinterpret_cast<const uint32_t *>(res_names),                           \
                             reinterpret_cast<const uint32_t *>(atom_names), num_atoms, batch, in_stride,          \
                             out_stride, out, num_atoms_of_type, offsets, atom_indexes, workspace,                 \
                             (cudaStream_t)stream);                                                                \
    }                                                                                                              \
    int tpl_typed_coords_backward_##SFX(const T *grad_typed, T *grad_flat, const int32_t *num_atoms_of_type,       \
                                        const int32_t *atom_indexes, int batch, int in_stride, int out_stride,     \
                                        void *stream) {                                                            \
        if (batch < 0 || in_stride < 0 || out_stride < 0) return TPL_ERR_ARGUMENT;                                 \
        if (batch == 0) return TPL_OK;                                                                             \
        if (!num_atoms_of_type || (in_stride > 0 && !grad_flat) || (out_stride > 0 && (!grad_typed || !atom_indexes))) \
            return TPL_ERR_ARGUMENT;                                                                               \
        return typed_backward(F64, grad_typed, grad_flat, num_atoms_of_type, atom_indexes, batch, in_stride,       \
                              out_stride, (cudaStream_t)stream);                                                   \
    }

TPL_TYPED_ENTRIES(float, f32, false)
TPL_TYPED_ENTRIES(double, f64, true)
#undef TPL_TYPED_ENTRIES

TPL_TRANSFORM_ENTRIES(float, f32)
TPL_TRANSFORM_ENTRIES(double, f64)
#undef TPL_TRANSFORM_ENTRIES

}  // extern "C"
