// Host-side declarations shared by the C-ABI layer and the kernel files.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/tpl_gb300.h"

namespace tpl {

// cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) once
// per (function, device) and size: the setting persists in the device's context, and
// repeating it would cost host time on every launch.  false if the call fails.
bool set_max_dynamic_smem(const void *func, int bytes);

// Number of SMs of the current device, queried once per device (at least 1).
int device_sm_count();

// FP32 / FP64 (cos, sin) of the three backbone bond angles plus the bond lengths,
// in joint order phi (N->CA), psi (CA->C), omega (C->N).  The FP32 pairs are picked
// by bond_constants() so that the rounding errors of their norms cancel over a
// residue (see tpl_capi.cu).
struct BondConsts {
    float cb[3], sb[3], d[3];
    double cbd[3], sbd[3], dd[3];
};
const BondConsts &bond_constants();

// Workspace header, shared by all launches that use one workspace buffer.  The
// ticket / done / epoch words make each persistent launch self-resetting, so that
// launches can be replayed from a CUDA graph without a memset.
struct WsHeader {
    unsigned status;      // first error code (tpl_status), 0 = ok
    unsigned fwd_ticket, fwd_done, fwd_epoch;
    unsigned bwd_ticket, bwd_done, bwd_epoch;
    unsigned tile;        // residues per tile used by the last forward
    unsigned test_skip_publish;  // fault injection for tests: 1 = chain 0, tile 0 never publishes
    unsigned pad[7];
};
static_assert(sizeof(WsHeader) == 64, "header size");

// Per (chain, tile) record of the decoupled look-back.
struct __align__(16) TileRecord {
    unsigned fflag, bflag, atoms, pad;  // atoms: residue-atom count carried by full-atom tiles
    double fagg[12];  // tile aggregate transform (forward)
    double finc[12];  // inclusive prefix transform through this tile
    double fexc[12];  // carry the forward used for this tile (read back by the backward)
    double bagg[6];   // tile sums (G, S) of the adjoint (backward)
    double binc[6];   // inclusive suffix sums from this tile to the chain end
};

inline size_t ws_bytes_for(int B, int ntiles) {
    return sizeof(WsHeader) + sizeof(TileRecord) * (size_t)B * (size_t)ntiles;
}

struct LaunchShape {
    int tile;       // residues per tile
    int threads;    // threads per CTA
    int grid;       // persistent CTAs
};

// Angles2Backbone launchers (tpl_a2b.cu); all return a tpl_status.
int a2b_forward_f32(const float *angles, const int32_t *lengths, float *coords, void *ws, int B, int L,
                    const tpl_options &opt, cudaStream_t st);
int a2b_backward_f32(float *grad_angles, const float *grad_coords, const float *angles, const int32_t *lengths,
                     void *ws, int B, int L, const tpl_options &opt, cudaStream_t st);
int a2b_forward_f64_plain(const double *angles, const int32_t *lengths, double *coords, int B, int L,
                          cudaStream_t st);
int a2b_backward_f64_plain(double *grad_angles, const double *grad_coords, const double *angles,
                           const int32_t *lengths, void *ws, int B, int L, cudaStream_t st);
int a2b_tile_for(const tpl_options &opt);
// One warp per chain (tpl_a2b_chain.cu; threads_per_cta = 32, residues_per_thread 4 or 8).
// The forward records the chain frame every a2b_chain_record_stride() residues in
// the workspace; the backward starts its chunks from those records.
int a2b_forward_chain(const float *angles, const int32_t *lengths, float *coords, void *ws, int B, int L,
                      const tpl_options &opt, cudaStream_t st);
int a2b_backward_chain(float *grad_angles, const float *grad_coords, const float *angles, const int32_t *lengths,
                       void *ws, int B, int L, const tpl_options &opt, cudaStream_t st);
int a2b_chain_record_stride();
// Backward from the forward's output coordinates (no re-walk; tpl_a2b_chain.cu).
int a2b_backward_coords(float *grad_angles, const float *grad_coords, const float *coords, const int32_t *lengths,
                        void *ws, int B, int L, const tpl_options &opt, cudaStream_t st);
int sincos_poly_f32(const float *a, float *s, float *c, int n, cudaStream_t st);
size_t a2b_ws(int B, int L, const tpl_options &o);  // workspace bytes of the FP32 Angles2Backbone entries
tpl_options resolve(const tpl_options *opt);
bool options_ok(const tpl_options &o);

// Angles2Coords launchers (tpl_a2c.cu).  ws holds at least a WsHeader (status word).
int a2c_forward(bool f64, const unsigned char *seq, int seq_stride, const void *angles, void *coords,
                uint32_t *res_names, uint32_t *atom_names, void *ws, int B, int L, int maxA,
                const tpl_options &opt, cudaStream_t st);
int a2c_backward_coords(float *grad_angles, const float *grad_coords, const float *coords, const unsigned char *seq,
                        int seq_stride, void *ws, int B, int L, int maxA, cudaStream_t st);
int a2c_backward(bool f64, void *grad_angles, const void *grad_coords, const unsigned char *seq, int seq_stride,
                 const void *angles, void *ws, int B, int L, int maxA, const tpl_options &opt, cudaStream_t st);
int num_atoms_host(const char *seq);

// CoordsTransform launchers (tpl_transform.cu); T = float or double.
template <typename T>
int coords_shift(const T *in, T *out, const T *add, int scale_by_count, const int *num_atoms, int B, int stride,
                 cudaStream_t st);
template <typename T>
int coords_rotate(const T *in, T *out, const T *R, int transpose, const int *num_atoms, int B, int stride,
                  cudaStream_t st);
template <typename T>
int coords_center(const T *in, T *center, const int *num_atoms, int B, int stride, cudaStream_t st);
template <typename T>
int coords_bbox(const T *in, T *lo, T *hi, const int *num_atoms, int B, int stride, cudaStream_t st);

// Coords2TypedCoords launchers (tpl_typed.cu); ws holds at least a WsHeader.
int typed_forward(bool f64, const void *coords, const uint32_t *res_names, const uint32_t *atom_names,
                  const int *num_atoms, int B, int in_stride, int out_stride, void *out, int *n_of_type, int *offsets,
                  int *atom_index, void *ws, cudaStream_t st);
int typed_backward(bool f64, const void *grad_typed, void *grad_flat, const int *n_of_type, const int *atom_index,
                   int B, int in_stride, int out_stride, cudaStream_t st);

// Coords2RMSD launchers (tpl_rmsd.cu).
int rmsd_forward(bool f64, const void *src, const void *dst, const int *num_atoms, int B, int stride, int center,
                 void *rmsd, void *ut, double *centroids, void *ws, cudaStream_t st);
int rmsd_backward(bool f64, const void *grad_rmsd, const void *src, const void *dst, const int *num_atoms,
                  const void *rmsd, const void *ut, const double *centroids, int B, int stride, int center,
                  void *grad_src, cudaStream_t st);

}  // namespace tpl
