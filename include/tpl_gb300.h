/*
 * tpl_gb300.h -- C ABI of the GB300 (sm_103a) chain-kinematics library
 * (libtpl_gb300.so).
 *
 * The library replaces the compute behind TorchProteinLibrary's two
 * internal-coordinate layers:
 *   ReducedModel.Angles2Backbone  (phi, psi, omega + lengths -> N, CA, C coords)
 *   FullAtomModel.Angles2Coords   (8 angles + sequences -> heavy-atom coords)
 * Each entry point below names the reference interface it stands in for
 * (paths relative to the reference project).
 *
 * Conventions
 *   - Plain pointers, sizes and a CUDA stream passed as `void *` (a cudaStream_t;
 *     NULL = legacy default stream).  No torch types.
 *   - Every pointer argument is a DEVICE pointer unless stated otherwise.
 *   - Layouts are the reference's: angles [batch, rows, max_len] row-major,
 *     coordinates [batch, 3 * atoms] with xyz interleaved, lengths int32.
 *   - The caller owns every buffer, including the workspace.  Entry points are
 *     asynchronous: they enqueue work on `stream` and return a tpl_status that
 *     covers argument checks and the launch itself.  Errors the kernels detect
 *     (a length outside [0, max_len], a look-back wait that timed out) are
 *     recorded in the workspace; tpl_workspace_status() reads them back.
 *   - No entry point allocates device memory or synchronises the stream,
 *     except tpl_workspace_status().
 */
#ifndef TPL_GB300_H
#define TPL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tpl_status {
    TPL_OK = 0,
    TPL_ERR_ARGUMENT = -1,          /* null pointer, negative size, bad option */
    TPL_ERR_WORKSPACE = -2,         /* workspace missing or too small */
    TPL_ERR_LAUNCH = -3,            /* CUDA reported an error at launch */
    TPL_ERR_LENGTH = -4,            /* a chain length outside [0, max_len] (device-detected) */
    TPL_ERR_SEQUENCE = -5,          /* a residue letter outside the 20 standard ones */
    TPL_ERR_LOOKBACK_TIMEOUT = -6,  /* a bounded device wait gave up: inter-tile look-back or bulk copy */
    TPL_ERR_ATOMS = -7,             /* a chain needs more atom slots than max_atoms */
    TPL_ERR_UNSUPPORTED = -8,       /* option combination without a compiled kernel */
    TPL_ERR_TOO_LARGE = -9,         /* problem exceeds the fixed scratch of tpl_a2b_forward_f32_noalloc */
    TPL_ERR_ATOM_TYPE = -10,        /* a (residue, atom) name pair outside the 11-type table */
    TPL_ERR_IO = -11                /* a file could not be opened */
} tpl_status;

/* Tuning knobs.  A NULL options pointer, or a zero field, selects the tuned default. */
typedef struct tpl_options {
    int residues_per_thread;   /* residues each thread scans serially: 1, 2, 4 or 8 (4 or 8 when
                                  threads_per_cta = 32 or 4) */
    int threads_per_cta;       /* scan scheme of Angles2Backbone FP32: 0 = automatic (one warp per
                                  chain when the batch has at least two chains per SM and
                                  residues_per_thread is 0, 4 or 8; warp tiles otherwise);
                                  32 = one warp walks a whole chain in chunks of 32 R residues (no
                                  look-back; the forward records the chain frame every 128
                                  residues in the workspace and the backward starts from those
                                  records); 4 = one CTA of four warps per chain, chunk k on warp
                                  k % 4, the chain frame handed from warp to warp in shared memory
                                  (same records); 1 = warp-granular tiles of 32 R residues joined by
                                  look-back; 128 = CTA tiles of 128 R residues.  Angles2Coords
                                  reads it as its threads per chain (0 = 256, 128, 256, 512). */
    int fp64_carry_min_len;    /* chains at least this long compose inter-tile carries in FP64.
                                  Tile schemes: 0 = default (always), -1 = never.  Four warps per
                                  chain: a positive length hands the chain frame from warp to warp
                                  in FP64; 0 (the default) and -1 keep it in FP32 (the tuned
                                  choice: the FP64 carry does not lower the error measurably).  One
                                  warp per chain keeps its frame in FP32. */
    int renormalize;           /* 0 = default (on), 1 = on, -1 = off: Newton-Schulz renormalisation
                                  of scan aggregates */
    int max_ctas;              /* cap on persistent CTAs; 0 = occupancy-derived */
    int copy_buffers;          /* chunk buffers of tpl_a2b_backward_coords_f32: 0 = default (1),
                                  1 = copy then evaluate, 2 = the next chunk's bulk copies in flight
                                  while a chunk is evaluated (residues_per_thread 4 only) */
} tpl_options;

/* Human-readable text for a tpl_status value (host). */
const char *tpl_status_string(int status);

/* Library version, major * 10000 + minor * 100 + patch (host). */
int tpl_version(void);

/* Bytes of workspace the Angles2Backbone FP32 entry points need for a batch of
 * `batch` chains stored with stride `max_len` (host). */
size_t tpl_a2b_workspace_bytes(int batch, int max_len, const tpl_options *opt);

/* Zero a workspace before its first use, or after an error (enqueued on stream). */
int tpl_workspace_init(void *workspace, size_t workspace_bytes, void *stream);

/* Synchronise `stream`, then return the first error the kernels recorded in
 * `workspace` (TPL_OK if none) through *status_out.  The recorded error is cleared. */
int tpl_workspace_status(void *workspace, void *stream, int *status_out);

/* Angles2Backbone forward, batched FP32.
 * Replaces Angles2BackboneGPU_forward (Layers/ReducedModel/Angles2Backbone/
 * angles2backbone_interface.cpp:7-26, kernel cBackboneProteinCUDAKernels.cu:6-41).
 *   angles  [batch, 3, max_len]  rows phi, psi, omega (radians)
 *   lengths [batch] int32        residues per chain, 0 <= lengths[b] <= max_len
 *   coords  [batch, 9 * max_len] N, CA, C xyz per residue; zero past 9 * lengths[b]
 * The workspace (the reference's `A` buffer) keeps one carry transform per tile
 * for the backward; it must be passed unchanged to tpl_a2b_backward_f32. */
int tpl_a2b_forward_f32(const float *angles, const int32_t *lengths, float *coords, void *workspace,
                        size_t workspace_bytes, int batch, int max_len, const tpl_options *opt, void *stream);

/* Angles2Backbone backward, batched FP32 adjoint.
 * Replaces Angles2BackboneGPU_backward (angles2backbone_interface.cpp:27-56,
 * kernels cBackboneProteinCUDAKernels.cu:84-163).  Writes dL/dangles
 * [batch, 3, max_len] (overwritten, zero past each length) from dL/dcoords
 * [batch, 9 * max_len].  No per-atom Jacobian (the reference's dr_dangle) is formed.
 * omega of each chain's last residue moves no atom; its gradient is 0 (the
 * reference reads one transform past the chain there). */
int tpl_a2b_backward_f32(float *grad_angles, const float *grad_coords, const float *angles,
                         const int32_t *lengths, void *workspace, size_t workspace_bytes, int batch, int max_len,
                         const tpl_options *opt, void *stream);

/* Angles2Backbone backward, batched FP32, from the forward's output coordinates.
 * Also replaces Angles2BackboneGPU_backward (angles2backbone_interface.cpp:27-56); the
 * reference's backward reads the forward's saved transforms `A`, whose translations
 * are these coordinates.  Same result as tpl_a2b_backward_f32 without recomputing
 * the chain: coords must be the unmodified output of tpl_a2b_forward_f32 for the
 * same angles and lengths.  It reads 36 B of coordinates per residue instead of
 * 12 B of angles and does a fraction of the arithmetic.  The workspace only needs
 * its status word (>= 64 bytes, zeroed once).  opt->residues_per_thread: 4 (default)
 * or 8 residues per lane; opt->threads_per_cta: 0 (default) or 32 = one warp per
 * chain, 4 = one CTA of four warps per chain with the carried sums handed from warp
 * to warp. */
int tpl_a2b_backward_coords_f32(float *grad_angles, const float *grad_coords, const float *coords,
                                const int32_t *lengths, void *workspace, size_t workspace_bytes, int batch,
                                int max_len, const tpl_options *opt, void *stream);

/* Angles2Backbone forward, plain FP64 form: one chain per CTA, one launch.
 * Same contract as tpl_a2b_forward_f32 in double precision; replaces
 * Angles2BackboneCPU_forward (angles2backbone_interface.cpp:60-80) on the GPU.
 * Needs no workspace. */
int tpl_a2b_forward_f64(const double *angles, const int32_t *lengths, double *coords, int batch, int max_len,
                        void *stream);

/* Angles2Backbone backward, plain FP64 form (replaces Angles2BackboneCPU_backward,
 * angles2backbone_interface.cpp:82-111).  The workspace needs
 * tpl_a2b_workspace_bytes(batch, max_len, NULL) bytes. */
int tpl_a2b_backward_f64(double *grad_angles, const double *grad_coords, const double *angles,
                         const int32_t *lengths, void *workspace, size_t workspace_bytes, int batch, int max_len,
                         void *stream);

/* Heavy atoms of a NUL-terminated one-letter sequence (host), or TPL_ERR_SEQUENCE
 * for a letter outside the 20 standard residues.  Replaces getSeqNumAtoms
 * (Layers/FullAtomModel/Angles2Coords/angles2coords_interface.cpp:139-144,
 * Math/nUtil.cpp:174-190; no terminal OXT). */
int tpl_num_atoms(const char *sequence);

/* Workspace bytes for the Angles2Coords entry points (a status word; the
 * full-atom kernels keep their carries on chip). */
size_t tpl_a2c_workspace_bytes(int batch, int max_len, int max_atoms, const tpl_options *opt);

/* Angles2Coords forward.  Replaces Angles2Coords_forward
 * (Layers/FullAtomModel/Angles2Coords/angles2coords_interface.cpp:8-74) with a GPU
 * path (the reference runs it on the CPU only).
 *   sequences  [batch, seq_stride] uint8, one NUL-terminated one-letter sequence per
 *              row (the chain length is the position of the NUL, at most max_len)
 *   angles     [batch, 8, max_len] rows phi, psi, omega, chi1..chi5; omega[i] is the
 *              dihedral between residues i and i+1
 *   coords     [batch, 3 * max_atoms] heavy-atom xyz in the reference's atom order,
 *              zero past each chain's atoms
 *   res_names, atom_names  [batch, max_atoms, 4] uint8 NUL-padded names, or both NULL
 *              to skip them (they depend on the sequences only)
 * Unknown letters, chains longer than max_len or with more than max_atoms atoms are
 * reported through the workspace status; such chains are zeroed.  One CTA walks a
 * chain (float32): opt->threads_per_cta 4 or 8 = four or eight warps on chunks of 32
 * residues, one per lane; 256 or 512 threads with one residue each; 128 threads with
 * two residues each; 0 (the default) = eight warps below 8 x (number of SMs) chains
 * (4 x with names), four from there.  float64 always uses 128 threads with one
 * residue each. */
int tpl_a2c_forward_f32(const uint8_t *sequences, int seq_stride, const float *angles, float *coords,
                        uint8_t *res_names, uint8_t *atom_names, void *workspace, size_t workspace_bytes, int batch,
                        int max_len, int max_atoms, const tpl_options *opt, void *stream);
int tpl_a2c_forward_f64(const uint8_t *sequences, int seq_stride, const double *angles, double *coords,
                        uint8_t *res_names, uint8_t *atom_names, void *workspace, size_t workspace_bytes, int batch,
                        int max_len, int max_atoms, const tpl_options *opt, void *stream);

/* Angles2Coords backward.  Replaces Angles2Coords_backward
 * (angles2coords_interface.cpp:76-115, cConformation.cpp:180-211): writes
 * dL/dangles [batch, 8, max_len] (overwritten) from dL/dcoords [batch, 3 * max_atoms].
 * Angles without a joint (omega of the last residue, chi angles a residue does not
 * have, Ala's chi1) and padding get 0, as in the reference. */
int tpl_a2c_backward_f32(float *grad_angles, const float *grad_coords, const uint8_t *sequences, int seq_stride,
                         const float *angles, void *workspace, size_t workspace_bytes, int batch, int max_len,
                         int max_atoms, const tpl_options *opt, void *stream);
int tpl_a2c_backward_f64(double *grad_angles, const double *grad_coords, const uint8_t *sequences, int seq_stride,
                         const double *angles, void *workspace, size_t workspace_bytes, int batch, int max_len,
                         int max_atoms, const tpl_options *opt, void *stream);

/* Angles2Coords backward, FP32, from the forward's output coordinates.  Also
 * replaces Angles2Coords_backward (angles2coords_interface.cpp:76-115,
 * cConformation.cpp:180-211), whose tree walk recomputes every joint transform.
 * Every joint's origin is an atom of the forward's output (N, CA and C for the
 * backbone; the first atom of each side-chain group) and every rotation axis is a
 * bond between two such atoms, so dL/dangle = u . sum over the joint's subtree of
 * (x - o) x g is evaluated from coords and grad_coords without rebuilding the
 * chain.  coords must be the unmodified output of tpl_a2c_forward_f32 for the same
 * sequences and angles.  Same outputs and zeros as tpl_a2c_backward_f32; the
 * gradient's error against FP64 is about 1e-5 of its largest entry, since the axes
 * come from FP32 coordinate differences.  The workspace only needs its status word
 * (>= 64 bytes, zeroed once).  Eight warps share a chain on chunks of 32 residues
 * below 4 x (number of SMs) chains, four from there. */
int tpl_a2c_backward_coords_f32(float *grad_angles, const float *grad_coords, const float *coords,
                                const uint8_t *sequences, int seq_stride, void *workspace, size_t workspace_bytes,
                                int batch, int max_len, int max_atoms, void *stream);

/* Angles2Backbone forward, batched FP32, for callers that cannot allocate device
 * memory.  This entry point has no counterpart in the reference.
 *
 * Some hosts cannot hand this library a workspace: a plugin or FFI caller that
 * only owns the input and output buffers it passes in, or a process whose
 * framework has already reserved the device memory, so that cudaMalloc fails.
 * This variant of tpl_a2b_forward_f32 takes the same inputs and outputs but keeps
 * its scratch (the look-back records of the tile scan) in a fixed 4 MiB array
 * that the library declares in device memory; every GPU that loads the library
 * holds that array until the process exits.  It calls no cudaMalloc or cudaFree.
 *
 *   - Size limit: 64 + 400 * batch * ceil(max_len / tile) bytes must fit in 4 MiB
 *     (tile = 32 * residues_per_thread for warp tiles, 128 * residues_per_thread for
 *     CTA tiles; 128 by default), e.g. 2048 chains of up to 640 residues.  Larger
 *     problems return TPL_ERR_TOO_LARGE before anything is enqueued.
 *   - The first call on a device looks up the array's device address on that
 *     device; make that first call before any CUDA stream capture.
 *   - All calls share the one array: it is cleared on `stream` at the start of every
 *     call, keeps the last call's contents afterwards, and calls that overlap on
 *     the GPU (two streams, or two host threads) race on it.
 *   - Its records are not kept for a backward pass: run tpl_a2b_forward_f32 with a
 *     workspace when the backward is needed.
 *   - The returned status covers the arguments and the launch.  Errors the kernels
 *     find on the device (a length outside [0, max_len], a bounded wait that gave
 *     up) are recorded in the array's status word; tpl_a2b_noalloc_status() reads
 *     them back.
 *   - The cached device address does not survive a cudaDeviceReset: do not call
 *     it across a device reset. */
int tpl_a2b_forward_f32_noalloc(const float *angles, const int32_t *lengths, float *coords, int batch, int max_len,
                                const tpl_options *opt, void *stream);

/* Error report of the last tpl_a2b_forward_f32_noalloc call on the current device.
 * This entry point has no counterpart in the reference.  It synchronises `stream`,
 * then returns through *status_out the first error the kernels recorded in the
 * fixed array (TPL_OK if none) and clears it; it allocates nothing.  The next
 * no-allocation call clears the record as well, so read it before that call. */
int tpl_a2b_noalloc_status(void *stream, int *status_out);

/* ---------------------------------------------------------------- CoordsTransform
 * Batched coordinate rows [batch, 3 * atoms_stride] (xyz per atom); the first
 * num_atoms[b] atoms of row b are transformed and the rest of the row is written
 * as zeros (the reference fills zero-initialised outputs).  Counts past
 * atoms_stride are clamped to it.  All entries launch on `stream` and return a
 * tpl_status.  _f64 variants take double.
 *
 * Translate: out = in + translation[b] (translation [batch, 3]); with
 * translation == NULL it is the masked copy that is the backward of
 * CoordsTranslateGPU_forward/_backward (Layers/FullAtomModel/CoordsTransform/
 * coordsTransformGPU_interface.cpp:8-56, kernels TransformCUDAKernels.cu:4-37). */
int tpl_coords_translate_f32(const float *in, float *out, const float *translation, const int32_t *num_atoms,
                             int batch, int atoms_stride, void *stream);
int tpl_coords_translate_f64(const double *in, double *out, const double *translation, const int32_t *num_atoms,
                             int batch, int atoms_stride, void *stream);
/* Rotate: out = R[b] in (transpose = 0, CoordsRotateGPU_forward) or R[b]^T in
 * (transpose = 1, CoordsRotateGPU_backward); rotation [batch, 3, 3] row-major.
 * Replaces coordsTransformGPU_interface.cpp:58-110, TransformCUDAKernels.cu:40-75. */
int tpl_coords_rotate_f32(const float *in, float *out, const float *rotation, int transpose,
                          const int32_t *num_atoms, int batch, int atoms_stride, void *stream);
int tpl_coords_rotate_f64(const double *in, double *out, const double *rotation, int transpose,
                          const int32_t *num_atoms, int batch, int atoms_stride, void *stream);
/* Centre: center[b] = mean of the first num_atoms[b] atoms (FP64 accumulation; 0 for
 * an empty chain, where the reference divides by zero), and its backward
 * grad_in[b, atom] = grad_center[b] / num_atoms[b].  Replaces Coords2CenterGPU_forward/
 * _backward (coordsTransformGPU_interface.cpp:112-160, TransformCUDAKernels.cu:77-107). */
int tpl_coords_center_f32(const float *in, float *center, const int32_t *num_atoms, int batch, int atoms_stride,
                          void *stream);
int tpl_coords_center_f64(const double *in, double *center, const int32_t *num_atoms, int batch, int atoms_stride,
                          void *stream);
int tpl_coords_center_backward_f32(const float *grad_center, float *grad_in, const int32_t *num_atoms, int batch,
                                   int atoms_stride, void *stream);
int tpl_coords_center_backward_f64(const double *grad_center, double *grad_in, const int32_t *num_atoms, int batch,
                                   int atoms_stride, void *stream);
/* Bounding box: lo[b] / hi[b] = per-coordinate min / max over the first
 * num_atoms[b] atoms (+inf / -inf for an empty chain).  Replaces getBBox
 * (coordsTransform_interface.cpp:175-200, Math/nUtil.cpp:27-57), which runs on the CPU. */
int tpl_coords_bbox_f32(const float *in, float *lo, float *hi, const int32_t *num_atoms, int batch,
                        int atoms_stride, void *stream);
int tpl_coords_bbox_f64(const double *in, double *lo, double *hi, const int32_t *num_atoms, int batch,
                        int atoms_stride, void *stream);

/* ------------------------------------------------------------- Coords2TypedCoords
 * Replaces Coords2TypedCoords_forward / _backward (Layers/FullAtomModel/
 * Coords2TypedCoords/coords2typedcoords_interface.cpp; atom types of
 * ProtUtil::get11AtomType, Math/nUtil.cpp:567-703), which run on the CPU.
 * Forward: the first num_atoms[b] atoms of coords [batch, 3 * in_stride] (names
 * res_names / atom_names [batch, in_stride, 4] bytes, as Angles2Coords writes them)
 * regrouped by type, stable within a type, into out [batch, 3 * out_stride];
 * num_atoms_of_type / offsets int32 [batch, 11]; atom_indexes int32
 * [batch, out_stride] (typed slot -> input atom).  Unused slots are zero.  An
 * unknown name pair is left out and records TPL_ERR_ATOM_TYPE in the workspace
 * (>= 64 bytes, zeroed once; read back with tpl_workspace_status).
 * Backward: grad_flat [batch, 3 * in_stride] = grad_typed scattered back through
 * atom_indexes, zero elsewhere. */
int tpl_typed_coords_forward_f32(const float *coords, const uint8_t *res_names, const uint8_t *atom_names,
                                 const int32_t *num_atoms, int batch, int in_stride, int out_stride, float *out,
                                 int32_t *num_atoms_of_type, int32_t *offsets, int32_t *atom_indexes,
                                 void *workspace, size_t workspace_bytes, void *stream);
int tpl_typed_coords_forward_f64(const double *coords, const uint8_t *res_names, const uint8_t *atom_names,
                                 const int32_t *num_atoms, int batch, int in_stride, int out_stride, double *out,
                                 int32_t *num_atoms_of_type, int32_t *offsets, int32_t *atom_indexes,
                                 void *workspace, size_t workspace_bytes, void *stream);
int tpl_typed_coords_backward_f32(const float *grad_typed, float *grad_flat, const int32_t *num_atoms_of_type,
                                  const int32_t *atom_indexes, int batch, int in_stride, int out_stride, void *stream);
int tpl_typed_coords_backward_f64(const double *grad_typed, double *grad_flat, const int32_t *num_atoms_of_type,
                                  const int32_t *atom_indexes, int batch, int in_stride, int out_stride, void *stream);

/* ------------------------------------------------------------------- PDB reading
 * Host functions (no GPU), the reader of PDB2CoordsUnordered
 * (Layers/FullAtomModel/PDB2Coords/pdb2coords_interface.cpp:75-127, parsing of
 * Layers/FullAtomModel/cPDBLoader.cpp:25-55): heavy-atom ATOM records (atom names
 * starting with C, N, O or S), coordinates parsed as float and widened to double,
 * names in NUL-padded 4-byte slots.  tpl_pdb_count_atoms gives one file's count;
 * tpl_pdb_read_batch fills rows of max_atoms atoms per file (coords
 * [batch, 3 max_atoms], names [batch, max_atoms, 4], res_nums [batch, max_atoms];
 * rows zero-padded) using `threads` host threads (0 = all cores).  It returns
 * TPL_ERR_IO if a file cannot be opened and TPL_ERR_ATOMS if a file holds more than
 * max_atoms atoms (num_atoms still reports the full count). */
int tpl_pdb_count_atoms(const char *filename, int32_t *num_atoms);
int tpl_pdb_read_batch(const char *const *filenames, int batch, int max_atoms, double *coords, uint8_t *chain_names,
                       uint8_t *res_names, int32_t *res_nums, uint8_t *atom_names, int32_t *num_atoms, int threads);

/* Diagnostics (no counterpart in the reference): s[i], c[i] = sin, cos of a[i] as
 * the FP32 Angles2Backbone kernels evaluate them (Cody-Waite reduction by pi/2 and
 * Taylor series), for n device floats on `stream`. */
int tpl_sincos_f32(const float *a, float *s, float *c, int n, void *stream);

/* Coords2RMSD forward: least RMSD between src and dst after optimal superposition
 * (quaternion method), per chain.  Replaces Coords2RMSDGPU_forward
 * (Layers/RMSD/Coords2RMSD/coords2rmsd_interface.cpp:52-111); center = 1 also folds
 * in the centring that Coords2RMSD.forward does with Coords2Center/CoordsTranslate
 * (TorchProteinLibrary/RMSD/Coords2RMSD/Coords2RMSD.py:71-78).
 *   src, dst   [batch, 3 * atoms_stride]   num_atoms int32 [batch]
 *   rmsd [batch], ut [batch, 3, 3] (the transposed rotation, as the reference's UT),
 *   centroids [batch, 6] doubles (src then dst centroid; may be NULL when center = 0) */
int tpl_rmsd_forward_f32(const float *src, const float *dst, const int32_t *num_atoms, int batch, int atoms_stride,
                         int center, float *rmsd, float *ut, double *centroids, void *workspace,
                         size_t workspace_bytes, void *stream);
int tpl_rmsd_forward_f64(const double *src, const double *dst, const int32_t *num_atoms, int batch, int atoms_stride,
                         int center, double *rmsd, double *ut, double *centroids, void *workspace,
                         size_t workspace_bytes, void *stream);

/* Coords2RMSD backward: dL/dsrc = dL/drmsd (x_i - UT y_i) / (rmsd N) on the centred
 * coordinates, zero past num_atoms.  Replaces Coords2RMSDFunction.backward
 * (TorchProteinLibrary/RMSD/Coords2RMSD/Coords2RMSD.py:40-62, a per-chain Python loop). */
int tpl_rmsd_backward_f32(const float *grad_rmsd, const float *src, const float *dst, const int32_t *num_atoms,
                          const float *rmsd, const float *ut, const double *centroids, int batch, int atoms_stride,
                          int center, float *grad_src, void *stream);
int tpl_rmsd_backward_f64(const double *grad_rmsd, const double *src, const double *dst, const int32_t *num_atoms,
                          const double *rmsd, const double *ut, const double *centroids, int batch, int atoms_stride,
                          int center, double *grad_src, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* TPL_GB300_H */
