/*
 * gisapr_gb300.h -- C ABI of the GB300 (sm_103a) candidate-scoring engine.
 *
 * Every pointer argument is a device pointer unless noted, every size is in
 * elements, arrays are dense C order, complex values are interleaved float
 * pairs (torch.complex64 layout). Work is enqueued on ``stream`` (a
 * cudaStream_t passed as void*; NULL is the legacy default stream) and the
 * calls return before it finishes. Each call returns GISAPR_OK or an error
 * code; gisapr_last_error() gives the message of the calling thread's last
 * failure. A context owns cuFFT plans, lookup tables and scratch buffers for
 * one device; it is not thread-safe, so use one context per host thread.
 * Scratch grows on first use of a size, so warm a size up once before
 * capturing a call into a CUDA graph.
 *
 * Each entry point names the reference interface it replaces. File paths are
 * those of GisAPR's sources: "v606" is
 * test1_with_isspa_weight_varingKK_search_translation_also_v606_torch_
 * optimized_standalone.py; "ZL/" is the GisAPR-Lite-v1.3.2 tree.
 */
#ifndef GISAPR_GB300_H
#define GISAPR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  GISAPR_OK = 0,
  GISAPR_ERR_ARGUMENT = 1,    /* bad size, shape or null pointer (Python: ValueError) */
  GISAPR_ERR_CUDA = 2,        /* CUDA runtime / launch failure (Python: RuntimeError) */
  GISAPR_ERR_CUFFT = 3,       /* cuFFT failure */
  GISAPR_ERR_UNSUPPORTED = 4  /* a size the library does not implement */
};

typedef struct gisapr_context* gisapr_ctx;

/* ABI version of this header (major * 100 + minor). */
int gisapr_abi_version(void);

/* Message of the calling thread's last failed call ("" if none). */
const char* gisapr_last_error(void);

/* Create / destroy a context bound to CUDA device ``device``. */
int gisapr_context_create(int device, gisapr_ctx* out);
int gisapr_context_destroy(gisapr_ctx ctx);

/*
 * Add Gaussian atoms to ``volume`` [box][box][box] in place.
 * Replaces the NVRTC kernel ``deposit(xyz, numbers, volume, n, box, width,
 * apix, rp, kn)`` of ZL/gisapr_cuda_density.py:21-55 (launched by
 * accumulate, :177-200) and the index_add_ loop of
 * pdb2mrc_gpu_ver_fp32_v3.py:71-97. xyz [n][3] float32 Angstrom, numbers [n]
 * float32 atomic numbers (0 = no density). Atoms are summed per voxel in
 * input order.
 */
int gisapr_deposit(gisapr_ctx ctx, void* stream, const float* xyz, const float* numbers, int n_atoms,
                   float* volume, int box, int width, double apix, double rp, double kn);

/*
 * gisapr_deposit without any device allocation. Same inputs, result and
 * per-voxel atom order as gisapr_deposit, for callers that cannot allocate
 * device memory (memory owned by another framework's pool, code running
 * while a CUDA graph is captured, loops that cannot take the device-wide
 * synchronisation of a cudaMalloc). This entry point has no counterpart in
 * the reference. Its per-atom scratch is a fixed array of 65,536 records
 * (3 MiB) in the library's static device memory, held by every GPU that
 * loads the library until the process exits; more atoms per call are
 * rejected with GISAPR_ERR_ARGUMENT. No context is needed. The first call
 * on a device resolves the array's device address and loads the two kernels
 * with that device current (a call with n_atoms == 0 does this too and
 * launches nothing), so make that first call before capturing a stream.
 * apix, rp and kn must be positive and finite. All calls share the
 * array: calls whose work overlaps on the GPU (other streams, other host
 * threads) race on it, so serialise them.
 */
int gisapr_deposit_noalloc(void* stream, const float* xyz, const float* numbers, int n_atoms,
                           float* volume, int box, int width, double apix, double rp, double kn);

/*
 * Density of a rigidly moved chain on top of a fixed context:
 * out = fixed + splat(q), q = pdb_8.3((xyz - pivot) @ rot + pivot + shift).
 * Replaces RigidDensityCache.generate (ZL/gisapr_batch_density.py:57-117)
 * with transformed_density_atoms / quantize_coordinates
 * (ZL/pdb_text.py:33-58, 204-223). pivot [3] float32 (the float32 mean of
 * the chain's first-model atoms), rot [3][3] float64 row-major (applied as a
 * row vector times rot), shift [3] float64 Angstrom. ``fixed`` may be NULL
 * (zeros); ``out`` may be NULL when only the FFT input is wanted.
 * ``write_padded`` != 0 also writes the sinc^2-weighted, zero-padded,
 * fftshifted (2*box)^3 volume into the context's FFT input for
 * gisapr_volume_spectrum(ctx, stream, NULL, ...).
 */
int gisapr_deposit_moved(gisapr_ctx ctx, void* stream, const float* xyz, const float* numbers,
                         int n_atoms, const float* pivot, const double* rot, const double* shift,
                         const float* fixed, float* out, int write_padded, int box, int width,
                         double apix, double rp, double kn);

/*
 * Half-volume spectrum of a box^3 density: pad box/2 per side, multiply by
 * sinc^2(|f|), fftshift, 3-D R2C (cuFFT). Replaces v606:1063-1073
 * (IntegratedProjector.build_templates pre-amble with
 * apply_sinc2_filter_inplace_3d, v606:837-853). ``volume`` NULL uses the
 * FFT input last written by gisapr_deposit_moved(..., write_padded=1).
 * spectrum: [2*box][2*box][box+1] complex, NOT fftshifted (the projector
 * applies the reference's (z, y) shift when it samples).
 */
int gisapr_volume_spectrum(gisapr_ctx ctx, void* stream, const float* volume, int box,
                           float* spectrum);

/*
 * The half-volume spectrum of gisapr_volume_spectrum for a power-of-two box
 * (32..256), computed from the box^3 density without the (2*box)^3 padded
 * volume (each 2N-point transform of N nonzero samples as two N-point ones)
 * and kept in the context in the blocked layout the slice gather reads, for
 * gisapr_project_templates with spectrum == NULL. Replaces the same
 * reference steps as gisapr_volume_spectrum (v606:1063-1073). volume:
 * [box][box][box] float32.
 */
int gisapr_volume_spectrum_blocked(gisapr_ctx ctx, void* stream, const float* volume, int box);

/*
 * Templates of ``n_build`` directions. Replaces the slice gather and the
 * per-orientation tail of IntegratedProjector.build_templates
 * (v606:1075-1147) with ProjectionWhitening (v606:899-992).
 * rot [n_dir][3][3] float32 (rotation_matrices_t), dirs [n_build] int32
 * direction indices, out_slot [n_build] int32 rows of ``bank`` to write (NULL:
 * row = dirs[i]), mask [box][box] float32 or NULL, fsc [newbox][newbox/2+1]
 * float32 packed FSC, bank [..][newbox][newbox/2+1] complex pre-shifted
 * packed templates. box: power of two, 32..256, or 96 or 192; newbox:
 * even, <= box, multiple of 16. spectrum NULL (power-of-two boxes): the
 * context's blocked spectrum of this box, as gisapr_volume_spectrum_blocked
 * or the last projector call with a spectrum left it.
 */
int gisapr_project_templates(gisapr_ctx ctx, void* stream, const float* spectrum, int box,
                             const float* rot, const int* dirs, int n_build, const int* out_slot,
                             const float* mask, const float* fsc, int newbox, float* bank);

/*
 * Failure reporting of the shared-memory projector (boxes 32, 64, 128): each
 * template's plane arrives in shared memory by bulk copies whose wait is
 * bounded. When a wait runs out, the CTA sets the context's projector
 * status word to 1, lets its copy land, writes NaN into the templates it
 * still had to build and returns, so scores computed from them are NaN.
 * gisapr_projector_status copies the word into *value (0 when no
 * projector call ran), resets it to 0 and synchronizes ``stream`` (the
 * stream the projector calls ran on). gisapr_set_projector_wait sets the
 * bound for later calls on the context: attempts < 0 restores the default
 * (2^24), 0 makes the wait give up at once (a way to exercise the failure
 * path without a fault). Neither has a counterpart in the reference, whose
 * projector has no bounded waits.
 */
int gisapr_projector_status(gisapr_ctx ctx, void* stream, int* value);
int gisapr_set_projector_wait(gisapr_ctx ctx, long long attempts);

/*
 * Kernel launches one gisapr_project_templates call of ``n_build``
 * templates enqueues at ``box`` (0 for n_build <= 0; -1 for an unsupported
 * box). Host only, no context; lets a caller count its launches or size a
 * captured graph. This query has no counterpart in the reference.
 */
int gisapr_project_launches(int box, int n_build);

/*
 * CTF * ISSPA weight per particle in the packed layout. Replaces
 * PackedCTFTorch.batch (v606:781-829). dfu/dfv/dfa [n] float32 (Angstrom,
 * degrees); tx, ty, tu4, tnc [K] float32 static tables (packed frequency x,
 * y, u^4 and the ISSPA noise curve, v606:745-777); out [n][K] float32.
 */
int gisapr_packed_ctf(void* stream, const float* dfu, const float* dfv, const float* dfa, int n,
                      const float* tx, const float* ty, const float* tu4, const float* tnc, int K,
                      float k1, float k2, float k3, float k5, float kk, float* out);

/*
 * Particle spectra for n particles x n_psi in-plane angles. Replaces
 * ParticleFourierPreparer.prepare (v606:1340-1374) with PsiGridBank
 * (v606:1193-1256). images [n][box][box] float32; psi_index [n][n_psi] int32
 * rows of psi_table [n_angles][4] float32 (cos, sin, offset_row, offset_col
 * of each effective psi, as PsiGridBank builds them); mask [box][box] or
 * NULL; ctf [n][newbox][newbox/2+1]; out [n][n_psi][newbox][newbox/2+1]
 * complex, conjugated, L2-normalised and pre-shifted.
 */
int gisapr_prepare_particles(gisapr_ctx ctx, void* stream, const float* images, int n, int n_psi,
                             const int* psi_index, const float* psi_table, const float* mask,
                             const float* ctf, int box, int newbox, float* out);

/*
 * For every particle b and every local direction entry e in
 * [local_ptr[b], local_ptr[b+1]) and psi s: the maximum of 1024 * n^2 *
 * irfft2(T[local_idx[e]] * P[b][s]) over the centred crop x crop window,
 * with its row-major first argmax. Replaces correlate_templates_and_particle
 * (v606:1418-1449) for a whole particle set. bank [..][n][n/2+1] and
 * stack [n_particles][n_psi][n][n/2+1] complex pre-shifted; local_ptr
 * [n_particles+1], local_idx [nnz] int32; out_score [nnz][n_psi] float32,
 * out_y / out_x [nnz][n_psi] int32 crop indices. crop: even, 2..16.
 */
int gisapr_correlate(gisapr_ctx ctx, void* stream, const float* bank, const float* stack,
                     const int* local_ptr, const int* local_idx, int n_particles, int n_psi, int n,
                     int crop, float* out_score, int* out_y, int* out_x);

/*
 * gisapr_correlate for n_cand candidates at once: candidate c's template bank
 * starts bank_stride complex elements after candidate c-1's, and its outputs
 * follow the previous candidate's (out_score [n_cand][nnz][n_psi]). Each
 * particle's spectra are staged on chip once for all candidates. nnz =
 * local_ptr[n_particles], passed so that no value is read back during graph
 * capture. Replaces the candidate loop of the Lite tree's round-batched
 * search (ZL/gisapr_batch_search.py:314-349).
 */
int gisapr_correlate_batch(gisapr_ctx ctx, void* stream, const float* bank, long long bank_stride, int n_cand,
                           const float* stack, const int* local_ptr, const int* local_idx, int n_particles,
                           int nnz, int n_psi, int n, int crop, float* out_score, int* out_y, int* out_x);

/*
 * Particle subsets per candidate. subset [n_cand][n_particles] (bytes,
 * device memory; NULL = every candidate scores every particle): candidate c
 * scores particle b when subset[c][b] != 0. The reference's round-batched
 * search scores every candidate on the job's whole particle set
 * (ZL/gisapr_batch_search.py:314-349, 361); a candidate with a subset gets
 * what that search gives on a job holding only those particles.
 *   gisapr_correlate_batch_subset: gisapr_correlate_batch that skips the
 *     (candidate, particle) pairs left out (their map entries are left
 *     as they were; a particle no candidate scores is not read).
 *   gisapr_particle_results_subset: a pair left out gets the record of a
 *     particle without directions (best_entry -1).
 *   gisapr_score_sum_subset: the sum over the candidate's particles only.
 * The mask is read when the kernels run, so a captured CUDA graph that names
 * it takes new subsets written between replays.
 */
int gisapr_correlate_batch_subset(gisapr_ctx ctx, void* stream, const float* bank, long long bank_stride,
                                  int n_cand, const float* stack, const int* local_ptr, const int* local_idx,
                                  int n_particles, int nnz, int n_psi, int n, int crop, const unsigned char* subset,
                                  float* out_score, int* out_y, int* out_x);
int gisapr_particle_results_subset(void* stream, const int* local_ptr, const float* score, const int* ys,
                                   const int* xs, int n_particles, int n_psi, int n_cand,
                                   const unsigned char* subset, int* best_entry, int* best_psi, float* peak,
                                   int* peak_y, int* peak_x, float* zscore);
int gisapr_score_sum_subset(void* stream, const int* local_ptr, const float* peak, int n_particles, int n_cand,
                            const unsigned char* subset, double* out);

/*
 * Launch-shape knobs of a context per transform size, chosen by the
 * autotuner (gisapr_gb300/autotune.py); no counterpart in the reference.
 *   GISAPR_TUNE_CORR_CLUSTER: CTAs per particle (thread-block cluster size,
 *     1..8; 0 = the default) of gisapr_correlate and gisapr_correlate_batch
 *     at correlation size ``size``. Results do not depend on it beyond
 *     float32 summation order of the cluster's partial maps.
 *   GISAPR_TUNE_TC_A_STAGES / GISAPR_TUNE_TC_B_STAGES: shared-memory ring
 *     depths of the tensor-core correlation at particle size ``size`` (A:
 *     bulk-copied template rows, 2..8; B: built particle rows, 2..3; 0 =
 *     the default: B two deep, A as deep as the shared memory allows).
 *     Depths that do not fit are reduced. Results do not depend on them.
 */
enum { GISAPR_TUNE_CORR_CLUSTER = 1, GISAPR_TUNE_TC_A_STAGES = 2, GISAPR_TUNE_TC_B_STAGES = 3 };
int gisapr_set_tuning(gisapr_ctx ctx, int key, int size, int value);
int gisapr_get_tuning(gisapr_ctx ctx, int key, int size, int* value);

/*
 * Tensor-core form of gisapr_correlate_batch (tcgen05 MMA, FP32 accumulate),
 * same inputs and output layout. The stage that contracts template and
 * particle columns over rows runs as a real GEMM on 16-bit operands, scaled
 * by 2^13 times a power of two per packed column. Replaces the same
 * reference interfaces as gisapr_correlate_batch (v606:1418-1449 per
 * candidate; ZL/gisapr_batch_search.py:314-349 for the candidate loop); the
 * precision modes have no reference counterpart:
 *   GISAPR_TC_FP16    fp16 operands, hi*hi only;
 *   GISAPR_TC_FP16X3  fp16 hi/lo split, hi*hi + hi*lo + lo*hi (about 22
 *                     significant bits per product);
 *   GISAPR_TC_BF16    bf16 operands, hi*hi only;
 *   GISAPR_TC_BF16X3  bf16 hi/lo split (about 16 significant bits).
 *   tbank: caller scratch of n_cand * gisapr_tc_bank_bytes(n_slot, n) bytes,
 *     rewritten on every call (the operand copy of the banks);
 *   work, n_work: device copy of the list made by gisapr_tc_plan_work
 *     (host arrays in, host array out: [n_work][2] (particle, tile of 128
 *     rows * psi groups + group of psi angles: three, two at crop 14),
 *     sorted by direction; work == NULL only counts; n_psi and crop must
 *     match the correlation call);
 *   col_scale_t, col_scale_p: device float [n/2+1] per stored bank column,
 *     powers of two multiplying the template and the particle operands
 *     (undone after accumulation), or NULL for 1;
 *   wait_limit: bound (iterations) of every on-chip hand-off wait, 0 for
 *     the default; on a timeout the kernel stops, waits for its own copies
 *     and MMAs in flight with the default bound and returns;
 *   status: device int; 1 if an on-chip barrier wait ran out (the outputs
 *     are then incomplete), 2 if a scaled template value left the operand
 *     type's range; the caller zeroes it.
 * Sizes: n in {32, 64, 96, 128, 192, 256}, crop even in 2..14 (10..14 at n = 256),
 * n_cand <= 128 per call (the
 * work list is planned for that n_cand: a tile holds 128 / ceil8(n_cand)
 * whole directions). gisapr_correlate_tc_batch is the _ex call with
 * split != 0 -> GISAPR_TC_FP16X3, else GISAPR_TC_FP16, no column scales and
 * the default wait bound.
 */
enum { GISAPR_TC_FP16 = 0, GISAPR_TC_FP16X3 = 1, GISAPR_TC_BF16 = 2, GISAPR_TC_BF16X3 = 3 };
long long gisapr_tc_bank_bytes(int n_slot, int n);
int gisapr_tc_plan_work(const int* local_ptr, const int* local_idx, int n_particles, int n_cand, int n_psi,
                        int crop, int* work, int max_work, int* n_work);
int gisapr_correlate_tc_batch(gisapr_ctx ctx, void* stream, const float* bank, long long bank_stride, int n_cand,
                              int n_slot, void* tbank, const float* stack, const int* local_ptr,
                              const int* local_idx, const int* work, int n_work, int nnz, int n_psi, int n, int crop,
                              int split, float* out_score, int* out_y, int* out_x, int* status);
int gisapr_correlate_tc_batch_ex(gisapr_ctx ctx, void* stream, const float* bank, long long bank_stride,
                                 int n_cand, int n_slot, void* tbank, const float* stack, const int* local_ptr,
                                 const int* local_idx, const int* work, int n_work, int nnz, int n_psi, int n,
                                 int crop, int precision, const float* col_scale_t, const float* col_scale_p,
                                 unsigned wait_limit, float* out_score, int* out_y, int* out_x, int* status);

/*
 * Per particle: first maximum over (local entry, psi), its crop position and
 * the z-score (peak - mean) / population sigma over all the particle's
 * scores. Replaces the numeric part of make_result_records (v606:1466-1491).
 * best_entry is a global entry index (-1 for a particle without directions).
 */
int gisapr_particle_results(void* stream, const int* local_ptr, const float* score, const int* ys,
                            const int* xs, int n_particles, int n_psi, int* best_entry,
                            int* best_psi, float* peak, int* peak_y, int* peak_x, float* zscore);

/* gisapr_particle_results for n_cand candidates laid out one after another. */
int gisapr_particle_results_batch(void* stream, const int* local_ptr, const float* score, const int* ys,
                                  const int* xs, int n_particles, int n_psi, int n_cand, int* best_entry,
                                  int* best_psi, float* peak, int* peak_y, int* peak_x, float* zscore);

/*
 * Candidate score sum over particles with directions of exp(peak / 1024),
 * float64 into out[0]. Replaces ZL/gisapr_batch_search.py:361 and the
 * "CC + simple sum" mode of new_method_to_fit_the_2nd_Gaussian_PEAK_v4.py:
 * 133-134.
 */
int gisapr_score_sum(void* stream, const int* local_ptr, const float* peak, int n_particles,
                     double* out);

/* gisapr_score_sum for n_cand candidates: peak [n_cand][n_particles], out [n_cand]. */
int gisapr_score_sum_batch(void* stream, const int* local_ptr, const float* peak, int n_particles, int n_cand,
                           double* out);

/*
 * Particle stack preparation (read_star_shift_crop_and_generate_new_star_v5.py:
 * 9-29, 42-134, 183-237), in float64. images: n float32 [h][w] images;
 * shifts: per image the integer shift {x, y} (the reference rounds
 * rlnOrigin/apix with floor(v + 0.5)), or NULL for none; the shifted image
 * (zero fill) is cropped to the centred ch x cw window, then flags select:
 * 1 = divide by the radial mean amplitude spectrum (getSpectrum_divideBy
 * Spectrum; bin tables: CSR bin_ptr[n_bins + 1] / bin_pix of row-major pixel
 * indices of the unshifted transform grid per bin round(centred radius),
 * bin_count = pixels per bin), 2 = least-squares plane removal and mean/sigma
 * normalisation (normalize), 4 = high-pass by highpass_mask (ch*cw doubles,
 * unshifted order). work: n*ch*cw*2 doubles; out: n float32 ch x cw images.
 * Every pointer but shifts is device memory.
 */
int gisapr_ingest_stack(gisapr_ctx ctx, void* stream, const float* images, int n, int h, int w, const int* shifts,
                        int ch, int cw, int flags, const int* bin_ptr, const int* bin_pix, const double* bin_count,
                        int n_bins, const double* highpass_mask, double* work, float* out);

/*
 * Geometric restraint (func_check_boundary_for_testing_v8.py:62-126,
 * GeometryRestraint). gisapr_restraint_edt thresholds the main-body density
 * [box]^3 (voxel > threshold) into mask (u8) and writes d2: per voxel the
 * exact squared Euclidean distance, in voxels, to the nearest mask voxel
 * (scipy distance_transform_edt(~mask) squared; 2^29 where the mask is
 * empty). scratch: box^3 ints. Replaces GeometryRestraint.__init__'s mask
 * and distance transform (v8:83-94).
 */
int gisapr_restraint_edt(gisapr_ctx ctx, void* stream, const float* density, int box, float threshold,
                         unsigned char* mask, int* d2, int* scratch);

/* out[3 * i + 0..2] = {0, INT_MAX, 0} for i < n (the reduction identities). */
int gisapr_restraint_init(void* stream, int* out, int n);

/*
 * One candidate (v8:96-126): over the half-open voxel box bounds = {z0, y0,
 * x0, z1, y1, x1} (host memory) of the chain density in volume (the moved chain splatted
 * with gisapr_deposit onto zeros), adds to out[0] the voxels above threshold
 * where mask is set (overlap), lowers out[1] to the minimum d2 of voxels
 * above threshold and sets out[2] if there is any. Every voxel read is reset
 * to zero, so volume is all-zero again when the chain lay inside bounds.
 */
int gisapr_restraint_eval(gisapr_ctx ctx, void* stream, float* volume, const unsigned char* mask, const int* d2,
                          int box, const int* bounds, float threshold, int* out);

#ifdef __cplusplus
}
#endif

#endif /* GISAPR_GB300_H */
