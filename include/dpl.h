/*
 * dpl.h -- C ABI of the GB300 phase-linking library (libdpl.so).
 *
 * Every entry point takes DEVICE pointers, sizes, parameters and a CUDA stream,
 * enqueues its kernels on that stream and returns without synchronising (except
 * where noted).  No entry point allocates device memory: scratch space is passed
 * in by the caller (`workspace`, sized by the matching *_workspace_size call).
 * Arrays are C-contiguous; complex values are interleaved float pairs
 * (numpy complex64 layout, 8-byte aligned); boolean arrays are one byte per element
 * (0/1).  Workspaces are 16-byte aligned (CUDA allocations are 256-byte aligned).
 * A misaligned complex array or workspace is DPL_ERR_INVALID_ARGUMENT.
 *
 * Each function names the reference (dolphin) interface it replaces; paths are
 * relative to the dolphin source tree (src/dolphin/...).
 */
#ifndef DPL_H_
#define DPL_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A cudaStream_t (the CUDA runtime and driver handle types are the same pointer). */
typedef struct CUstream_st* dpl_stream_t;

typedef enum dpl_status {
    DPL_OK = 0,
    DPL_ERR_INVALID_ARGUMENT = 1, /* maps to ValueError */
    DPL_ERR_ALL_NAN_SLC = 2,      /* maps to PhaseLinkRuntimeError (phase_link/_core.py:564-571) */
    DPL_ERR_CUDA = 3,             /* a CUDA call failed; maps to RuntimeError */
    DPL_ERR_WORKSPACE = 4,        /* workspace smaller than *_workspace_size() */
    DPL_ERR_UNSUPPORTED = 5,      /* parameters outside the supported range (e.g. nslc > 64) */
    DPL_ERR_TIMEOUT = 6           /* a bounded device-side wait gave up; no result written */
} dpl_status;

/* Element types of raster arguments that accept several. */
typedef enum dpl_dtype {
    DPL_DTYPE_F32 = 0,
    DPL_DTYPE_U8 = 1,
    DPL_DTYPE_I8 = 2,
    DPL_DTYPE_I16 = 3,
    DPL_DTYPE_U16 = 4,
    DPL_DTYPE_I32 = 5
} dpl_dtype;

/* Message for the last non-OK status returned on the calling host thread. */
const char* dpl_last_error_message(void);

/* Library ABI version (major * 1000 + minor). */
int dpl_version(void);

/* Largest number of SLCs a phase-linking call accepts. */
int dpl_max_nslc(void);

/* ---------------------------------------------------------------------------------
 * Amplitude dispersion / PS selection.
 * Replaces: calc_ps_block(stack_mag, amp_dispersion_threshold, min_count)  -- ps.py:169-244
 *
 * stack_mag : (nslc, npix) float32, may hold NaN
 * mean      : (npix) float32 out  -- nanmean, NaN/inf -> 0
 * amp_disp  : (npix) float32 out  -- nanstd/nanmean, 0 where count < min_count
 * ps        : (npix) uint8 out    -- amp_disp < threshold and amp_disp != 0
 * The comparison is done in float32 against `threshold` (numpy's rule for a Python
 * float threshold); pass threshold_is_f64=1 to compare in float64 against
 * `threshold64` (numpy's rule for a numpy float64 threshold).
 * ------------------------------------------------------------------------------- */
dpl_status dpl_ps_block(const float* stack_mag, int64_t nslc, int64_t npix, float threshold,
                        int threshold_is_f64, double threshold64, int64_t min_count,
                        float* mean, float* amp_disp, uint8_t* ps, dpl_stream_t stream);

/* ---------------------------------------------------------------------------------
 * SHP selection by the GLRT on Rayleigh scale parameters.
 * Replaces: shp._glrt.estimate_neighbors(mean, var, halfwin_rowcol, strides, nslc, alpha)
 *           -- shp/_glrt.py:13-130 (dispatched from shp/__init__.py:83-99)
 *
 * mean, var : (rows, cols) float32
 * threshold : chi2.ppf(1 - alpha, df=1), rounded to float32 by the caller
 * is_shp    : (rows / sy, cols / sx, 2*hy+1, 2*hx+1) uint8 out
 * workspace : dpl_shp_glrt_workspace_size(rows, cols) bytes
 * ------------------------------------------------------------------------------- */
size_t dpl_shp_glrt_workspace_size(int64_t rows, int64_t cols);
dpl_status dpl_shp_glrt(const float* mean, const float* var, int64_t rows, int64_t cols, int hy,
                        int hx, int sy, int sx, int nslc, float threshold, uint8_t* is_shp,
                        void* workspace, size_t workspace_bytes, dpl_stream_t stream);

/* ---------------------------------------------------------------------------------
 * SHP selection by the two-sample Kolmogorov-Smirnov test.
 * Replaces: shp._ks.estimate_neighbors(amp_stack, halfwin_rowcol, alpha, strides, is_sorted)
 *           -- shp/_ks.py:22-98 with _set_neighbors / _get_max_cdf_dist (:139-218)
 *
 * amp_stack : (nslc, rows, cols) float32 (sorted along axis 0 if is_sorted)
 * cutoff    : critical ECDF distance (shp/_ks.py:221-239), float64
 * is_shp    : (rows / sy, cols / sx, 2*hy+1, 2*hx+1) uint8 out
 * workspace : dpl_shp_ks_workspace_size(nslc, rows, cols) bytes
 * ------------------------------------------------------------------------------- */
size_t dpl_shp_ks_workspace_size(int64_t nslc, int64_t rows, int64_t cols);
dpl_status dpl_shp_ks(const float* amp_stack, int64_t nslc, int64_t rows, int64_t cols, int hy,
                      int hx, int sy, int sx, double cutoff, int is_sorted, uint8_t* is_shp,
                      void* workspace, size_t workspace_bytes, dpl_stream_t stream);

/* ---------------------------------------------------------------------------------
 * Phase linking.
 * Replaces: phase_link.run_phase_linking(...)  -- phase_link/_core.py:67-249
 *           (run_cpl :252-376, process_coherence_matrices :379-534)
 * ------------------------------------------------------------------------------- */
typedef struct dpl_pl_params {
    int64_t nslc, rows, cols;      /* slc_stack shape */
    int hy, hx;                    /* half_window (y, x) */
    int sy, sx;                    /* strides (y, x) */
    int use_evd;                   /* 1: EVD for every pixel */
    double beta;                   /* |Gamma| regularisation (Python float; rounded like jax) */
    double zero_correlation_threshold;
    int reference_idx;             /* negative counts from the end */
    int mask_input_ps;
    int use_max_ps;
    int use_slc_amp;
    int baseline_lag;              /* <= 0: off */
    int first_real_slc_idx;
    int compute_crlb;
    int cov_form;                  /* 0: tensor-core covariance, bf16 hi/lo (default); 1: SIMT covariance (plain
                                      form); 2: covariance and solver in FP64 (the double-precision reference
                                      form); 3: tensor-core covariance with tf32 operands (one product) */
    /* Not in the reference (zero = default).  Register-solver instance: row slots K (even,
     * >= nslc; 0 = nslc rounded up to even) and threads per pixel (8, 16 or 32 for K <= 32,
     * at least K; 0 = the smallest power of two >= max(K, 8); K > 32 always uses two warps);
     * a tuner's choices: the same algorithm, group reductions may round differently. */
    int solver_slots;
    int solver_lanes;
    /* Not in the reference.  Pixels whose eigen-iteration misses the stopping rule within
     * 49 steps (the reference returns that last iterate, _eigenvalues.py:194-202):
     * 0 (default) -- solved again by a dense Hermitian eigensolver (|Gamma| inverted in
     * double precision; Householder tridiagonalisation, Sturm multisection and inverse
     * iteration for the wanted eigenpair) and flagged in outputs->nonconverged; 1 -- keep
     * the last iterate, as the reference does.  Applies to the tensor-core form (the
     * forms that store the coherence). */
    int nonconverged_mode;
} dpl_pl_params;

typedef struct dpl_pl_inputs {
    const float* slc;              /* (nslc, rows, cols) complex64 */
    const uint8_t* nodata_mask;    /* (rows, cols) or NULL */
    const uint8_t* ps_mask;        /* (rows, cols) or NULL */
    const uint8_t* neighbors;      /* (out_rows, out_cols, 2hy+1, 2hx+1) or NULL (rectangular window) */
    const float* avg_mag;          /* (rows, cols) or NULL (nanmean |slc| is used) */
} dpl_pl_inputs;

typedef struct dpl_pl_outputs {
    float* cpx_phase;              /* (nslc, out_rows, out_cols) complex64 */
    float* temp_coh;               /* (out_rows, out_cols) float32 */
    int32_t* shp_counts;           /* (out_rows, out_cols) int32; may be NULL when neighbors is NULL */
    float* eigenvalues;            /* (out_rows, out_cols) float32 */
    uint8_t* estimator;            /* (out_rows, out_cols) uint8: 0 EVD, 1 EMI */
    float* crlb_std_dev;           /* (nslc, out_rows, out_cols) float32 */
    float* closure_phases;         /* (out_rows, out_cols, nslc - 2) float32; may be NULL */
    uint8_t* nonconverged;         /* (out_rows, out_cols) uint8 or NULL (not in the reference): 1 where the
                                      dense eigensolver replaced an iterate that missed the stopping rule */
} dpl_pl_outputs;

size_t dpl_phase_link_workspace_size(const dpl_pl_params* params);

/* Enqueues the whole pipeline, then synchronises the stream once to report an
 * all-NaN SLC (DPL_ERR_ALL_NAN_SLC, with the reference's message) or a PS window
 * whose brightness is undefined (DPL_ERR_INVALID_ARGUMENT). */
dpl_status dpl_phase_link(const dpl_pl_params* params, const dpl_pl_inputs* inputs,
                          const dpl_pl_outputs* outputs, void* workspace,
                          size_t workspace_bytes, dpl_stream_t stream);

/* The two halves of dpl_phase_link (no reference counterpart: the reference runs
 * synchronously).  dpl_phase_link_async enqueues the pipeline and returns without
 * synchronising, so a sequence of calls (e.g. several ministacks) can be captured in a
 * CUDA graph; the per-call status stays in the workspace.  dpl_phase_link_status
 * synchronises `stream` and reports that status exactly as dpl_phase_link does. */
dpl_status dpl_phase_link_async(const dpl_pl_params* params, const dpl_pl_inputs* inputs,
                                const dpl_pl_outputs* outputs, void* workspace,
                                size_t workspace_bytes, dpl_stream_t stream);
dpl_status dpl_phase_link_status(const dpl_pl_params* params, void* workspace,
                                 size_t workspace_bytes, dpl_stream_t stream);

/* Deferred form of dpl_phase_link_status, for block loops that keep the host ahead of
 * the GPU (no reference counterpart).  dpl_phase_link_status_copy enqueues on `stream`
 * a copy of the call's three 32-bit status words from the workspace into `words`
 * (pinned host or device memory, 12 bytes); the workspace may be reused once the copy
 * has run.  After the caller has synchronised, dpl_phase_link_status_words maps the
 * host copy to the status and message dpl_phase_link would have returned. */
dpl_status dpl_phase_link_status_copy(const dpl_pl_params* params, void* workspace,
                                      size_t workspace_bytes, void* words, dpl_stream_t stream);
dpl_status dpl_phase_link_status_words(int64_t nslc, const void* words);

/* Batches (not in the reference's API; its sequential workflow runs one ministack after
 * another, workflows/sequential.py:105-147).  Enqueues `count` (<= 16) independent
 * dpl_phase_link calls -- ministacks of uneven N, each with its own params, inputs and
 * outputs -- on `stream` without synchronising.  The tensor-core covariance of all of
 * them is one persistent launch whose CTAs take (stack, 16x16-pixel tile) items from a
 * work queue, largest N first; the other stages run per stack.  The results are those
 * of the separate calls.  workspace: dpl_phase_link_batch_workspace_size bytes, 256-byte
 * aligned.  dpl_phase_link_batch_status synchronises `stream` and reports the first
 * failing call's error, in order, as dpl_phase_link would. */
size_t dpl_phase_link_batch_workspace_size(const dpl_pl_params* params, int count);
dpl_status dpl_phase_link_batch(const dpl_pl_params* params, const dpl_pl_inputs* inputs,
                                const dpl_pl_outputs* outputs, int count, void* workspace,
                                size_t workspace_bytes, dpl_stream_t stream);
dpl_status dpl_phase_link_batch_status(const dpl_pl_params* params, int count, void* workspace,
                                       size_t workspace_bytes, dpl_stream_t stream);

/* ---------------------------------------------------------------------------------
 * Stage entry points (used to check each stage against the oracle).
 * ------------------------------------------------------------------------------- */

/* Replaces: covariance.estimate_stack_covariance(slc_stack, half_window, strides,
 *           neighbor_arrays) -- phase_link/covariance.py:24-107.
 * C : (out_rows, out_cols, nslc, nslc) complex64 out.  NaN samples are masked. */
size_t dpl_covariance_workspace_size(int64_t nslc, int64_t rows, int64_t cols);
dpl_status dpl_covariance(const float* slc, int64_t nslc, int64_t rows, int64_t cols, int hy,
                          int hx, int sy, int sx, const uint8_t* neighbors, int cov_form, float* C,
                          void* workspace, size_t workspace_bytes, dpl_stream_t stream);

/* Replaces: _core.process_coherence_matrices(C_arrays, ...) -- phase_link/_core.py:379-534,
 *           followed by metrics.estimate_temp_coh (metrics.py:10-40) and
 *           compute_nearest_closure_phases_batch (_closure_phase.py:23-40).
 * C            : (npix, nslc, nslc) complex64 (baseline_lag, if any, already applied)
 * eig_vecs     : (npix, nslc) complex64 out, referenced to reference_idx
 * eig_vals     : (npix) float32;  estimator : (npix) uint8
 * crlb_std_dev : (npix, nslc) float32 (zeros if !compute_crlb)
 * temp_coh     : (npix) float32;  closure_phases : (npix, nslc - 2) float32 or NULL
 * num_looks    : sqrt(hy * hx) in the reference
 * workspace    : dpl_process_coherence_workspace_size(npix) bytes */
size_t dpl_process_coherence_workspace_size(int64_t npix);
dpl_status dpl_process_coherence(const float* C, int64_t npix, int nslc, int use_evd, double beta,
                                 double zero_correlation_threshold, int reference_idx,
                                 double num_looks, int first_real_slc_idx, int compute_crlb,
                                 float* eig_vecs, float* eig_vals, uint8_t* estimator,
                                 float* crlb_std_dev, float* temp_coh, float* closure_phases,
                                 void* workspace, size_t workspace_bytes, dpl_stream_t stream);

/* Replaces: _compress.compress(slc_stack, pl_cpx_phase, first_real_slc_idx, slc_mean,
 *           reference_idx) -- phase_link/_compress.py:11-65 (with utils.upsample_nearest,
 *           utils.py:281-324).
 * slc          : (nslc, rows, cols) complex64
 * pl_cpx_phase : (nslc, pl_rows, pl_cols) complex64, upsampled by block repetition
 *                (rows / pl_rows, cols / pl_cols), zero beyond the repeats
 * slc_mean     : (rows, cols) float32 in/out or NULL (then mean |z| over the real SLCs);
 *                set to NaN where the projected phase is exactly 0, as the reference does
 * has_reference: re-reference pl_cpx_phase to reference_idx (0 <= idx < nslc) first
 * comp_slc     : (rows, cols) complex64 out */
dpl_status dpl_compress(const float* slc, int64_t nslc, int64_t rows, int64_t cols,
                        const float* pl_cpx_phase, int64_t pl_rows, int64_t pl_cols,
                        int first_real_slc_idx, float* slc_mean, int has_reference,
                        int reference_idx, float* comp_slc, dpl_stream_t stream);

/* ---------------------------------------------------------------------------------
 * Phase-similarity raster (similarity.py).
 * ------------------------------------------------------------------------------- */

/* Replaces: get_circle_idxs(max_radius, min_radius, sort_output) -- similarity.py:176-254.
 * Host-only (no device work).  Writes up to `capacity` (row, col) pairs to `offsets`
 * ((capacity, 2) int32, may be NULL) and the number of offsets to `count`, in the
 * reference's order (ring by ring), or sorted lexicographically if sort_output != 0.
 * max_radius < 1 is an error (the reference raises). */
dpl_status dpl_circle_offsets(int max_radius, int min_radius, int sort_output, int32_t* offsets,
                              int64_t capacity, int64_t* count);

/* Largest search_radius dpl_similarity accepts (16; the reference's workflows use 7 and
 * 11). */
int dpl_similarity_max_radius(void);

/* Replaces the preparation in _create_loop_and_run -- similarity.py:96-117 -- and, with
 * nearest_n > 0, _calc_nearest_diffs / _create_nearest_n_pairs -- similarity.py:355-375
 * (pairs (i, j), i < j <= i + nearest_n, of the nlayers + 1 dates of a single-reference
 * stack; timeseries.get_incidence_matrix, timeseries.py:594-644).
 * stack       : (nlayers, rows, cols) complex64 (is_complex != 0) or float32 phase
 * mask        : (rows, cols) uint8 or NULL (all pixels)
 * unit        : (unit_layers, rows, cols) complex64 out -- exp(i angle z), exp(i phase) or
 *               exp(i (phi_j - phi_i)); NaN on pixels that are not valid.  unit_layers
 *               must be nlayers, or the number of nearest-n pairs.
 * valid       : (rows, cols) uint8 out -- mask and not invalid, where invalid means the
 *               layer-by-layer float32 sum of nan_to_num(z) is exactly 0 (with
 *               nearest_n > 0 also: some layer's phase is not finite, which makes every
 *               pair NaN in the reference's matrix product). */
dpl_status dpl_similarity_prep(const float* stack, int is_complex, int64_t nlayers, int64_t rows,
                               int64_t cols, const uint8_t* mask, int nearest_n, float* unit,
                               int64_t unit_layers, uint8_t* valid, dpl_stream_t stream);

/* Replaces: median_similarity / max_similarity(ifg_stack, search_radius, mask) --
 * similarity.py:31-93, loop _make_loop_function, similarity.py:120-173.
 * unit  : (nlayers, rows, cols) complex64 from dpl_similarity_prep
 * kind  : 0 median (nanmedian), 1 max (nanmax) of the similarities
 *         mean_t Re(u_t(p) conj u_t(q)) over the circle's neighbours q of p, each
 *         coordinate clipped to the image, p itself and NaN similarities left out
 * out   : (rows, cols) float32 out; NaN where no similarity is left.
 * 1 <= search_radius <= dpl_similarity_max_radius(). */
dpl_status dpl_similarity(const float* unit, int64_t nlayers, int64_t rows, int64_t cols,
                          int search_radius, int kind, float* out, dpl_stream_t stream);

/* ---------------------------------------------------------------------------------
 * Wrapped-phase workflow helpers.
 * ------------------------------------------------------------------------------- */

/* Replaces: utils.grow_nodata_region(arr, nodata, n_pixels) -- utils.py:613-660, applied
 * to the strided outputs of each block in workflows/single.py:352-362.
 * in, out : (rows, cols) of `dtype` (dpl_dtype); out must not alias in
 * A pixel of out is `nodata` where any pixel of the (2 n_pixels + 1)^2 square around it
 * (clipped to the image) is nodata in `in`, else the pixel of `in`.  Nodata means equal
 * to `nodata`, or NaN if nodata_is_nan (integer arrays then have none). */
dpl_status dpl_grow_nodata_region(const void* in, void* out, int dtype, int64_t rows, int64_t cols,
                                  double nodata, int nodata_is_nan, int n_pixels, dpl_stream_t stream);

/* ---------------------------------------------------------------------------------
 * Learned EMI warm start (no counterpart in the reference, whose EMI inverse iteration
 * starts from a constant vector, phase_link/_eigenvalues.py:139-205).
 * ------------------------------------------------------------------------------- */

/* dpl_process_coherence with optional per-pixel EMI starting vectors `vstart`
 * ((npix, nslc) complex64, NULL: constant start).  A pixel whose iteration from its
 * starting vector does not meet the stopping rule (|v_k+1 - v_k| <= 1e-5 within 49
 * steps), or whose vector is zero or not finite, is iterated again from the constant
 * start (plain EMI).  iterations: (npix) int16 out or NULL -- eigen-iterations used. */
dpl_status dpl_process_coherence_warm(const float* C, int64_t npix, int nslc, int use_evd, double beta,
                                      double zero_correlation_threshold, int reference_idx,
                                      double num_looks, int first_real_slc_idx, int compute_crlb,
                                      const float* vstart, float* eig_vecs, float* eig_vals,
                                      uint8_t* estimator, float* crlb_std_dev, float* temp_coh,
                                      float* closure_phases, int16_t* iterations, void* workspace,
                                      size_t workspace_bytes, dpl_stream_t stream);

/* Network input: |C_ij| of the nslc (nslc - 1) / 2 lower pairs (i > j, row by row) of
 * each pixel's coherence, (npix, nslc(nslc-1)/2) float32.  layout 0: planar coherence
 * (npix, nslc^2) floats (diagonal, then (Re, Im) per pair); layout 1: full (npix, nslc,
 * nslc) complex64. */
dpl_status dpl_mlp_features(const float* C, int nslc, int64_t npix, int layout, float* X,
                            dpl_stream_t stream);

/* out_j = V_j * f_j (conj_frame: V_j * conj(f_j)) with f_j = exp(i angle C_j0), f_0 = 1:
 * the network's outputs live in the frame of each pixel's phases relative to SLC 0.
 * C (npix, nslc, nslc) complex64; V, out (npix, nslc) complex64. */
dpl_status dpl_mlp_frame(const float* C, int nslc, int64_t npix, const float* V, int conj_frame,
                         float* out, dpl_stream_t stream);

/* C = act(alpha * op(A) op(B)^T + bias) (+ beta * C), fp32: element (i, k) of op(A) at
 * A[i * sai + k * sak], (j, k) of op(B) at B[j * sbj + k * sbk], C row stride sci; bias
 * per column j or NULL; act = ReLU if relu, else identity.  M x N x K. */
dpl_status dpl_gemm_f32(int M, int N, int K, const float* A, int64_t sai, int64_t sak,
                        const float* B, int64_t sbj, int64_t sbk, float* C, int64_t sci,
                        const float* bias, float alpha, float beta, int relu, dpl_stream_t stream);

/* Training-step kernels: dH *= (H > 0); dY = 2 (Y - T) / count with per-block partial
 * sums of (Y - T)^2 in loss_parts[ceil(count / 256)]; column sums of an (M, N) matrix;
 * Adam (step >= 1, bias-corrected). */
dpl_status dpl_relu_grad(const float* H, float* dH, int64_t count, dpl_stream_t stream);
dpl_status dpl_mse_grad(const float* Y, const float* T, float* dY, int64_t count,
                        float* loss_parts, dpl_stream_t stream);
dpl_status dpl_colsum(const float* X, int M, int N, float* out, dpl_stream_t stream);
dpl_status dpl_adam(float* w, const float* grad, float* m, float* v, int64_t count, float lr,
                    float b1, float b2, float eps, int step, dpl_stream_t stream);

/* Tensor-core inference of a three-layer network (bf16 operands, fp32 accumulation in
 * tensor memory): Y = L3(relu(L2(relu(L1(X))))), L(h) = h W^T + b, every width 1..256.
 * dpl_mlp_pack converts one layer's W (nout, nin) fp32 into the packed bf16 blocks the
 * forward pass streams (dpl_mlp_packed_bytes(nout, nin) bytes, 16-byte aligned).
 * X (npix, n0) fp32, Y (npix, n3) fp32 out, b_l (n_l) fp32; status: one device int,
 * set to DPL_ERR_TIMEOUT if a bounded wait gave up (the caller zeroes and reads it). */
size_t dpl_mlp_packed_bytes(int nout, int nin);
dpl_status dpl_mlp_pack(const float* W, int nout, int nin, void* packed, dpl_stream_t stream);
dpl_status dpl_mlp_forward_tc(const float* X, int64_t npix, int n0, int n1, int n2, int n3,
                              const void* W1, const float* b1, const void* W2, const float* b2,
                              const void* W3, const float* b3, float* Y, int* status,
                              dpl_stream_t stream);

/* No counterpart in the reference: dpl_process_coherence without a caller-supplied
 * workspace, for callers that cannot allocate device memory per call (a C/GDAL-style
 * host that owns no device allocator and cannot size one, or a multi-stream pipeline
 * where cudaMalloc/cudaFree would synchronise the device).  Same arguments, meaning
 * and results as dpl_process_coherence; allocates nothing.
 * Scratch: a static device array of 64 + dpl_process_coherence_noalloc_max_pixels()
 *   ints (1,048,576 pixels, 4 MiB) per device.  npix above that limit returns
 *   DPL_ERR_UNSUPPORTED.  The call zeroes the array's counter on `stream` itself;
 *   nothing needs to start at zero.
 * Set-up: the first call on a device (with that device current) resolves the array's
 *   address (cudaGetSymbolAddress, which also loads the module's data if it is not yet
 *   loaded); make that first call before any stream capture.
 * Calls that overlap on one device (other streams or threads) share the array and
 *   race: serialise them. */
int64_t dpl_process_coherence_noalloc_max_pixels(void);
dpl_status dpl_process_coherence_noalloc(const float* C, int64_t npix, int nslc, int use_evd,
                                         double beta, double zero_correlation_threshold,
                                         int reference_idx, double num_looks,
                                         int first_real_slc_idx, int compute_crlb,
                                         float* eig_vecs, float* eig_vals, uint8_t* estimator,
                                         float* crlb_std_dev, float* temp_coh,
                                         float* closure_phases, dpl_stream_t stream);

/* Kernel timing (no reference counterpart: a measurement hook).  While enabled,
 * dpl_phase_link records CUDA event pairs on its stream around the covariance
 * kernel (slot 0) and the solver kernel (slot 1; the plain form fuses both into
 * slot 0).  Each call returns (and clears) per slot the summed elapsed milliseconds
 * and launch counts recorded since the previous call -- total_ms[2], launches[2] --
 * waiting for them to complete, then sets the enable state. */
dpl_status dpl_kernel_timing(int enable, double* total_ms, int64_t* launches);

/* FP32 fused multiply-add throughput probe, the measured FP32 peak that the benchmark
 * puts under the CUDA-core kernels' roofline (no reference counterpart).  Launches
 * `blocks` x 256 threads, each running 8 independent chains of `iters` FMAs (16 * iters
 * flop per thread), and writes one float per thread to `out` (blocks * 256 floats). */
dpl_status dpl_fp32_fma_probe(float* out, int blocks, int iters, dpl_stream_t stream);

/* FP64 fused multiply-add throughput probe (no reference counterpart): the same shape
 * as dpl_fp32_fma_probe in double precision -- `blocks` x 256 threads, 8 independent
 * chains of `iters` double FMAs each (16 * iters flop per thread), one double per
 * thread written to `out` (blocks * 256 doubles).  It measures the rate that decides
 * which parts of the solver may run in FP64. */
dpl_status dpl_fp64_fma_probe(double* out, int blocks, int iters, dpl_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* DPL_H_ */
