/*
 * sid.h -- C ABI of libsid, the GB300 (sm_103a) implementation of SID's
 * light-field projection / deconvolution / NNLS hot path.
 *
 * Conventions
 *   - Arrays are MATLAB column-major with the reference's shapes.
 *   - Sizes are int64_t.  Every call returns an int status: SID_OK (0) or a
 *     negative code; sid_last_error() returns a thread-local message.
 *   - Unless a name ends in _host, array arguments are DEVICE pointers and the
 *     call is ordered on `stream` (a cudaStream_t passed as void*, NULL = the
 *     legacy default stream).  _host entry points take host arrays, copy them
 *     in, compute and copy the result out before returning (the MEX path for
 *     non-gpuArray inputs).
 *   - The caller owns every array it passes.  A plan owns its PSF copy,
 *     spectra and workspaces; one plan serves one stream at a time.
 */
#ifndef SID_H
#define SID_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    SID_OK = 0,
    SID_EINVAL = -1,   /* bad argument (shape, pointer, option) */
    SID_ENOMEM = -2,   /* device allocation failed */
    SID_ECUDA = -3,    /* CUDA runtime error */
    SID_ETIMEOUT = -4, /* a device-side wait exceeded its budget */
    SID_ENOCONV = -5,  /* solver hit its iteration cap (NQP.m:116-119) */
    SID_ENOTSUP = -6   /* the plan was not built for the requested method */
};

/* Plan flags: which operator forms to build at plan creation. */
#define SID_PLAN_DIRECT       0x1 /* FP32 lenslet taps for the direct kernels */
#define SID_PLAN_SPECTRAL_F32 0x2 /* lenslet-grid spectra, FP32 */
#define SID_PLAN_SPECTRAL_I16 0x4 /* lenslet-grid spectra in 16-bit block floating point
                                     (int16 mantissas, one FP32 step per frequency row),
                                     FP32 arithmetic: the forward of the mixed forms */
#define SID_PLAN_SPECTRAL_F24 0x8 /* lenslet-grid spectra as 24-bit floats (sign, 8-bit
                                     exponent, 15-bit mantissa: 16 significant bits),
                                     FP32 arithmetic: the back projection of
                                     SID_METHOD_SPECTRAL_MIXED */
#define SID_PLAN_SPECTRAL_TC  0x10 /* with SPECTRAL_F24: a transposed copy of the 24-bit
                                     spectra, so that the batched calls
                                     (sid_*_batched) of SID_METHOD_SPECTRAL_MIXED
                                     contract up to 64 volumes per pass on the tensor
                                     cores, forward and back with the 24-bit spectra */

/* Projection methods. */
#define SID_METHOD_DIRECT       0
#define SID_METHOD_SPECTRAL_F32 1
#define SID_METHOD_SPECTRAL_I16 2
/* Forward projection with the 16-bit block-floating-point spectra, back
 * projection with the 24-bit float spectra (plan flags SPECTRAL_I16 and
 * SPECTRAL_F24).  The 16-bit error is absolute (relative to each frequency
 * row's largest entry), which the forward image tolerates (no sensor pixel is
 * near zero) but a back projection does not: ISRA divides by the back
 * projection (deconvRL.m:52) and voxels whose PSF falls mostly outside the
 * sensor have tiny back projections.  The 24-bit floats keep 16 significant
 * bits of every entry, which holds ISRA within the mixed-precision bar. */
#define SID_METHOD_SPECTRAL_MIXED 3
/* The same with FP32 back-projection spectra (plan flags SPECTRAL_I16 and
 * SPECTRAL_F32). */
#define SID_METHOD_SPECTRAL_MIXED_F32 4

typedef struct sid_plan sid_plan;

/* Thread-local description of the last failure. */
const char* sid_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
int sid_version(void);

/* ---- Projector plan ------------------------------------------------------
 * H: HOST array, M x M x Nnum x Nnum x Z single (psf_ballistic.H).
 * CAindex: HOST Z x 2 int32, 1-based per-depth crop (psf_ballistic.CAindex),
 *   or NULL for the uncropped PSF (the forwardProjectGPU semantics).
 * X, Y: volume / sensor size.  flags: SID_PLAN_* bits.
 * Replaces the PSF upload that forwardProjectGPU.m:19 and
 * backwardProjectGPU_new.m:19 repeat for every slice of every call. */
int sid_plan_create(const float* H, int64_t M, int64_t Nnum, int64_t Z,
                    const int32_t* CAindex, int64_t X, int64_t Y, int flags,
                    sid_plan** plan);
/* Frees the plan's solver and projection workspaces (they are allocated again
 * on demand), keeping the operator data (taps, spectra, weak-voxel lists).
 * No reference counterpart: the MATLAB functions allocate per call. */
int sid_plan_release_workspaces(sid_plan* plan);
int sid_plan_destroy(sid_plan* plan);
/* info[0..13] = M, Nnum, Z, X, Y, Lx, Ly, D (taps per axis), L (DFT length),
 * device bytes held, flags, adjoint-taps-separate, weakly observed voxels (column
 * mass A'1 below 1e-2 of the largest unless set otherwise; the spectral back
 * projections recompute them exactly from the lenslet taps), kernel launches
 * that recomputation adds to each spectral back projection. */
int sid_plan_info(const sid_plan* plan, int64_t* info);
/* Spectral back projections recompute the weakly observed voxels exactly from
 * the lenslet taps: those whose column mass A'1 (the PSF mass landing on the
 * sensor) is below `frac` of the largest (default 1e-2; 0 turns it off).  Their
 * FFT-based values carry only absolute accuracy, which the multiplicative
 * solvers' divisions by A'(.) amplify.  Rebuilds the list (synchronous). */
int sid_plan_set_weak_fraction(sid_plan* plan, double frac);
/* The runs the weakly observed voxels are recomputed in (host only): for a
 * strictly ascending list of polyphase voxel indices (plane (c N + b) N + a,
 * then v, then u), runs[4r..4r+3] = plane, fixed coordinate, first voxel and
 * length (<= 24) of run r: column runs (fixed u, v = first..) plane by plane,
 * then row runs (fixed v, u = first..); every voxel lies in exactly one run. */
int sid_weak_runs_plan(const int32_t* list, int64_t n, int64_t N, int64_t Lx, int64_t Ly, int32_t* runs, int64_t cap,
                       int64_t* ncols, int64_t* nrows);

/* TOTALprojection = forwardProjectGPU(H, realspace)   forwardProjectGPU.m:1
 *                 = forwardProjectACC(H, realspace, CAindex)  forwardProjectACC.m:1
 * V: X x Y x Z single, I: X x Y single (device). */
int sid_forward(sid_plan* plan, int method, const float* V, float* I, void* stream);
/* Backprojection = backwardProjectGPU_new(H, projection)  backwardProjectGPU_new.m:1
 *                = backwardProjectACC_new(H, projection, CAindex)  backwardProjectACC_new.m:1
 * I: X x Y single, V: X x Y x Z single (device). */
int sid_adjoint(sid_plan* plan, int method, const float* I, float* V, void* stream);
/* Host-array forms of the two calls above. */
int sid_forward_host(sid_plan* plan, int method, const float* V, float* I);
int sid_adjoint_host(sid_plan* plan, int method, const float* I, float* V);

/* Wait for `stream`, then report SID_ETIMEOUT if a device-side wait of a
 * kernel launched on this plan ran out of budget since the last check. */
int sid_plan_sync(sid_plan* plan, void* stream);

/* CUDA-event timing of the plan's dominant kernel launches (the spectral
 * contraction, or the direct projection kernel), recorded on the launch
 * stream.  Enable, run, then read the summed milliseconds and the number of
 * timed launches (reading resets the counters). */
int sid_plan_timing_enable(sid_plan* plan, int on);
int sid_plan_timing_read(sid_plan* plan, double* total_ms, int64_t* launches);

/* Neuron-kernel composition (reconstruct_S.m:110-114,126-127,188-189): with a
 * kernel set, every projection of the plan is P(convn(X, kernel, 'same')) and
 * every back projection convn(P'(y), kernel, 'same') -- one kernel both ways,
 * as the reference composes them -- for the projector calls and all solvers.
 * kernel: HOST kx x ky x kz single, column-major (e.g. generate_kernel.m:1);
 * each size <= 64.  NULL or a zero size removes it. */
int sid_plan_set_kernel(sid_plan* plan, const float* kernel, int64_t kx, int64_t ky, int64_t kz);

/* ---- Deconvolution -------------------------------------------------------
 * Xguess = deconvRL(fwd, bwd, Htf, maxIter, Xguess, opts)   deconvRL.m:1
 * ISRA: X <- X .* Htf ./ (A'A X + lambda) with inf -> 0 and NaN -> 0
 * (deconvRL.m:46-87, mode 'basic', p = 1; lambda = 0 is the unpenalised form).
 * Htf, X: X x Y x Z single (device); X holds Xguess on entry. */
int sid_deconv_isra(sid_plan* plan, int method, const float* Htf, float* X,
                    int maxIter, float lambda, void* stream);

/* [Xguess, Xguess_history] = deconvRL(forwardFUN, backwardFUN, Htf, maxIter, Xguess, opts)
 *                                            deconvRL.m:1 (every mode)
 * mode 0 'basic': lambda3[0] is opts.lambda (p must be 1 when it is nonzero:
 * p ~= 1 reads the reference's undefined Filter, deconvRL.m:57); mode 1
 * 'TV': lambda3 is opts.lambda (1 x 3, one weight per axis), pnorm 1
 * (sign of forward differences, deconvRL.m:67-74) or 2 (7-point filter,
 * deconvRL.m:75-78); other pnorm values return X unchanged, as the
 * reference's 'p>2 not supported' return does.  lambda3: 3 floats (host).
 * history (optional, device): maxIter x X x Y x Z single, Xguess_history
 * (deconvRL.m:10,90-92). */
int sid_deconv_isra_ex(sid_plan* plan, int method, const float* Htf, float* X, int maxIter, int mode, int pnorm,
                       const float* lambda3, float* history, void* stream);

/* Several volumes at once (reconstruct_S.m:162-212 reconstructs components
 * side by side): nb volumes / images given as host arrays of device pointers
 * (each X x Y x Z or X x Y single).  The spectral forms contract up to four
 * volumes per pass over the tap spectra on the FP32 pipes, so the spectra
 * stream once per four volumes, and the results equal nb single calls up to
 * FP32 rounding; on a plan built with SID_PLAN_SPECTRAL_TC the mixed form
 * contracts up to 64 volumes per pass (as many as the device memory holds
 * workspaces for: 64, 32, 16 or 8) on the tensor cores with the 24-bit
 * spectra both ways (BF16 operand splits that carry them exactly, FP32
 * accumulation), within the mixed form's accuracy of the FP64 projections.
 * The direct form runs volume by volume.
 *   sid_forward_batched:     I[b] = forwardProjectGPU(H, V[b])      forwardProjectGPU.m:1
 *   sid_adjoint_batched:     V[b] = backwardProjectGPU_new(H, I[b]) backwardProjectGPU_new.m:1
 *   sid_deconv_isra_batched: X[b] = deconvRL(fwd, bwd, Htf[b], maxIter, X[b], opts) in mode
 *                            'basic' with opts.lambda = lambda     deconvRL.m:1 */
int sid_forward_batched(sid_plan* plan, int method, int64_t nb, const float* const* V, float* const* I, void* stream);
int sid_adjoint_batched(sid_plan* plan, int method, int64_t nb, const float* const* I, float* const* V, void* stream);
int sid_deconv_isra_batched(sid_plan* plan, int method, int64_t nb, const float* const* Htf, float* const* X,
                            int maxIter, float lambda, void* stream);
/* X[b] = LS_deconv(fwd, bwd, X[b], max_iter, opts) in the plain mode (no TV
 * terms) for nb volumes, X[b] holding df = Htf on entry (LS_deconv.m:1);
 * lamb_L1: nb values (host), one per volume; lamb_L2 shared. */
int sid_deconv_ls_batched(sid_plan* plan, int method, int64_t nb, float* const* X, int max_iter,
                          const float* lamb_L1, float lamb_L2, void* stream);
/* Host-array form of sid_deconv_isra (copies in, iterates, copies X out). */
int sid_deconv_isra_host(sid_plan* plan, int method, const float* Htf, float* X,
                         int maxIter, float lambda);
/* Poisson-likelihood Richardson-Lucy, the multiplicative update whose fixed
 * point maximises sum(y log AX - AX): X <- X .* A'(y ./ AX) ./ A'1, with
 * y ./ AX -> 0 where it is not finite, inf -> 0 and NaN -> 0 in the update as in
 * deconvRL.m:85-87.  (The reference's deconvRL, labelled RL, is the ISRA form
 * above; this is the Poisson counterpart whose gradient A'(1 - y ./ AX) the
 * log-likelihood checks use.)  y: X x Y single sensor image (device);
 * X: X x Y x Z single (device), Xguess on entry. */
int sid_deconv_rl_poisson(sid_plan* plan, int method, const float* y, float* X, int maxIter,
                          void* stream);
/* Xguess = LS_deconv(fwd, bwd, df, opts)   LS_deconv.m:1
 * Projected gradient with exact line search on ||y - A x||^2 + lamb_L2 ||x||^2
 * + lamb_L1 ||x||_1, x >= 0 (LS_deconv.m:49-93; TV terms not supported).
 * X: X x Y x Z single (device); holds df = A'y on entry, the solution on exit. */
int sid_deconv_ls(sid_plan* plan, int method, float* X, int max_iter,
                  float lamb_L1, float lamb_L2, void* stream);

/* Xguess = LS_deconv(forwardFUN, backwardFUN, df, opts) with the TV terms
 *                                            LS_deconv.m:1
 * lamb_TV_L2: 3 floats (host), the per-axis weights of the 7-point
 * Laplacian term convn(X, filter, 'same') in Q (LS_deconv.m:49-62,73);
 * lamb_TV_L1 enters only the reference's step-length test: alpha comes from
 * Q itself when lamb_TV_L1 * lamb_TV_L2 * lamb_L2 is nonzero in every
 * component, else from ||A df_||^2 (LS_deconv.m:82-87). */
int sid_deconv_ls_ex(sid_plan* plan, int method, float* X, int max_iter, float lamb_L1, float lamb_L2,
                     const float* lamb_TV_L2, float lamb_TV_L1, void* stream);

/* ---- Library generation -----------------------------------------------------
 * forward_model = generate_LFM_library_GPU(recon, centers, neur_id, psf, options)
 *                                              generate_LFM_library_GPU.m:1
 * All neurons in one batched launch.  recon: HOST array of n_comp DEVICE
 * pointers, each an X x Y x Z single volume; centers: HOST n_neur x 3 double
 * (1-based, column-major); neur_id: HOST n_neur x n_comp uint8 (column-major);
 * neur_rad, axial: options.neur_rad / options.axial.  out (device):
 * out_layout 0 = n_neur x P (the reference's forward_model), 1 = P x n_neur.
 * Needs a plan built with SID_PLAN_DIRECT.  Synchronises the stream. */
int sid_library(sid_plan* plan, const float* const* recon, int64_t n_comp, const double* centers,
                const uint8_t* neur_id, int64_t n_neur, int64_t neur_rad, double axial, float* out,
                int out_layout, void* stream);
/* The same library through the tensor-core spectral projector on lenslet
 * windows around each neuron's box (tap spectra on a small lenslet grid, built
 * at the first call and kept on the plan; up to 64 neurons per contraction
 * pass, each pass reducing only over its neurons' depths).  Arguments and
 * layouts as sid_library; the spectra carry 16 significant bits (about 1e-5
 * relative per row against 1e-7 for sid_library's FP32 taps).  Any plan
 * (odd PSF crop widths); boxes of at most 6 lattice points per phase. */
int sid_library_spectral(sid_plan* plan, const float* const* recon, int64_t n_comp, const double* centers,
                         const uint8_t* neur_id, int64_t n_neur, int64_t neur_rad, double axial, float* out,
                         int out_layout, void* stream);
/* forward_model = generate_LFM_library_CPU(centers, psf_ballistic, r, dim, m, kernel)
 *                                              generate_LFM_library_CPU.m:1
 * Each neuron is the kernel W (kernel: kx x ky x kz single, HOST, MATLAB
 * order; or, when kernel is NULL, the ball x^2 + y^2 + (z r/rr)^2 <= r^2 over
 * meshgrid(-r:r, -r:r, -rr:rr) with rr = r / dim_z) painted at round(W index -
 * [r+1, r+1, rr+1] + centre) (voxels outside the volume dropped),
 * forward-projected (project_forward_patched.m: for odd Nnum its centred patch
 * projection is the frame's conv2 'same' projection) and divided by its L2
 * norm.  method SID_METHOD_DIRECT (FP32 lenslet taps) or
 * SID_METHOD_SPECTRAL_MIXED (tensor-core windows).  centers: HOST n_neur x 3
 * double, 1-based; out (device) as sid_library: dense rows, the reference's
 * sparse matrix holds their nonzeros.  Synchronises the stream. */
int sid_library_kernel(sid_plan* plan, int method, const double* centers, int64_t n_neur, double r, double dim_z,
                       const float* kernel, int64_t kx, int64_t ky, int64_t kz, float* out, int out_layout,
                       void* stream);
/* The voxels the call above paints (host only): counts[n] per neuron; when xyz
 * is not NULL, 0-based (x, y, z) triples (and the kernel values) of all neurons
 * back to back, at most cap of them. */
int sid_library_kernel_voxels(const double* centers, int64_t n_neur, double r, double dim_z, const float* kernel,
                              int64_t kx, int64_t ky, int64_t kz, int64_t X, int64_t Y, int64_t Z, int64_t* counts,
                              int32_t* xyz, float* values, int64_t cap);
/* The crop boxes sid_library and sid_library_spectral use (host only):
 * boxes[6n..6n+5] = 0-based half-open x0 x1 y0 y1 z0 z1 of neuron n
 * (generate_LFM_library_GPU.m:68-88). */
int sid_library_boxes(const double* centers, int64_t n_neur, int64_t neur_rad, double axial, int64_t X,
                      int64_t Y, int64_t Z, int32_t* boxes);

/* ---- NNLS contractions -----------------------------------------------------
 * A solver context owns the workspaces of the contractions and NNLS solvers
 * (16-bit operand copies, split-K partials, iteration state). */
typedef struct sid_ctx sid_ctx;
int sid_ctx_create(sid_ctx** ctx);
int sid_ctx_destroy(sid_ctx* ctx);
/* Wait for `stream`; SID_ETIMEOUT if a device-side wait ran out of budget. */
int sid_ctx_sync(sid_ctx* ctx, void* stream);
/* CUDA-event timing of the tensor-core GEMM launches (with their split-K sum
 * or mirror) inside sid_gram / sid_cross, without the operand conversions:
 * enable, run, then read the total and the number of timed calls (read resets). */
int sid_ctx_timing_enable(sid_ctx* ctx, int on);
int sid_ctx_timing_read(sid_ctx* ctx, double* total_ms, int64_t* launches);
/* The tensor-core GEMM's tile plan (host only; the project's autotuner): for
 * C (m x n) = A'B with a k-deep reduction (symmetric: A'A, tiles on and above
 * the diagonal) on `sms` SMs, the tile width bn (256, 192, 128 or 64 columns
 * of 128-row tiles) and the number of K splits the contractions use. */
int sid_gemm_tile_plan(int64_t m, int64_t n, int64_t k, int symmetric, int sms, int* bn, int* splitk);

/* Precision of the contractions. */
#define SID_PREC_FP32  0 /* FP32 SIMT: the plain path */
#define SID_PREC_SPLIT 1 /* tcgen05 tensor cores on 16-bit hi/lo splits, FP32 accumulation */
#define SID_PREC_BF16  2 /* one 16-bit tensor-core pass */
/* Element types of movie arrays. */
#define SID_DTYPE_F32 0
#define SID_DTYPE_F16 1
#define SID_DTYPE_U16 2 /* camera frames (sid_image_rect) */

/* G = A'*A (K x K, column-major)   LS_nnls.m:82, fast_nnls.m:54, T_update.m:24
 * A: P x K single (device, column-major). */
int sid_gram(sid_ctx* ctx, const float* A, int64_t P, int64_t K, float* G, int prec, void* stream);
/* h = A'*Y (K x F)   LS_nnls.m:76, fast_nnls.m:57, T_update.m:25
 * Y: P x F single or half (ydtype). */
int sid_cross(sid_ctx* ctx, const float* A, const void* Y, int ydtype, int64_t P, int64_t K, int64_t F,
              float* h, int prec, void* stream);

/* ---- Movie scans -------------------------------------------------------------
 * [bg_spatial, bg_temporal] = rank_1_factorization(Y, maxIter)   rank_1_factorization.m:1
 * std_image = compute_std_image(Y, bg_spatial, bg_temporal)      compute_std_image.m:1
 * (the two calls of sid_main.m:95,101).  Y: P x F movie (device, column-major,
 * SID_DTYPE_F32 or SID_DTYPE_F16); bg_spatial: P floats, bg_temporal: F floats
 * (device outputs); maxIter >= 1.  std_image (P floats, device) may be NULL;
 * when given it is computed in the same pass over Y as the last spatial
 * update.  Negative variances (rounding) give 0 rather than MATLAB's complex
 * square root. */
int sid_rank1_background(sid_ctx* ctx, const void* Y, int ydtype, int64_t P, int64_t F, int maxIter,
                         float* bg_spatial, float* bg_temporal, float* std_image, void* stream);
/* std_image = compute_std_image(Y, y_1, y_2)   compute_std_image.m:1.  y_1 (P) and
 * y_2 (F) are device floats or NULL for zeros (compute_std_image.m:17-19). */
int sid_std_image(sid_ctx* ctx, const void* Y, int ydtype, int64_t P, int64_t F, const float* y1,
                  const float* y2, float* std_image, void* stream);

/* ---- Post-processing of the demixing (merge_filters.m, SNR_order.m) --------
 * merge_filters(forward_model, timeseries, template, indices_in_orig, opts)
 *                                                   merge_filters.m:1
 * Merges components whose templates overlap by more than a third of the
 * smaller one and whose traces correlate above `limit` (opts.limit, default
 * 0.9), with MATLAB's single arithmetic and its two bg_sub crops
 * (merge_filters.m:19-29).  ts: K x F single traces (device, the background
 * row last when bg_sub); templ: (K - bg_sub) x P single 0/1 templates
 * (device, merged in place: absorbing rows OR-ed, absorbed rows zeroed,
 * :33-36); keep: HOST int32[K] output, 1 for the rows of forward_model /
 * timeseries / indices_in_orig (and template, first K - bg_sub) that survive
 * (:38-50).  The overlap Gram runs exactly on the tensor cores. */
int sid_merge_filters(sid_ctx* ctx, const float* ts, int64_t K, int64_t F, float* templ, int64_t P, double limit,
                      int bg_sub, int32_t* keep, void* stream);
/* n = SNR_order(traces, opts)   SNR_order.m:1.  traces: K x F single (device);
 * order: HOST int32[K] output, 0-based row order by decreasing peak-to-noise
 * ratio, the background row (K-1) last when bg_sub. */
int sid_snr_order(sid_ctx* ctx, const float* traces, int64_t K, int64_t F, int bg_sub, int32_t* order,
                  void* stream);

/* ---- Sensor frames: lenslet rectification (ImageRect.m) --------------------
 * IMG_RESAMPLE = ImageRect(IMG_BW, xCenter, yCenter, dx, M, Crop, XcutLeft,
 *                          XcutRight, YcutUp, YcutDown)          ImageRect.m:1
 * frames: rows x cols x nframes (device, column-major), SID_DTYPE_U16 or
 * SID_DTYPE_F32; mask: rows x cols single (device) or NULL, multiplied in
 * first as read_sensor_movie.m:94-99 does; cuts: HOST int32[4] = XcutLeft,
 * XcutRight, YcutUp, YcutDown (used when crop).  out: out_rows x out_cols x
 * nframes single (device) -- the P x F movie of read_sensor_movie.m --
 * bilinear as interp2, NaN outside the image.  sid_image_rect_size gives
 * out_rows / out_cols (host only). */
int sid_image_rect_size(int64_t rows, int64_t cols, double xCenter, double yCenter, double dx, int64_t M, int crop,
                        const int32_t* cuts, int64_t* out_rows, int64_t* out_cols);
int sid_image_rect(sid_ctx* ctx, const void* frames, int dtype, int64_t rows, int64_t cols, int64_t nframes,
                   const float* mask, double xCenter, double yCenter, double dx, int64_t M, int crop,
                   const int32_t* cuts, float* out, void* stream);

/* ---- NNLS solvers -----------------------------------------------------------
 * Options mirror the reference's opts fields and defaults. */
typedef struct {
    double lambda;     /* L1 weight: LS_nnls h = A'Y - lambda; fast_nnls df = -A'Y + lambda */
    int64_t sample;    /* convergence-fit window: LS_nnls 300, fast_nnls 30 */
    double tol;        /* LS_nnls 1e-7, fast_nnls 1e-6 */
    double tol_;       /* fit-residual tolerance: LS_nnls 1e-2, fast_nnls 1e-1 */
    int64_t max_iter;  /* 2000 */
    int use_std;       /* LS_nnls: least standard deviation instead of least squares */
    int tol_p;         /* fast_nnls: 1 = log l1 step, 2 = log l2 step */
} sid_nnls_opts;
void sid_ls_nnls_defaults(sid_nnls_opts* opts);   /* LS_nnls.m:59-73 */
void sid_fast_nnls_defaults(sid_nnls_opts* opts); /* fast_nnls.m:21-51 */

/* [X, G] = LS_nnls(A, Y, opts, G, x)   LS_nnls.m:1
 * A: P x K single; Y: P x F single or half (ydtype); all device arrays.
 * G: K x K, read when g_given, else written when non-NULL.
 * X: K x F, the start point when x_given (else zeros), the solution on return.
 * iters (optional, F int32): iteration at which each column retired.
 * prec: SID_PREC_FP32 or SID_PREC_SPLIT. */
int sid_ls_nnls(sid_ctx* ctx, const float* A, const void* Y, int ydtype, int64_t P, int64_t K, int64_t F,
                const sid_nnls_opts* opts, float* G, int g_given, float* X, int x_given, int prec,
                int32_t* iters, void* stream);
/* [xx, Q] = fast_nnls(A, Y, opts) with opts.warm_start = warm_start (K x F, or
 * NULL for a zero start)   fast_nnls.m:1.  Q_out (optional): the normalised
 * Gram.  X: K x F solution (diag(h) * x, fast_nnls.m:197-199). */
int sid_fast_nnls(sid_ctx* ctx, const float* A, const void* Y, int ydtype, int64_t P, int64_t K, int64_t F,
                  const sid_nnls_opts* opts, const float* warm_start, float* X, float* Q_out, int prec,
                  int32_t* iters, void* stream);

/* [xx, Q, df, h] = fast_nnls(A, Y, opts, Q, df, h) with every input and output
 *                                            fast_nnls.m:1
 * total: opts.total (one step length for all columns, fast_nnls.m:101-117;
 * the reference's loop then ends at max_iter without copying x into xx, so X
 * is diag(h) * ones, and df_out carries the iterations' result).
 * warm_mode: 0 none; 1 opts.warm_start == 1 (x = inv(Q)(-df) clamped at 0,
 * fast_nnls.m:66-69; Q singular is SID_EINVAL); 2 opts.warm_start = W (K x F).
 * Q_in (K x K, normalised) and h_in (K) given together: the caller's Q and h
 * (fast_nnls.m:58-62, nargin > 3); df_in (K x F): the caller's df.  A and Y
 * are read only to form what is not given (they may be NULL when Q, h and df
 * all are).  Outputs (optional except X): Q_out, h_out, and df_out (total
 * mode; the reference's df has no columns left otherwise). */
int sid_fast_nnls_ex(sid_ctx* ctx, const float* A, const void* Y, int ydtype, int64_t P, int64_t K, int64_t F,
                     const sid_nnls_opts* opts, int total, int warm_mode, const float* W, const float* Q_in,
                     const float* df_in, const float* h_in, float* X, float* Q_out, float* df_out, float* h_out,
                     int prec, int32_t* iters, void* stream);

/* forward_model = update_spatial_component(timeseries, sensor_movie, template, opts)
 *                                            update_spatial_component.m:1
 * Every template pixel's regularised NNLS (reg_nnls.m:40-69, NQP.m:42-178 with
 * default options, FP64 active set) in one launch.  T: R x F single (the
 * timeseries; with bg_sub the last row is the background); Y: P x F single or
 * half; tmpl: (R - bg_sub) x P uint8 template; forward_model: R x P single
 * (dense).  Pixels covered by up to 32 components solve with their working
 * arrays in registers and local memory; more crowded pixels (any number of
 * components) are listed and solved by a second launch whose working arrays sit
 * in device scratch.  status (optional, P int32): 0 ok, 2 NQP iteration cap;
 * SID_ENOCONV if any pixel hit the cap. */
int sid_spatial_update(sid_ctx* ctx, const float* T, const void* Y, int ydtype, const uint8_t* tmpl, int64_t R,
                       int64_t F, int64_t P, double lamb_L1, double lamb_L2, double lamb_orth_L1, int use_std,
                       int bg_sub, float* forward_model, int32_t* status, void* stream);

/* [x, w, info] = NQP(Q, b) for B independent problems of one size
 *                                            NQP.m:42-178 (default options)
 * argmin_{x >= 0} 0.5 x'Qx + q'x, Lawson-Hanson active set with an incremental
 * Cholesky factor, FP64, one thread per problem; the solver reg_nnls.m:69 and
 * the spatial update call.  Q: n x n x B (column-major, device), q: n x B;
 * x: n x B; w (optional): n x B, NQP's final w; iters / status (optional, B
 * int32): iterations taken, 0 ok or 2 at the iteration cap.  n <= 4096 (above
 * 32 the working arrays of each problem sit in device scratch).
 * SID_ENOCONV if any problem hit the cap (NQP.m:116-119's error).
 * Synchronises the stream. */
int sid_nqp_batched(sid_ctx* ctx, const double* Q, const double* q, int n, int64_t B, double* x, double* w,
                    int32_t* iters, int32_t* status, void* stream);

/* x = reg_nnls(A, d, opts) (reg_nnls.m:1): min_{x >= 0} ||A x - d||^2 with the
 * reference's options, as one NQP whose system libsid forms in FP64
 * (reg_nnls.m:40-66: Q = A'A [- t t'/m] + lamb_L2 I + lamb_orth_L1 hilf,
 * q = -A'd [+ t sum(d)/m] + lamb_L1, t = column sums of A when use_std) and
 * solves with the Lawson-Hanson kernel (NQP.m:42-178).  A: m x n double, d: m
 * double, x: n double (device); hilf: n x n double or NULL (ones - eye, with
 * the last row and column zero when bg_sub, reg_nnls.m:31-38).  n <= 4096. */
int sid_reg_nnls(sid_ctx* c, const double* A, int64_t m, int n, const double* d, double lamb_L1, double lamb_L2,
                 double lamb_orth_L1, int use_std, int bg_sub, const double* hilf, double* x, void* stream);

/* ---- Quantiles and component reconstruction ---------------------------------
 * MATLAB quantile of a vector (sorted non-NaN data at probabilities
 * (k - 0.5)/n, linear interpolation, clamped to the extremes; NaN when no
 * value is left): out[i] = quantile(x(exclude == 0), p[i]) for np <= 64
 * probabilities.  x: n single (device); exclude: n uint8 (device) or NULL;
 * out: HOST doubles.  Synchronises the stream.  (reconstruct_S.m:132,137,169,193) */
int sid_quantile(sid_ctx* ctx, const float* x, int64_t n, const uint8_t* exclude, const double* p, int np,
                 double* out, void* stream);

typedef struct {
    double q;       /* background quantile of the non-microlens pixels (0.8) */
    double lamb_L1; /* L1 weight, capped by the (1 - 1e-4) quantile of Htf (0) */
    double lamb_L2; /* L2 weight (0) */
    int solver;     /* 0 = 'fast_nnls' (LS_deconv, the default), 1 = 'ISRA' (deconvRL) */
    int max_iter;   /* iterations of the solver (8) */
} sid_recon_opts;
void sid_recon_defaults(sid_recon_opts* opts); /* reconstruct_S.m:47-95 */
/* recon_nnmf{ii} for one component image (reconstruct_S.m:130-148, 168-205):
 * background clip at quantile q of the pixels with microlenses == 0, divide
 * by the maximum, back-project img/||img||, cap lamb_L1, solve, scale by
 * ||img||.  img: X x Y single, microlenses: X x Y uint8 or NULL, X: X x Y x Z
 * single output (all device).  lamb_used (optional, host): the capped lamb_L1.
 * Reads the capped weight back to the host (one stream synchronisation). */
int sid_reconstruct_component(sid_plan* plan, int method, const float* img, const uint8_t* microlenses,
                              const sid_recon_opts* opts, float* X, double* lamb_used, void* stream);
/* The same for nc components (the components reconstruct_S.m:162-212 runs side
 * by side): imgs / X are host arrays of nc device pointers, lamb_used (optional,
 * host) nc values.  The back projections and the solver run on groups of
 * components (up to 64 on the tensor cores, else 32) through sid_adjoint_batched and sid_deconv_ls_batched /
 * sid_deconv_isra_batched (on the tensor cores with a SID_PLAN_SPECTRAL_TC plan
 * and SID_METHOD_SPECTRAL_MIXED).  One stream synchronisation per group. */
int sid_reconstruct_components(sid_plan* plan, int method, int64_t nc, const float* const* imgs,
                               const uint8_t* microlenses, const sid_recon_opts* opts, float* const* X,
                               double* lamb_used, void* stream);

/* ---- NMF steps (fast_NMF.m:185-186) ------------------------------------------
 * One projected-gradient step with exact line search on T or on S for
 * Y ~ S*T.  Y: P x F single or half (ydtype); S: P x R single; T: R x F
 * single; all device arrays, updated in place (NaNs zeroed first, as the
 * reference does).  Options mirror the reference's opts fields; zero = off. */
typedef struct {
    double lamb_temp;    /* T_update: L1 weight on T */
    double lamb_corr;    /* T_update: correlation penalty (rows of T renormalised, S rescaled) */
    double lamb_temp_TV; /* T_update: temporal total variation, [-1 2 -1] */
    double lamb_spat;    /* S_update: L1 weight on S */
    double lamb_spat_TV; /* S_update: must be 0 (the reference's term calls an undefined 'laplace') */
    double lamb_orth_L1; /* S_update: Q_T += lamb_orth_L1 * hilf; S columns renormalised */
    double lamb_orth_L2; /* S_update: L2 orthogonality (step floored at 1e-6) */
    int use_std;         /* both: least standard deviation (needs ymean = opts.Y) */
    int pointwise;       /* both: one step per frame (T) / per pixel (S) */
} sid_nmf_opts;
void sid_nmf_defaults(sid_nmf_opts* opts);

/* [S, T] = T_update(Y, T, S, opts)   T_update.m:1
 * active: P uint8 (opts.active; NULL = every pixel); ymean: P single (opts.Y,
 * read with use_std).  S is written too: NaNs zeroed and, with lamb_corr > 0,
 * its columns rescaled by the norms of T's rows.  prec: precision of S'S and
 * S'Y (an FP16 movie always uses SID_PREC_SPLIT, with a power-of-two operand
 * scale kept on the device).  No host round trip: the call can be captured in
 * a CUDA graph once an ordinary call has sized its workspaces. */
int sid_t_update(sid_ctx* ctx, const void* Y, int ydtype, float* T, float* S, int64_t P, int64_t R, int64_t F,
                 const uint8_t* active, const float* ymean, const sid_nmf_opts* opts, int prec, void* stream);
/* [S, T] = S_update(Y, S, T, opts)   S_update.m:1
 * ymean: P single (opts.Y, use_std); hilf: R x R single (opts.hilf, read when
 * an orthogonality weight is set).  T is written too: NaNs zeroed and, with an
 * orthogonality weight, its rows rescaled by the norms of S's columns.
 * prec: precision of the pixel-long products -- S'S (L2 orthogonality) and
 * the pixel-by-rank products Y*T', S*Q_T, v*Q_T, which at SID_PREC_SPLIT and
 * SID_PREC_BF16 run on the tensor cores (split: FP16 hi/lo of power-of-two
 * scaled operands, the scales found, applied and undone on the device) and at
 * SID_PREC_FP32 on the FP32 SIMT GEMM.  No host round trip: the call can be
 * captured in a CUDA graph once an ordinary call has sized its workspaces. */
int sid_s_update(sid_ctx* ctx, const void* Y, int ydtype, float* S, float* T, int64_t P, int64_t R, int64_t F,
                 const float* ymean, const float* hilf, const sid_nmf_opts* opts, int prec, void* stream);

/* ---- Timeseries extraction (incremental_temporal_update_gpu.m:76-100) ----------
 * Least-squares branch: Q = inv(F*F')*F once (:83-84), then T = Q*(Y ./ b) for
 * each chunk of frames (:66-68, 89, 99).  The handle keeps a pixel-major copy
 * of F and inv(F*F') in FP64 (blocked Cholesky, then inverse); a chunk costs
 * the contraction F*Y and the FP64 product inv(F*F')*(F*Y), the reference's
 * product re-associated so that the K x P matrix Q is never formed.  The
 * non-negative branch (opts.non_neg_on) is sid_ls_nnls. */
typedef struct sid_pinv sid_pinv;
/* F: K x P single (layout 0, the reference's forward_model) or P x K
 * (layout 1, the library's pixel-major columns), device.  prec: precision of
 * F*F' and F*Y (SID_PREC_FP32 or SID_PREC_SPLIT).  Synchronises the stream;
 * SID_EINVAL when F*F' is not positive definite.  The handle uses ctx for
 * its contractions: keep ctx alive and do not use it on another stream meanwhile. */
int sid_pinv_create(sid_ctx* ctx, const float* F, int64_t K, int64_t P, int layout, int prec, sid_pinv** out,
                    void* stream);
/* T (K x n, leading dimension ldt) = Q * (Y ./ baseline): Y P x n single or
 * half (ydtype); baseline: n single per-frame divisors, or NULL. */
int sid_pinv_apply(sid_pinv* q, const void* Y, int ydtype, int64_t n, const float* baseline, float* T, int64_t ldt,
                   void* stream);
int sid_pinv_destroy(sid_pinv* q);

/* ---- Allocation-free Gram product ---------------------------------------------
 * No counterpart in the reference: an addition for callers that cannot let a
 * library allocate device memory (a MEX function whose memory belongs to
 * MATLAB's gpuArray manager, or a program that reserves all device memory up
 * front).  G = A'*A in FP32 (same result as sid_gram with SID_PREC_FP32),
 * without a context: split-K partials live in a fixed 16 MiB device array
 * compiled into libsid, so K is limited to 2048 (SID_EINVAL beyond).  The
 * array is shared by every call and keeps the last call's contents; calls
 * whose kernels overlap on the GPU race on it.  The first call in a CUDA
 * context looks the array up (cudaGetSymbolAddress) and should precede any
 * stream capture; the address is kept per context (driver context ID), so a
 * device reset or a second context on the device looks it up again.
 * A: P x K single, G: K x K single (device). */
int sid_gram_noalloc(const float* A, int64_t P, int64_t K, float* G, void* stream);

/* ---- Self-test of the bounded device waits --------------------------------------
 * No counterpart in the reference (library diagnostics).  Runs one CTA shaped
 * like a tensor-core pipeline at its abort point (TMEM held, one mbarrier, no
 * copies or MMAs in flight) whose waiter polls the mbarrier at most `polls`
 * times (1..2^20).  arrive = 0: nobody arrives, the wait runs out, the kernel
 * frees TMEM and returns, and the call returns SID_ETIMEOUT (the mapping every
 * pipelined entry point uses).  arrive = 1: the barrier completes and the call
 * returns SID_OK.  Synchronises the device. */
int sid_selftest_wait_timeout(uint32_t polls, int arrive);

#ifdef __cplusplus
}
#endif

#endif /* SID_H */
