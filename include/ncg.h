/*
 * ncg.h -- C-ABI of the GB300 (sm_103a) KDE/VKDE proposal engine.
 *
 * A drop-in for NumCosmo's NcmStatsDistKDE / NcmStatsDistVKDE hot path as used
 * by the APES walker (numcosmo/ncm/fit/ncm_fit_esmcmc_walker_apes.c:646-891):
 * prepare, prepare_interp, eval_m2lnp, eval, kernel_choose and sample, with
 * the Gaussian and Student-t(nu) kernels.  All work runs on one GPU through
 * hand-written CUDA kernels; the handle owns its device state.
 *
 * Plain C, no GLib: matrices are row-major double arrays (the NcmMatrix
 * layout, numcosmo/ncm/algebra/ncm_matrix.h:66-74); a covariance
 * decomposition U is upper triangular with Sigma = U^T U.  Every function
 * returns an ncg_status_t; misuse that aborts in the reference (g_error /
 * g_assert) returns an error code here.  The caller owns every buffer it
 * passes; calls on one handle are serialised on the handle's CUDA stream,
 * different handles may be used from different threads.
 */
#ifndef NCG_H
#define NCG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */

typedef enum ncg_status
{
  NCG_OK                   = 0,
  NCG_ERR_INVALID_ARG      = 1,  /* bad pointer / size / option                      */
  NCG_ERR_SAMPLE_TOO_SMALL = 2,  /* n_obs <= dim: numcosmo/ncm/stats/ncm_stats_dist.c:748-749 */
  NCG_ERR_TOO_FEW_LOCAL    = 3,  /* local_frac*n < 2: numcosmo/ncm/stats/ncm_stats_dist_vkde.c:505-510 */
  NCG_ERR_NOT_PD           = 4,  /* diagonal fallback not PD: numcosmo/ncm/stats/ncm_stats_dist_kde.c:365 */
  NCG_ERR_NOT_PREPARED     = 5,  /* eval/sample before prepare                        */
  NCG_ERR_NONFINITE        = 6,  /* NaN/Inf in an input                               */
  NCG_ERR_UNSUPPORTED      = 7,  /* option outside the GPU path (e.g. dimension > 32) */
  NCG_ERR_CUDA             = 8,  /* CUDA runtime error; see ncg_last_error()          */
  NCG_ERR_OUT_OF_MEMORY    = 9,  /* device allocation failed or budget exceeded      */
  NCG_ERR_TIMEOUT          = 10, /* a bounded device wait gave up                     */
  NCG_ERR_BAD_WEIGHTS      = 11, /* sum of NNLS weights <= 0: ncm_stats_dist.c:1089   */
  NCG_ERR_BUSY             = 12, /* serving queue full / slot not free                */
} ncg_status_t;

/* Message for a status code (static string). */
const char *ncg_status_string (ncg_status_t status);
/* Detail of the last error raised on the calling thread ("" when none). */
const char *ncg_last_error (void);

/* --------------------------------------------------------------- options */

/* NcmStatsDistKDE vs NcmStatsDistVKDE */
typedef enum ncg_kind { NCG_KDE = 0, NCG_VKDE = 1 } ncg_kind_t;

/* NcmStatsDistKernelGauss vs NcmStatsDistKernelST */
typedef enum ncg_kernel { NCG_KERNEL_GAUSS = 0, NCG_KERNEL_ST = 1 } ncg_kernel_t;

/* NcmStatsDistCV, numcosmo/ncm/stats/ncm_stats_dist.h:77-85.  NONE; SPLIT_NOFIT (the
 * first ceil(n split_frac) observations are the kernels; prepare fits the
 * over-smoothing to the -2 ln p of the rest by the reference's Nelder-Mead, and
 * prepare_interp fits the kernels' weights on all n observations); LOO (every
 * observation is a kernel; prepare fits the over-smoothing to the AMISE, in closed
 * form for a Gaussian KDE, by the reference's Monte Carlo otherwise, with its
 * draws from MT19937 seeded 4357, the seed GSL gives 0); SPLIT (kernels as under
 * SPLIT_NOFIT, no fit in prepare; prepare_interp restarts the weight fit at ten
 * over-smoothings drawn from the handle's own generator, MT19937 seeded 4357 at
 * its first use, then fits ln over_smooth by the reference's levmar
 * Levenberg-Marquardt to the observations' -2 ln p and fits the weights there). */
typedef enum ncg_cv { NCG_CV_NONE = 0, NCG_CV_SPLIT = 1, NCG_CV_SPLIT_NOFIT = 2, NCG_CV_LOO = 3 } ncg_cv_t;

/* NcmStatsDistKDECovType, numcosmo/ncm/stats/ncm_stats_dist_kde.h:56-68 (all four run here:
 * SAMPLE, FIXED, ROBUST_DIAG and ROBUST; a robust global estimate takes at most 16384 samples) */
typedef enum ncg_cov_type { NCG_COV_SAMPLE = 0, NCG_COV_FIXED = 1, NCG_COV_ROBUST_DIAG = 2, NCG_COV_ROBUST = 3 } ncg_cov_type_t;

/* Arithmetic of eval_m2lnp: plain FP64; or mixed: the whitening as split-
 * precision tensor-core GEMMs (tcgen05, FP16x3 on kind::f16) with FP32
 * accumulation and log-sum-exp for VKDE at every dimension (padded 4..32)
 * whose operand passes its accuracy check (ncg_sd_get_tc_check), FP32 CUDA
 * cores with hi/lo-split differences elsewhere (KDE, or a failed check);
 * MIXED_SIMT forces the latter.  Covariances and their Cholesky factors stay
 * FP64 in every mode; in the mixed modes prepare_interp's NNLS builds A^T A
 * and factors it in FP32 on the tensor cores (TF32x3) as the preconditioner
 * of FP64 conjugate gradients, handing a set the preconditioner cannot solve
 * to the FP64 Cholesky. */
typedef enum ncg_precision { NCG_PREC_FP64 = 0, NCG_PREC_MIXED = 1, NCG_PREC_MIXED_SIMT = 2 } ncg_precision_t;

/* GObject properties of the reference with their defaults. */
typedef struct ncg_sd_config
{
  double  over_smooth;      /* "over-smooth" 1.0, numcosmo/ncm/stats/ncm_stats_dist.c:404-410 */
  double  shrink;           /* "shrink" 0.01, numcosmo/ncm/stats/ncm_stats_dist.c:436-442 */
  double  local_frac;       /* "local-frac" 0.05, numcosmo/ncm/stats/ncm_stats_dist_vkde.c:276-283 */
  int32_t use_rot_href;     /* "use-rot-href" FALSE, numcosmo/ncm/stats/ncm_stats_dist_vkde.c:284-290 */
  int32_t nearPD_maxiter;   /* "nearPD-maxiter" 200, numcosmo/ncm/stats/ncm_stats_dist_kde.c:290-296 */
  int32_t cv_type;          /* ncg_cv_t, "CV-type" NONE */
  int32_t cov_type;         /* ncg_cov_type_t, "cov-type" SAMPLE */
  int32_t precision;        /* ncg_precision_t, default FP64 */
  int32_t device;           /* CUDA device ordinal, default 0 */
  int32_t async_alloc;      /* 1: the handle's device buffers come from the stream-ordered allocator on
                               its stream (no device-wide synchronisation when they grow or are freed);
                               only for handles whose buffers no other stream uses (not in a batch).
                               Default 0.  No counterpart in the reference. */
} ncg_sd_config_t;

/* Fill cfg with the reference defaults. */
void ncg_sd_config_init (ncg_sd_config_t *cfg);

/* ------------------------------------------------------------ the handle */

typedef struct ncg_sd ncg_sd_t;

/* ncm_stats_dist_kde_new / ncm_stats_dist_vkde_new with a
 * ncm_stats_dist_kernel_{gauss,st}_new kernel:
 * numcosmo/ncm/stats/ncm_stats_dist_kde.h:74, ncm_stats_dist_vkde.h:53,
 * ncm_stats_dist_kernel_gauss.h:41, ncm_stats_dist_kernel_st.h:41.
 * nu is ignored for the Gaussian kernel.  cfg may be NULL (defaults). */
ncg_status_t ncg_sd_new (ncg_kind_t kind, ncg_kernel_t kernel, uint32_t dim, double nu,
                         const ncg_sd_config_t *cfg, ncg_sd_t **out);

/* ncm_stats_dist_free / ncm_stats_dist_clear: ncm_stats_dist.h:88-89 */
ncg_status_t ncg_sd_free (ncg_sd_t *sd);

/* Run this handle's work on an existing cudaStream_t (NULL: the handle's own). */
ncg_status_t ncg_sd_set_stream (ncg_sd_t *sd, void *cuda_stream);
ncg_status_t ncg_sd_synchronize (ncg_sd_t *sd);

/* property setters: ncm_stats_dist.h:100,106; ncm_stats_dist_vkde.h:58,61;
 * ncm_stats_dist_kde.h:79,82 */
ncg_status_t ncg_sd_set_over_smooth (ncg_sd_t *sd, double over_smooth);
ncg_status_t ncg_sd_set_shrink (ncg_sd_t *sd, double shrink);
/* ncm_stats_dist_set_split_frac: ncm_stats_dist.h:103 (0.01 <= split_frac <= 1;
 * a new handle has 0.5, the "split-frac" property's construct-time default,
 * ncm_stats_dist.c:428-434) */
ncg_status_t ncg_sd_set_split_frac (ncg_sd_t *sd, double split_frac);
/* ncm_stats_dist_get_over_smooth: ncm_stats_dist.h:101 (after a SPLIT_NOFIT prepare, the
 * fitted value; the bandwidth follows it) */
ncg_status_t ncg_sd_get_over_smooth (ncg_sd_t *sd, double *over_smooth);
ncg_status_t ncg_sd_set_local_frac (ncg_sd_t *sd, double local_frac);
ncg_status_t ncg_sd_set_use_rot_href (ncg_sd_t *sd, int32_t use_rot_href);
ncg_status_t ncg_sd_set_nearPD_maxiter (ncg_sd_t *sd, int32_t maxiter);
ncg_status_t ncg_sd_set_cov_type (ncg_sd_t *sd, ncg_cov_type_t cov_type);
/* ncm_stats_dist_kde_set_cov_fixed: dim x dim covariance used with NCG_COV_FIXED
 * (ncm_stats_dist_kde.c:825-845): the global covariance and the VKDE whitening,
 * factored as given by ncg_sd_prepare (NCG_ERR_NOT_PD if it is not positive
 * definite: no nearPD repair; the reference checks when the matrix is set);
 * VKDE neighbourhoods keep their sample covariances */
ncg_status_t ncg_sd_set_cov_fixed (ncg_sd_t *sd, const double *cov);
ncg_status_t ncg_sd_set_precision (ncg_sd_t *sd, ncg_precision_t precision);

/* ncm_stats_dist_reset: ncm_stats_dist.h:141 */
ncg_status_t ncg_sd_reset (ncg_sd_t *sd);
/* ncm_stats_dist_add_obs (copies the point): ncm_stats_dist.h:130 */
ncg_status_t ncg_sd_add_obs (ncg_sd_t *sd, const double *y);
/* n calls of add_obs over the rows of Y (n x dim) */
ncg_status_t ncg_sd_add_obs_batch (ncg_sd_t *sd, const double *Y, uint64_t n);

/* ncm_stats_dist_prepare: ncm_stats_dist.h:119 */
ncg_status_t ncg_sd_prepare (ncg_sd_t *sd);
/* ncm_stats_dist_prepare_interp: ncm_stats_dist.h:120; m2lnp has one value
 * per observation (n_obs; the weights are n_kernels long).  May shrink the
 * sample (the reference's range cut).  Under a split, where the reference
 * would index a weight past n_kernels or fail its count assertion
 * (ncm_stats_dist.c:938-966), returns NCG_ERR_INVALID_ARG. */
ncg_status_t ncg_sd_prepare_interp (ncg_sd_t *sd, const double *m2lnp);

/* ncm_stats_dist_eval_m2lnp: ncm_stats_dist.h:123 (one point, host memory) */
ncg_status_t ncg_sd_eval_m2lnp (ncg_sd_t *sd, const double *x, double *m2lnp);
/* the same at m points X (m x dim, host memory) in one launch */
ncg_status_t ncg_sd_eval_m2lnp_batch (ncg_sd_t *sd, const double *X, uint64_t m, double *m2lnp);
/* the same with device pointers, asynchronous on the handle's stream */
ncg_status_t ncg_sd_eval_m2lnp_device (ncg_sd_t *sd, const double *d_X, uint64_t m, double *d_m2lnp);

/* eval_m2lnp in the FP64 form on device pointers, for callers that must not
 * allocate device memory while they evaluate: a pipeline that keeps other
 * streams busy (cudaMalloc can synchronise the whole device and stall them),
 * or a caller that owns all device memory under a fixed budget and forbids
 * allocations hidden inside library calls.  It calls no cudaMalloc, cudaFree
 * or other allocating routine: its per-call scratch is a file-scope device
 * array of 4 MiB that every GPU loading the library holds until the process
 * exits.  At most 262144 points per call (larger m: NCG_ERR_INVALID_ARG).  The
 * distribution must be prepared (prepare allocates, once, at set-up).  The
 * first call on a device looks up the array's device address, so make that
 * first call before any stream capture; the address is kept for the life of
 * the process and does not survive cudaDeviceReset (a new context reloads the
 * module), so do not call this entry point on a device after resetting it.  Calls share the array: calls whose
 * kernels overlap on the GPU (different streams, or concurrent threads)
 * race; nothing in it needs clearing between calls.  Asynchronous on the
 * handle's stream.  No counterpart in the reference. */
ncg_status_t ncg_sd_eval_m2lnp_device_noalloc (ncg_sd_t *sd, const double *d_X, uint64_t m, double *d_m2lnp);

/* ncm_stats_dist_eval (linear density): ncm_stats_dist.h:122 */
ncg_status_t ncg_sd_eval (ncg_sd_t *sd, const double *x, double *p);
ncg_status_t ncg_sd_eval_batch (ncg_sd_t *sd, const double *X, uint64_t m, double *p);

/* ncm_stats_dist_kernel_choose: ncm_stats_dist.h:125, with the uniform draw
 * p = ncm_rng_uniform_gen (rng, 0, 1) supplied by the caller per choice. */
ncg_status_t ncg_sd_kernel_choose_batch (ncg_sd_t *sd, const double *u, uint64_t n, int32_t *idx);

/* ncm_stats_dist_sample: ncm_stats_dist.h:126.  Per draw j the caller
 * supplies the RNG stream the reference would consume, in its order:
 * u[j] (kernel choice), z[j*dim .. j*dim+dim-1] (unit gaussians) and, for the
 * Student-t kernel, chisq[j] (a chi^2_nu draw; NULL for Gauss).  Outputs the
 * points x (n x dim) and the chosen kernels idx (may be NULL). */
ncg_status_t ncg_sd_sample_batch (ncg_sd_t *sd, const double *u, const double *z,
                                  const double *chisq, uint64_t n, double *x, int32_t *idx);
/* the same with device buffers, asynchronous on the handle's stream; d_idx
 * may be NULL */
ncg_status_t ncg_sd_sample_batch_device (ncg_sd_t *sd, const double *d_u, const double *d_z,
                                         const double *d_chisq, uint64_t n, double *d_x, int32_t *d_idx);

/* Device workspace for prepare_interp's O(n^2) matrices (the interpolation
 * matrix and the normal-equation factors).  By default the handle allocates
 * and keeps them; with a workspace set they are carved from the caller's
 * arena (256-byte aligned, at least ncg_sd_workspace_bytes for the sample
 * size) on every prepare_interp, so one arena can serve many handles in
 * turn.  NULL returns to handle-owned buffers.  No counterpart in the
 * reference (its matrices are GLib allocations). */
ncg_status_t ncg_sd_workspace_bytes (ncg_sd_t *sd, uint64_t n, size_t *bytes);   /* n = 0: current sample */
ncg_status_t ncg_sd_set_workspace (ncg_sd_t *sd, void *d_ws, size_t bytes);

/* getters: ncm_stats_dist.h:95-98,128,132-137 */
ncg_status_t ncg_sd_get_dim (ncg_sd_t *sd, uint32_t *dim);
ncg_status_t ncg_sd_get_sample_size (ncg_sd_t *sd, uint64_t *n);
ncg_status_t ncg_sd_get_n_kernels (ncg_sd_t *sd, uint64_t *n);   /* of the last prepare */
ncg_status_t ncg_sd_get_href (ncg_sd_t *sd, double *href);
ncg_status_t ncg_sd_get_rnorm (ncg_sd_t *sd, double *rnorm);
ncg_status_t ncg_sd_get_weights (ncg_sd_t *sd, double *w);                 /* n_kernels */
ncg_status_t ncg_sd_get_sample (ncg_sd_t *sd, double *X);                  /* n x dim */
ncg_status_t ncg_sd_get_cov_decomp (ncg_sd_t *sd, uint32_t i, double *U);  /* dim x dim */
ncg_status_t ncg_sd_get_full_cov_decomp (ncg_sd_t *sd, double *U);
ncg_status_t ncg_sd_get_full_cov (ncg_sd_t *sd, double *cov);
ncg_status_t ncg_sd_get_lnnorm (ncg_sd_t *sd, uint32_t i, double *lnnorm); /* incl. dim*ln(href) */
/* ncm_stats_dist_get_Ki: numcosmo/ncm/stats/ncm_stats_dist.h:139.  Everything
 * about kernel i: its location y_i (dim), its covariance cov_i = href^2 U_i^T U_i
 * (dim x dim, row-major), its normalisation n_i = exp(lnnorm_i) (incl. dim*ln(href))
 * and its weight w_i. */
ncg_status_t ncg_sd_get_Ki (ncg_sd_t *sd, uint32_t i, double *y_i, double *cov_i, double *n_i, double *w_i);
/* The neighbour lists behind the VKDE local covariances: for each of the n
 * kernels its k nearest centres in the globally whitened space (k from
 * ncg_sd_get_knn_k), ordered by squared distance and then index, as the
 * reference's kd-tree returns them (numcosmo/external/misc/kdtree.c:193-320,
 * rb_knn_list.c:32-40).  idx is n x k.  KDE handles: NCG_ERR_UNSUPPORTED.
 * Inspection entry point: the reference keeps these lists inside
 * _ncm_stats_dist_vkde_build_cov_array_kdtree (ncm_stats_dist_vkde.c:363-451)
 * and has no getter for them. */
ncg_status_t ncg_sd_get_knn (ncg_sd_t *sd, int32_t *idx);
/* which branch prepare_interp took: 0 NNLS fit, 1 range heuristic, 2 cut + refit */
ncg_status_t ncg_sd_get_interp_branch (ncg_sd_t *sd, int32_t *branch);
/* number of kernels whose covariance needed the nearPD / diagonal fallback */
ncg_status_t ncg_sd_get_chol_fallbacks (ncg_sd_t *sd, uint64_t *count);
/* The arithmetic that eval_m2lnp uses with the current precision setting, and
 * (mixed settings) the largest infinity-norm condition number of the per-kernel
 * FP32 whitening.  The mixed form keeps its -2lnp error within 1e-6 relative
 * only for well-conditioned whitening; above a condition number of 1000 a
 * mixed request is served by the FP64 form.  No counterpart in the reference
 * (it has only the FP64 form). */
typedef enum ncg_eval_path { NCG_PATH_FP64 = 0, NCG_PATH_TC = 1, NCG_PATH_SIMT = 2 } ncg_eval_path_t;
ncg_status_t ncg_sd_get_eval_path (ncg_sd_t *sd, int32_t *path, double *kappa_max);
/* The tensor-core form folds the centre subtraction into its GEMM, so its
 * FP32 cancellation grows with |W'_i theta'_i|; before first use the handle
 * evaluates up to 128 kernel centres with it and with the FP64 form and keeps
 * it only if the largest relative difference (floored at 1) is at most 5e-7,
 * else serves mixed requests with the FP32 SIMT form.  err = that difference
 * (-1 before the check).  No counterpart in the reference. */
ncg_status_t ncg_sd_get_tc_check (ncg_sd_t *sd, double *err);
/* Measurement hook: with timing on, each tensor-core eval records two CUDA
 * events on the handle's stream around its main kernel (not the point
 * packing or the merge); get_kernel_time waits for the second and returns
 * the elapsed milliseconds of the last such eval (NCG_ERR_NOT_PREPARED if
 * none ran since timing was switched on).  No counterpart in the reference. */
ncg_status_t ncg_sd_set_kernel_timing (ncg_sd_t *sd, int32_t on);
ncg_status_t ncg_sd_get_kernel_time (ncg_sd_t *sd, double *ms);
/* the k of the kNN local covariance (VKDE) */
ncg_status_t ncg_sd_get_knn_k (ncg_sd_t *sd, uint32_t *k);
/* Counters of the last prepare_interp NNLS fit: active-set solves, conjugate-
 * gradient iterations of the mixed solver, FP32 factorisations that needed a
 * diagonal shift, and solves served by the FP64 Cholesky (every solve in the
 * FP64 form; the mixed form's fallback).  stats[4] = {solves, cg_iters,
 * shifted, fp64}.  No counterpart in the reference (its only solver is the
 * FP64 one of ncm_nnls.c). */
ncg_status_t ncg_sd_get_interp_stats (ncg_sd_t *sd, int32_t stats[4]);
/* How many FP64 active-set solves of the last prepare_interp found their
 * normal equations not positive definite and took the symmetric (LU) solve
 * of ncm_nnls.c:573-606 (lu), and how many of those met an exactly zero pivot
 * and took the least-squares (QR) solve of ncm_nnls.c:608-638 (qr).  The
 * reference counts neither; it takes the same branches. */
ncg_status_t ncg_sd_get_interp_fallbacks (ncg_sd_t *sd, int32_t *lu, int32_t *qr);
/* ncm_stats_dist_compute_IM with unit f: the interpolation matrix, n_obs x
 * n_kernels row-major (square but under a split) */
ncg_status_t ncg_sd_compute_IM (ncg_sd_t *sd, double *IM);

/* ----------------------------------------------------------------- RNG */

/* NcmRNG replacement for the streams sample consumes: MT19937 (Matsumoto &
 * Nishimura 1998) with the uniform, gaussian (polar Box-Muller) and chi^2
 * (Marsaglia-Tsang gamma) transforms.  ncm_rng_seeded_new:
 * numcosmo/ncm/core/ncm_rng.h:60.  Draw order mirrors ncm_rng.c:709-772. */
typedef struct ncg_rng ncg_rng_t;

ncg_status_t ncg_rng_new (uint32_t seed, ncg_rng_t **out);
ncg_status_t ncg_rng_free (ncg_rng_t *rng);
/* the generator's state (MT19937 words and position, ncg_rng_state_bytes bytes),
 * for checkpoints; ncm_rng_get_state / ncm_rng_set_state carry GSL's state the same way */
size_t       ncg_rng_state_bytes (void);
ncg_status_t ncg_rng_get_state (const ncg_rng_t *rng, void *state);
ncg_status_t ncg_rng_set_state (ncg_rng_t *rng, const void *state);
uint32_t     ncg_rng_get_u32 (ncg_rng_t *rng);
double       ncg_rng_uniform (ncg_rng_t *rng);       /* [0,1), u32 / 2^32 */
double       ncg_rng_uniform_pos (ncg_rng_t *rng);   /* (0,1)               */
double       ncg_rng_ugaussian (ncg_rng_t *rng);
double       ncg_rng_chisq (ncg_rng_t *rng, double nu);
/* Draw the stream of n sample calls in the reference's order
 * (ncm_stats_dist.c:1618-1627 then kernel sample): per call one uniform, dim
 * gaussians and, for Student-t, one chi^2_nu. chisq may be NULL for Gauss. */
ncg_status_t ncg_rng_sample_stream (ncg_rng_t *rng, ncg_kernel_t kernel, uint32_t dim, double nu,
                                    uint64_t n, double *u, double *z, double *chisq);
/* The draws of n calls of ncm_stats_dist_sample2 (ncm_stats_dist.c:1633-1651,
 * the antithetic pairs of the LOO AMISE integral), in its order: per pair
 * u[j] (one kernel choice), then z1[j*dim ..] and (Student-t) chisq1[j] for
 * the first point, z2[j*dim ..] and chisq2[j] for the second. */
ncg_status_t ncg_rng_sample2_stream (ncg_rng_t *rng, ncg_kernel_t kernel, uint32_t dim, double nu, uint64_t n,
                                     double *u, double *z1, double *chisq1, double *z2, double *chisq2);

/* ------------------------------------------------- many problems at once
 *
 * No counterpart in the reference: APES evaluates one NcmStatsDist at a time
 * (ncm_fit_esmcmc_walker_apes.c:828-873).  A batch borrows prepared handles
 * (same device as the batch; the handles must outlive the batch or be
 * removed with ncg_batch_clear) and evaluates -2 ln p of all of them in one
 * persistent launch, replayed from a captured CUDA graph.  Points and
 * results are concatenated in the order of ncg_batch_add: problem i's m_i x
 * dim_i points start at x_off[i] (in doubles) and its m_i results at
 * out_off[i] (ncg_batch_layout).  A launch reads the handles' current
 * state: re-preparing a handle or refitting its weights re-plans the batch
 * on the next call.  precision: NCG_PREC_FP64, or NCG_PREC_MIXED (FP32 SIMT
 * tiles; a problem whose whitening is ill-conditioned gets FP64 tiles).
 * Each problem's result equals its one-problem eval with the same tile
 * arithmetic up to the slicing of its kernel range. */
typedef struct ncg_batch ncg_batch_t;

/* plan parameters (chosen by ncg_batch_autotune, or set) */
typedef struct ncg_batch_params
{
  double  items_per_cta;   /* work items per resident CTA (>= 1): sets each problem's kernel slices */
  int32_t ctas_per_sm;     /* resident CTAs per SM of the persistent grid (0 = as many as fit) */
  int32_t order;           /* 0 problem-major, 1 largest item first */
  int32_t split;           /* 0 one launch; 1 two launches (dim <= 16 | > 16), two branches of the graph */
  int32_t tc;              /* mixed only: 1 = VKDE problems whose tensor-core operand passes its check run on
                              the tensor-core kernel (one launch each, parallel graph branches);
                              both precisions: 2 = the branch schedule, no persistent launch: every problem
                              is one launch of the kernel its own eval uses (tensor cores, FP32 SIMT or FP64
                              tiles), spread largest first over 16 parallel graph branches */
} ncg_batch_params_t;

ncg_status_t ncg_batch_params_init (ncg_batch_params_t *p);
ncg_status_t ncg_batch_new (int device, ncg_batch_t **out);
void         ncg_batch_free (ncg_batch_t *b);
ncg_status_t ncg_batch_add (ncg_batch_t *b, ncg_sd_t *sd, uint64_t m, int32_t *slot);
ncg_status_t ncg_batch_clear (ncg_batch_t *b);
/* x_off, out_off: n_problems entries each (may be NULL); totals = {points
 * doubles, results} */
ncg_status_t ncg_batch_layout (ncg_batch_t *b, int64_t *x_off, int64_t *out_off, int64_t totals[2]);
ncg_status_t ncg_batch_set_params (ncg_batch_t *b, int32_t precision, const ncg_batch_params_t *p);
ncg_status_t ncg_batch_get_params (ncg_batch_t *b, int32_t precision, ncg_batch_params_t *p);
/* time candidate plans on the device and keep the fastest; best_ms may be NULL */
ncg_status_t ncg_batch_autotune (ncg_batch_t *b, int32_t precision, int32_t reps, double *best_ms);
/* device buffers; ordered on `stream` (a cudaStream_t, NULL = the legacy stream) */
ncg_status_t ncg_batch_eval_m2lnp_device (ncg_batch_t *b, int32_t precision, const double *d_X, double *d_out,
                                          void *stream);
/* host buffers; returns when the results are in `out` */
ncg_status_t ncg_batch_eval_m2lnp (ncg_batch_t *b, int32_t precision, const double *X, double *out);
/* Prepare every problem of the batch (ncm_stats_dist_prepare, ncm_stats_dist.h:119, for each handle,
 * whose sample must be set) from a pool of nthreads host threads (<= 0: one per host core, at most
 * 64), each handle on its own stream, so the problems' device work overlaps.  Each handle ends as its
 * own ncg_sd_prepare would leave it.  On failure the status of the lowest failing problem is
 * returned and ncg_last_error names it.  No counterpart in the reference (one NcmStatsDist at a
 * time). */
ncg_status_t ncg_batch_prepare (ncg_batch_t *b, int32_t nthreads);
/* The same for ncm_stats_dist_prepare_interp (ncm_stats_dist.h:120): m2lnp holds each problem's
 * -2 ln L at its sample points, concatenated in the order of ncg_batch_add (sample sizes as before
 * the call; a range cut may shrink them). */
ncg_status_t ncg_batch_prepare_interp (ncg_batch_t *b, const double *m2lnp, int32_t nthreads);
/* stats[7] = {work items, persistent launches, problems on FP64 tiles, pairs, graph captures, graph
 * launches, problems on the tensor-core kernel} */
ncg_status_t ncg_batch_get_stats (ncg_batch_t *b, int32_t precision, int64_t stats[7]);

/* ---------------------------------------------------------------- serving
 *
 * A request loop over many concurrent APES chains.  No counterpart in the
 * reference: NcmFitESMCMC runs one chain in-process.  A chain is a walker
 * ensemble (n walkers of dimension dim, two halves of N = n/2) with its own
 * StatsDist handle, RNG stream and Gaussian target; one request = one APES
 * half-move of that chain (ncm_fit_esmcmc_walker_apes.c:739-919), step k
 * moving half k mod 2:
 *   prepare_interp of the handle on the other half's N walkers and their -2 ln L,
 *   N proposals sampled from the fit,
 *   eval_m2lnp at the 2N points (proposals and the moving half's walkers),
 *   -2 ln L of the target at the proposals, Metropolis-Hastings accept.
 * `slots` worker threads run steps at once, each on its chain's stream, so
 * steps that arrive while others are on the GPU start as soon as a slot and
 * memory are free and overlap on the device.  A chain's state (walkers,
 * factors, weights) stays resident in device memory between its steps;
 * chains are admitted by the device-memory budget (resident state plus the
 * slots' O(n^2) prepare_interp workspaces) and an idle chain is evicted
 * (state kept on the host) when a waiting chain needs the room.  A chain's
 * steps run in submission order and each step's result depends only on the
 * chain, never on what else runs. */
typedef struct ncg_server ncg_server_t;

typedef struct ncg_server_config
{
  int32_t  device;
  int32_t  slots;          /* steps on the device at once (default 4)                  */
  int32_t  precision;      /* NCG_PREC_FP64 or NCG_PREC_MIXED (default)                 */
  int32_t  pad_;
  uint64_t hbm_budget;     /* bytes for resident chains + workspaces (default 40 GB) */
} ncg_server_config_t;

typedef struct ncg_chain_desc
{
  int32_t  kind, kernel;   /* ncg_kind_t, ncg_kernel_t */
  uint32_t dim;
  int32_t  pad_;
  uint64_t n;              /* walkers, even (each step's fit has n/2 kernels) */
  double   nu;             /* Student-t degrees of freedom */
  double   over_smooth, local_frac;
  uint32_t seed;           /* the chain's MT19937 stream */
  int32_t  pad2_;
  const double *X0;        /* n x dim initial walkers (copied) */
  const double *target_L;  /* dim x dim lower Cholesky factor of the target covariance (copied) */
  /* NcmFitESMCMCWalkerAPES options (numcosmo/ncm/fit/ncm_fit_esmcmc_walker_apes.c:646-919) */
  double   random_walk_prob; /* "random-walk-prob": weight of the truncated Gaussian random walk
                                (std 0.25 sqrt(cov_ii) of the fit) in the proposal mixture; 0: off */
  uint32_t exploration;      /* first half-moves accepted on the target ratio alone ("exploration") */
  int32_t  pad3_;
  const double *lb, *ub;     /* dim parameter bounds (copied; NULL: unbounded); proposals outside
                                are drawn again, as ncm_mset_fparam_valid_bounds rejects them */
} ncg_chain_desc_t;

typedef struct ncg_step_result
{
  int64_t  request;
  int32_t  chain, status;  /* status: ncg_status_t of the step */
  uint64_t step;           /* the chain's step index */
  uint64_t accepted;       /* proposals accepted */
  uint64_t pairs;          /* kernel-point pairs, N = n/2: 2N^2 eval + N^2 interpolation matrix */
  double   mean_m2lnL;     /* mean target -2 ln L of the walkers after the step */
  double   state_sum;      /* sum of the walker coordinates after the step */
  double   t_arrive, t_start, t_done;   /* seconds on the server clock */
  char     detail[128];    /* the error text of a failed step */
} ncg_step_result_t;

typedef struct ncg_server_stats
{
  uint64_t submitted, completed, failed, admitted, evicted;
  uint64_t reserved_bytes, peak_reserved_bytes;
  double   p50_ms, p99_ms, mean_ms, max_ms;   /* latency = done - arrival */
  double   span_s;                            /* first arrival to last completion */
  double   pairs;                             /* over the completed steps */
} ncg_server_stats_t;

ncg_status_t ncg_server_config_init (ncg_server_config_t *cfg);
ncg_status_t ncg_server_new (const ncg_server_config_t *cfg, ncg_server_t **out);
/* stops accepting, waits for the running steps, frees everything */
void         ncg_server_free (ncg_server_t *s);
ncg_status_t ncg_server_add_chain (ncg_server_t *s, const ncg_chain_desc_t *c, int32_t *chain_id);
ncg_status_t ncg_server_submit (ncg_server_t *s, int32_t chain_id, int64_t *request_id);
ncg_status_t ncg_server_wait (ncg_server_t *s, int64_t request_id, ncg_step_result_t *res);
ncg_status_t ncg_server_drain (ncg_server_t *s);
ncg_status_t ncg_server_get_stats (ncg_server_t *s, ncg_server_stats_t *st);
/* walkers (n x dim) and their -2 ln L after the chain's last completed step */
ncg_status_t ncg_server_get_chain (ncg_server_t *s, int32_t chain_id, double *X, double *m2lnL);
double       ncg_server_clock (ncg_server_t *s);
/* Checkpoint and resume of the chains' state (walkers, -2 ln L, target factor,
 * steps taken, the RNG state): the server must be idle (NCG_ERR_BUSY while a
 * step is pending or running).  The file is written beside `path` and renamed
 * over it, so a crash leaves the previous checkpoint.  restore adds the saved
 * chains, in order, to a server (ids first_id .. first_id + count - 1); their next
 * steps continue the saved trajectories bit for bit.  The format is this
 * library's own (little-endian, versioned, FNV-1a checksum); the reference's
 * catalogue (ncm_mset_catalog.c, FITS) stores sampled points, not resumable
 * sampler state. */
ncg_status_t ncg_server_checkpoint (ncg_server_t *s, const char *path);
/* a chain's description (X0 and target_L set to NULL) and its completed steps */
ncg_status_t ncg_server_get_chain_info (ncg_server_t *s, int32_t chain_id, ncg_chain_desc_t *desc, uint64_t *steps);
ncg_status_t ncg_server_restore (ncg_server_t *s, const char *path, int32_t *first_id, int32_t *count);

/* ------------------------------------------------- failure detection test
 *
 * Every wait of a device kernel on another CTA or on an asynchronous copy is
 * bounded: the tensor-core eval's mbarrier waits give up after 1.5 s of
 * %globaltimer, the preconditioner's chained triangular solves after 2^21
 * polls; the kernel then ends and the call returns NCG_ERR_TIMEOUT, with the
 * CUDA context still usable.  This hook makes the next launch of one such
 * kernel (process-wide, one shot) wait for something that never comes, so a
 * test can check that path end to end without faulting or hanging the GPU:
 *   NCG_FAULT_EVAL_TC_WAIT  the tensor-core eval's copy warp issues no copies
 *                           (its MMA warp's first wait runs out);
 *   NCG_FAULT_CHAIN_WAIT    the chained forward solve publishes its values
 *                           under an epoch no reader waits for.
 * No counterpart in the reference (its CPU path has no device waits). */
typedef enum ncg_fault { NCG_FAULT_NONE = 0, NCG_FAULT_EVAL_TC_WAIT = 1, NCG_FAULT_CHAIN_WAIT = 2 } ncg_fault_t;
ncg_status_t ncg_debug_inject_wait_fault (int32_t fault);

/* ---------------------------------------------------------- measurement
 *
 * Measured FP64 FMA rate of a device: a launch of SMs x 8 CTAs of 256
 * threads, each thread eight independent FMA chains, timed with CUDA events
 * after a warm-up launch; tflops = 2 x FMAs / time.  It is the denominator of
 * the FP64 eval's roofline fraction.  No counterpart in the reference. */
ncg_status_t ncg_measure_fp64_peak (int32_t device, double *tflops);

/* -------------------------------------------------------------- version */

/* "ncg <version> sm_103a" */
const char *ncg_version (void);

#ifdef __cplusplus
}
#endif

#endif /* NCG_H */
