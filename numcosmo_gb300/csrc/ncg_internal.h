/*
 * ncg_internal.h -- declarations shared by the C host layer (ncg_api.c) and
 * the CUDA translation units (ncg_*.cu).  Not part of the public ABI.
 *
 * Device layout of one prepared distribution (n kernels, dimension d, padded
 * dimension dp = ncg_pad_dim(d) in {4,8,...,32}):
 *   X      [n][d]     centres (the sample), FP64
 *   Y      [n][d]     whitened centres  X U^{-1}  (invUsample), FP64
 *   cov,U  [d][d]     global covariance and its upper Cholesky factor
 *   Ui     [n][d][d]  VKDE per-kernel upper factors (zero lower triangle)
 *   lnnorm [n]        VKDE per-kernel kernel lnnorm (without d ln h)
 *   w      [n]        weights;  c[n] = ln w_i - lnnorm_i (VKDE) or ln w_i (KDE)
 *   pack64 [n][s64]   eval operand per kernel, s64 = dp + dp(dp+1)/2 (VKDE:
 *                     centre, then U_i^{-T}/h packed lower by rows) or dp (KDE:
 *                     whitened centre / h); zero padded past d.
 *   packmx            the mixed-precision operand (see ncg_eval.cu)
 */
#ifndef NCG_INTERNAL_H
#define NCG_INTERNAL_H

#include <stdint.h>
#include <cuda_runtime_api.h>

#include "ncg.h"

#ifdef __cplusplus
extern "C" {
#endif

#define NCG_DMAX 32
#define NCG_KNN_KMAX 4096
#define NCG_ROBUST_MAX_ROWS 16384   /* rows of a robust-covariance set (one Qn sorts them in shared memory) */

/* ln(2 pi), ln(pi) */
#define NCG_LN2PI 1.8378770664093454835606594728112
#define NCG_LNPI 1.1447298858494001741434273513531

#ifdef __CUDACC__
#define NCG_HD __host__ __device__
#else
#define NCG_HD
#endif

NCG_HD static inline int
ncg_pad_dim (int d)
{
  return (d <= 4) ? 4 : ((d + 3) / 4) * 4;
}

NCG_HD static inline int
ncg_pack64_stride (int kind, int dp)
{
  return (kind == NCG_VKDE) ? dp + dp * (dp + 1) / 2 : dp;
}

/* Device-side counters of one prepare, read back by the host. */
typedef struct ncg_prep_status
{
  int32_t n_fallback;     /* factors that needed nearPD or the diagonal */
  int32_t n_fail;         /* factors whose diagonal fallback failed too */
  int32_t n_nonfinite;    /* non-finite inputs met                      */
  int32_t n_flagged;      /* factors queued for the nearPD pass         */
  int32_t n_badindex;     /* neighbour indices outside [0, n) (a bug)   */
  int32_t pad_;
  double  kernel_lnnorm;  /* lnnorm of the global factor                */
} ncg_prep_status_t;

/* Per-launch parameters of the eval kernels. */
typedef struct ncg_eval_args
{
  int32_t kind, kernel, d, dp;
  int32_t n;              /* kernels        */
  int64_t m;              /* points         */
  double  nu, kappa;      /* kappa = -(nu + d)/2 */
  double  final_shift;    /* KDE: kernel_lnnorm, VKDE: 0 */
  double  d_ln_href;      /* d * ln(href)   */
  double  inv_href;       /* 1 / href       */
  double  c_shift;        /* mixed form: constant taken out of c[] */
} ncg_eval_args_t;

/* ---- wait-fault test hook (ncg_api.c): 1 if `fault` was armed (and disarms it) ---- */
int         ncg_fault_take (int fault);

/* ---- prepare (ncg_prepare.cu) ---- */
cudaError_t ncg_launch_global_cov_chol (const double *X, int n, int d, double *cov, double *U,
                                        int32_t *flag, ncg_prep_status_t *st, cudaStream_t s);
cudaError_t ncg_launch_nearpd (double *cov_then_U, int count, const int32_t *ids, int d, int maxiter,
                               int32_t *flag, ncg_prep_status_t *st, cudaStream_t s);
cudaError_t ncg_launch_global_lnnorm (const double *U, int d, int kernel, double nu,
                                      ncg_prep_status_t *st, cudaStream_t s);
cudaError_t ncg_launch_whiten (const double *X, const double *U, int n, int d, double *Y, cudaStream_t s);
cudaError_t ncg_launch_knn (const double *Y, int n, int nq, int d, int k, int32_t *knn,
                            uint64_t *keys_scratch, cudaStream_t s);
size_t      ncg_knn_scratch_bytes (int n, int d, int k);
cudaError_t ncg_launch_local_cov_chol (const double *X, const int32_t *knn, int n, int nq, int d, int k,
                                       double *Ui, int32_t *flag, ncg_prep_status_t *st, cudaStream_t s);
cudaError_t ncg_launch_chol_slots (double *Ui, int n, int d, int32_t *flag, ncg_prep_status_t *st, cudaStream_t s);
/* robust covariance types, ncg_robust.cu */
size_t      ncg_robust_work_doubles (int nsets, int d);
cudaError_t ncg_launch_robust_cov (const double *X, int n, int d, const int32_t *idx, int m, int nsets, int ogk,
                                   double *work, double *out, int32_t *bad, cudaStream_t s);
cudaError_t ncg_launch_vkde_finish (const double *X, double *Ui, const int32_t *flag, int n, int d,
                                    int kernel, double nu, double href, double *lnnorm, double *pack64,
                                    cudaStream_t s);
cudaError_t ncg_launch_kde_finish (const double *Y, const double *U, int n, int d, double href,
                                   double *pack64, double *Vg, cudaStream_t s);
cudaError_t ncg_launch_mean (const double *X, int n, int d, double *mu, cudaStream_t s);
cudaError_t ncg_launch_global_vg (const double *U, int d, double scale, double *Vg, cudaStream_t s);
cudaError_t ncg_launch_weights_c (const double *w, const double *lnnorm, int n, int kind,
                                  double *c, double *wcum_dirty, cudaStream_t s);
cudaError_t ncg_launch_fill (double *p, double v, int64_t n, cudaStream_t s);
cudaError_t ncg_launch_compact_flags (const int32_t *flag, int n, int32_t *ids, int32_t *count,
                                      cudaStream_t s);

/* ---- eval (ncg_eval.cu) ---- */
size_t      ncg_eval_scratch_bytes (const ncg_eval_args_t *a, int precision);
cudaError_t ncg_launch_eval_m2lnp_fp64 (const ncg_eval_args_t *a, const double *Xq, const double *pack64,
                                        const double *c, const double *Vg, double *out, void *scratch,
                                        int linear, cudaStream_t s);
cudaError_t ncg_launch_build_packmx (const ncg_eval_args_t *a, const double *X, const double *pack64,
                                     const double *c, const double *Ui, const double *Ug, const double *Vg,
                                     const double *mu, float *packmx, cudaStream_t s);
size_t      ncg_packmx_bytes (int kind, int n, int dp);
cudaError_t ncg_launch_eval_m2lnp_mixed (const ncg_eval_args_t *a, const double *Xq, const float *packmx,
                                         const double *mu, const double *Vg, double *out, void *scratch,
                                         cudaStream_t s);
cudaError_t ncg_launch_merge_f2 (const void *part, int nparts, int64_t m, double shift, const double *dshift,
                                 double d_ln_href, double *out, cudaStream_t s);
const double *ncg_packmx_cshift (const float *packmx, int kind, int n, int dp);
const double *ncg_packmx_kappa_max (const float *packmx, int kind, int n, int dp);
size_t      ncg_noalloc_scratch_bytes (void);
int64_t     ncg_noalloc_max_points (void);
cudaError_t ncg_launch_eval_m2lnp_fp64_noalloc (const ncg_eval_args_t *a, const double *Xq, const double *pack64,
                                                const double *c, const double *Vg, double *out, cudaStream_t s);
cudaError_t ncg_launch_dfma_peak (double *out, int blocks, int iters, cudaStream_t s);
/* raise (never lower) a kernel's dynamic shared-memory limit on the current device; limit[NCG_MAX_DEVICES] */
#define NCG_MAX_DEVICES 64
cudaError_t ncg_raise_smem_limit (const void *fn, size_t bytes, int *limit);
cudaError_t ncg_launch_nonfinite (const double *X, int64_t n, int32_t *flag, cudaStream_t s);

/* The mixed form whitens with FP32 arithmetic; its chi^2 error grows with the
 * infinity-norm condition number of the per-kernel whitening W'_i.  Above this
 * bound the mixed request is served by the FP64 form. */
#define NCG_MIXED_KAPPA_MAX 1000.0

/* ---- tensor-core eval (ncg_eval_tc.cu) ---- */
int         ncg_tc_supported (int kind, int dp);
size_t      ncg_tc_B_bytes (int n, int dp);
size_t      ncg_tc_scratch_bytes (int64_t m, int n, int dp);
cudaError_t ncg_launch_build_tc_B (const float *packmx, int kind, int n, int dp, int kernel, double nu, uint8_t *B,
                                   cudaStream_t s);
/* ev (may be NULL): two events recorded on s around the main kernel only */
cudaError_t ncg_launch_eval_tc (const ncg_eval_args_t *a, const double *Xq, const uint8_t *B, const double *mu,
                                const double *Vg, const double *cshift, void *scratch, double *out, int *flag_host,
                                cudaEvent_t *ev, cudaStream_t s);
cudaError_t ncg_launch_compute_IM (const ncg_eval_args_t *a, const double *X, const double *pack64,
                                   const double *lnnorm, double kernel_lnnorm, const double *f,
                                   double *IM, cudaStream_t s);
cudaError_t ncg_launch_reduce_minmax (const double *v, int n, double *out2, cudaStream_t s);

/* ---- multi-problem eval (ncg_batch.cu) ----
 * One problem of a persistent multi-problem launch.  x_off / out_off index
 * the launch's concatenated point and output arrays (in doubles); part holds
 * the problem's [ns][m] (gamma, lambda) pairs (double2 for FP64 tiles, float2
 * for mixed ones); tile_cnt[bx] counts the finished slices of each point tile
 * and is reset by the tile's merger, so it is zero between launches. */
typedef struct ncg_bprob
{
  ncg_eval_args_t a;
  const double *pack64, *c, *Vg, *mu, *dshift;
  const float *packmx;
  int64_t x_off, out_off;
  void *part;
  int32_t *tile_cnt;
  int32_t kper, ns, bx, cls;
} ncg_bprob_t;

/* class of a problem: tile arithmetic (0 FP64, 1 mixed SIMT), padded
 * dimension, kind and kernel */
#define NCG_BCLS(mixed, dp, kind, kernel) ((((mixed) * 8 + ((dp) / 4 - 1)) * 2 + (kind)) * 2 + (kernel))
#define NCG_BATCH_NCLS 64

/* which classes a persistent launch carries */
enum { NCG_BSET_ALL = 0, NCG_BSET_SMALL = 1, NCG_BSET_LARGE = 2 };   /* all dp; dp <= 16; dp > 16 */
#define NCG_BSET_SPLIT_DP 16

int         ncg_batch_chunk (int cls);
size_t      ncg_batch_smem_bytes (int mixed, int set);
int         ncg_batch_ctas_per_sm (int mixed, int set);
cudaError_t ncg_launch_batch_eval (int mixed, int set, const ncg_bprob_t *probs, const int32_t *items, int nitems,
                                   int32_t *counter, const double *Xq, double *out, int grid, cudaStream_t s);

/* ---- serving loop device steps (ncg_serve.cu) ---- */
cudaError_t ncg_launch_serve_target (const double *X, int64_t n, int d, const double *L, double *out, cudaStream_t s);
cudaError_t ncg_launch_serve_accept (double *X, double *m2lnL, const double *prop, const double *m2lnL_prop,
                                     const double *q, const double *u, int64_t n, int d, int explore,
                                     unsigned long long *accepted, cudaStream_t s);
cudaError_t ncg_launch_serve_mix (double *q, const double *X, const double *prop, const double *rw, int64_t n, int d,
                                  double p, cudaStream_t s);

/* ---- sample (ncg_sample.cu) ---- */
cudaError_t ncg_launch_wcum (const double *w, int n, double *wcum, cudaStream_t s);
cudaError_t ncg_launch_kernel_choose (const double *wcum, int n, const double *u, int64_t m,
                                      int32_t *idx, cudaStream_t s);
cudaError_t ncg_launch_sample (int kind, int kernel, int d, double nu, double href,
                               const double *wcum, int n, const double *X, const double *Ui,
                               const double *U, const double *u, const double *z, const double *chisq,
                               int64_t m, double *x, int32_t *idx, cudaStream_t s);
cudaError_t ncg_launch_sample_at (int kind, int kernel, int d, double nu, double href, const double *X,
                                  const double *Ui, const double *U, const int32_t *kidx, const double *z,
                                  const double *chisq, int64_t m, double *x, cudaStream_t s);
cudaError_t ncg_launch_im_rowsums (const double *IM, int n, double *rowx, double *diag, cudaStream_t s);

/* ---- dense linear algebra for prepare_interp (ncg_linalg.cu) ---- */
cudaError_t ncg_launch_syrk_upper (const double *A, int nrows, int ncols, double *M, cudaStream_t s);
size_t      ncg_gemv_t_scratch (int nrows, int ncols);
cudaError_t ncg_launch_gemv_ex (const double *A, int nrows, int ncols, int trans, double alpha,
                                const double *x, double beta, double *y, double *part, cudaStream_t s);
cudaError_t ncg_launch_normalize_weights (double *w, int n, double shrink, int32_t *bad, cudaStream_t s);
cudaError_t ncg_launch_gather_sub (const double *M, int n, const int32_t *P, int np, double *Msub,
                                   const double *b, double *bsub, cudaStream_t s);
cudaError_t ncg_launch_potrf (double *A, int n, int32_t *info, double *work, cudaStream_t s);
cudaError_t ncg_launch_potrs (const double *U, int n, double *b, double *work, cudaStream_t s);
/* the NNLS solve's fallbacks: symmetric solve of the upper-stored A (n x n,
 * overwritten) with right-hand side b (overwritten by x), *info = k + 1 at an
 * exactly zero pivot; least squares A[:, P] x = f by Householder QR (Q:
 * nrows x np work, y: nrows work, sc: 3 scalars) */
cudaError_t ncg_launch_sysv (double *A, int n, double *b, int32_t *info, cudaStream_t s);
cudaError_t ncg_launch_gels (const double *A, int nrows, int ncols, const int32_t *P, int np, const double *f,
                             double *Q, double *y, double *sc, double *x, cudaStream_t s);

/* mixed NNLS: FP32 preconditioner, FP64 conjugate-gradient refinement */
enum { NCG_PCG_RZ = 0, NCG_PCG_PQ, NCG_PCG_RZN, NCG_PCG_ZRP, NCG_PCG_RR, NCG_PCG_BB, NCG_PCG_ERR, NCG_PCG_NSC = 8 };
cudaError_t ncg_launch_syrk_upper_f32 (const double *A, int nrows, int ncols, float *M, cudaStream_t s);
cudaError_t ncg_launch_colsumsq (const double *A, int nrows, int ncols, double *out, cudaStream_t s);
cudaError_t ncg_launch_gather_scaled_f32 (const float *M32, int n, const int32_t *P, int np, const double *diagM,
                                          double shift, float *Msub, double *Dsub, const double *b, double *bsub,
                                          cudaStream_t s);
cudaError_t ncg_launch_potrf_f32 (float *A, int n, int32_t *info, float *pk, cudaStream_t s);
/* tensor-core (TF32x3) symmetric rank-K updates, ncg_syrk_tc.cu */
size_t      ncg_syrk_tc_pack_bytes (int nn, int K);
cudaError_t ncg_launch_syrk_tc (const void *pk, int K, int nn, float *C, int ldc, int mode, int *err,
                                cudaStream_t s);
cudaError_t ncg_launch_syrk_upper_tc_f64 (const double *A, int nrows, int ncols, float *C, void *scratch,
                                          size_t cap, int *err, cudaStream_t s);
cudaError_t ncg_launch_pcg_matvec (const double *A, int nrows, int n, const int32_t *P, int np, const double *v,
                                   double *vf, double *yf, double *qf, double *part, double *q, cudaStream_t s);
size_t      ncg_pcg_trinv_bytes (int n);
size_t      ncg_pcg_sync_bytes (int n);
size_t      ncg_pcg_chain_bytes (int n);
cudaError_t ncg_launch_trinv_diag_f32 (const float *U, int n, float *V, cudaStream_t s);
cudaError_t ncg_launch_pcg_precond (const float *R, const float *V, const double *D, int np, const double *r,
                                    void *chain, uint32_t *epoch, double *z, int32_t *sync, double *err,
                                    cudaStream_t s);
cudaError_t ncg_launch_pcg_dot (const double *u0, const double *v0, const double *u1, const double *v1,
                                const double *w, int n, double *sc, int out0, int out1, cudaStream_t s);
cudaError_t ncg_launch_pcg_step (double *x, double *r, double *rprev, const double *p, const double *q, int n,
                                 const double *sc, cudaStream_t s);
cudaError_t ncg_launch_pcg_dir (double *p, const double *z, int n, double *sc, cudaStream_t s);
cudaError_t ncg_launch_rsub (const double *b, double *r, int n, cudaStream_t s);
cudaError_t ncg_launch_scatter_x (const double *xsub, const int32_t *P, int np, int n, double *x,
                                  cudaStream_t s);
cudaError_t ncg_launch_residual_norm (const double *A, int nrows, int ncols, const double *x,
                                      const double *f, double *res, double *rnorm2, cudaStream_t s);

#ifdef __cplusplus
}
#endif

#endif /* NCG_INTERNAL_H */
