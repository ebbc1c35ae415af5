/*
 * ncg_oracle.h -- CPU oracle for the KDE/VKDE proposal path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C99 restatement of NumCosmo's
 * NcmStatsDist / NcmStatsDistKDE / NcmStatsDistVKDE FP64 CPU path, used by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the
 * checker.  The product library (numcosmo_gb300/csrc) never links or calls it.
 *
 * Pinning: the k-nearest-neighbour step is checked against the reference's own
 * vendored kd-tree (numcosmo/external/misc/kdtree.c, rb_knn_list.c) compiled
 * from the reference sources into oracle/_ref; the kernel formulas are checked
 * against the closed forms of tests/c/ncm/stats/test_ncm_stats_dist_kernel.c.
 * The rest (Welford covariance, Cholesky, nearPD, NNLS) cannot be run from the
 * reference here (GLib/GSL/LAPACK are absent) and is cross-checked against
 * independent numpy/scipy computations instead: parity there is unpinned.
 *
 * Conventions (as in the reference): matrices are row-major; a covariance
 * decomposition U is upper triangular with Sigma = U^T U
 * (numcosmo/ncm/algebra/ncm_lapack.h:32-33 swaps UPLO for the row-major view).
 */
#ifndef NCG_ORACLE_H
#define NCG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_KDE = 0, ORC_VKDE = 1 };
enum { ORC_GAUSS = 0, ORC_ST = 1 };
/* NcmStatsDistKDECovType (numcosmo/ncm/stats/ncm_stats_dist_kde.h:56-68); FIXED is not restated */
enum { ORC_COV_SAMPLE = 0, ORC_COV_FIXED = 1, ORC_COV_ROBUST_DIAG = 2, ORC_COV_ROBUST = 3 };

enum
{
  ORC_OK                   = 0,
  ORC_ERR_SAMPLE_TOO_SMALL = 2,
  ORC_ERR_TOO_FEW_LOCAL    = 3,
  ORC_ERR_NOT_PD           = 4,
  ORC_ERR_NOT_PREPARED     = 5,
  ORC_ERR_BAD_INPUT        = 6,
  ORC_ERR_INVALID          = 7,
};

/* NcmStatsDistCV (numcosmo/ncm/stats/ncm_stats_dist.h:77-85); prepare runs
 * NONE and SPLIT_NOFIT, prepare_interp NONE */
enum { ORC_CV_NONE = 0, ORC_CV_SPLIT = 1, ORC_CV_SPLIT_NOFIT = 2, ORC_CV_LOO = 3 };

typedef struct orc_sd orc_sd;

/* ---- building blocks (each cites the reference function it restates) ---- */
double orc_kernel_rot_bandwidth (int kernel, double nu, int d, double n);
double orc_kernel_lnnorm (int kernel, double nu, int d, const double *U);
double orc_kernel_eval_unnorm (int kernel, double nu, int d, double chi2);
void   orc_kernel_sum0 (int kernel, double nu, int d, int n, const double *chi2,
                        const double *w, const double *lnu, double *lnK,
                        double *gamma, double *lambda);
void   orc_kernel_sum1 (int kernel, double nu, int d, int n, const double *chi2,
                        const double *w, double lnnorm, double *lnK,
                        double *gamma, double *lambda);
void   orc_welford_cov (const double *X, const int *rows, int nrows, int d, double *cov);
int    orc_cholesky_upper (double *A, int d);
double orc_cholesky_lndet (const double *U, int d);
int    orc_nearPD (double *A, int d, int maxiter);
int    orc_cholesky_decomp_fallback (const double *cov, double *U, int d, int maxiter);
int    orc_sym_eigen (const double *A, int n, double *eval, double *evec);
double orc_qn (double *v, int m);
void   orc_cov_robust_diag (const double *X, const int *rows, int nrows, int d, double *cov);
void   orc_cov_robust_ogk (const double *X, const int *rows, int nrows, int d, double *cov);
void   orc_knn (const double *Y, int n, int d, int k, int *out, int nthreads);
void orc_knn_q (const double *Y, int n, int nq, int d, int k, int *out, int nthreads);
void orc_sd_set_cv (orc_sd *sd, int cv_type, double split_frac);
/* the LOO Monte Carlo's draws, in the order ncm_stats_dist_sample2 takes them
 * (per pair: u, z1[d], c1 (Student-t), z2[d], c2); every AMISE evaluation
 * starts again at the first pair, as the reference reseeds its generator */
void orc_sd_set_loo_draws (orc_sd *sd, long npairs, const double *u, const double *z1, const double *c1,
                           const double *z2, const double *c2);
int  orc_sd_get_loo_short (orc_sd *sd);
/* CV_SPLIT's restarts: unit gaussians consumed in order across calls (the
 * reference's own generator, seeded at init) */
void orc_sd_set_split_draws (orc_sd *sd, long n, const double *g);
/* skip the CV type's bandwidth fit (the weight fit at a given bandwidth) */
void orc_sd_set_no_fit (orc_sd *sd, int no_fit);
/* dlevmar_dif restated for one parameter (see ncg_oracle.c) */
typedef void (*orc_lm_fn) (double p, double *hx, int n, void *ctx);
int  orc_lm1_dif (orc_lm_fn func, double *p, int n, int itmax, const double *opts, void *ctx);
int orc_sd_get_nk (orc_sd *sd);
double orc_sd_get_over_smooth (orc_sd *sd);
/* solves of the last orc_nnls_solve that took the LU / the QR fallback */
void orc_nnls_fallbacks (int *lu, int *qr);
double orc_nnls_solve (const double *A, int nrows, int ncols, const double *f,
                       double *x, int nthreads);

/* ---- the StatsDist object ---- */
orc_sd *orc_sd_new (int kind, int kernel, double nu, int d);
void    orc_sd_free (orc_sd *sd);
void    orc_sd_set_params (orc_sd *sd, double over_smooth, double shrink,
                           double local_frac, int use_rot_href, int nearPD_maxiter);
void    orc_sd_set_threads (orc_sd *sd, int nthreads);
void    orc_sd_set_cov_type (orc_sd *sd, int cov_type);
void    orc_sd_set_cov_fixed (orc_sd *sd, const double *cov);
void    orc_sd_set_sample (orc_sd *sd, const double *X, int n);
int     orc_sd_prepare (orc_sd *sd);
int     orc_sd_prepare_interp (orc_sd *sd, const double *m2lnp);
double  orc_sd_eval_m2lnp (orc_sd *sd, const double *x);
void    orc_sd_eval_m2lnp_batch (orc_sd *sd, const double *X, int m, double *out);
double  orc_sd_eval (orc_sd *sd, const double *x);
void    orc_sd_eval_batch (orc_sd *sd, const double *X, int m, double *out);
int     orc_sd_compute_IM (orc_sd *sd, double *IM);
int     orc_sd_kernel_choose (orc_sd *sd, double u);
int     orc_sd_sample (orc_sd *sd, double u, const double *z, double chisq, double *x);
void    orc_sd_sample_batch (orc_sd *sd, int n, const double *u, const double *z,
                             const double *chisq, double *x, int *idx);

/* getters */
int     orc_sd_get_n (orc_sd *sd);
int     orc_sd_get_k (orc_sd *sd);
double  orc_sd_get_href (orc_sd *sd);
double  orc_sd_get_rnorm (orc_sd *sd);
double  orc_sd_get_kernel_lnnorm (orc_sd *sd);
int     orc_sd_get_interp_branch (orc_sd *sd);
int     orc_sd_get_chol_fallbacks (orc_sd *sd);
void    orc_sd_get_weights (orc_sd *sd, double *w);
void    orc_sd_get_sample (orc_sd *sd, double *X);
void    orc_sd_get_cov (orc_sd *sd, double *cov);
void    orc_sd_get_U (orc_sd *sd, double *U);
void    orc_sd_get_invUsample (orc_sd *sd, double *Y);
void    orc_sd_get_Ui (orc_sd *sd, int i, double *U);
void    orc_sd_get_lnnorms (orc_sd *sd, double *lnnorms);
void    orc_sd_get_knn (orc_sd *sd, int *knn);

#ifdef __cplusplus
}
#endif

#endif /* NCG_ORACLE_H */
