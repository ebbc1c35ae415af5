/*
 * ncg_host.h -- the handle structure shared by the host C files.
 */
#ifndef NCG_HOST_H
#define NCG_HOST_H

#include <stdint.h>
#include <cuda_runtime_api.h>

#include "ncg_internal.h"

typedef struct ncg_caps
{
  size_t X, Y, cov, U, Ui, lnnorm, w, c, wcum, pack64, Vg, packmx, knn, flag, ids, keys, st, scratch, q, qo, qi, f,
         mu, cal, rq, cv, loo;
} ncg_caps_t;

/* prepare_interp / NNLS device state (ncg_interp.c) */
typedef struct ncg_nnls_dev
{
  double *IM, *M, *b, *f1, *x, *xsub, *Msub, *bsub, *res, *mg, *part, *red;
  int32_t *P, *info;
  size_t cIM, cM, cb, cf1, cx, cxsub, cMsub, cbsub, cres, cmg, cpart, cred, cP, cinfo;
  /* mixed solver: FP32 A^T A and factor, FP64 diagonal and CG vectors */
  float *M32, *R32, *t32, *Vi, *pk32;
  double *diagM, *D, *xv, *pv, *qv, *zv, *rv, *rp, *vf, *yf, *qf, *sc;
  int32_t *csync;
  size_t cM32, cR32, ct32, cVi, cpk32, cdiagM, cD, cxv, cpv, cqv, czv, crv, crp, cvf, cyf, cqf, csc, ccsync;
  /* the least-squares fallback's Householder work: A_P (n x np) and f | 3 scalars */
  double *Q, *qy;
  size_t cQ, cqy;
  int M64_ready;          /* the FP64 A^T A exists (mixed solver fallback) */
  uint32_t cs_epoch;      /* launches of the chained solves (their words carry it) */
} ncg_nnls_dev_t;

/* counters of the last prepare_interp */
typedef struct ncg_interp_stats
{
  int32_t n_solves;       /* active-set solves                               */
  int32_t n_cg_iters;     /* conjugate-gradient iterations (mixed solver)    */
  int32_t n_shifted;      /* FP32 factorisations that needed a diagonal shift */
  int32_t n_fp64;         /* solves served by the FP64 factorisation         */
  int32_t n_lu;           /* of those, solves whose normal equations were not
                             positive definite (the symmetric LU fallback)   */
  int32_t n_qr;           /* of those, solves that went on to least squares  */
} ncg_interp_stats_t;

struct ncg_sd
{
  ncg_kind_t kind;
  ncg_kernel_t kernel;
  uint32_t d;
  int dp;
  double nu;
  ncg_sd_config_t cfg;
  double *cov_fixed;

  /* host copy of the sample */
  double *hX;
  uint64_t n, cap_n;
  uint64_t nk;            /* kernels of the last prepare: n, or ceil(n split_frac) with a split CV */
  double split_frac;      /* "split-frac" of the split cross-validation types */

  /* prepared state */
  int prepared, wcum_ready, packmx_ready, tcB_ready, interp_branch, last_path;
  uint64_t gen;           /* bumps whenever the prepared state or the weights change */
  double mixed_kappa;     /* max_i cond(W'_i) of the mixed operand */
  int tc_ok;              /* the tensor-core operand passed its accuracy check */
  double tc_err;          /* its measured error on the kernel centres */
  int32_t *h_flag;        /* mapped pinned: error word of the last tensor-core launch */
  int32_t *d_flag_alias;  /* its device address, written by the merge kernel */
  uint8_t *dtcB;          /* tensor-core kernel tiles */
  size_t cap_tcB;
  uint32_t k;
  uint64_t n_fallback;
  double href, kernel_lnnorm, rnorm;
  double *hw;

  /* device */
  cudaStream_t stream;
  int own_stream;
  cudaMemPool_t pool;     /* with async_alloc: the pool to allocate from (NULL: the device's default) */
  double *drq;            /* robust covariance work (sigma, sigma_z, C, E per set) */
  double *dX, *dY, *dcov, *dU, *dUi, *dlnnorm, *dw, *dc, *dwcum, *dpack64, *dVg, *dq, *dqo, *df, *dmu, *dcal, *dcv;
  float *dpackmx;
  int32_t *dknn, *dflag, *dids, *dqi;
  void *dkeys, *dscratch;
  void *dloo;             /* the LOO Monte Carlo's windows (kernels, draws, points) */
  ncg_rng_t *cv_rng;      /* the split fit's generator (the reference's own, seeded 0 at init) */
  ncg_prep_status_t *dst;
  ncg_caps_t cap;
  ncg_nnls_dev_t nn;
  ncg_interp_stats_t istats;

  /* CUDA events around the tensor-core eval kernel (ncg_sd_set_kernel_timing) */
  int ktime_on, ktime_valid;
  cudaEvent_t kev[2];

  /* caller-owned device arena for the O(n^2) NNLS matrices (NULL: owned) */
  void *ws_base;
  size_t ws_size, ws_off;
};

void         ncg_set_error (const char *fmt, ...);
ncg_status_t ncg_cuda_status (cudaError_t e, const char *where);
ncg_status_t ncg_dev_reserve (void **p, size_t *cap, size_t bytes);
ncg_status_t ncg_sd_reserve (ncg_sd_t *sd, void **p, size_t *cap, size_t bytes);
void         ncg_sd_release (ncg_sd_t *sd, void *p);
double       ncg_rot_bandwidth (int kernel, double nu, int d, double n);
void         ncg_nnls_free (ncg_sd_t *sd);
void         ncg_sd_fill_args (ncg_sd_t *sd, uint64_t m, ncg_eval_args_t *a);
size_t       ncg_sd_workspace_bytes_for (uint64_t n, int mixed);
size_t       ncg_sd_workspace_bytes_rect (uint64_t nobs, uint64_t nk, int mixed);
uint64_t     ncg_sd_kernels_for (const ncg_sd_t *sd, uint64_t n);
ncg_status_t ncg_sd_im_rowsums (ncg_sd_t *sd, double *rowx, double *diag);
double       ncg_sd_href_for (ncg_sd_t *sd);
ncg_status_t ncg_sd_href_operand (ncg_sd_t *sd);
void         ncg_sd_prepare_reserve (ncg_sd_t *sd);
void         ncg_sd_interp_reserve (ncg_sd_t *sd);
ncg_status_t ncg_sd_ensure_packmx (ncg_sd_t *sd);
ncg_status_t ncg_sd_ensure_tc (ncg_sd_t *sd);      /* tensor-core operand + its check (VKDE) */

#endif /* NCG_HOST_H */
