/*
 * ncg_api.c -- host side of the C-ABI (include/ncg.h).
 *
 * Owns the handle: the host copy of the sample (add_obs copies, as
 * ncm_stats_dist_add_obs does, numcosmo/ncm/stats/ncm_stats_dist.c:1680-1686),
 * the device buffers, and the control flow of prepare / prepare_interp, which
 * runs the CUDA kernels of ncg_prepare.cu, ncg_eval.cu, ncg_sample.cu and
 * ncg_linalg.cu.  No numerical work of the path runs on the host apart from
 * scalar formulas (href) and the prepare_interp range cut (a sort of the
 * caller's m2lnp values), which the reference also runs serially.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "ncg_internal.h"
#include "ncg_host.h"

#define NCG_VERSION_STRING "ncg 0.1.0 sm_103a"

static __thread char g_err[512];

void
ncg_set_error (const char *fmt, ...)
{
  va_list ap;

  va_start (ap, fmt);
  vsnprintf (g_err, sizeof (g_err), fmt, ap);
  va_end (ap);
}

const char *
ncg_last_error (void)
{
  return g_err;
}

const char *
ncg_version (void)
{
  return NCG_VERSION_STRING;
}

const char *
ncg_status_string (ncg_status_t s)
{
  switch (s)
  {
    case NCG_OK: return "ok";
    case NCG_ERR_INVALID_ARG: return "invalid argument";
    case NCG_ERR_SAMPLE_TOO_SMALL: return "the sample is too small";
    case NCG_ERR_TOO_FEW_LOCAL: return "too few observations for the local covariance (local_frac * n < 2)";
    case NCG_ERR_NOT_PD: return "covariance is not positive definite after the nearPD and diagonal fallbacks";
    case NCG_ERR_NOT_PREPARED: return "distribution not prepared";
    case NCG_ERR_NONFINITE: return "non-finite input";
    case NCG_ERR_UNSUPPORTED: return "option not supported on the GPU path";
    case NCG_ERR_CUDA: return "CUDA error";
    case NCG_ERR_OUT_OF_MEMORY: return "out of device memory or over budget";
    case NCG_ERR_TIMEOUT: return "device wait timed out";
    case NCG_ERR_BAD_WEIGHTS: return "the fitted weights sum to a non-positive value";
    case NCG_ERR_BUSY: return "busy";
    default: return "unknown status";
  }
}

ncg_status_t
ncg_cuda_status (cudaError_t e, const char *where)
{
  if (e == cudaSuccess)
    return NCG_OK;

  ncg_set_error ("%s: %s", where, cudaGetErrorString (e));

  if (e == cudaErrorMemoryAllocation)
    return NCG_ERR_OUT_OF_MEMORY;

  return NCG_ERR_CUDA;
}

#define CK(call, where)                                   \
  do {                                                    \
    ncg_status_t _s = ncg_cuda_status ((call), (where));  \
    if (_s != NCG_OK)                                     \
      return _s;                                          \
  } while (0)

ncg_status_t
ncg_measure_fp64_peak (int32_t device, double *tflops)
{
  const int iters = 2048;
  cudaStream_t st = NULL;
  cudaEvent_t e0 = NULL, e1 = NULL;
  double *out = NULL;
  int nsm = 0;
  float ms = 0.0f;
  ncg_status_t r;

  if (tflops == NULL)
    return NCG_ERR_INVALID_ARG;

  if ((r = ncg_cuda_status (cudaSetDevice (device), "cudaSetDevice")) != NCG_OK)
    return r;

  if ((r = ncg_cuda_status (cudaDeviceGetAttribute (&nsm, cudaDevAttrMultiProcessorCount, device), "SM count")) != NCG_OK)
    return r;

  const int blocks = 8 * nsm;

  r = ncg_cuda_status (cudaStreamCreateWithFlags (&st, cudaStreamNonBlocking), "cudaStreamCreate");

  if (r == NCG_OK)
    r = ncg_cuda_status (cudaMalloc ((void **) &out, sizeof (double) * 256 * (size_t) blocks), "cudaMalloc");

  if (r == NCG_OK)
    r = ncg_cuda_status (cudaEventCreate (&e0), "cudaEventCreate");

  if (r == NCG_OK)
    r = ncg_cuda_status (cudaEventCreate (&e1), "cudaEventCreate");

  if (r == NCG_OK)
    r = ncg_cuda_status (ncg_launch_dfma_peak (out, blocks, iters / 8, st), "dfma warm-up");

  if (r == NCG_OK)
    r = ncg_cuda_status (cudaEventRecord (e0, st), "cudaEventRecord");

  if (r == NCG_OK)
    r = ncg_cuda_status (ncg_launch_dfma_peak (out, blocks, iters, st), "dfma");

  if (r == NCG_OK)
    r = ncg_cuda_status (cudaEventRecord (e1, st), "cudaEventRecord");

  if (r == NCG_OK)
    r = ncg_cuda_status (cudaEventSynchronize (e1), "cudaEventSynchronize");

  if (r == NCG_OK)
    r = ncg_cuda_status (cudaEventElapsedTime (&ms, e0, e1), "cudaEventElapsedTime");

  if (r == NCG_OK)
    *tflops = 2.0 * 8.0 * 16.0 * iters * 256.0 * blocks / (ms * 1e-3) / 1e12;

  if (e0)
    cudaEventDestroy (e0);

  if (e1)
    cudaEventDestroy (e1);

  if (out)
    cudaFree (out);

  if (st)
    cudaStreamDestroy (st);

  return r;
}

void
ncg_sd_config_init (ncg_sd_config_t *cfg)
{
  if (cfg == NULL)
    return;

  cfg->over_smooth    = 1.0;
  cfg->shrink         = 0.01;
  cfg->local_frac     = 0.05;
  cfg->use_rot_href   = 0;
  cfg->nearPD_maxiter = 200;
  cfg->cv_type        = NCG_CV_NONE;
  cfg->cov_type       = NCG_COV_SAMPLE;
  cfg->precision      = NCG_PREC_FP64;
  cfg->device         = 0;
  cfg->async_alloc    = 0;
}

/* grow a device buffer to at least bytes */
ncg_status_t
ncg_dev_reserve (void **p, size_t *cap, size_t bytes)
{
  if (*cap >= bytes && *p != NULL)
    return NCG_OK;

  if (*p)
    cudaFree (*p);

  *p   = NULL;
  *cap = 0;

  if (bytes == 0)
    return NCG_OK;

  CK (cudaMalloc (p, bytes), "cudaMalloc");
  *cap = bytes;

  return NCG_OK;
}

/* a handle's buffer: ncg_dev_reserve, or with async_alloc the stream-ordered
 * allocator on the handle's stream */
ncg_status_t
ncg_sd_reserve (ncg_sd_t *sd, void **p, size_t *cap, size_t bytes)
{
  if (!sd->cfg.async_alloc)
    return ncg_dev_reserve (p, cap, bytes);

  if (*cap >= bytes && *p != NULL)
    return NCG_OK;

  if (*p)
    cudaFreeAsync (*p, sd->stream);

  *p   = NULL;
  *cap = 0;

  if (bytes == 0)
    return NCG_OK;

  if (sd->pool)
    CK (cudaMallocFromPoolAsync (p, bytes, sd->pool, sd->stream), "cudaMallocFromPoolAsync");
  else
    CK (cudaMallocAsync (p, bytes, sd->stream), "cudaMallocAsync");
  *cap = bytes;

  return NCG_OK;
}

void
ncg_sd_release (ncg_sd_t *sd, void *p)
{
  if (p == NULL)
    return;

  if (sd->cfg.async_alloc)
    cudaFreeAsync (p, sd->stream);
  else
    cudaFree (p);
}

static void
_dev_free_all (ncg_sd_t *sd)
{
  void **bufs[] = {
    (void **) &sd->dX, (void **) &sd->dY, (void **) &sd->dcov, (void **) &sd->dU, (void **) &sd->dUi,
    (void **) &sd->dlnnorm, (void **) &sd->dw, (void **) &sd->dc, (void **) &sd->dwcum, (void **) &sd->dpack64,
    (void **) &sd->dVg, (void **) &sd->dpackmx, (void **) &sd->dknn, (void **) &sd->dflag, (void **) &sd->dids,
    (void **) &sd->dkeys, (void **) &sd->dst, (void **) &sd->dscratch, (void **) &sd->dq,
    (void **) &sd->dqo, (void **) &sd->dqi, (void **) &sd->df, (void **) &sd->dmu, (void **) &sd->dcal, (void **) &sd->dcv, (void **) &sd->dloo,
    (void **) &sd->drq,
  };

  for (size_t i = 0; i < sizeof (bufs) / sizeof (bufs[0]); i++)
  {
    ncg_sd_release (sd, *bufs[i]);
    *bufs[i] = NULL;
  }

  memset (&sd->cap, 0, sizeof (sd->cap));
  ncg_nnls_free (sd);
}

ncg_status_t
ncg_sd_new (ncg_kind_t kind, ncg_kernel_t kernel, uint32_t dim, double nu, const ncg_sd_config_t *cfg,
            ncg_sd_t **out)
{
  ncg_sd_t *sd;

  if (out == NULL)
    return NCG_ERR_INVALID_ARG;

  *out = NULL;

  if ((kind != NCG_KDE && kind != NCG_VKDE) || (kernel != NCG_KERNEL_GAUSS && kernel != NCG_KERNEL_ST))
  {
    ncg_set_error ("ncg_sd_new: unknown kind or kernel");

    return NCG_ERR_INVALID_ARG;
  }

  if (dim == 0 || dim > NCG_DMAX)
  {
    ncg_set_error ("ncg_sd_new: dimension %u outside 1..%d", dim, NCG_DMAX);

    return NCG_ERR_UNSUPPORTED;
  }

  if (kernel == NCG_KERNEL_ST && !(nu >= 1.0))
  {
    ncg_set_error ("ncg_sd_new: Student-t nu must be >= 1 (ncm_stats_dist_kernel_st.c:208-214)");

    return NCG_ERR_INVALID_ARG;
  }

  sd = calloc (1, sizeof (ncg_sd_t));

  if (sd == NULL)
    return NCG_ERR_OUT_OF_MEMORY;

  sd->kind       = kind;
  sd->kernel     = kernel;
  sd->d          = dim;
  sd->dp         = ncg_pad_dim ((int) dim);
  sd->nu         = (kernel == NCG_KERNEL_ST) ? nu : 0.0;
  sd->split_frac = 0.5;   /* the "split-frac" property's construct-time default (ncm_stats_dist.c:428-434) */

  if (cfg)
    sd->cfg = *cfg;
  else
    ncg_sd_config_init (&sd->cfg);

  {
    ncg_status_t s = ncg_cuda_status (cudaSetDevice (sd->cfg.device), "cudaSetDevice");

    if (s == NCG_OK)
      s = ncg_cuda_status (cudaStreamCreateWithFlags (&sd->stream, cudaStreamNonBlocking), "cudaStreamCreate");

    if (s == NCG_OK)
      s = ncg_cuda_status (cudaHostAlloc ((void **) &sd->h_flag, sizeof (int32_t) * 4, cudaHostAllocMapped),
                           "cudaHostAlloc");

    if (s == NCG_OK)
      s = ncg_cuda_status (cudaHostGetDevicePointer ((void **) &sd->d_flag_alias, sd->h_flag, 0),
                           "cudaHostGetDevicePointer");

    if (s != NCG_OK)
    {
      if (sd->stream)
        cudaStreamDestroy (sd->stream);

      free (sd);

      return s;
    }

    sd->h_flag[0] = 0;
  }

  sd->own_stream = 1;
  *out           = sd;

  return NCG_OK;
}

ncg_status_t
ncg_sd_free (ncg_sd_t *sd)
{
  if (sd == NULL)
    return NCG_OK;

  cudaSetDevice (sd->cfg.device);

  if (sd->stream)
    cudaStreamSynchronize (sd->stream);

  _dev_free_all (sd);

  ncg_sd_release (sd, sd->dtcB);
  sd->dtcB = NULL;

  if (sd->stream)
    cudaStreamSynchronize (sd->stream);

  if (sd->h_flag)
    cudaFreeHost (sd->h_flag);

  if (sd->kev[0])
  {
    cudaEventDestroy (sd->kev[0]);
    cudaEventDestroy (sd->kev[1]);
  }

  if (sd->own_stream && sd->stream)
    cudaStreamDestroy (sd->stream);

  if (sd->cv_rng)
    ncg_rng_free (sd->cv_rng);

  free (sd->hX);
  free (sd->cov_fixed);
  free (sd->hw);
  free (sd);

  return NCG_OK;
}

ncg_status_t
ncg_sd_set_stream (ncg_sd_t *sd, void *cuda_stream)
{
  if (sd == NULL)
    return NCG_ERR_INVALID_ARG;

  cudaStreamSynchronize (sd->stream);

  if (cuda_stream == NULL)
  {
    if (!sd->own_stream)
    {
      CK (cudaStreamCreateWithFlags (&sd->stream, cudaStreamNonBlocking), "cudaStreamCreate");
      sd->own_stream = 1;
    }
  }
  else
  {
    if (sd->own_stream)
      cudaStreamDestroy (sd->stream);

    sd->stream     = (cudaStream_t) cuda_stream;
    sd->own_stream = 0;
  }

  return NCG_OK;
}

/* error word of the last tensor-core launch, valid after a stream sync */
static ncg_status_t
_check_device_flag (ncg_sd_t *sd)
{
  if (sd->h_flag && sd->h_flag[0])
  {
    sd->h_flag[0] = 0;
    ncg_set_error ("tensor-core eval: a bounded pipeline wait timed out; results of that call are invalid");

    return NCG_ERR_TIMEOUT;
  }

  return NCG_OK;
}

ncg_status_t
ncg_sd_synchronize (ncg_sd_t *sd)
{
  if (sd == NULL)
    return NCG_ERR_INVALID_ARG;

  CK (cudaStreamSynchronize (sd->stream), "cudaStreamSynchronize");

  return _check_device_flag (sd);
}

#define SETTER(name, field, type, check)          \
  ncg_status_t name (ncg_sd_t * sd, type v)       \
  {                                               \
    if (sd == NULL || !(check))                   \
      return NCG_ERR_INVALID_ARG;                 \
    sd->cfg.field = v;                            \
    sd->prepared  = 0;                            \
    return NCG_OK;                                \
  }

SETTER (ncg_sd_set_over_smooth, over_smooth, double, v > 0.0)
SETTER (ncg_sd_set_shrink, shrink, double, v >= 0.0 && v <= 1.0)
SETTER (ncg_sd_set_local_frac, local_frac, double, v > 0.0 && v <= 1.0)
SETTER (ncg_sd_set_use_rot_href, use_rot_href, int32_t, 1)
SETTER (ncg_sd_set_nearPD_maxiter, nearPD_maxiter, int32_t, v >= 0)

ncg_status_t
ncg_sd_set_cov_type (ncg_sd_t *sd, ncg_cov_type_t cov_type)
{
  if (sd == NULL)
    return NCG_ERR_INVALID_ARG;

  if (cov_type < NCG_COV_SAMPLE || cov_type > NCG_COV_ROBUST)
    return NCG_ERR_INVALID_ARG;

  sd->cfg.cov_type = cov_type;
  sd->prepared     = 0;

  return NCG_OK;
}

ncg_status_t
ncg_sd_set_cov_fixed (ncg_sd_t *sd, const double *cov)
{
  if (sd == NULL || cov == NULL)
    return NCG_ERR_INVALID_ARG;

  for (uint32_t i = 0; i < sd->d * sd->d; i++)
    if (!isfinite (cov[i]))
      return NCG_ERR_NONFINITE;

  if (sd->cov_fixed == NULL)
    sd->cov_fixed = malloc (sizeof (double) * sd->d * sd->d);

  memcpy (sd->cov_fixed, cov, sizeof (double) * sd->d * sd->d);
  sd->prepared = 0;

  return NCG_OK;
}

ncg_status_t
ncg_sd_set_precision (ncg_sd_t *sd, ncg_precision_t precision)
{
  if (sd == NULL || (precision != NCG_PREC_FP64 && precision != NCG_PREC_MIXED && precision != NCG_PREC_MIXED_SIMT))
    return NCG_ERR_INVALID_ARG;

  sd->cfg.precision = precision;

  return NCG_OK;
}

ncg_status_t
ncg_sd_reset (ncg_sd_t *sd)
{
  if (sd == NULL)
    return NCG_ERR_INVALID_ARG;

  sd->n        = 0;
  sd->prepared = 0;

  return NCG_OK;
}

ncg_status_t
ncg_sd_add_obs_batch (ncg_sd_t *sd, const double *Y, uint64_t n)
{
  if (sd == NULL || (Y == NULL && n > 0))
    return NCG_ERR_INVALID_ARG;

  for (uint64_t i = 0; i < n * sd->d; i++)
    if (!isfinite (Y[i]))
    {
      ncg_set_error ("add_obs: non-finite coordinate at row %llu", (unsigned long long) (i / sd->d));

      return NCG_ERR_NONFINITE;
    }

  if (sd->n + n > sd->cap_n)
  {
    uint64_t nc = sd->cap_n ? sd->cap_n : 256;

    while (nc < sd->n + n)
      nc *= 2;

    double *p = realloc (sd->hX, sizeof (double) * nc * sd->d);

    if (p == NULL)
      return NCG_ERR_OUT_OF_MEMORY;

    sd->hX    = p;
    sd->cap_n = nc;
  }

  memcpy (sd->hX + sd->n * sd->d, Y, sizeof (double) * n * sd->d);
  sd->n       += n;
  sd->prepared = 0;

  return NCG_OK;
}

ncg_status_t
ncg_sd_add_obs (ncg_sd_t *sd, const double *y)
{
  return ncg_sd_add_obs_batch (sd, y, 1);
}

/* href: ncm_stats_dist.c:476-482 (base, KDE) and ncm_stats_dist_vkde.c:317-335 */
double
ncg_rot_bandwidth (int kernel, double nu, int d, double n)
{
  if (kernel == NCG_KERNEL_GAUSS)
    return pow (4.0 / (n * (d + 2.0)), 1.0 / (d + 4.0));
  else
  {
    const double nuc = (nu >= 3.0) ? nu : 3.0;
    const double dd  = (double) d;

    return pow (16.0 * ((nuc - 2) * (nuc - 2)) * (1.0 + dd + nuc) * (3.0 + dd + nuc) /
                ((2.0 + dd) * (dd + nuc) * (2.0 + dd + nuc) * (dd + 2.0 * nuc) * (2.0 + dd + 2.0 * nuc) * n),
                1.0 / (dd + 4.0));
  }
}

static double
_get_href (ncg_sd_t *sd)
{
  const double base = sd->cfg.over_smooth * ncg_rot_bandwidth (sd->kernel, sd->nu, (int) sd->d, (double) sd->nk);

  if (sd->kind == NCG_KDE)
    return base;

  if (sd->cfg.use_rot_href)
    return base / sd->cfg.local_frac;

  return sd->cfg.over_smooth;
}

#define RESERVE(ptr, field, bytes) \
  do { ncg_status_t _r = ncg_sd_reserve (sd, (void **) &sd->ptr, &sd->cap.field, (bytes)); if (_r != NCG_OK) return _r; } while (0)

static ncg_status_t
_reserve_prepare (ncg_sd_t *sd, uint32_t k)
{
  const size_t n = sd->n, d = sd->d, dp = sd->dp;     /* observations bound every kernel buffer */

  RESERVE (dX, X, n * d * sizeof (double));
  RESERVE (dY, Y, n * d * sizeof (double));
  RESERVE (dcov, cov, d * d * sizeof (double));
  RESERVE (dU, U, d * d * sizeof (double));
  RESERVE (dw, w, n * sizeof (double));
  RESERVE (dc, c, n * sizeof (double));
  RESERVE (dwcum, wcum, (n + 1) * sizeof (double));
  RESERVE (dlnnorm, lnnorm, n * sizeof (double));
  RESERVE (dpack64, pack64, n * (size_t) ncg_pack64_stride (sd->kind, (int) dp) * sizeof (double));
  RESERVE (dVg, Vg, (dp * (dp + 1) / 2 + 4) * sizeof (double));
  RESERVE (dmu, mu, dp * sizeof (double));
  RESERVE (dflag, flag, (n + 1) * sizeof (int32_t));
  RESERVE (dids, ids, (n + 2) * sizeof (int32_t));
  RESERVE (dst, st, sizeof (ncg_prep_status_t));

  if (sd->cfg.cov_type == NCG_COV_ROBUST_DIAG || sd->cfg.cov_type == NCG_COV_ROBUST)
    RESERVE (drq, rq, ncg_robust_work_doubles ((sd->kind == NCG_VKDE) ? (int) n : 1, (int) d) * sizeof (double));

  if (sd->kind == NCG_VKDE)
  {
    RESERVE (dUi, Ui, n * d * d * sizeof (double));
    RESERVE (dknn, knn, n * (size_t) k * sizeof (int32_t));

    {
      const size_t kb = ncg_knn_scratch_bytes ((int) n, (int) d, (int) k);

      if (kb)
        RESERVE (dkeys, keys, kb);
    }
  }

  return NCG_OK;
}

/* The device buffers a prepare of the current sample needs, reserved now with
 * the sizes ncg_sd_prepare reserves, so that handles prepared at the same time
 * from several host threads allocate nothing meanwhile (cudaMalloc
 * synchronises the whole device and would serialise them).  Anything the
 * prepare would reject is left for the prepare to report. */
void
ncg_sd_prepare_reserve (ncg_sd_t *sd)
{
  uint32_t k = 0;

  if (sd == NULL || sd->n == 0 || sd->n > 0x7fffffffULL || cudaSetDevice (sd->cfg.device) != cudaSuccess)
    return;

  if (sd->kind == NCG_VKDE)
  {
    const double lf = sd->cfg.local_frac * (double) sd->n;

    if (lf < 2)
      return;

    k = (uint32_t) (size_t) ((lf > 2) ? lf : 2);

    if (k > NCG_KNN_KMAX || k > sd->n)
      return;
  }

  (void) _reserve_prepare (sd, k);
}

/* nearPD pass over the flagged factors of M (count known on the host) */
static ncg_status_t
_nearpd_pass (ncg_sd_t *sd, double *M, int nmat, int32_t nflagged)
{
  if (nmat == 1)
  {
    CK (ncg_launch_nearpd (M, 1, NULL, (int) sd->d, sd->cfg.nearPD_maxiter, sd->dflag, sd->dst, sd->stream),
        "nearpd");
  }
  else
  {
    int32_t *cnt = sd->dids + sd->n;   /* trailing counter slot */

    CK (cudaMemsetAsync (cnt, 0, sizeof (int32_t), sd->stream), "memset");
    CK (ncg_launch_compact_flags (sd->dflag, nmat, sd->dids, cnt, sd->stream), "compact_flags");
    CK (ncg_launch_nearpd (M, nflagged, sd->dids, (int) sd->d, sd->cfg.nearPD_maxiter, sd->dflag, sd->dst,
                           sd->stream), "nearpd");
  }

  return NCG_OK;
}

/* ------------------------------------------------ split cross-validation */

/* The objective of _ncm_stats_dist_m2lnp (ncm_stats_dist.c:484-511):
 * over_smooth = exp(lnos), the eval operand rebuilt for the new bandwidth, and
 * the sum in observation order of the FP64 -2 ln p of the held-out
 * observations n_kernels .. n_obs - 1. */
static ncg_status_t
_split_obj (ncg_sd_t *sd, double lnos, double *hbuf, double *f)
{
  const uint64_t nh = sd->n - sd->nk;
  const int d       = (int) sd->d;
  ncg_eval_args_t a;
  double sum        = 0.0;

  sd->cfg.over_smooth = exp (lnos);
  sd->href            = _get_href (sd);

  if (sd->kind == NCG_VKDE)
    CK (ncg_launch_vkde_finish (sd->dX, sd->dUi, sd->dflag, (int) sd->nk, d, sd->kernel, sd->nu, sd->href,
                                sd->dlnnorm, sd->dpack64, sd->stream), "vkde_finish");
  else
    CK (ncg_launch_kde_finish (sd->dY, sd->dU, (int) sd->n, d, sd->href, sd->dpack64, sd->dVg, sd->stream),
        "kde_finish");

  if (nh > 0)
  {
    ncg_sd_fill_args (sd, nh, &a);
    RESERVE (dscratch, scratch, ncg_eval_scratch_bytes (&a, NCG_PREC_FP64));
    RESERVE (dcv, cv, nh * sizeof (double));
    CK (ncg_launch_eval_m2lnp_fp64 (&a, sd->dX + sd->nk * sd->d, sd->dpack64, sd->dc, sd->dVg, sd->dcv,
                                    sd->dscratch, 0, sd->stream), "eval_fp64");
    CK (cudaMemcpyAsync (hbuf, sd->dcv, nh * sizeof (double), cudaMemcpyDeviceToHost, sd->stream), "D2H");
    CK (cudaStreamSynchronize (sd->stream), "sync");

    for (uint64_t i = 0; i < nh; i++)
      sum += hbuf[i];
  }

  *f = sum;

  return NCG_OK;
}

/* The eval operand for the current href: VKDE W_i / h and lnnorms, KDE the
 * whitened observations / h (every observation, compute_IM reads them all) */
static ncg_status_t
_href_operand (ncg_sd_t *sd)
{
  const int d = (int) sd->d;

  if (sd->kind == NCG_VKDE)
    CK (ncg_launch_vkde_finish (sd->dX, sd->dUi, sd->dflag, (int) sd->nk, d, sd->kernel, sd->nu, sd->href,
                                sd->dlnnorm, sd->dpack64, sd->stream), "vkde_finish");
  else
    CK (ncg_launch_kde_finish (sd->dY, sd->dU, (int) sd->n, d, sd->href, sd->dpack64, sd->dVg, sd->stream),
        "kde_finish");

  return NCG_OK;
}

double
ncg_sd_href_for (ncg_sd_t *sd)
{
  return _get_href (sd);
}

ncg_status_t
ncg_sd_href_operand (ncg_sd_t *sd)
{
  return _href_operand (sd);
}

typedef ncg_status_t (*_obj_fn) (ncg_sd_t *sd, double lnos, void *ctx, double *f);

static ncg_status_t
_split_obj_cb (ncg_sd_t *sd, double lnos, void *ctx, double *f)
{
  return _split_obj (sd, lnos, (double *) ctx, f);
}

/* The bandwidth fits of _ncm_stats_dist_prepare (ncm_stats_dist.c:764-781)
 * run _ncm_stats_dist_minimize_obj (:660-701): one-dimensional Nelder-Mead
 * over ln over_smooth in the form of GSL's nmsimplex2 (the reference's
 * minimiser), from its published description -- a simplex of the start and
 * the start plus 0.1; reflect the worst vertex through the others' centroid,
 * try the doubled step when that is the new best, else contract halfway
 * towards the worst vertex and, failing that, shrink towards the best;
 * size = the vertices' RMS distance from their centroid, stop below 1e-3 or
 * after 1000 iterations.  As in the reference, the bandwidth left set is the
 * one of the last objective evaluation.  Mixed operands are rebuilt on the
 * next mixed eval. */
static ncg_status_t
_nm_fit (ncg_sd_t *sd, _obj_fn obj, void *ctx)
{
  double x[2], f[2];
  ncg_status_t r = NCG_OK;

#define OBJ(xv, fv) do { if ((r = obj (sd, (xv), ctx, &(fv))) != NCG_OK) goto out; } while (0)

  x[0] = log (sd->cfg.over_smooth);
  x[1] = x[0] + 0.1;
  OBJ (x[0], f[0]);
  OBJ (x[1], f[1]);

  for (int iter = 1; iter <= 1000; iter++)
  {
    const int hi    = (f[1] > f[0]) ? 1 : 0;
    const int lo    = 1 - hi;
    const double c  = x[lo];                 /* centroid of the vertices but the worst */
    const double xr = 2.0 * c - x[hi];
    double fr;

    OBJ (xr, fr);

    if (isfinite (fr) && fr < f[lo])
    {
      const double xe = 3.0 * c - 2.0 * x[hi];
      double fe;

      OBJ (xe, fe);

      if (isfinite (fe) && fe < f[lo])
      {
        x[hi] = xe;
        f[hi] = fe;
      }
      else
      {
        x[hi] = xr;
        f[hi] = fr;
      }
    }
    else if (!isfinite (fr) || fr > f[lo])
    {
      if (isfinite (fr) && fr <= f[hi])
      {
        x[hi] = xr;
        f[hi] = fr;
      }

      {
        const double xc = 0.5 * c + 0.5 * x[hi];
        double fc;

        OBJ (xc, fc);

        if (isfinite (fc) && fc <= f[hi])
        {
          x[hi] = xc;
          f[hi] = fc;
        }
        else
        {
          x[hi] = 0.5 * (x[hi] + x[lo]);
          OBJ (x[hi], f[hi]);
        }
      }
    }
    else
    {
      x[hi] = xr;
      f[hi] = fr;
    }

    if (0.5 * fabs (x[0] - x[1]) < 1.0e-3)
      break;
  }

#undef OBJ

out:
  sd->packmx_ready = 0;
  sd->tcB_ready    = 0;

  return r;
}

/* CV_SPLIT_NOFIT (ncm_stats_dist.c:768-770): Nelder-Mead on the held-out
 * -2 ln p of _ncm_stats_dist_m2lnp */
static ncg_status_t
_split_nofit_fit (ncg_sd_t *sd)
{
  double *hbuf = malloc (sizeof (double) * (size_t) (sd->n - sd->nk + 1));
  ncg_status_t r;

  if (hbuf == NULL)
    return NCG_ERR_OUT_OF_MEMORY;

  r = _nm_fit (sd, _split_obj_cb, hbuf);
  free (hbuf);

  return r;
}

/* ---------------------------------------------- leave-one-out (AMISE) fit */

typedef struct
{
  double *rowx, *diag;        /* n row sums without the diagonal, the diagonal */
  double *m2, *x, *p, *z1, *z2, *c1, *c2, *u;
  int32_t *idx, *kidx, *dkidx;
  double *dz, *dc, *dx;
  int32_t *sorted;
  uint64_t win;
} _loo_ctx;

/* _ncm_stats_dist_amise_kde_gauss (ncm_stats_dist.c:513-557): the sum of the
 * unit-f interpolation matrix over n^2 at href = sqrt(2) h, minus twice its
 * off-diagonal sum over n (n - 1) at h */
static ncg_status_t
_amise_kde_gauss (ncg_sd_t *sd, double lnos, void *vctx, double *f)
{
  _loo_ctx *cx   = vctx;
  const int n    = (int) sd->nk;
  const double n2 = (double) n * (double) n;
  const double nn1 = (double) ((unsigned) n * (unsigned) (n - 1));
  double amise   = 0.0;
  ncg_status_t r;

  sd->cfg.over_smooth = exp (lnos);
  sd->href            = sqrt (2.0) * _get_href (sd);

  if ((r = _href_operand (sd)) != NCG_OK || (r = ncg_sd_im_rowsums (sd, cx->rowx, cx->diag)) != NCG_OK)
    return r;

  for (int i = 0; i < n; i++)
    amise += (cx->rowx[i] + cx->diag[i]) / n2;

  sd->cfg.over_smooth = exp (lnos);
  sd->href            = _get_href (sd);

  if ((r = _href_operand (sd)) != NCG_OK || (r = ncg_sd_im_rowsums (sd, cx->rowx, cx->diag)) != NCG_OK)
    return r;

  for (int i = 0; i < n; i++)
    amise -= 2.0 * cx->rowx[i] / nn1;

  *f = amise;

  return NCG_OK;
}

typedef struct { double v; int32_t idx; } _loo_sv;

static int
_loo_sv_cmp (const void *a, const void *b)
{
  const _loo_sv *pa = a, *pb = b;

  if (pa->v < pb->v) return -1;
  if (pa->v > pb->v) return 1;
  return (pa->idx < pb->idx) ? -1 : (pa->idx > pb->idx);
}

/* _ncm_stats_dist_amise (ncm_stats_dist.c:561-658): minus twice the
 * off-diagonal interpolation-matrix sum over n (n - 1), plus the mean density
 * at antithetic pairs (ncm_stats_dist_sample2: kernel i of the order sorted by
 * (row sum)/n and kernel n - 1 - i) from a generator reseeded at every call,
 * run to a relative standard error below 1e-2 after 100 pairs.  The pairs are
 * drawn, sampled and evaluated a window at a time (the generator is local, so
 * draws past the stopping pair are discarded); the running mean and
 * covariance follow ncm_stats_vec_update (ncm_stats_vec.c:511-565) pair by pair. */
static ncg_status_t
_amise_mc (ncg_sd_t *sd, double lnos, void *vctx, double *f)
{
  _loo_ctx *cx    = vctx;
  const int n     = (int) sd->nk, d = (int) sd->d, st = (sd->kernel == NCG_KERNEL_ST);
  const double nn1 = (double) ((unsigned) n * (unsigned) (n - 1));
  const uint64_t W = cx->win;
  double amise    = 0.0, mean = 0.0;
  double w = 0.0, w2 = 0.0, bias = 0.0, m0 = 0.0, m1 = 0.0, v0 = 0.0, v1 = 0.0, c01 = 0.0;
  ncg_rng_t *rng  = NULL;
  _loo_sv *srt;
  ncg_status_t r;
  int64_t it = 0;
  int done = 0;

  sd->cfg.over_smooth = exp (lnos);
  sd->href            = _get_href (sd);

  if ((r = _href_operand (sd)) != NCG_OK || (r = ncg_sd_im_rowsums (sd, cx->rowx, cx->diag)) != NCG_OK)
    return r;

  if ((srt = malloc (sizeof (_loo_sv) * n)) == NULL)
    return NCG_ERR_OUT_OF_MEMORY;

  for (int i = 0; i < n; i++)
  {
    amise     -= 2.0 * cx->rowx[i] / nn1;
    srt[i].v   = (cx->rowx[i] + cx->diag[i]) / n;
    srt[i].idx = i;
  }

  /* gsl_sort_index: ascending (ties, absent for distinct sums, by index) */
  qsort (srt, n, sizeof (_loo_sv), _loo_sv_cmp);

  for (int i = 0; i < n; i++)
    cx->sorted[i] = srt[i].idx;

  free (srt);

  /* ncm_rng_seeded_new (NULL, 0): MT19937 seeded as GSL seeds it for 0 */
  if ((r = ncg_rng_new (4357u, &rng)) != NCG_OK)
    return r;

  while (!done)
  {
    r = ncg_rng_sample2_stream (rng, (ncg_kernel_t) sd->kernel, (uint32_t) d, sd->nu, W, cx->u, cx->z1,
                                st ? cx->c1 : NULL, cx->z2, st ? cx->c2 : NULL);

    if (r == NCG_OK)
      r = ncg_sd_kernel_choose_batch (sd, cx->u, W, cx->idx);

    if (r != NCG_OK)
      break;

    /* points 2j (first of pair j) and 2j + 1 (second) */
    for (uint64_t j = 0; j < W; j++)
    {
      const int i = cx->idx[j];

      cx->kidx[2 * j]     = cx->sorted[i];
      cx->kidx[2 * j + 1] = cx->sorted[n - 1 - i];
      memcpy (cx->x + (2 * j) * d, cx->z1 + j * d, sizeof (double) * d);
      memcpy (cx->x + (2 * j + 1) * d, cx->z2 + j * d, sizeof (double) * d);

      if (st)
      {
        cx->p[2 * j]     = cx->c1[j];
        cx->p[2 * j + 1] = cx->c2[j];
      }
    }

    {
      ncg_eval_args_t a;

      ncg_sd_fill_args (sd, 2 * W, &a);
      r = ncg_cuda_status (cudaMemcpyAsync (cx->dkidx, cx->kidx, sizeof (int32_t) * 2 * W, cudaMemcpyHostToDevice,
                                            sd->stream), "H2D kernels");
      if (r == NCG_OK)
        r = ncg_cuda_status (cudaMemcpyAsync (cx->dz, cx->x, sizeof (double) * 2 * W * d, cudaMemcpyHostToDevice,
                                              sd->stream), "H2D z");
      if (r == NCG_OK && st)
        r = ncg_cuda_status (cudaMemcpyAsync (cx->dc, cx->p, sizeof (double) * 2 * W, cudaMemcpyHostToDevice,
                                              sd->stream), "H2D chisq");
      if (r == NCG_OK)
        r = ncg_cuda_status (ncg_launch_sample_at (sd->kind, sd->kernel, d, sd->nu, sd->href, sd->dX, sd->dUi, sd->dU,
                                                   cx->dkidx, cx->dz, st ? cx->dc : NULL, (int64_t) (2 * W), cx->dx,
                                                   sd->stream), "sample_at");
      if (r == NCG_OK)
        r = ncg_sd_reserve (sd, (void **) &sd->dscratch, &sd->cap.scratch, ncg_eval_scratch_bytes (&a, NCG_PREC_FP64));
      if (r == NCG_OK)
        r = ncg_cuda_status (ncg_launch_eval_m2lnp_fp64 (&a, cx->dx, sd->dpack64, sd->dc, sd->dVg, cx->dz,
                                                         sd->dscratch, 1, sd->stream), "eval");
      if (r == NCG_OK)
        r = ncg_cuda_status (cudaMemcpyAsync (cx->p, cx->dz, sizeof (double) * 2 * W, cudaMemcpyDeviceToHost,
                                              sd->stream), "D2H p");
      if (r == NCG_OK)
        r = ncg_cuda_status (cudaStreamSynchronize (sd->stream), "sync");
    }

    if (r != NCG_OK)
      break;

    for (uint64_t j = 0; j < W && !done; j++, it++)
    {
      const double x0 = cx->p[2 * j], x1 = cx->p[2 * j + 1];
      const double cw = w + 1.0;

      {
        const double delta = x0 - m0;
        const double R     = delta * 1.0 / cw;
        const double dvar  = w * delta * R;

        m0 += R;
        v0 += dvar;
        c01 += 1.0 * (x0 - m0) * (x1 - m1);
      }
      {
        const double delta = x1 - m1;
        const double R     = delta * 1.0 / cw;
        const double dvar  = w * delta * R;

        m1 += R;
        v1 += dvar;
      }

      w     = cw;
      w2   += 1.0;
      bias  = 1.0 / (w - w2 / w);

      if (it >= 100)
      {
        const double var = 0.25 * (v0 * bias + v1 * bias + 2.0 * (c01 * bias));
        const double msd = sqrt (var / ((it - 100) + 101.0)) / (mean = 0.5 * (m0 + m1));

        if (msd < 1.0e-2)
          done = 1;
      }
    }

    if (!done && it >= 100 + 100000000LL)
      done = 1;
  }

  ncg_rng_free (rng);

  if (r != NCG_OK)
    return r;

  *f = amise + mean;

  return NCG_OK;
}

/* CV_LOO (ncm_stats_dist.c:760-765): Nelder-Mead on the AMISE, in closed
 * form for a Gaussian KDE, by Monte Carlo otherwise */
static ncg_status_t
_loo_fit (ncg_sd_t *sd)
{
  const int n = (int) sd->nk, d = (int) sd->d;
  const uint64_t W = 1024;
  _loo_ctx cx;
  ncg_status_t r = NCG_ERR_OUT_OF_MEMORY;

  memset (&cx, 0, sizeof (cx));
  cx.win    = W;
  cx.rowx   = malloc (sizeof (double) * n);
  cx.diag   = malloc (sizeof (double) * n);
  cx.sorted = malloc (sizeof (int32_t) * n);
  cx.u      = malloc (sizeof (double) * W);
  cx.z1     = malloc (sizeof (double) * W * d);
  cx.z2     = malloc (sizeof (double) * W * d);
  cx.c1     = malloc (sizeof (double) * W);
  cx.c2     = malloc (sizeof (double) * W);
  cx.x      = malloc (sizeof (double) * 2 * W * d);
  cx.p      = malloc (sizeof (double) * 2 * W);
  cx.idx    = malloc (sizeof (int32_t) * W);
  cx.kidx   = malloc (sizeof (int32_t) * 2 * W);

  if (cx.rowx && cx.diag && cx.sorted && cx.u && cx.z1 && cx.z2 && cx.c1 && cx.c2 && cx.x && cx.p && cx.idx && cx.kidx)
  {
    const int closed = (sd->kind == NCG_KDE && sd->kernel == NCG_KERNEL_GAUSS);

    r = NCG_OK;

    if (!closed)
    {
      /* device buffers of the Monte Carlo windows: kernels, draws (the draws'
       * buffer then takes the densities), chi^2, points */
      char *b = NULL;
      const size_t need = 256 + sizeof (int32_t) * 2 * W + sizeof (double) * (2 * W * d + 2 * W + 2 * W * d) + 3 * 256;

      r = ncg_sd_reserve (sd, (void **) &sd->dloo, &sd->cap.loo, need);

      if (r == NCG_OK)
      {
        b        = (char *) sd->dloo;
        cx.dkidx = (int32_t *) b;
        b       += (sizeof (int32_t) * 2 * W + 255) / 256 * 256;
        cx.dz    = (double *) b;
        b       += (sizeof (double) * 2 * W * d + 255) / 256 * 256;
        cx.dc    = (double *) b;
        b       += (sizeof (double) * 2 * W + 255) / 256 * 256;
        cx.dx    = (double *) b;
      }
    }

    if (r == NCG_OK)
      r = _nm_fit (sd, closed ? _amise_kde_gauss : _amise_mc, &cx);
  }

  free (cx.rowx);
  free (cx.diag);
  free (cx.sorted);
  free (cx.u);
  free (cx.z1);
  free (cx.z2);
  free (cx.c1);
  free (cx.c2);
  free (cx.x);
  free (cx.p);
  free (cx.idx);
  free (cx.kidx);

  return r;
}

ncg_status_t
ncg_sd_prepare (ncg_sd_t *sd)
{
  ncg_prep_status_t st;
  const int d = (int) (sd ? sd->d : 0);
  uint32_t k  = 0;

  if (sd == NULL)
    return NCG_ERR_INVALID_ARG;

  sd->prepared = 0;

  const int robust = sd->cfg.cov_type == NCG_COV_ROBUST_DIAG || sd->cfg.cov_type == NCG_COV_ROBUST;

  if (sd->n <= (uint64_t) d)
  {
    ncg_set_error ("_ncm_stats_dist_prepare: the sample is too small (n = %llu, dim = %d)", (unsigned long long) sd->n, d);

    return NCG_ERR_SAMPLE_TOO_SMALL;
  }

  /* n_kernels, ncm_stats_dist.c:714-740: the first ceil(n split_frac)
   * observations are the kernels under a split cross-validation */
  uint64_t nk = sd->n;

  if (sd->cfg.cv_type == NCG_CV_SPLIT_NOFIT || sd->cfg.cv_type == NCG_CV_SPLIT)
  {
    if (!(sd->split_frac >= 0.01 && sd->split_frac <= 1.0))
    {
      ncg_set_error ("a split CV needs a split fraction in [0.01, 1] (ncg_sd_set_split_frac)");

      return NCG_ERR_INVALID_ARG;
    }

    nk = (uint64_t) ceil ((double) sd->n * sd->split_frac);

    if (nk <= (uint64_t) d)
    {
      ncg_set_error ("split CV: %llu kernels for dimension %d", (unsigned long long) nk, d);

      return NCG_ERR_SAMPLE_TOO_SMALL;
    }
  }

  if (sd->n > 0x7fffffffULL)
    return NCG_ERR_UNSUPPORTED;

  if (sd->kind == NCG_VKDE)
  {
    const double lf = sd->cfg.local_frac * (double) sd->n;

    if (lf < 2)
    {
      ncg_set_error ("Too few observations: local_frac * n = %g < 2", lf);

      return NCG_ERR_TOO_FEW_LOCAL;
    }

    k = (uint32_t) (size_t) ((lf > 2) ? lf : 2);

    if (k > NCG_KNN_KMAX || k > sd->n)
    {
      ncg_set_error ("kNN size %u above the device limit %d", k, NCG_KNN_KMAX);

      return NCG_ERR_UNSUPPORTED;
    }
  }

  if (robust && (sd->n < 4 || (sd->kind == NCG_VKDE && k < 4)))
  {
    /* ncm_stats_vec.c:1841-1843, 1911-1913 */
    ncg_set_error ("robust covariance: too few points to estimate the covariance [%u].",
                   (sd->kind == NCG_VKDE) ? k : (uint32_t) sd->n);

    return NCG_ERR_SAMPLE_TOO_SMALL;
  }

  if (robust && sd->n > NCG_ROBUST_MAX_ROWS)
  {
    ncg_set_error ("robust covariance of %llu samples: at most %d on the device", (unsigned long long) sd->n,
                   NCG_ROBUST_MAX_ROWS);

    return NCG_ERR_UNSUPPORTED;
  }

  if (sd->cfg.cov_type == NCG_COV_FIXED && sd->cov_fixed == NULL)
  {
    ncg_set_error ("cov_type is FIXED but no fixed covariance was set");

    return NCG_ERR_INVALID_ARG;
  }

  CK (cudaSetDevice (sd->cfg.device), "cudaSetDevice");

  {
    ncg_status_t r = _reserve_prepare (sd, k);

    if (r != NCG_OK)
      return r;
  }

  const int n        = (int) sd->n;
  const int nkk      = (int) nk;
  cudaStream_t s     = sd->stream;

  sd->nk             = nk;
  sd->k              = k;
  sd->href           = _get_href (sd);
  sd->n_fallback     = 0;
  sd->wcum_ready     = 0;
  sd->packmx_ready   = 0;
  sd->interp_branch  = 0;
  sd->rnorm          = 0.0;

  CK (cudaMemcpyAsync (sd->dX, sd->hX, sizeof (double) * (size_t) n * d, cudaMemcpyHostToDevice, s), "H2D sample");
  CK (cudaMemsetAsync (sd->dst, 0, sizeof (ncg_prep_status_t), s), "memset");

  if (sd->cfg.cov_type == NCG_COV_FIXED)
  {
    CK (cudaMemcpyAsync (sd->dcov, sd->cov_fixed, sizeof (double) * d * d, cudaMemcpyHostToDevice, s), "H2D cov");
    CK (ncg_launch_global_cov_chol (sd->dX, 0, d, sd->dcov, sd->dU, sd->dflag, sd->dst, s), "global_chol");
  }
  else if (robust)
  {
    /* ncm_stats_dist_kde.c:423-440 */
    CK (ncg_launch_robust_cov (sd->dX, n, d, NULL, nkk, 1, sd->cfg.cov_type == NCG_COV_ROBUST, sd->drq, sd->dcov,
                               &sd->dst->n_badindex, s),
        "robust global cov");
    CK (ncg_launch_global_cov_chol (sd->dX, 0, d, sd->dcov, sd->dU, sd->dflag, sd->dst, s), "global_chol");
  }
  else
  {
    CK (ncg_launch_global_cov_chol (sd->dX, nkk, d, sd->dcov, sd->dU, sd->dflag, sd->dst, s), "global_cov_chol");
  }

  CK (cudaMemcpyAsync (&st, sd->dst, sizeof (st), cudaMemcpyDeviceToHost, s), "D2H status");
  CK (cudaStreamSynchronize (s), "sync");

  if (st.n_flagged)
  {
    if (sd->cfg.cov_type == NCG_COV_FIXED)
    {
      ncg_set_error ("ncm_stats_dist_kde_set_cov_fixed: matrix cov_fixed is not positive definite.");

      return NCG_ERR_NOT_PD;
    }

    ncg_status_t r = _nearpd_pass (sd, sd->dU, 1, 1);

    if (r != NCG_OK)
      return r;

    CK (cudaMemsetAsync (&sd->dst->n_flagged, 0, sizeof (int32_t), s), "memset");
  }

  CK (ncg_launch_global_lnnorm (sd->dU, d, sd->kernel, sd->nu, sd->dst, s), "global_lnnorm");
  CK (ncg_launch_whiten (sd->dX, sd->dU, n, d, sd->dY, s), "whiten");
  CK (ncg_launch_mean (sd->dX, nkk, d, sd->dmu, s), "mean");

  if (sd->kind == NCG_VKDE)
  {
    CK (ncg_launch_knn (sd->dY, n, nkk, d, (int) k, sd->dknn, (uint64_t *) sd->dkeys, s), "knn");
    if (robust)
    {
      /* ncm_stats_dist_vkde.c:467-472: the robust estimate over each kernel's neighbours */
      CK (ncg_launch_robust_cov (sd->dX, n, d, sd->dknn, (int) k, nkk, sd->cfg.cov_type == NCG_COV_ROBUST,
                                 sd->drq, sd->dUi, &sd->dst->n_badindex, s), "robust local cov");
      CK (ncg_launch_chol_slots (sd->dUi, nkk, d, sd->dflag, sd->dst, s), "chol slots");
    }
    else
    {
      CK (ncg_launch_local_cov_chol (sd->dX, sd->dknn, n, nkk, d, (int) k, sd->dUi, sd->dflag, sd->dst, s),
          "local_cov_chol");
    }
    CK (cudaMemcpyAsync (&st, sd->dst, sizeof (st), cudaMemcpyDeviceToHost, s), "D2H status");
    CK (cudaStreamSynchronize (s), "sync");

    if (st.n_flagged)
    {
      ncg_status_t r = _nearpd_pass (sd, sd->dUi, nkk, st.n_flagged);

      if (r != NCG_OK)
        return r;
    }

    CK (ncg_launch_vkde_finish (sd->dX, sd->dUi, sd->dflag, nkk, d, sd->kernel, sd->nu, sd->href, sd->dlnnorm,
                                sd->dpack64, s), "vkde_finish");
    /* global whitening of the points for the mixed form (unscaled U^{-T}) */
    CK (ncg_launch_global_vg (sd->dU, d, 1.0, sd->dVg, s), "global_vg");
  }
  else
  {
    /* the operand of every observation (the first n_kernels are the kernels;
     * compute_IM reads the held-out rows too) */
    CK (ncg_launch_kde_finish (sd->dY, sd->dU, n, d, sd->href, sd->dpack64, sd->dVg, s), "kde_finish");
  }

  CK (ncg_launch_fill (sd->dw, 1.0 / (1.0 * nkk), nkk, s), "fill weights");
  CK (ncg_launch_weights_c (sd->dw, sd->dlnnorm, nkk, sd->kind, sd->dc, NULL, s), "weights_c");
  CK (cudaMemcpyAsync (&st, sd->dst, sizeof (st), cudaMemcpyDeviceToHost, s), "D2H status");
  CK (cudaStreamSynchronize (s), "sync");

  sd->kernel_lnnorm = st.kernel_lnnorm;
  sd->n_fallback    = (uint64_t) st.n_fallback;

  if (st.n_badindex)
  {
    ncg_set_error ("kNN produced %d out-of-range neighbour indices", st.n_badindex);

    return NCG_ERR_CUDA;
  }

  if (st.n_fail)
  {
    ncg_set_error ("%d covariance factor(s) not positive definite after nearPD and diagonal fallback", st.n_fail);

    return NCG_ERR_NOT_PD;
  }

  sd->prepared = 1;
  sd->gen++;

  if (sd->cfg.cv_type == NCG_CV_SPLIT_NOFIT)
    return _split_nofit_fit (sd);

  if (sd->cfg.cv_type == NCG_CV_LOO)
    return _loo_fit (sd);

  return NCG_OK;
}

/* ---------------------------------------------------------------- eval */

void
ncg_sd_fill_args (ncg_sd_t *sd, uint64_t m, ncg_eval_args_t *a)
{
  a->kind        = sd->kind;
  a->kernel      = sd->kernel;
  a->d           = (int32_t) sd->d;
  a->dp          = sd->dp;
  a->n           = (int32_t) sd->nk;
  a->m           = (int64_t) m;
  a->nu          = (sd->kernel == NCG_KERNEL_ST) ? sd->nu : 1.0;
  a->kappa       = -0.5 * (sd->nu + sd->d);
  a->final_shift = (sd->kind == NCG_KDE) ? sd->kernel_lnnorm : 0.0;
  a->d_ln_href   = sd->d * log (sd->href);
  a->inv_href    = 1.0 / sd->href;
  a->c_shift     = 0.0;
}

ncg_status_t
ncg_sd_ensure_packmx (ncg_sd_t *sd)
{
  if (sd->packmx_ready)
    return NCG_OK;

  ncg_eval_args_t a;

  ncg_sd_fill_args (sd, 1, &a);
  RESERVE (dpackmx, packmx, ncg_packmx_bytes (sd->kind, (int) sd->nk, sd->dp));
  CK (ncg_launch_build_packmx (&a, sd->dX, sd->dpack64, sd->dc, sd->dUi, sd->dU, sd->dVg, sd->dmu, sd->dpackmx,
                               sd->stream), "build_packmx");
  CK (cudaMemcpyAsync (&sd->mixed_kappa, ncg_packmx_kappa_max (sd->dpackmx, sd->kind, (int) sd->nk, sd->dp),
                       sizeof (double), cudaMemcpyDeviceToHost, sd->stream), "D2H kappa");
  CK (cudaStreamSynchronize (sd->stream), "sync");
  sd->packmx_ready = 1;
  sd->tcB_ready    = 0;

  return NCG_OK;
}

/* Points used to check the tensor-core operand: up to this many kernel
 * centres.  At a centre y = W'(x' - theta') = 0 is formed from W'x' and b of
 * the size of W'theta', the worst case of the operand's FP32 cancellation. */
#define NCG_TC_CHECK_POINTS 128

/* The tensor-core operand (built once per packed state) and its accuracy
 * check: -2 ln p at up to NCG_TC_CHECK_POINTS kernel centres by the
 * tensor-core kernel against the FP64 kernel; the handle uses the tensor
 * cores only if the largest relative difference (floored at 1) is at most
 * half the mixed form's 1e-6 bound, else the FP32 SIMT form. */
ncg_status_t
ncg_sd_ensure_tc (ncg_sd_t *sd)
{
  ncg_eval_args_t a;
  const uint64_t ncal = (sd->nk < NCG_TC_CHECK_POINTS) ? sd->nk : NCG_TC_CHECK_POINTS;
  double *hx, *hout;
  ncg_status_t r;

  if (sd->tcB_ready)
    return NCG_OK;

  r = ncg_sd_reserve (sd, (void **) &sd->dtcB, &sd->cap_tcB, ncg_tc_B_bytes ((int) sd->nk, sd->dp));

  if (r != NCG_OK)
    return r;

  CK (ncg_launch_build_tc_B (sd->dpackmx, sd->kind, (int) sd->nk, sd->dp, sd->kernel, sd->nu, sd->dtcB, sd->stream),
      "build_tc_B");

  ncg_sd_fill_args (sd, ncal, &a);

  {
    const size_t s64 = ncg_eval_scratch_bytes (&a, NCG_PREC_FP64), stc = ncg_tc_scratch_bytes ((int64_t) ncal, (int) sd->nk, sd->dp);

    RESERVE (dscratch, scratch, s64 > stc ? s64 : stc);
  }

  RESERVE (dcal, cal, sizeof (double) * ncal * (sd->d + 2));

  hx   = malloc (sizeof (double) * ncal * (sd->d + 2));
  hout = hx + ncal * sd->d;

  if (hx == NULL)
    return NCG_ERR_OUT_OF_MEMORY;

  for (uint64_t j = 0; j < ncal; j++)
    memcpy (hx + j * sd->d, sd->hX + (j * sd->nk / ncal) * sd->d, sizeof (double) * sd->d);

  r = ncg_cuda_status (cudaMemcpyAsync (sd->dcal, hx, sizeof (double) * ncal * sd->d, cudaMemcpyHostToDevice,
                                        sd->stream), "H2D check points");

  if (r == NCG_OK)
    r = ncg_cuda_status (ncg_launch_eval_m2lnp_fp64 (&a, sd->dcal, sd->dpack64, sd->dc, sd->dVg,
                                                     sd->dcal + ncal * sd->d, sd->dscratch, 0, sd->stream),
                         "check eval_fp64");

  if (r == NCG_OK)
    r = ncg_cuda_status (ncg_launch_eval_tc (&a, sd->dcal, sd->dtcB, sd->dmu, sd->dVg,
                                             ncg_packmx_cshift (sd->dpackmx, sd->kind, (int) sd->nk, sd->dp),
                                             sd->dscratch, sd->dcal + ncal * (sd->d + 1), sd->d_flag_alias, NULL,
                                             sd->stream), "check eval_tc");

  if (r == NCG_OK)
    r = ncg_cuda_status (cudaMemcpyAsync (hout, sd->dcal + ncal * sd->d, sizeof (double) * 2 * ncal,
                                          cudaMemcpyDeviceToHost, sd->stream), "D2H check");

  if (r == NCG_OK)
    r = ncg_cuda_status (cudaStreamSynchronize (sd->stream), "sync");

  if (r == NCG_OK)
  {
    double e = 0.0;

    for (uint64_t j = 0; j < ncal; j++)
    {
      const double ref = hout[j], got = hout[ncal + j];
      const double rel = fabs (got - ref) / fmax (fabs (ref), 1.0);

      e = (rel > e || isnan (rel)) ? rel : e;
    }

    sd->tc_err    = e;
    sd->tc_ok     = (e <= 0.5e-6) && *sd->h_flag == 0;
    sd->tcB_ready = 1;
  }

  free (hx);

  return r;
}

/* which arithmetic serves this call: FP64, tensor cores or FP32 SIMT */
static int
_eval_path (ncg_sd_t *sd, int linear, ncg_status_t *r)
{
  *r = NCG_OK;

  if (linear || sd->cfg.precision == NCG_PREC_FP64)
    return NCG_PATH_FP64;

  if ((*r = ncg_sd_ensure_packmx (sd)) != NCG_OK)
    return NCG_PATH_FP64;

  if (!(sd->mixed_kappa <= NCG_MIXED_KAPPA_MAX))
    return NCG_PATH_FP64;

  if (sd->cfg.precision == NCG_PREC_MIXED && ncg_tc_supported (sd->kind, sd->dp))
  {
    if ((*r = ncg_sd_ensure_tc (sd)) != NCG_OK)
      return NCG_PATH_FP64;

    if (sd->tc_ok)
      return NCG_PATH_TC;
  }

  return NCG_PATH_SIMT;
}

static ncg_status_t
_eval_device (ncg_sd_t *sd, const double *dXq, uint64_t m, double *dout, int linear)
{
  ncg_eval_args_t a;
  ncg_status_t r;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  if (m == 0)
    return NCG_OK;

  const int path = _eval_path (sd, linear, &r);

  if (r != NCG_OK)
    return r;

  sd->last_path = path;
  ncg_sd_fill_args (sd, m, &a);

  if (path == NCG_PATH_FP64)
  {
    RESERVE (dscratch, scratch, ncg_eval_scratch_bytes (&a, NCG_PREC_FP64));
    CK (ncg_launch_eval_m2lnp_fp64 (&a, dXq, sd->dpack64, sd->dc, sd->dVg, dout, sd->dscratch, linear, sd->stream),
        "eval_fp64");
  }
  else
  {
    if (path == NCG_PATH_TC)
    {
      RESERVE (dscratch, scratch, ncg_tc_scratch_bytes ((int64_t) m, (int) sd->nk, sd->dp));
      CK (ncg_launch_eval_tc (&a, dXq, sd->dtcB, sd->dmu, sd->dVg,
                              ncg_packmx_cshift (sd->dpackmx, sd->kind, (int) sd->nk, sd->dp), sd->dscratch, dout,
                              sd->d_flag_alias, sd->ktime_on ? sd->kev : NULL, sd->stream), "eval_tc");
      sd->ktime_valid = sd->ktime_on;
    }
    else
    {
      RESERVE (dscratch, scratch, ncg_eval_scratch_bytes (&a, NCG_PREC_MIXED_SIMT));
      CK (ncg_launch_eval_m2lnp_mixed (&a, dXq, sd->dpackmx, sd->dmu, sd->dVg, dout, sd->dscratch, sd->stream),
          "eval_mixed");
    }
  }

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_eval_path (ncg_sd_t *sd, int32_t *path, double *kappa_max)
{
  ncg_status_t r;

  if (sd == NULL || path == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  *path = _eval_path (sd, 0, &r);

  if (kappa_max)
    *kappa_max = (sd->cfg.precision == NCG_PREC_FP64) ? 0.0 : sd->mixed_kappa;

  return r;
}

ncg_status_t
ncg_sd_get_tc_check (ncg_sd_t *sd, double *err)
{
  if (sd == NULL || err == NULL)
    return NCG_ERR_INVALID_ARG;

  *err = sd->tcB_ready ? sd->tc_err : -1.0;

  return NCG_OK;
}

ncg_status_t
ncg_sd_set_kernel_timing (ncg_sd_t *sd, int32_t on)
{
  if (sd == NULL)
    return NCG_ERR_INVALID_ARG;

  if (on && !sd->kev[0])
  {
    CK (cudaEventCreate (&sd->kev[0]), "cudaEventCreate");
    CK (cudaEventCreate (&sd->kev[1]), "cudaEventCreate");
  }

  sd->ktime_on    = on ? 1 : 0;
  sd->ktime_valid = 0;

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_kernel_time (ncg_sd_t *sd, double *ms)
{
  float f = 0.0f;

  if (sd == NULL || ms == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->ktime_valid)
    return NCG_ERR_NOT_PREPARED;

  CK (cudaEventSynchronize (sd->kev[1]), "cudaEventSynchronize");
  CK (cudaEventElapsedTime (&f, sd->kev[0], sd->kev[1]), "cudaEventElapsedTime");
  *ms = f;

  return NCG_OK;
}

ncg_status_t
ncg_sd_eval_m2lnp_device (ncg_sd_t *sd, const double *d_X, uint64_t m, double *d_m2lnp)
{
  if (sd == NULL || (m > 0 && (d_X == NULL || d_m2lnp == NULL)))
    return NCG_ERR_INVALID_ARG;

  return _eval_device (sd, d_X, m, d_m2lnp, 0);
}

/* The FP64 eval with its per-call scratch in a static device array (see
 * ncg_eval.cu), for callers that must not allocate while they evaluate.  Only
 * checks, a device switch and two kernel launches: no allocation. */
ncg_status_t
ncg_sd_eval_m2lnp_device_noalloc (ncg_sd_t *sd, const double *d_X, uint64_t m, double *d_m2lnp)
{
  ncg_eval_args_t a;

  if (sd == NULL || (m > 0 && (d_X == NULL || d_m2lnp == NULL)))
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  if (m == 0)
    return NCG_OK;

  if (m > (uint64_t) ncg_noalloc_max_points ())
  {
    ncg_set_error ("ncg_sd_eval_m2lnp_device_noalloc: %llu points exceed its static scratch of %zu bytes "
                   "(at most %lld points per call)", (unsigned long long) m, ncg_noalloc_scratch_bytes (),
                   (long long) ncg_noalloc_max_points ());

    return NCG_ERR_INVALID_ARG;
  }

  CK (cudaSetDevice (sd->cfg.device), "cudaSetDevice");
  ncg_sd_fill_args (sd, m, &a);
  CK (ncg_launch_eval_m2lnp_fp64_noalloc (&a, d_X, sd->dpack64, sd->dc, sd->dVg, d_m2lnp, sd->stream), "eval_noalloc");

  return NCG_OK;
}

static ncg_status_t
_eval_host (ncg_sd_t *sd, const double *X, uint64_t m, double *out, int linear)
{
  if (sd == NULL || (m > 0 && (X == NULL || out == NULL)))
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  if (m == 0)
    return NCG_OK;

  RESERVE (dq, q, m * sd->d * sizeof (double));
  RESERVE (dqo, qo, m * sizeof (double));
  CK (cudaMemcpyAsync (sd->dq, X, m * sd->d * sizeof (double), cudaMemcpyHostToDevice, sd->stream), "H2D points");

  /* NaN / Inf among the points: checked on the device beside the eval (a
   * word of mapped host memory, read after the call's synchronisation) */
  ((volatile int32_t *) sd->h_flag)[1] = 0;
  CK (ncg_launch_nonfinite (sd->dq, (int64_t) (m * sd->d), sd->d_flag_alias + 1, sd->stream), "nonfinite");

  {
    ncg_status_t r = _eval_device (sd, sd->dq, m, sd->dqo, linear);

    if (r != NCG_OK)
      return r;
  }

  CK (cudaMemcpyAsync (out, sd->dqo, m * sizeof (double), cudaMemcpyDeviceToHost, sd->stream), "D2H results");
  CK (cudaStreamSynchronize (sd->stream), "sync");

  if (((volatile int32_t *) sd->h_flag)[1])
  {
    ncg_set_error ("eval: non-finite coordinate among the %llu points", (unsigned long long) m);

    return NCG_ERR_NONFINITE;
  }

  return _check_device_flag (sd);
}

ncg_status_t
ncg_sd_eval_m2lnp_batch (ncg_sd_t *sd, const double *X, uint64_t m, double *m2lnp)
{
  return _eval_host (sd, X, m, m2lnp, 0);
}

ncg_status_t
ncg_sd_eval_m2lnp (ncg_sd_t *sd, const double *x, double *m2lnp)
{
  return _eval_host (sd, x, 1, m2lnp, 0);
}

ncg_status_t
ncg_sd_eval_batch (ncg_sd_t *sd, const double *X, uint64_t m, double *p)
{
  return _eval_host (sd, X, m, p, 1);
}

ncg_status_t
ncg_sd_eval (ncg_sd_t *sd, const double *x, double *p)
{
  return _eval_host (sd, x, 1, p, 1);
}

/* -------------------------------------------------------------- sample */

static ncg_status_t
_ensure_wcum (ncg_sd_t *sd)
{
  if (!sd->wcum_ready)
  {
    CK (ncg_launch_wcum (sd->dw, (int) sd->nk, sd->dwcum, sd->stream), "wcum");
    sd->wcum_ready = 1;
  }

  return NCG_OK;
}

ncg_status_t
ncg_sd_kernel_choose_batch (ncg_sd_t *sd, const double *u, uint64_t n, int32_t *idx)
{
  if (sd == NULL || (n > 0 && (u == NULL || idx == NULL)))
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  if (n == 0)
    return NCG_OK;

  {
    ncg_status_t r = _ensure_wcum (sd);

    if (r != NCG_OK)
      return r;
  }

  RESERVE (dq, q, n * sizeof (double));
  RESERVE (dqi, qi, n * sizeof (int32_t));
  CK (cudaMemcpyAsync (sd->dq, u, n * sizeof (double), cudaMemcpyHostToDevice, sd->stream), "H2D u");
  CK (ncg_launch_kernel_choose (sd->dwcum, (int) sd->nk, sd->dq, (int64_t) n, sd->dqi, sd->stream), "choose");
  CK (cudaMemcpyAsync (idx, sd->dqi, n * sizeof (int32_t), cudaMemcpyDeviceToHost, sd->stream), "D2H idx");
  CK (cudaStreamSynchronize (sd->stream), "sync");

  return NCG_OK;
}

ncg_status_t
ncg_sd_sample_batch (ncg_sd_t *sd, const double *u, const double *z, const double *chisq, uint64_t n, double *x,
                     int32_t *idx)
{
  const size_t d = sd ? sd->d : 0;

  if (sd == NULL || (n > 0 && (u == NULL || z == NULL || x == NULL)))
    return NCG_ERR_INVALID_ARG;

  if (sd->kernel == NCG_KERNEL_ST && n > 0 && chisq == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  if (n == 0)
    return NCG_OK;

  {
    ncg_status_t r = _ensure_wcum (sd);

    if (r != NCG_OK)
      return r;
  }

  /* staging layout in dq: u[n] | z[n*d] | chisq[n] | x[n*d] */
  RESERVE (dq, q, n * (2 * d + 2) * sizeof (double));
  RESERVE (dqi, qi, n * sizeof (int32_t));

  double *du = sd->dq, *dz = du + n, *dch = dz + n * d, *dx = dch + n;

  CK (cudaMemcpyAsync (du, u, n * sizeof (double), cudaMemcpyHostToDevice, sd->stream), "H2D u");
  CK (cudaMemcpyAsync (dz, z, n * d * sizeof (double), cudaMemcpyHostToDevice, sd->stream), "H2D z");

  if (sd->kernel == NCG_KERNEL_ST)
    CK (cudaMemcpyAsync (dch, chisq, n * sizeof (double), cudaMemcpyHostToDevice, sd->stream), "H2D chisq");

  CK (ncg_launch_sample (sd->kind, sd->kernel, (int) d, sd->nu, sd->href, sd->dwcum, (int) sd->nk, sd->dX, sd->dUi,
                         sd->dU, du, dz, dch, (int64_t) n, dx, sd->dqi, sd->stream), "sample");
  CK (cudaMemcpyAsync (x, dx, n * d * sizeof (double), cudaMemcpyDeviceToHost, sd->stream), "D2H x");

  if (idx)
    CK (cudaMemcpyAsync (idx, sd->dqi, n * sizeof (int32_t), cudaMemcpyDeviceToHost, sd->stream), "D2H idx");

  CK (cudaStreamSynchronize (sd->stream), "sync");

  return NCG_OK;
}

ncg_status_t
ncg_sd_sample_batch_device (ncg_sd_t *sd, const double *d_u, const double *d_z, const double *d_chisq, uint64_t n,
                            double *d_x, int32_t *d_idx)
{
  if (sd == NULL || (n > 0 && (d_u == NULL || d_z == NULL || d_x == NULL)))
    return NCG_ERR_INVALID_ARG;

  if (sd->kernel == NCG_KERNEL_ST && n > 0 && d_chisq == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  if (n == 0)
    return NCG_OK;

  {
    ncg_status_t r = _ensure_wcum (sd);

    if (r != NCG_OK)
      return r;
  }

  if (d_idx == NULL)
  {
    RESERVE (dqi, qi, n * sizeof (int32_t));
    d_idx = sd->dqi;
  }

  CK (ncg_launch_sample (sd->kind, sd->kernel, (int) sd->d, sd->nu, sd->href, sd->dwcum, (int) sd->nk, sd->dX,
                         sd->dUi, sd->dU, d_u, d_z, d_chisq, (int64_t) n, d_x, d_idx, sd->stream), "sample");

  return NCG_OK;
}

/* ------------------------------------------------------------- getters */

ncg_status_t
ncg_sd_get_dim (ncg_sd_t *sd, uint32_t *dim)
{
  if (sd == NULL || dim == NULL)
    return NCG_ERR_INVALID_ARG;

  *dim = sd->d;

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_sample_size (ncg_sd_t *sd, uint64_t *n)
{
  if (sd == NULL || n == NULL)
    return NCG_ERR_INVALID_ARG;

  *n = sd->n;

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_n_kernels (ncg_sd_t *sd, uint64_t *n)
{
  if (sd == NULL || n == NULL)
    return NCG_ERR_INVALID_ARG;

  *n = sd->prepared ? sd->nk : sd->n;

  return NCG_OK;
}

/* "split-frac": ncm_stats_dist_set_split_frac (ncm_stats_dist.c:1303-1311,
 * the reference asserts 0.01 <= split_frac <= 1) */
ncg_status_t
ncg_sd_set_split_frac (ncg_sd_t *sd, double split_frac)
{
  if (sd == NULL || !(split_frac >= 0.01 && split_frac <= 1.0))
    return NCG_ERR_INVALID_ARG;

  sd->split_frac = split_frac;
  sd->prepared   = 0;

  return NCG_OK;
}

/* ncm_stats_dist_get_over_smooth (the value a split cross-validation fit left) */
ncg_status_t
ncg_sd_get_over_smooth (ncg_sd_t *sd, double *over_smooth)
{
  if (sd == NULL || over_smooth == NULL)
    return NCG_ERR_INVALID_ARG;

  *over_smooth = sd->cfg.over_smooth;

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_href (ncg_sd_t *sd, double *href)
{
  if (sd == NULL || href == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  *href = sd->href;

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_rnorm (ncg_sd_t *sd, double *rnorm)
{
  if (sd == NULL || rnorm == NULL)
    return NCG_ERR_INVALID_ARG;

  *rnorm = sd->rnorm;

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_interp_branch (ncg_sd_t *sd, int32_t *branch)
{
  if (sd == NULL || branch == NULL)
    return NCG_ERR_INVALID_ARG;

  *branch = sd->interp_branch;

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_chol_fallbacks (ncg_sd_t *sd, uint64_t *count)
{
  if (sd == NULL || count == NULL)
    return NCG_ERR_INVALID_ARG;

  *count = sd->n_fallback;

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_interp_stats (ncg_sd_t *sd, int32_t stats[4])
{
  if (sd == NULL || stats == NULL)
    return NCG_ERR_INVALID_ARG;

  stats[0] = sd->istats.n_solves;
  stats[1] = sd->istats.n_cg_iters;
  stats[2] = sd->istats.n_shifted;
  stats[3] = sd->istats.n_fp64;

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_interp_fallbacks (ncg_sd_t *sd, int32_t *lu, int32_t *qr)
{
  if (sd == NULL || lu == NULL || qr == NULL)
    return NCG_ERR_INVALID_ARG;

  *lu = sd->istats.n_lu;
  *qr = sd->istats.n_qr;

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_knn_k (ncg_sd_t *sd, uint32_t *k)
{
  if (sd == NULL || k == NULL)
    return NCG_ERR_INVALID_ARG;

  *k = sd->k;

  return NCG_OK;
}

static ncg_status_t
_d2h (ncg_sd_t *sd, void *dst, const void *src, size_t bytes)
{
  CK (cudaMemcpyAsync (dst, src, bytes, cudaMemcpyDeviceToHost, sd->stream), "D2H");
  CK (cudaStreamSynchronize (sd->stream), "sync");

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_weights (ncg_sd_t *sd, double *w)
{
  if (sd == NULL || w == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  return _d2h (sd, w, sd->dw, sd->nk * sizeof (double));
}

ncg_status_t
ncg_sd_get_sample (ncg_sd_t *sd, double *X)
{
  if (sd == NULL || X == NULL)
    return NCG_ERR_INVALID_ARG;

  memcpy (X, sd->hX, sd->n * sd->d * sizeof (double));

  return NCG_OK;
}

ncg_status_t
ncg_sd_get_full_cov (ncg_sd_t *sd, double *cov)
{
  if (sd == NULL || cov == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  return _d2h (sd, cov, sd->dcov, sd->d * sd->d * sizeof (double));
}

ncg_status_t
ncg_sd_get_full_cov_decomp (ncg_sd_t *sd, double *U)
{
  if (sd == NULL || U == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  return _d2h (sd, U, sd->dU, sd->d * sd->d * sizeof (double));
}

ncg_status_t
ncg_sd_get_cov_decomp (ncg_sd_t *sd, uint32_t i, double *U)
{
  if (sd == NULL || U == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  if (i >= sd->nk)
    return NCG_ERR_INVALID_ARG;

  if (sd->kind == NCG_KDE)
    return ncg_sd_get_full_cov_decomp (sd, U);

  return _d2h (sd, U, sd->dUi + (size_t) i * sd->d * sd->d, sd->d * sd->d * sizeof (double));
}

ncg_status_t
ncg_sd_get_lnnorm (ncg_sd_t *sd, uint32_t i, double *lnnorm)
{
  if (sd == NULL || lnnorm == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  if (i >= sd->nk)
    return NCG_ERR_INVALID_ARG;

  if (sd->kind == NCG_KDE)
  {
    *lnnorm = sd->kernel_lnnorm + sd->d * log (sd->href);

    return NCG_OK;
  }

  {
    double v;
    ncg_status_t r = _d2h (sd, &v, sd->dlnnorm + i, sizeof (double));

    if (r != NCG_OK)
      return r;

    *lnnorm = v + sd->d * log (sd->href);
  }

  return NCG_OK;
}

/* ncm_stats_dist_get_Ki (numcosmo/ncm/stats/ncm_stats_dist.c:1811-1829): the
 * i-th kernel's location (the sample point), its covariance
 * h^2 U_i^T U_i (ncm_matrix_triang_to_sym on the upper factor, then the
 * href^2 scaling), exp(lnnorm_i) with the d ln h term and its weight.  The
 * product sums k = 0..min(r, c) in ascending order. */
ncg_status_t
ncg_sd_get_Ki (ncg_sd_t *sd, uint32_t i, double *y_i, double *cov_i, double *n_i, double *w_i)
{
  double U[NCG_DMAX * NCG_DMAX], lnnorm, w;
  ncg_status_t r;

  if (sd == NULL || y_i == NULL || cov_i == NULL || n_i == NULL || w_i == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  if (i >= sd->nk)
    return NCG_ERR_INVALID_ARG;

  if ((r = ncg_sd_get_cov_decomp (sd, i, U)) != NCG_OK)
    return r;

  if ((r = ncg_sd_get_lnnorm (sd, i, &lnnorm)) != NCG_OK)
    return r;

  if ((r = _d2h (sd, &w, sd->dw + i, sizeof (double))) != NCG_OK)
    return r;

  {
    const int d     = (int) sd->d;
    const double h2 = sd->href * sd->href;

    for (int a = 0; a < d; a++)
      for (int b = 0; b < d; b++)
      {
        const int kmax = (a < b) ? a : b;
        double acc     = 0.0;

        for (int k = 0; k <= kmax; k++)
          acc += U[k * d + a] * U[k * d + b];

        cov_i[a * d + b] = acc * h2;
      }

    memcpy (y_i, sd->hX + (size_t) i * d, (size_t) d * sizeof (double));
  }

  *n_i = exp (lnnorm);
  *w_i = w;

  return NCG_OK;
}

/* The k nearest neighbours of every kernel centre found by the last VKDE
 * prepare, in the order the local covariance consumes them (squared
 * whitened distance, then index). */
ncg_status_t
ncg_sd_get_knn (ncg_sd_t *sd, int32_t *idx)
{
  if (sd == NULL || idx == NULL)
    return NCG_ERR_INVALID_ARG;

  if (sd->kind != NCG_VKDE)
    return NCG_ERR_UNSUPPORTED;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  return _d2h (sd, idx, sd->dknn, (size_t) sd->nk * sd->k * sizeof (int32_t));
}

/* ------------------------------------------------------- wait-fault hook */

static int g_fault = NCG_FAULT_NONE;

ncg_status_t
ncg_debug_inject_wait_fault (int32_t fault)
{
  if (fault < NCG_FAULT_NONE || fault > NCG_FAULT_CHAIN_WAIT)
    return NCG_ERR_INVALID_ARG;

  __atomic_store_n (&g_fault, fault, __ATOMIC_SEQ_CST);

  return NCG_OK;
}

int
ncg_fault_take (int fault)
{
  int want = fault;

  return __atomic_compare_exchange_n (&g_fault, &want, NCG_FAULT_NONE, 0, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
}
