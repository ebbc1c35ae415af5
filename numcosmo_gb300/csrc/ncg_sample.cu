/*
 * ncg_sample.cu -- kernel_choose and sample.
 *
 *  wcum            the reference's lazily built cumulative weights: a
 *                  sequential FP64 prefix sum then a multiplication by the
 *                  reciprocal of the total (numcosmo/ncm/stats/ncm_stats_dist.c:1565-1590).
 *                  One thread, same operation order, so the table is
 *                  bit-identical and the chosen indices are exact.
 *  kernel_choose   binary search of p on wcum (ncm_stats_dist.c:1592-1606).
 *  sample          x = theta_i + s U_i^T (h z), s = 1 (Gauss) or
 *                  sqrt(nu / chisq) (Student-t)
 *                  (ncm_stats_dist.c:1618-1627, ncm_stats_dist_kernel_gauss.c:335-355,
 *                   ncm_stats_dist_kernel_st.c:388-414).
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "ncg_internal.h"

__global__ void
_wcum_kernel (const double *__restrict__ w, int n, double *__restrict__ wcum)
{
  if (blockIdx.x != 0 || threadIdx.x != 0)
    return;

  double cum = 0.0;

  wcum[0] = cum;

  for (int i = 0; i < n; i++)
  {
    cum         = __dadd_rn (cum, w[i]);
    wcum[i + 1] = cum;
  }

  const double s = __ddiv_rn (1.0, cum);

  for (int i = 0; i <= n; i++)
    wcum[i] = __dmul_rn (wcum[i], s);
}

extern "C" cudaError_t
ncg_launch_wcum (const double *w, int n, double *wcum, cudaStream_t s)
{
  _wcum_kernel<<<1, 32, 0, s>>> (w, n, wcum);

  return cudaGetLastError ();
}

__device__ __forceinline__ int
_choose (const double *__restrict__ wcum, int n, double p)
{
  int ilo = 0, ihi = n;

  while (ihi > ilo + 1)
  {
    const int mi = (ihi + ilo) / 2;

    if (wcum[mi] > p)
      ihi = mi;
    else
      ilo = mi;
  }

  return ilo;
}

__global__ void
_choose_kernel (const double *__restrict__ wcum, int n, const double *__restrict__ u, int64_t m,
                int32_t *__restrict__ idx)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;

  if (j < m)
    idx[j] = _choose (wcum, n, u[j]);
}

extern "C" cudaError_t
ncg_launch_kernel_choose (const double *wcum, int n, const double *u, int64_t m, int32_t *idx, cudaStream_t s)
{
  if (m <= 0)
    return cudaSuccess;

  _choose_kernel<<<(unsigned) ((m + 255) / 256), 256, 0, s>>> (wcum, n, u, m, idx);

  return cudaGetLastError ();
}

__global__ void
_sample_kernel (int kind, int kernel, int d, double nu, double href, const double *__restrict__ wcum, int n,
                const double *__restrict__ X, const double *__restrict__ Ui, const double *__restrict__ U,
                const double *__restrict__ u, const double *__restrict__ z, const double *__restrict__ chisq,
                int64_t m, double *__restrict__ x, int32_t *__restrict__ idx, const int32_t *__restrict__ kidx)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;

  if (j >= m)
    return;

  /* the chosen kernel, or (kidx) the caller's */
  const int i      = kidx ? kidx[j] : _choose (wcum, n, u[j]);
  const double *Uk = (kind == NCG_VKDE) ? Ui + (size_t) i * d * d : U;
  const double *mu = X + (size_t) i * d;
  double v[NCG_DMAX];

  for (int c = 0; c < d; c++)
    v[c] = z[j * d + c] * href;

  /* v := U^T v (dtrmv Upper/Trans), bottom row first so it works in place */
  for (int r = d - 1; r >= 0; r--)
  {
    double s = 0.0;

    for (int c = 0; c <= r; c++)
      s += Uk[c * d + r] * v[c];

    v[r] = s;
  }

  if (kernel == NCG_KERNEL_ST)
  {
    const double chi_scale = sqrt (nu / chisq[j]);

    for (int c = 0; c < d; c++)
      v[c] = v[c] * chi_scale;
  }

  for (int c = 0; c < d; c++)
    x[j * d + c] = v[c] + mu[c];

  if (idx)
    idx[j] = i;
}

extern "C" cudaError_t
ncg_launch_sample (int kind, int kernel, int d, double nu, double href, const double *wcum, int n,
                   const double *X, const double *Ui, const double *U, const double *u, const double *z,
                   const double *chisq, int64_t m, double *x, int32_t *idx, cudaStream_t s)
{
  if (m <= 0)
    return cudaSuccess;

  _sample_kernel<<<(unsigned) ((m + 127) / 128), 128, 0, s>>> (kind, kernel, d, nu, href, wcum, n, X, Ui, U, u, z,
                                                                chisq, m, x, idx, NULL);

  return cudaGetLastError ();
}

/* the kernel draws of ncm_stats_dist_kernel_{gauss,st}_sample from the given
 * kernels kidx[j] (ncm_stats_dist_sample2 picks them from a sorted order) */
extern "C" cudaError_t
ncg_launch_sample_at (int kind, int kernel, int d, double nu, double href, const double *X, const double *Ui,
                      const double *U, const int32_t *kidx, const double *z, const double *chisq, int64_t m, double *x,
                      cudaStream_t s)
{
  if (m <= 0)
    return cudaSuccess;

  _sample_kernel<<<(unsigned) ((m + 127) / 128), 128, 0, s>>> (kind, kernel, d, nu, href, NULL, 0, X, Ui, U, NULL, z,
                                                                chisq, m, x, NULL, kidx);

  return cudaGetLastError ();
}
