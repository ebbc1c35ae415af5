/*
 * ncg_serve.cu -- the device steps of one APES move that are not StatsDist
 * calls, for the serving loop (ncg_server.c):
 *
 *   target   -2 ln L of the chain's Gaussian target at the proposals:
 *            |L^{-1} x|^2 with L the lower Cholesky factor of its covariance
 *   accept   the Metropolis-Hastings test of an independence proposal drawn
 *            from the fitted density q: ln r = -(m2lnL* - m2lnL_k)/2 +
 *            (m2lnq* - m2lnq_k)/2 (NcmFitESMCMCWalkerAPES, numcosmo/ncm/fit/
 *            ncm_fit_esmcmc_walker_apes.c:872-919); accepted walkers take
 *            the proposal and its -2 ln L.  The accept count is a sum of
 *            integers, so its value does not depend on the order.  In the
 *            exploration phase the ratio is the target's alone (:910-912).
 *   mix      the transition densities of the proposal mixture with the
 *            truncated Gaussian random walk (_ncm_fit_esmcmc_walker_apes_
 *            transition_prob, :816-859), in place of the fit's m2lnq.
 */
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "ncg_internal.h"

#define SV_THREADS 128

__global__ void __launch_bounds__ (SV_THREADS)
_target_kernel (const double *__restrict__ X, int64_t n, int d, const double *__restrict__ L,
                double *__restrict__ out)
{
  const int64_t j = (int64_t) blockIdx.x * SV_THREADS + threadIdx.x;

  if (j >= n)
    return;

  const double *x = X + j * d;
  double y[NCG_DMAX];
  double s = 0.0;

  for (int r = 0; r < d; r++)
  {
    double v = x[r];

    for (int c = 0; c < r; c++)
      v = fma (-L[r * d + c], y[c], v);

    y[r] = v / L[r * d + r];
    s    = fma (y[r], y[r], s);
  }

  out[j] = s;
}

extern "C" cudaError_t
ncg_launch_serve_target (const double *X, int64_t n, int d, const double *L, double *out, cudaStream_t s)
{
  if (n <= 0)
    return cudaSuccess;

  if (d > NCG_DMAX)
    return cudaErrorInvalidValue;

  _target_kernel<<<(unsigned) ((n + SV_THREADS - 1) / SV_THREADS), SV_THREADS, 0, s>>> (X, n, d, L, out);

  return cudaGetLastError ();
}

/* ln of the standard normal mass in [zl, zu] (negative orientation gives the
 * same magnitude), ncm_util_log_normal_gaussian_integral (numcosmo/ncm/core/
 * ncm_util.c:646-693): erfc tails beyond 3 / sqrt 2 on either side */
__device__ double
_log_ngi (double zl, double zu)
{
  const double b = 3.0;
  double ul, uu;

  if (zl == zu)
    return -CUDART_INF;

  if (zl < zu)
  {
    ul = zl * CUDART_SQRT_HALF;
    uu = zu * CUDART_SQRT_HALF;
  }
  else
  {
    ul = zu * CUDART_SQRT_HALF;
    uu = zl * CUDART_SQRT_HALF;
  }

  if (ul > b)
    return log (fabs (0.5 * (erfc (ul) - erfc (uu))));

  if (uu < -b)
    return log (fabs (0.5 * (erfc (-ul) - erfc (-uu))));

  if (uu > b && ul < -b)
    return log1p (-0.5 * (erfc (uu) + erfc (-ul)));

  return log (fabs (0.5 * (erf (uu) - erf (ul))));
}

/* -2 ln of the truncated random walk's density at `to` from `from`
 * (ncm_fit_esmcmc_walker_apes.c:832-843); rw = std | lb | ub */
__device__ double
_m2lnp_rw (const double *from, const double *to, const double *rw, int d)
{
  double m = 0.0;

  for (int i = 0; i < d; i++)
  {
    const double sd = rw[i], lb = rw[d + i], ub = rw[2 * d + i];
    const double ln_norm = 0.91893853320467274178 + log (sd) + _log_ngi ((lb - from[i]) / sd, (ub - from[i]) / sd);
    const double t       = (to[i] - from[i]) / sd;

    m += t * t + 2.0 * ln_norm;
  }

  return m;
}

/* -2 ln of the mixture (1 - p) q + p rw, as the reference combines them (:845-853) */
__device__ double
_mix2 (double m2_sd, double m2_rw, double p)
{
  m2_rw += -2.0 * log (p);
  m2_sd += -2.0 * log1p (-p);

  return (m2_sd < m2_rw) ? m2_sd - 2.0 * log1p (exp (-0.5 * (m2_rw - m2_sd)))
                         : m2_rw - 2.0 * log1p (exp (-0.5 * (m2_sd - m2_rw)));
}

__global__ void __launch_bounds__ (SV_THREADS)
_mix_kernel (double *__restrict__ q, const double *__restrict__ X, const double *__restrict__ prop,
             const double *__restrict__ rw, int64_t n, int d, double p)
{
  const int64_t j = (int64_t) blockIdx.x * SV_THREADS + threadIdx.x;

  if (j >= n)
    return;

  const double *x = X + j * d, *y = prop + j * d;

  q[j]     = _mix2 (q[j], _m2lnp_rw (x, y, rw, d), p);       /* m2lnp_star: theta_k -> theta* */
  q[n + j] = _mix2 (q[n + j], _m2lnp_rw (y, x, rw, d), p);   /* m2lnp_cur: theta* -> theta_k */
}

extern "C" cudaError_t
ncg_launch_serve_mix (double *q, const double *X, const double *prop, const double *rw, int64_t n, int d, double p,
                      cudaStream_t s)
{
  if (n <= 0)
    return cudaSuccess;

  _mix_kernel<<<(unsigned) ((n + SV_THREADS - 1) / SV_THREADS), SV_THREADS, 0, s>>> (q, X, prop, rw, n, d, p);

  return cudaGetLastError ();
}

/* q = [m2lnq at the proposals (n) | m2lnq at the walkers (n)] */
__global__ void __launch_bounds__ (SV_THREADS)
_accept_kernel (double *__restrict__ X, double *__restrict__ m2lnL, const double *__restrict__ prop,
                const double *__restrict__ m2lnL_prop, const double *__restrict__ q, const double *__restrict__ u,
                int64_t n, int d, int explore, unsigned long long *accepted)
{
  const int64_t j = (int64_t) blockIdx.x * SV_THREADS + threadIdx.x;
  int acc         = 0;

  if (j < n)
  {
    const double lnr = explore ? -0.5 * (m2lnL_prop[j] - m2lnL[j])
                               : -0.5 * (m2lnL_prop[j] - m2lnL[j]) + 0.5 * (q[j] - q[n + j]);

    if (log (u[j]) < lnr)
    {
      for (int c = 0; c < d; c++)
        X[j * d + c] = prop[j * d + c];

      m2lnL[j] = m2lnL_prop[j];
      acc      = 1;
    }
  }

  acc = __syncthreads_count (acc);

  if (threadIdx.x == 0 && acc > 0)
    atomicAdd (accepted, (unsigned long long) acc);
}

extern "C" cudaError_t
ncg_launch_serve_accept (double *X, double *m2lnL, const double *prop, const double *m2lnL_prop, const double *q,
                         const double *u, int64_t n, int d, int explore, unsigned long long *accepted,
                         cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync (accepted, 0, sizeof (unsigned long long), s);

  if (e != cudaSuccess || n <= 0)
    return e;

  _accept_kernel<<<(unsigned) ((n + SV_THREADS - 1) / SV_THREADS), SV_THREADS, 0, s>>> (X, m2lnL, prop, m2lnL_prop,
                                                                                       q, u, n, d, explore, accepted);

  return cudaGetLastError ();
}
