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
 *            integers, so its value does not depend on the order.
 */
#include <cuda_runtime.h>
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

/* q = [m2lnq at the proposals (n) | m2lnq at the walkers (n)] */
__global__ void __launch_bounds__ (SV_THREADS)
_accept_kernel (double *__restrict__ X, double *__restrict__ m2lnL, const double *__restrict__ prop,
                const double *__restrict__ m2lnL_prop, const double *__restrict__ q, const double *__restrict__ u,
                int64_t n, int d, unsigned long long *accepted)
{
  const int64_t j = (int64_t) blockIdx.x * SV_THREADS + threadIdx.x;
  int acc         = 0;

  if (j < n)
  {
    const double lnr = -0.5 * (m2lnL_prop[j] - m2lnL[j]) + 0.5 * (q[j] - q[n + j]);

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
                         const double *u, int64_t n, int d, unsigned long long *accepted, cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync (accepted, 0, sizeof (unsigned long long), s);

  if (e != cudaSuccess || n <= 0)
    return e;

  _accept_kernel<<<(unsigned) ((n + SV_THREADS - 1) / SV_THREADS), SV_THREADS, 0, s>>> (X, m2lnL, prop, m2lnL_prop,
                                                                                       q, u, n, d, accepted);

  return cudaGetLastError ();
}
