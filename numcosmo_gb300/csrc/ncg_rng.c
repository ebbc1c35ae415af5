/*
 * ncg_rng.c -- host RNG producing the streams ncg_sd_sample_batch consumes.
 *
 * Stands in for NcmRNG (numcosmo/ncm/core/ncm_rng.c), which wraps GSL's
 * generators (GSL is not part of NumCosmo's sources).  Core: MT19937 of
 * Matsumoto & Nishimura (1998) with the 2002 initialisation.  Transforms:
 * uniform = u32 / 2^32; uniform_pos rejects 0; unit gaussian by Knuth's polar
 * Box-Muller method (TAOCP vol. 2, 3.4.1 algorithm P); chi^2_nu = 2 Gamma(nu/2)
 * with Marsaglia & Tsang (2000) for shape >= 1 and the u^{1/a} boost below 1.
 * The draw order of one sample call follows ncm_stats_dist.c:1618-1627 and the
 * kernels' sample functions: uniform, dim gaussians, then (Student-t) chi^2.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ncg_internal.h"

#define MT_N 624
#define MT_M 397

struct ncg_rng
{
  uint32_t mt[MT_N];
  int mti;
};

static void
_mt_seed (ncg_rng_t *r, uint32_t s)
{
  r->mt[0] = s;

  for (int i = 1; i < MT_N; i++)
    r->mt[i] = 1812433253U * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t) i;

  r->mti = MT_N;
}

uint32_t
ncg_rng_get_u32 (ncg_rng_t *r)
{
  static const uint32_t mag01[2] = { 0x0U, 0x9908b0dfU };
  uint32_t y;

  if (r->mti >= MT_N)
  {
    int kk;

    for (kk = 0; kk < MT_N - MT_M; kk++)
    {
      y         = (r->mt[kk] & 0x80000000U) | (r->mt[kk + 1] & 0x7fffffffU);
      r->mt[kk] = r->mt[kk + MT_M] ^ (y >> 1) ^ mag01[y & 0x1U];
    }

    for (; kk < MT_N - 1; kk++)
    {
      y         = (r->mt[kk] & 0x80000000U) | (r->mt[kk + 1] & 0x7fffffffU);
      r->mt[kk] = r->mt[kk + (MT_M - MT_N)] ^ (y >> 1) ^ mag01[y & 0x1U];
    }

    y                 = (r->mt[MT_N - 1] & 0x80000000U) | (r->mt[0] & 0x7fffffffU);
    r->mt[MT_N - 1]   = r->mt[MT_M - 1] ^ (y >> 1) ^ mag01[y & 0x1U];
    r->mti            = 0;
  }

  y  = r->mt[r->mti++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680U;
  y ^= (y << 15) & 0xefc60000U;
  y ^= (y >> 18);

  return y;
}

ncg_status_t
ncg_rng_new (uint32_t seed, ncg_rng_t **out)
{
  ncg_rng_t *r;

  if (out == NULL)
    return NCG_ERR_INVALID_ARG;

  r = malloc (sizeof (ncg_rng_t));

  if (r == NULL)
    return NCG_ERR_OUT_OF_MEMORY;

  _mt_seed (r, seed);
  *out = r;

  return NCG_OK;
}

ncg_status_t
ncg_rng_free (ncg_rng_t *rng)
{
  free (rng);

  return NCG_OK;
}

size_t
ncg_rng_state_bytes (void)
{
  return sizeof (uint32_t) * (MT_N + 1);
}

ncg_status_t
ncg_rng_get_state (const ncg_rng_t *rng, void *state)
{
  uint32_t *w = state;

  if (rng == NULL || state == NULL)
    return NCG_ERR_INVALID_ARG;

  memcpy (w, rng->mt, sizeof (uint32_t) * MT_N);
  w[MT_N] = (uint32_t) rng->mti;

  return NCG_OK;
}

ncg_status_t
ncg_rng_set_state (ncg_rng_t *rng, const void *state)
{
  const uint32_t *w = state;

  if (rng == NULL || state == NULL || w[MT_N] > MT_N)
    return NCG_ERR_INVALID_ARG;

  memcpy (rng->mt, w, sizeof (uint32_t) * MT_N);
  rng->mti = (int) w[MT_N];

  return NCG_OK;
}

double
ncg_rng_uniform (ncg_rng_t *rng)
{
  return ncg_rng_get_u32 (rng) / 4294967296.0;
}

double
ncg_rng_uniform_pos (ncg_rng_t *rng)
{
  double u;

  do {
    u = ncg_rng_uniform (rng);
  } while (u == 0.0);

  return u;
}

double
ncg_rng_ugaussian (ncg_rng_t *rng)
{
  double x, y, r2;

  do {
    x  = -1.0 + 2.0 * ncg_rng_uniform_pos (rng);
    y  = -1.0 + 2.0 * ncg_rng_uniform_pos (rng);
    r2 = x * x + y * y;
  } while (r2 > 1.0 || r2 == 0.0);

  return y * sqrt (-2.0 * log (r2) / r2);
}

static double
_gamma_ge1 (ncg_rng_t *rng, double a)
{
  const double dd = a - 1.0 / 3.0;
  const double c  = 1.0 / sqrt (9.0 * dd);

  for (;;)
  {
    double x, v, u;

    do {
      x = ncg_rng_ugaussian (rng);
      v = 1.0 + c * x;
    } while (v <= 0.0);

    v = v * v * v;
    u = ncg_rng_uniform_pos (rng);

    if (u < 1.0 - 0.0331 * x * x * x * x)
      return dd * v;

    if (log (u) < 0.5 * x * x + dd * (1.0 - v + log (v)))
      return dd * v;
  }
}

static double
_gamma (ncg_rng_t *rng, double a)
{
  if (a < 1.0)
  {
    const double u = ncg_rng_uniform_pos (rng);

    return _gamma_ge1 (rng, 1.0 + a) * pow (u, 1.0 / a);
  }

  return _gamma_ge1 (rng, a);
}

double
ncg_rng_chisq (ncg_rng_t *rng, double nu)
{
  return 2.0 * _gamma (rng, nu / 2.0);
}

ncg_status_t
ncg_rng_sample_stream (ncg_rng_t *rng, ncg_kernel_t kernel, uint32_t dim, double nu, uint64_t n, double *u,
                       double *z, double *chisq)
{
  if (rng == NULL || u == NULL || z == NULL || dim == 0)
    return NCG_ERR_INVALID_ARG;

  if (kernel == NCG_KERNEL_ST && (chisq == NULL || !(nu > 0.0)))
    return NCG_ERR_INVALID_ARG;

  for (uint64_t j = 0; j < n; j++)
  {
    u[j] = ncg_rng_uniform (rng);

    for (uint32_t c = 0; c < dim; c++)
      z[j * dim + c] = ncg_rng_ugaussian (rng);

    if (kernel == NCG_KERNEL_ST)
      chisq[j] = ncg_rng_chisq (rng, nu);
  }

  return NCG_OK;
}

ncg_status_t
ncg_rng_sample2_stream (ncg_rng_t *rng, ncg_kernel_t kernel, uint32_t dim, double nu, uint64_t n, double *u,
                        double *z1, double *chisq1, double *z2, double *chisq2)
{
  if (rng == NULL || u == NULL || z1 == NULL || z2 == NULL || dim == 0)
    return NCG_ERR_INVALID_ARG;

  if (kernel == NCG_KERNEL_ST && (chisq1 == NULL || chisq2 == NULL || !(nu > 0.0)))
    return NCG_ERR_INVALID_ARG;

  for (uint64_t j = 0; j < n; j++)
  {
    u[j] = ncg_rng_uniform (rng);

    for (uint32_t c = 0; c < dim; c++)
      z1[j * dim + c] = ncg_rng_ugaussian (rng);

    if (kernel == NCG_KERNEL_ST)
      chisq1[j] = ncg_rng_chisq (rng, nu);

    for (uint32_t c = 0; c < dim; c++)
      z2[j * dim + c] = ncg_rng_ugaussian (rng);

    if (kernel == NCG_KERNEL_ST)
      chisq2[j] = ncg_rng_chisq (rng, nu);
  }

  return NCG_OK;
}
