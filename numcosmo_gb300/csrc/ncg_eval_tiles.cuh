/*
 * ncg_eval_tiles.cuh -- the per-CTA work of eval_m2lnp: EV_THREADS points
 * (one per thread) against one slice of the kernel range, leaving per point
 * the reference's (gamma, lambda) pair of the slice.  Shared by the
 * one-problem launches (ncg_eval.cu, grid = point tiles x slices) and the
 * persistent multi-problem launch (ncg_batch.cu, tiles taken from a work
 * list), so a problem gets the same arithmetic in both.
 *
 * Restates, batched over points, _ncm_stats_dist_vkde_eval_weights_m2lnp
 * (numcosmo/ncm/stats/ncm_stats_dist_vkde.c:682-723) and
 * _ncm_stats_dist_kde_eval_weights_m2lnp (numcosmo/ncm/stats/ncm_stats_dist_kde.c:640-681)
 * with the kernels' eval_sum0/sum1_gamma_lambda
 * (ncm_stats_dist_kernel_gauss.c:246-333, ncm_stats_dist_kernel_st.c:295-386).
 * The kernels of a slice are staged in shared memory in chunks of KC (all
 * threads read the same kernel: broadcast); the chunk size changes only the
 * staging, never the order of the arithmetic.
 *
 * FP64 form: everything in double.  Mixed form (SIMT): the difference
 * x - theta_i is formed from hi/lo float splits of both operands (exact to
 * float rounding of the difference), whitening and chi^2 in FP32 FMA,
 * log-sum-exp in FP32 with the per-kernel constants shifted by their
 * maximum.
 */
#ifndef NCG_EVAL_TILES_CUH
#define NCG_EVAL_TILES_CUH

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "ncg_internal.h"

#define EV_THREADS 128

/* FP64 operand stride (doubles per kernel) and the one-problem chunk size */
template <int DP, int KIND>
struct NcgEv64
{
  static constexpr int P   = DP * (DP + 1) / 2;
  static constexpr int S   = (KIND == NCG_VKDE) ? DP + P : DP;
  static constexpr int raw = 32768 / ((S + 1) * 8);
  static constexpr int KC  = raw < 4 ? 4 : (raw > 256 ? 256 : raw);
};

/* mixed operand stride (floats per kernel, multiple of 4):
 *  VKDE: theta_hi[dp] theta_lo[dp] W[dp(dp+1)/2] c'
 *  KDE : yhat_hi[dp]  yhat_lo[dp]  c'
 * KC is the one-problem chunk size, KCB the persistent kernel's (shared
 * memory per CTA <= 40 KiB so several CTAs fit an SM) */
template <int DP, int KIND>
struct NcgEvMx
{
  static constexpr int P   = DP * (DP + 1) / 2;
  static constexpr int RAW = (KIND == NCG_VKDE) ? 2 * DP + P + 1 : 2 * DP + 1;
  static constexpr int S   = (RAW + 3) / 4 * 4;
  static constexpr int KC  = 64;
  static constexpr int kb  = 10240 / S;
  static constexpr int KCB = kb < 4 ? 4 : (kb > 64 ? 64 : kb);
};

template <int DP, int KIND, int KERN, int KC>
__device__ __forceinline__ void
ncg_tile_eval64 (const ncg_eval_args_t a, const double *__restrict__ Xq, const double *__restrict__ pack,
                 const double *__restrict__ cvec, const double *__restrict__ Vg, double2 *__restrict__ part,
                 int kper, int bx, int sy, double *__restrict__ sm, double *__restrict__ sc)
{
  constexpr int S  = NcgEv64<DP, KIND>::S;

  const int64_t j  = (int64_t) bx * EV_THREADS + threadIdx.x;
  const bool valid = j < a.m;
  double x[DP];

#pragma unroll
  for (int c = 0; c < DP; c++)
    x[c] = (valid && c < a.d) ? Xq[j * a.d + c] : 0.0;

  if (KIND == NCG_KDE)
  {
    double v[DP];
    int p = 0;

#pragma unroll
    for (int r = 0; r < DP; r++)
    {
      double s = 0.0;

#pragma unroll
      for (int c = 0; c <= r; c++)
        s = fma (Vg[p++], x[c], s);

      v[r] = s;
    }

#pragma unroll
    for (int c = 0; c < DP; c++)
      x[c] = v[c];
  }

  double gmax = -CUDART_INF, lam = 0.0;
  const int i0 = sy * kper;
  const int i1 = min (a.n, i0 + kper);
  const double inv_nu = 1.0 / a.nu;

  for (int ic = i0; ic < i1; ic += KC)
  {
    const int kc = min (KC, i1 - ic);

    __syncthreads ();

    for (int e = threadIdx.x; e < kc * S; e += EV_THREADS)
      sm[e] = pack[(size_t) ic * S + e];

    for (int e = threadIdx.x; e < kc; e += EV_THREADS)
      sc[e] = cvec[ic + e];

    __syncthreads ();

    for (int kk = 0; kk < kc; kk++)
    {
      const double *pk = sm + kk * S;
      double chi2      = 0.0;

      if (KIND == NCG_VKDE)
      {
        double dl[DP];

#pragma unroll
        for (int c = 0; c < DP; c++)
          dl[c] = x[c] - pk[c];

        const double *W = pk + DP;
        int p           = 0;

#pragma unroll
        for (int r = 0; r < DP; r++)
        {
          double y = 0.0;

#pragma unroll
          for (int c = 0; c <= r; c++)
            y = fma (W[p++], dl[c], y);

          chi2 = fma (y, y, chi2);
        }
      }
      else
      {
#pragma unroll
        for (int c = 0; c < DP; c++)
        {
          const double t = pk[c] - x[c];

          chi2 = fma (t, t, chi2);
        }
      }

      const double lnt = (KERN == NCG_KERNEL_ST) ? fma (a.kappa, log1p (chi2 * inv_nu), sc[kk])
                                                 : fma (-0.5, chi2, sc[kk]);

      if (lnt > gmax)
      {
        lam  = (lam + 1.0) * exp (gmax - lnt);
        gmax = lnt;
      }
      else if (lnt > -CUDART_INF)
      {
        lam += exp (lnt - gmax);
      }
    }
  }

  if (valid)
    part[(size_t) sy * a.m + j] = make_double2 (gmax, lam);
}

template <int DP, int KIND, int KERN, int KC>
__device__ __forceinline__ void
ncg_tile_evalmx (const ncg_eval_args_t a, const double *__restrict__ Xq, const float *__restrict__ pack,
                 const double *__restrict__ Vg, const double *__restrict__ mu, float2 *__restrict__ part, int kper,
                 int bx, int sy, float *__restrict__ sm)
{
  constexpr int P  = DP * (DP + 1) / 2;
  constexpr int S  = NcgEvMx<DP, KIND>::S;

  const int64_t j  = (int64_t) bx * EV_THREADS + threadIdx.x;
  const bool valid = j < a.m;
  float xh[DP], xl[DP];

  {
    double x[DP];

#pragma unroll
    for (int c = 0; c < DP; c++)
      x[c] = (valid && c < a.d) ? Xq[j * a.d + c] - (mu ? mu[c] : 0.0) : 0.0;

    /* global whitening in FP64: KDE v = U^{-T} x / h, VKDE x' = U^{-T} (x - mu) */
    {
      double v[DP];
      int p = 0;

#pragma unroll
      for (int r = 0; r < DP; r++)
      {
        double s = 0.0;

#pragma unroll
        for (int c = 0; c <= r; c++)
          s = fma (Vg[p++], x[c], s);

        v[r] = s;
      }

#pragma unroll
      for (int c = 0; c < DP; c++)
        x[c] = v[c];
    }

#pragma unroll
    for (int c = 0; c < DP; c++)
    {
      xh[c] = __double2float_rn (x[c]);
      xl[c] = __double2float_rn (x[c] - (double) xh[c]);
    }
  }

  float gmax = -CUDART_INF_F, lam = 0.0f;
  const int i0 = sy * kper;
  const int i1 = min (a.n, i0 + kper);
  const float kappa  = (float) a.kappa;
  const float inv_nu = (float) (1.0 / a.nu);

  for (int ic = i0; ic < i1; ic += KC)
  {
    const int kc = min (KC, i1 - ic);

    __syncthreads ();

    {
      const float4 *src = (const float4 *) (pack + (size_t) ic * S);
      float4 *dst       = (float4 *) sm;

      for (int e = threadIdx.x; e < kc * S / 4; e += EV_THREADS)
        dst[e] = src[e];
    }

    __syncthreads ();

    for (int kk = 0; kk < kc; kk++)
    {
      const float *pk = sm + kk * S;
      float dl[DP];

#pragma unroll
      for (int c = 0; c < DP; c++)
        dl[c] = (xh[c] - pk[c]) + (xl[c] - pk[DP + c]);

      float chi2 = 0.0f;

      if (KIND == NCG_VKDE)
      {
        const float *W = pk + 2 * DP;
        int p          = 0;

#pragma unroll
        for (int r = 0; r < DP; r++)
        {
          float y = 0.0f;

#pragma unroll
          for (int c = 0; c <= r; c++)
            y = fmaf (W[p++], dl[c], y);

          chi2 = fmaf (y, y, chi2);
        }
      }
      else
      {
#pragma unroll
        for (int c = 0; c < DP; c++)
          chi2 = fmaf (dl[c], dl[c], chi2);
      }

      const float cc  = pk[(KIND == NCG_VKDE) ? 2 * DP + P : 2 * DP];
      const float lnt = (KERN == NCG_KERNEL_ST) ? fmaf (kappa, log1pf (chi2 * inv_nu), cc) : fmaf (-0.5f, chi2, cc);

      if (lnt > gmax)
      {
        lam  = (lam + 1.0f) * __expf (gmax - lnt);
        gmax = lnt;
      }
      else if (lnt > -CUDART_INF_F)
      {
        lam += __expf (lnt - gmax);
      }
    }
  }

  if (valid)
    part[(size_t) sy * a.m + j] = make_float2 (gmax, lam);
}

#endif /* NCG_EVAL_TILES_CUH */
