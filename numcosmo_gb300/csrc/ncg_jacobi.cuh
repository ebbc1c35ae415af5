/*
 * ncg_jacobi.cuh -- CTA-parallel cyclic Jacobi eigen-decomposition of a small
 * symmetric matrix (d <= NCG_DMAX) in shared memory, NPD_THREADS threads:
 * used by the nearPD fallback (ncg_prepare.cu) and the OGK robust covariance
 * (ncg_robust.cu), where the reference calls LAPACK dsyevr.
 */
#ifndef NCG_JACOBI_CUH
#define NCG_JACOBI_CUH

#include <cuda_runtime.h>

#include "ncg_internal.h"

#define NPD_THREADS 128
#define NPD_LD (NCG_DMAX + 1)

/* player at seat i of round r of the round-robin schedule over m (even) */
static __device__ __forceinline__ int
_rr_seat (int i, int r, int m)
{
  return (i == 0) ? 0 : ((i - 1 + r) % (m - 1)) + 1;
}

/* sum over the threads of the CTA in a fixed order */
static __device__ __forceinline__ double
_npd_block_sum (double v, double *red)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync (0xffffffffu, v, o);

  __syncthreads ();

  if (lane == 0)
    red[wid] = v;

  __syncthreads ();

  double t = 0.0;

  for (int w = 0; w < NPD_THREADS / 32; w++)
    t += red[w];

  return t;
}

/* eigen-decomposition of the symmetric W (destroyed); V gets the vectors as
 * columns, eva the values (unsorted) */
static __device__ void
_npd_jacobi (double (*W)[NPD_LD], double (*V)[NPD_LD], int d, double *eva, double2 *cs, double *red)
{
  const int tid = threadIdx.x;
  const int m   = d + (d & 1);
  const int np  = m / 2;

  for (int e = tid; e < d * d; e += NPD_THREADS)
    V[e / d][e % d] = (e / d == e % d) ? 1.0 : 0.0;

  __syncthreads ();

  for (int sweep = 0; sweep < 100; sweep++)
  {
    double off = 0.0, dg = 0.0;

    for (int e = tid; e < d * d; e += NPD_THREADS)
    {
      const int p = e / d, q = e % d;
      const double v = W[p][q];

      if (q > p)
        off += v * v;
      else if (q == p)
        dg += v * v;
    }

    off = _npd_block_sum (off, red);
    dg  = _npd_block_sum (dg, red);

    if (off <= 1.0e-30 * dg || off == 0.0)
      break;

    for (int r = 0; r < m - 1; r++)
    {
      if (tid < np)
      {
        int p = _rr_seat (tid, r, m), q = _rr_seat (m - 1 - tid, r, m);
        double c = 1.0, sn = 0.0;

        if (p > q)
        {
          const int t = p;

          p = q;
          q = t;
        }

        if (q < d)
        {
          const double apq = W[p][q];

          if (apq != 0.0)
          {
            const double theta = (W[q][q] - W[p][p]) / (2.0 * apq);
            const double t     = (theta >= 0.0 ? 1.0 : -1.0) / (fabs (theta) + sqrt (theta * theta + 1.0));

            c  = 1.0 / sqrt (t * t + 1.0);
            sn = t * c;
          }
        }

        cs[tid] = make_double2 (c, sn);
      }

      __syncthreads ();

      /* W J and V J: columns p, q of every row */
      for (int e = tid; e < 2 * np * d; e += NPD_THREADS)
      {
        const int which = e / (np * d);
        const int k     = (e / d) % np, row = e % d;
        int p = _rr_seat (k, r, m), q = _rr_seat (m - 1 - k, r, m);
        const double2 g = cs[k];

        if (p > q)
        {
          const int t = p;

          p = q;
          q = t;
        }

        if (q >= d || g.y == 0.0)
          continue;

        double (*Z)[NPD_LD] = which ? V : W;
        const double zp = Z[row][p], zq = Z[row][q];

        Z[row][p] = g.x * zp - g.y * zq;
        Z[row][q] = g.y * zp + g.x * zq;
      }

      __syncthreads ();

      /* J^T (W J): rows p, q of every column */
      for (int e = tid; e < np * d; e += NPD_THREADS)
      {
        const int k = e / d, col = e % d;
        int p = _rr_seat (k, r, m), q = _rr_seat (m - 1 - k, r, m);
        const double2 g = cs[k];

        if (p > q)
        {
          const int t = p;

          p = q;
          q = t;
        }

        if (q >= d || g.y == 0.0)
          continue;

        const double wp = W[p][col], wq = W[q][col];

        W[p][col] = g.x * wp - g.y * wq;
        W[q][col] = g.y * wp + g.x * wq;
      }

      __syncthreads ();
    }
  }

  if (tid < d)
    eva[tid] = W[tid][tid];

  __syncthreads ();
}

#endif /* NCG_JACOBI_CUH */
