/*
 * ncg_prepare.cu -- device side of NcmStatsDistKDE / NcmStatsDistVKDE prepare.
 *
 *  global_cov_chol  Welford covariance of all centres + upper Cholesky
 *                   (numcosmo/ncm/stats/ncm_stats_dist_kde.c:379-450,
 *                    numcosmo/ncm/stats/ncm_stats_vec.c:511-565,2376-2398)
 *  whiten           invUsample = X U^{-1}  (ncm_stats_dist_kde.c:477-480)
 *  knn              exact k nearest neighbours in the whitened space, ordered
 *                   by (squared distance, index) as the reference kd-tree
 *                   (numcosmo/external/misc/kdtree.c:28-38,193-320,
 *                    numcosmo/external/misc/rb_knn_list.c:32-40)
 *  local_cov_chol   per-kernel Welford covariance of the neighbours (in that
 *                   order) + Cholesky (ncm_stats_dist_vkde.c:426-488)
 *  nearpd           Higham nearPD / diagonal fallback for the factors that
 *                   failed (ncm_stats_dist_vkde.c:338-360,
 *                   numcosmo/ncm/algebra/ncm_matrix.c:1248-1344)
 *  vkde_finish      lnnorm_i (ncm_stats_dist_kernel_{gauss,st}.c get_lnnorm)
 *                   and the eval operand U_i^{-T}/h
 *
 * The covariance, Cholesky, whitening and distance arithmetic use explicitly
 * rounded operations (no FMA contraction) in the reference's operation order,
 * so the factors and the kNN sets are bit-identical to a CPU evaluation of
 * the same formulas compiled without contraction.
 */
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "ncg_internal.h"

#include <mutex>

/* Raise a kernel's dynamic shared-memory limit on the current device to at
 * least `bytes`, never lowering it: host threads that launch the same kernel
 * with different sizes at the same time (several handles prepared at once)
 * cannot then launch under a smaller limit another thread set in between.
 * limit[dev] remembers what was set, under one lock for all kernels. */
static std::mutex g_smem_mu;

extern "C" cudaError_t
ncg_raise_smem_limit (const void *fn, size_t bytes, int *limit)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice (&dev);

  if (e != cudaSuccess)
    return e;

  if (dev < 0 || dev >= NCG_MAX_DEVICES)
    return cudaErrorInvalidDevice;

  std::lock_guard<std::mutex> lock (g_smem_mu);

  if ((size_t) limit[dev] >= bytes)
    return cudaSuccess;

  e = cudaFuncSetAttribute (fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);

  if (e == cudaSuccess)
    limit[dev] = (int) bytes;

  return e;
}

#define WT 32          /* Welford rows staged per chunk */
#define PREP_THREADS 128

struct WelfordSmem
{
  double xs[WT][NCG_DMAX];
  double mh[WT][NCG_DMAX];
  double mprev[NCG_DMAX];
  double A[NCG_DMAX * NCG_DMAX];
  int    rows[WT];
  int    info;
};

/* (r, c), r < c, of the e-th strictly-upper element, row by row */
__device__ __forceinline__ void
_upper_rc (int e, int d, int *r, int *c)
{
  int rr = 0, rem = e;

  while (rem >= d - 1 - rr)
  {
    rem -= d - 1 - rr;
    rr++;
  }

  *r = rr;
  *c = rr + 1 + rem;
}

/* Unit-weight Welford mean/covariance of X[rows[t]] for t < cnt (rows NULL:
 * row t), restating ncm_stats_vec.c:511-565 and get_cov_matrix :2376-2398.
 * Result (full symmetric, bias-corrected) in sm.A.  All threads call it. */
__device__ void
_welford_block (const double *__restrict__ X, const int32_t *__restrict__ rows, int cnt, int d, int nmax,
                int32_t *bad, WelfordSmem &sm)
{
  const int tid = threadIdx.x, nth = blockDim.x;
  const int E   = d * (d - 1) / 2;
  double Cacc[4];
  int er[4], ec[4];
  double mean = 0.0, var = 0.0;

#pragma unroll
  for (int q = 0; q < 4; q++)
  {
    const int e = tid + q * nth;

    Cacc[q] = 0.0;
    er[q]   = 0;
    ec[q]   = 0;

    if (e < E)
      _upper_rc (e, d, &er[q], &ec[q]);
  }

  if (tid < d)
    sm.mprev[tid] = 0.0;

  for (int t0 = 0; t0 < cnt; t0 += WT)
  {
    const int tn = min (WT, cnt - t0);

    __syncthreads ();

    if (tid < tn)
    {
      int r = rows ? rows[t0 + tid] : t0 + tid;

      if (r < 0 || r >= nmax)
      {
        atomicAdd (bad, 1);
        r = 0;
      }

      sm.rows[tid] = r;
    }

    __syncthreads ();

    for (int idx = tid; idx < tn * d; idx += nth)
    {
      const int tt = idx / d, c = idx - tt * d;

      sm.xs[tt][c] = X[(size_t) sm.rows[tt] * d + c];
    }

    __syncthreads ();

    if (tid < d)
    {
      for (int tt = 0; tt < tn; tt++)
      {
        const double weight    = (double) (t0 + tt);
        const double curweight = __dadd_rn (weight, 1.0);
        const double delta     = __dsub_rn (sm.xs[tt][tid], mean);
        const double R         = __ddiv_rn (delta, curweight);
        const double dvar      = __dmul_rn (__dmul_rn (weight, delta), R);

        mean            = __dadd_rn (mean, R);
        var             = __dadd_rn (var, dvar);
        sm.mh[tt][tid]  = mean;
      }
    }

    __syncthreads ();

#pragma unroll
    for (int q = 0; q < 4; q++)
    {
      if (tid + q * nth < E)
      {
        const int r = er[q], c = ec[q];
        double acc  = Cacc[q];

        for (int tt = 0; tt < tn; tt++)
        {
          const double a = __dsub_rn (sm.xs[tt][r], sm.mh[tt][r]);
          const double b = __dsub_rn (sm.xs[tt][c], (tt > 0) ? sm.mh[tt - 1][c] : sm.mprev[c]);

          acc = __dadd_rn (acc, __dmul_rn (a, b));
        }

        Cacc[q] = acc;
      }
    }

    __syncthreads ();

    if (tid < d)
      sm.mprev[tid] = sm.mh[tn - 1][tid];
  }

  {
    const double W    = (double) cnt;
    const double bias = __ddiv_rn (1.0, __dsub_rn (W, __ddiv_rn (W, W)));

#pragma unroll
    for (int q = 0; q < 4; q++)
    {
      if (tid + q * nth < E)
      {
        const double v = __dmul_rn (Cacc[q], bias);

        sm.A[er[q] * d + ec[q]] = v;
        sm.A[ec[q] * d + er[q]] = v;
      }
    }

    if (tid < d)
      sm.A[tid * d + tid] = __dmul_rn (var, bias);
  }

  __syncthreads ();
}

/* In-place upper Cholesky of sm.A (Sigma = U^T U), column by column in the
 * order of orc_cholesky_upper.  Returns LAPACK-style info in all threads. */
__device__ int
_chol_block (double *A, int d, int *info)
{
  const int tid = threadIdx.x, nth = blockDim.x;

  if (tid == 0)
    *info = 0;

  __syncthreads ();

  for (int j = 0; j < d; j++)
  {
    if (tid == 0)
    {
      double ajj = A[j * d + j];

      for (int k = 0; k < j; k++)
        ajj = __dsub_rn (ajj, __dmul_rn (A[k * d + j], A[k * d + j]));

      if (!(ajj > 0.0))
      {
        A[j * d + j] = ajj;
        *info        = j + 1;
      }
      else
      {
        A[j * d + j] = __dsqrt_rn (ajj);
      }
    }

    __syncthreads ();

    if (*info != 0)
      return *info;

    {
      const double ajj = A[j * d + j];

      for (int i = j + 1 + tid; i < d; i += nth)
      {
        double aji = A[j * d + i];

        for (int k = 0; k < j; k++)
          aji = __dsub_rn (aji, __dmul_rn (A[k * d + j], A[k * d + i]));

        A[j * d + i] = __ddiv_rn (aji, ajj);
      }
    }

    __syncthreads ();
  }

  return 0;
}

/* frexp-guarded 2 ln det (ncm_matrix.c:1158-1186) */
__device__ double
_chol_lndet (const double *U, int d, int ld)
{
  const double lb = 1.0e-200, ub = 1.0e+200;
  double detL     = 1.0;
  long exponent   = 0;

  for (int i = 0; i < d; i++)
  {
    const double Lii   = fabs (U[i * ld + i]);
    const double ndetL = detL * Lii;

    if ((ndetL < lb) || (ndetL > ub))
    {
      int e = 0;

      detL      = frexp (ndetL, &e);
      exponent += e;
    }
    else
    {
      detL = ndetL;
    }
  }

  return 2.0 * (log (detL) + exponent * 0.69314718055994530941723212145818);
}

/* kernel lnnorm: ncm_stats_dist_kernel_gauss.c:201-207, ncm_stats_dist_kernel_st.c:240-252 */
__device__ double
_kernel_lnnorm (int kernel, double nu, int d, double lndet)
{
  if (kernel == NCG_KERNEL_GAUSS)
    return 0.5 * (d * NCG_LN2PI + lndet);

  return (lgamma (nu / 2.0) - lgamma ((nu + d) / 2.0)) + (d / 2.0) * (NCG_LNPI + log (nu)) + 0.5 * lndet;
}

/* ------------------------------------------------------------------------ */

__global__ void __launch_bounds__ (PREP_THREADS)
_global_cov_chol_kernel (const double *__restrict__ X, int n, int d, double *cov, double *U,
                         int32_t *flag, ncg_prep_status_t *st)
{
  __shared__ WelfordSmem sm;
  const int tid = threadIdx.x;

  if (n > 0)
  {
    _welford_block (X, NULL, n, d, n, &st->n_badindex, sm);

    for (int i = tid; i < d * d; i += blockDim.x)
      cov[i] = sm.A[i];
  }
  else
  {
    /* fixed covariance supplied in cov (ncm_stats_dist_kde.c:825-845) */
    for (int i = tid; i < d * d; i += blockDim.x)
      sm.A[i] = cov[i];
  }

  __syncthreads ();

  if (_chol_block (sm.A, d, &sm.info) != 0)
  {
    /* leave the covariance in U for the nearPD pass */
    for (int i = tid; i < d * d; i += blockDim.x)
      U[i] = cov[i];

    if (tid == 0)
    {
      flag[0] = 1;
      atomicAdd (&st->n_flagged, 1);
    }

    return;
  }

  for (int i = tid; i < d * d; i += blockDim.x)
  {
    const int r = i / d, c = i - r * d;

    U[i] = (c >= r) ? sm.A[i] : 0.0;
  }

  if (tid == 0)
    flag[0] = 0;
}

extern "C" cudaError_t
ncg_launch_global_cov_chol (const double *X, int n, int d, double *cov, double *U, int32_t *flag,
                            ncg_prep_status_t *st, cudaStream_t s)
{
  _global_cov_chol_kernel<<<1, PREP_THREADS, 0, s>>> (X, n, d, cov, U, flag, st);

  return cudaGetLastError ();
}

__global__ void
_global_lnnorm_kernel (const double *U, int d, int kernel, double nu, ncg_prep_status_t *st)
{
  if (threadIdx.x == 0 && blockIdx.x == 0)
    st->kernel_lnnorm = _kernel_lnnorm (kernel, nu, d, _chol_lndet (U, d, d));
}

extern "C" cudaError_t
ncg_launch_global_lnnorm (const double *U, int d, int kernel, double nu, ncg_prep_status_t *st,
                          cudaStream_t s)
{
  _global_lnnorm_kernel<<<1, 32, 0, s>>> (U, d, kernel, nu, st);

  return cudaGetLastError ();
}

/* ------------------------------------------------------------------------ */

/* Y = X U^{-1} row by row (dtrsm Right/Upper/NoTrans, kde.c:477-480) */
__global__ void
_whiten_kernel (const double *__restrict__ X, const double *__restrict__ U, int n, int d,
                double *__restrict__ Y)
{
  __shared__ double sU[NCG_DMAX * NCG_DMAX];

  for (int i = threadIdx.x; i < d * d; i += blockDim.x)
    sU[i] = U[i];

  __syncthreads ();

  const int row = blockIdx.x * blockDim.x + threadIdx.x;

  if (row >= n)
    return;

  double y[NCG_DMAX];
  const double *x = X + (size_t) row * d;

  for (int j = 0; j < d; j++)
  {
    double s = x[j];

    for (int k = 0; k < j; k++)
      s = __dsub_rn (s, __dmul_rn (y[k], sU[k * d + j]));

    y[j] = __ddiv_rn (s, sU[j * d + j]);
  }

  for (int j = 0; j < d; j++)
    Y[(size_t) row * d + j] = y[j];
}

extern "C" cudaError_t
ncg_launch_whiten (const double *X, const double *U, int n, int d, double *Y, cudaStream_t s)
{
  const int th = 128;

  _whiten_kernel<<<(n + th - 1) / th, th, 0, s>>> (X, U, n, d, Y);

  return cudaGetLastError ();
}

/* ------------------------------------------------------------------------ */
/* Exact kNN: all squared distances of one query into shared memory (or a    */
/* per-CTA global slice for large n), MSB-first radix select of the k-th     */
/* (distance, index) key, ordered compaction of ties, bitonic sort.          */
/* ------------------------------------------------------------------------ */

#define KNN_THREADS 512
#define KNN_SMEM_NMAX 16384

static inline int
_pow2_ceil (int k)
{
  int p = 1;

  while (p < k)
    p <<= 1;

  return p;
}

__global__ void __launch_bounds__ (KNN_THREADS)
_knn_kernel (const double *__restrict__ Y, int n, int nq, int d, int k, int kp2, int32_t *__restrict__ out,
             uint64_t *__restrict__ gkeys)
{
  extern __shared__ __align__ (16) unsigned char knn_smem[];
  __shared__ double yq[NCG_DMAX];
  __shared__ unsigned int hist[256];
  __shared__ unsigned long long s_prefix;
  __shared__ int s_need, s_cnt_lt, s_eq_base;
  __shared__ int warp_tot[KNN_THREADS / 32];

  const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, wid = tid >> 5;
  uint64_t *selk = (uint64_t *) knn_smem;
  int32_t *seli  = (int32_t *) (selk + kp2);
  uint64_t *keys = gkeys ? gkeys + (size_t) blockIdx.x * n : (uint64_t *) (seli + kp2 + (kp2 & 1));

  for (int q = blockIdx.x; q < nq; q += gridDim.x)
  {
    __syncthreads ();

    if (tid < d)
      yq[tid] = Y[(size_t) q * d + tid];

    __syncthreads ();

    /* squared distances summed in coordinate order, candidate minus query */
    for (int j = tid; j < n; j += nth)
    {
      const double *p = Y + (size_t) j * d;
      double dist     = 0.0;

      for (int c = 0; c < d; c++)
      {
        const double df = __dsub_rn (p[c], yq[c]);

        dist = __dadd_rn (dist, __dmul_rn (df, df));
      }

      keys[j] = (uint64_t) __double_as_longlong (dist);
    }

    if (tid == 0)
    {
      s_prefix = 0ULL;
      s_need   = k;
      s_cnt_lt = 0;
    }

    __syncthreads ();

    /* radix select of the k-th smallest key */
    unsigned long long mask = 0ULL;

    for (int pass = 7; pass >= 0; pass--)
    {
      const int sh = 8 * pass;

      for (int b = tid; b < 256; b += nth)
        hist[b] = 0;

      __syncthreads ();

      const unsigned long long prefix = s_prefix;

      for (int j = tid; j < n; j += nth)
      {
        const unsigned long long key = keys[j];

        if ((key & mask) == prefix)
          atomicAdd (&hist[(key >> sh) & 255ULL], 1U);
      }

      __syncthreads ();

      if (tid == 0)
      {
        int need = s_need;
        int b    = 0;

        for (b = 0; b < 256; b++)
        {
          if ((int) hist[b] >= need)
            break;

          need -= hist[b];
        }

        if (b > 255)
          b = 255;

        s_need   = need;
        s_prefix = prefix | ((unsigned long long) b << sh);
      }

      mask |= (255ULL << sh);
      __syncthreads ();
    }

    const unsigned long long T = s_prefix;
    const int need_eq          = s_need;   /* how many keys equal to T are kept */

    if (tid == 0)
      s_eq_base = 0;

    __syncthreads ();

    /* compaction: keys < T anywhere (sorted later), keys == T by index order */
    for (int base = 0; base < n; base += nth)
    {
      const int j      = base + tid;
      const bool valid = j < n;
      const unsigned long long key = valid ? keys[j] : ~0ULL;
      const bool lt    = valid && key < T;
      const bool eq    = valid && key == T;

      if (lt)
      {
        const int pos = atomicAdd (&s_cnt_lt, 1);

        if (pos < k - need_eq)
        {
          selk[pos] = key;
          seli[pos] = j;
        }
      }

      const unsigned int bal = __ballot_sync (0xffffffffu, eq);

      if (lane == 0)
        warp_tot[wid] = __popc (bal);

      __syncthreads ();

      if (eq)
      {
        int rank = s_eq_base + __popc (bal & ((1u << lane) - 1u));

        for (int w = 0; w < wid; w++)
          rank += warp_tot[w];

        if (rank < need_eq)
        {
          selk[(k - need_eq) + rank] = key;
          seli[(k - need_eq) + rank] = j;
        }
      }

      __syncthreads ();

      if (tid == 0)
      {
        int tot = 0;

        for (int w = 0; w < nth / 32; w++)
          tot += warp_tot[w];

        s_eq_base += tot;
      }

      __syncthreads ();
    }

    for (int t = k + tid; t < kp2; t += nth)
    {
      selk[t] = ~0ULL;
      seli[t] = 0x7fffffff;
    }

    __syncthreads ();

    /* bitonic sort of (key, index) ascending */
    for (int size = 2; size <= kp2; size <<= 1)
    {
      for (int stride = size >> 1; stride > 0; stride >>= 1)
      {
        for (int t = tid; t < kp2; t += nth)
        {
          const int u = t ^ stride;

          if (u > t)
          {
            const bool up = ((t & size) == 0);
            const uint64_t ka = selk[t], kb = selk[u];
            const int32_t ia = seli[t], ib = seli[u];
            const bool gt = (ka > kb) || (ka == kb && ia > ib);

            if (gt == up)
            {
              selk[t] = kb;
              selk[u] = ka;
              seli[t] = ib;
              seli[u] = ia;
            }
          }
        }

        __syncthreads ();
      }
    }

    for (int t = tid; t < k; t += nth)
      out[(size_t) q * k + t] = seli[t];
  }
}

extern "C" size_t
ncg_knn_scratch_bytes (int n, int d, int k)
{
  (void) d;
  (void) k;

  if (n <= KNN_SMEM_NMAX)
    return 0;

  return (size_t) 4 * 152 * (size_t) n * sizeof (uint64_t);
}

/* the k nearest of the n points Y to each of the first nq of them (the
 * kernels; with a split cross-validation the other observations only enter
 * as neighbours) */
extern "C" cudaError_t
ncg_launch_knn (const double *Y, int n, int nq, int d, int k, int32_t *knn, uint64_t *keys_scratch, cudaStream_t s)
{
  const int kp2      = _pow2_ceil (k);
  const bool in_smem = (n <= KNN_SMEM_NMAX);
  size_t smem        = (size_t) kp2 * (sizeof (uint64_t) + sizeof (int32_t)) + 8;
  int grid           = nq;

  if (k > NCG_KNN_KMAX || k > n || nq > n || nq <= 0)
    return cudaErrorInvalidValue;

  if (in_smem)
    smem += (size_t) n * sizeof (uint64_t);
  else
  {
    if (keys_scratch == NULL)
      return cudaErrorInvalidValue;

    grid = (nq < 4 * 152) ? nq : 4 * 152;
  }

  /* raised whatever the size: the kernel's static arrays count against the
   * 48 KiB default too */
  static int limit[NCG_MAX_DEVICES];
  cudaError_t e = ncg_raise_smem_limit ((const void *) _knn_kernel, smem, limit);

  if (e != cudaSuccess)
    return e;

  _knn_kernel<<<grid, KNN_THREADS, smem, s>>> (Y, n, nq, d, k, kp2, knn, in_smem ? NULL : keys_scratch);

  return cudaGetLastError ();
}

/* ------------------------------------------------------------------------ */

__global__ void __launch_bounds__ (PREP_THREADS)
_local_cov_chol_kernel (const double *__restrict__ X, const int32_t *__restrict__ knn, int n, int nq, int d, int k,
                        double *__restrict__ Ui, int32_t *__restrict__ flag, ncg_prep_status_t *st)
{
  __shared__ WelfordSmem sm;
  const int tid = threadIdx.x;

  for (int i = blockIdx.x; i < nq; i += gridDim.x)
  {
    double *Uo = Ui + (size_t) i * d * d;

    _welford_block (X, knn + (size_t) i * k, k, d, n, &st->n_badindex, sm);

    /* keep the covariance in the output slot until the factor succeeds */
    for (int e = tid; e < d * d; e += blockDim.x)
      Uo[e] = sm.A[e];

    __syncthreads ();

    const int info = _chol_block (sm.A, d, &sm.info);

    if (info != 0)
    {
      if (tid == 0)
      {
        flag[i] = 1;
        atomicAdd (&st->n_flagged, 1);
      }
    }
    else
    {
      for (int e = tid; e < d * d; e += blockDim.x)
      {
        const int r = e / d, c = e - r * d;

        Uo[e] = (c >= r) ? sm.A[e] : 0.0;
      }

      if (tid == 0)
        flag[i] = 0;
    }

    __syncthreads ();
  }
}

/* the nq kernels' local covariances from their neighbour lists (indices
 * into the n observations) and their upper Cholesky factors */
extern "C" cudaError_t
ncg_launch_local_cov_chol (const double *X, const int32_t *knn, int n, int nq, int d, int k, double *Ui,
                           int32_t *flag, ncg_prep_status_t *st, cudaStream_t s)
{
  const int grid = (nq < 152 * 16) ? nq : 152 * 16;

  _local_cov_chol_kernel<<<grid, PREP_THREADS, 0, s>>> (X, knn, n, nq, d, k, Ui, flag, st);

  return cudaGetLastError ();
}

/* upper Cholesky of the covariance each slot of Ui holds (the robust types
 * compute it elsewhere); flags as _local_cov_chol_kernel */
__global__ void __launch_bounds__ (PREP_THREADS)
_chol_slots_kernel (double *__restrict__ Ui, int n, int d, int32_t *__restrict__ flag, ncg_prep_status_t *st)
{
  __shared__ WelfordSmem sm;
  const int tid = threadIdx.x;

  for (int i = blockIdx.x; i < n; i += gridDim.x)
  {
    double *Uo = Ui + (size_t) i * d * d;

    for (int e = tid; e < d * d; e += blockDim.x)
      sm.A[e] = Uo[e];

    __syncthreads ();

    const int info = _chol_block (sm.A, d, &sm.info);

    if (info != 0)
    {
      if (tid == 0)
      {
        flag[i] = 1;
        atomicAdd (&st->n_flagged, 1);
      }
    }
    else
    {
      for (int e = tid; e < d * d; e += blockDim.x)
      {
        const int r = e / d, c = e - r * d;

        Uo[e] = (c >= r) ? sm.A[e] : 0.0;
      }

      if (tid == 0)
        flag[i] = 0;
    }

    __syncthreads ();
  }
}

extern "C" cudaError_t
ncg_launch_chol_slots (double *Ui, int n, int d, int32_t *flag, ncg_prep_status_t *st, cudaStream_t s)
{
  const int grid = (n < 152 * 16) ? n : 152 * 16;

  _chol_slots_kernel<<<grid, PREP_THREADS, 0, s>>> (Ui, n, d, flag, st);

  return cudaGetLastError ();
}

/* ------------------------------------------------------------------------ */
/* nearPD fallback: one CTA per failed factor, all state in shared memory.    */
/*                                                                          */
/* Restates ncm_matrix_nearPD (numcosmo/ncm/algebra/ncm_matrix.c:1248-1344)   */
/* with cholesky_decomp = TRUE, as the oracle does: Higham's alternating      */
/* projections with the unit diagonal restored, negative eigenvalues raised  */
/* to min_pos_ev * DBL_EPSILON, until the Cholesky of the iterate succeeds or */
/* maxiter is passed; then the diagonal fallback of _cholesky_decomp.         */
/* The eigen-decomposition (dsyevr in the reference) is a cyclic Jacobi with */
/* the round-robin pair order: each round rotates d/2 disjoint pairs at once */
/* (the rotations of disjoint pairs commute), d-1 rounds a sweep, the        */
/* oracle's stopping rule (off-diagonal mass <= 1e-30 of the diagonal's).    */
/* The Cholesky test is right-looking over the threads with the same         */
/* operations in the same order as the serial one (bit-identical).           */
/* ------------------------------------------------------------------------ */

#include "ncg_jacobi.cuh"

/* upper Cholesky of S in place, right-looking over the threads; returns
 * 0 or the failing column + 1 (same value in every thread) */
__device__ int
_npd_chol (double (*S)[NPD_LD], int d)
{
  const int tid = threadIdx.x;

  for (int j = 0; j < d; j++)
  {
    const double ajj = S[j][j];

    if (!(ajj > 0.0))
    {
      __syncthreads ();

      return j + 1;
    }

    const double ujj = __dsqrt_rn (ajj);

    for (int i = j + 1 + tid; i < d; i += NPD_THREADS)
      S[j][i] = __ddiv_rn (S[j][i], ujj);

    __syncthreads ();

    if (tid == 0)
      S[j][j] = ujj;

    const int w = d - j - 1;

    for (int e = tid; e < w * w; e += NPD_THREADS)
    {
      const int r = j + 1 + e / w, c = j + 1 + e % w;

      if (c >= r)
        S[r][c] = __dsub_rn (S[r][c], __dmul_rn (S[j][r], S[j][c]));
    }

    __syncthreads ();
  }

  return 0;
}

__global__ void __launch_bounds__ (NPD_THREADS)
_nearpd_kernel (double *M, int count, const int32_t *ids, int d, int maxiter, int32_t *flag,
                ncg_prep_status_t *st)
{
  __shared__ double Y[NCG_DMAX][NPD_LD];    /* the iterate                  */
  __shared__ double R[NCG_DMAX][NPD_LD];    /* its copy / Cholesky work     */
  __shared__ double DS[NCG_DMAX][NPD_LD];   /* Dykstra correction           */
  __shared__ double V[NCG_DMAX][NPD_LD];    /* eigenvectors (columns)       */
  __shared__ double diag[NCG_DMAX], eva[NCG_DMAX], red[NPD_THREADS / 32];
  __shared__ double2 cs[NCG_DMAX / 2];
  __shared__ int perm[NCG_DMAX];
  __shared__ double s_minpos;

  const int t   = blockIdx.x;
  const int tid = threadIdx.x;

  if (t >= count)
    return;

  const int i = ids ? ids[t] : t;
  double *A   = M + (size_t) i * d * d;   /* covariance in, factor out */
  int ret     = 0;

  for (int e = tid; e < d * d; e += NPD_THREADS)
  {
    Y[e / d][e % d]  = A[e];
    DS[e / d][e % d] = 0.0;
  }

  __syncthreads ();

  if (tid < d)
    diag[tid] = Y[tid][tid];

  for (int iter = 0;; iter++)
  {
    /* Y -= D_S and R = Y (kept for D_S); Y is then taken apart by Jacobi */
    for (int e = tid; e < d * d; e += NPD_THREADS)
    {
      const int r = e / d, c = e % d;
      const double y = Y[r][c] - DS[r][c];

      Y[r][c] = y;
      R[r][c] = y;
    }

    __syncthreads ();

    _npd_jacobi (Y, V, d, eva, cs, red);

    /* eigenvalues ascending (the oracle's insertion sort), floor of the
     * negative ones at min_pos_ev * DBL_EPSILON */
    if (tid == 0)
    {
      double mp = CUDART_INF;

      for (int k = 0; k < d; k++)
      {
        perm[k] = k;

        if (eva[k] > 0.0)
          mp = fmin (eva[k], mp);
      }

      for (int p = 1; p < d; p++)
      {
        const int cur = perm[p];
        int q         = p - 1;

        while (q >= 0 && eva[perm[q]] > eva[cur])
        {
          perm[q + 1] = perm[q];
          q--;
        }

        perm[q + 1] = cur;
      }

      s_minpos = mp;
    }

    __syncthreads ();

    if (tid < d)
    {
      const double ev = eva[tid];

      eva[tid] = sqrt ((ev < 0.0) ? s_minpos * 2.220446049250313080847e-16 : ev);
    }

    __syncthreads ();

    /* Y = sum_k (s_k v_k)(s_k v_k)^T in ascending eigenvalue order, then
     * D_S = Y - R and the diagonal restored */
    for (int e = tid; e < d * d; e += NPD_THREADS)
    {
      const int r = e / d, c = e % d;

      if (c < r)
        continue;

      double sum = 0.0;

      for (int k = 0; k < d; k++)
      {
        const int pk  = perm[k];
        const double sk = eva[pk];

        sum += (V[r][pk] * sk) * (V[c][pk] * sk);
      }

      DS[r][c] = sum - R[r][c];
      DS[c][r] = sum - R[c][r];
      Y[r][c]  = (r == c) ? diag[r] : sum;
      Y[c][r]  = (r == c) ? diag[r] : sum;
    }

    __syncthreads ();

    for (int e = tid; e < d * d; e += NPD_THREADS)
      R[e / d][e % d] = Y[e / d][e % d];

    __syncthreads ();

    if ((ret = _npd_chol (R, d)) == 0)
      break;

    if (iter > maxiter)
      break;
  }

  if (ret != 0)
  {
    /* diagonal fallback */
    for (int e = tid; e < d * d; e += NPD_THREADS)
      R[e / d][e % d] = (e / d == e % d) ? diag[e / d] : 0.0;

    __syncthreads ();

    if (_npd_chol (R, d) != 0 && tid == 0)
    {
      atomicAdd (&st->n_fail, 1);
      flag[i] = 2;
    }
  }

  __syncthreads ();

  for (int e = tid; e < d * d; e += NPD_THREADS)
  {
    const int r = e / d, c = e % d;

    A[e] = (c >= r) ? R[r][c] : 0.0;
  }

  if (tid == 0)
  {
    atomicAdd (&st->n_fallback, 1);

    if (flag[i] != 2)
      flag[i] = 0;
  }
}

extern "C" cudaError_t
ncg_launch_nearpd (double *cov_then_U, int count, const int32_t *ids, int d, int maxiter, int32_t *flag,
                   ncg_prep_status_t *st, cudaStream_t s)
{
  if (count <= 0)
    return cudaSuccess;

  if (d > NCG_DMAX)
    return cudaErrorInvalidValue;

  _nearpd_kernel<<<count, NPD_THREADS, 0, s>>> (cov_then_U, count, ids, d, maxiter, flag, st);

  return cudaGetLastError ();
}

/* ids of the flagged factors (order irrelevant) */
__global__ void
_compact_flags_kernel (const int32_t *flag, int n, int32_t *ids, int32_t *count)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;

  if (i < n && flag[i] == 1)
    ids[atomicAdd (count, 1)] = i;
}

extern "C" cudaError_t
ncg_launch_compact_flags (const int32_t *flag, int n, int32_t *ids, int32_t *count, cudaStream_t s)
{
  _compact_flags_kernel<<<(n + 255) / 256, 256, 0, s>>> (flag, n, ids, count);

  return cudaGetLastError ();
}

/* ------------------------------------------------------------------------ */
/* lnnorm_i and the FP64 eval operand: centre (dp) + U_i^{-T}/h packed lower  */
/* by rows (dp(dp+1)/2), zero padded past d.  One warp per kernel; lane c    */
/* computes column c of W = (U_i^T)^{-1}.                                    */
/* ------------------------------------------------------------------------ */

#define FIN_WARPS 2

__global__ void __launch_bounds__ (FIN_WARPS * 32)
_vkde_finish_kernel (const double *__restrict__ X, const double *__restrict__ Ui, const int32_t *flag,
                     int n, int d, int kernel, double nu, double inv_href, double *__restrict__ lnnorm,
                     double *__restrict__ pack)
{
  __shared__ double sU[FIN_WARPS][NCG_DMAX * NCG_DMAX];
  __shared__ double sW[FIN_WARPS][NCG_DMAX * NCG_DMAX];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int dp   = ncg_pad_dim (d);
  const int P    = dp * (dp + 1) / 2;
  const int S    = dp + P;

  for (int i = blockIdx.x * FIN_WARPS + w; i < n; i += gridDim.x * FIN_WARPS)
  {
    const double *U = Ui + (size_t) i * d * d;
    double *pk      = pack + (size_t) i * S;

    for (int e = lane; e < d * d; e += 32)
      sU[w][e] = U[e];

    __syncwarp ();

    if (lane < d)
    {
      const int c = lane;

      sW[w][c * d + c] = 1.0 / sU[w][c * d + c];

      for (int r = c + 1; r < d; r++)
      {
        double s = 0.0;

        for (int m = c; m < r; m++)
          s += sU[w][m * d + r] * sW[w][m * d + c];

        sW[w][r * d + c] = -s / sU[w][r * d + r];
      }
    }

    __syncwarp ();

    for (int e = lane; e < dp; e += 32)
      pk[e] = (e < d) ? X[(size_t) i * d + e] : 0.0;

    for (int e = lane; e < P; e += 32)
    {
      /* e -> (r, c), c <= r, packed by rows */
      int r = (int) ((sqrt (8.0 * e + 1.0) - 1.0) * 0.5);

      while (r * (r + 1) / 2 > e)
        r--;

      while ((r + 1) * (r + 2) / 2 <= e)
        r++;

      const int c = e - r * (r + 1) / 2;

      pk[dp + e] = (r < d && c < d) ? sW[w][r * d + c] * inv_href : 0.0;
    }

    if (lane == 0)
      lnnorm[i] = _kernel_lnnorm (kernel, nu, d, _chol_lndet (sU[w], d, d));

    __syncwarp ();
  }
}

extern "C" cudaError_t
ncg_launch_vkde_finish (const double *X, double *Ui, const int32_t *flag, int n, int d, int kernel,
                        double nu, double href, double *lnnorm, double *pack64, cudaStream_t s)
{
  int grid = (n + FIN_WARPS - 1) / FIN_WARPS;

  if (grid > 152 * 32)
    grid = 152 * 32;

  _vkde_finish_kernel<<<grid, FIN_WARPS * 32, 0, s>>> (X, Ui, flag, n, d, kernel, nu, 1.0 / href, lnnorm,
                                                        pack64);

  return cudaGetLastError ();
}

/* KDE operand: whitened centres / h (dp), and Vg = U^{-T}/h packed lower for
 * whitening the evaluation points. */
__global__ void
_kde_finish_kernel (const double *__restrict__ Y, const double *__restrict__ U, int n, int d,
                    double inv_href, double *__restrict__ pack, double *__restrict__ Vg)
{
  const int dp = ncg_pad_dim (d);
  const int i  = blockIdx.x * blockDim.x + threadIdx.x;

  if (i < n)
    for (int e = 0; e < dp; e++)
      pack[(size_t) i * dp + e] = (e < d) ? Y[(size_t) i * d + e] * inv_href : 0.0;

  if (blockIdx.x == 0 && threadIdx.x == 0)
  {
    double W[NCG_DMAX * NCG_DMAX];

    for (int c = 0; c < d; c++)
    {
      W[c * d + c] = 1.0 / U[c * d + c];

      for (int r = c + 1; r < d; r++)
      {
        double s = 0.0;

        for (int m = c; m < r; m++)
          s += U[m * d + r] * W[m * d + c];

        W[r * d + c] = -s / U[r * d + r];
      }
    }

    int e = 0;

    for (int r = 0; r < dp; r++)
      for (int c = 0; c <= r; c++)
        Vg[e++] = (r < d && c < d) ? W[r * d + c] * inv_href : 0.0;
  }
}

extern "C" cudaError_t
ncg_launch_kde_finish (const double *Y, const double *U, int n, int d, double href, double *pack64,
                       double *Vg, cudaStream_t s)
{
  _kde_finish_kernel<<<(n + 127) / 128, 128, 0, s>>> (Y, U, n, d, 1.0 / href, pack64, Vg);

  return cudaGetLastError ();
}

/* mean of the centres, one thread per coordinate (the anchor of the mixed form) */
__global__ void
_mean_kernel (const double *__restrict__ X, int n, int d, double *__restrict__ mu)
{
  const int c = threadIdx.x;

  if (c >= d)
    return;

  double s = 0.0;

  for (int i = 0; i < n; i++)
    s += X[(size_t) i * d + c];

  mu[c] = s / n;
}

extern "C" cudaError_t
ncg_launch_mean (const double *X, int n, int d, double *mu, cudaStream_t s)
{
  _mean_kernel<<<1, 32, 0, s>>> (X, n, d, mu);

  return cudaGetLastError ();
}

/* Vg = scale * U^{-T}, packed lower by rows with dp padding (the global
 * whitening of the evaluation points) */
__global__ void
_global_vg_kernel (const double *__restrict__ U, int d, double scale, double *__restrict__ Vg)
{
  if (blockIdx.x != 0 || threadIdx.x != 0)
    return;

  const int dp = ncg_pad_dim (d);
  double W[NCG_DMAX * NCG_DMAX];

  for (int c = 0; c < d; c++)
  {
    W[c * d + c] = 1.0 / U[c * d + c];

    for (int r = c + 1; r < d; r++)
    {
      double s = 0.0;

      for (int m = c; m < r; m++)
        s += U[m * d + r] * W[m * d + c];

      W[r * d + c] = -s / U[r * d + r];
    }
  }

  int e = 0;

  for (int r = 0; r < dp; r++)
    for (int c = 0; c <= r; c++)
      Vg[e++] = (r < d && c < d) ? W[r * d + c] * scale : 0.0;
}

extern "C" cudaError_t
ncg_launch_global_vg (const double *U, int d, double scale, double *Vg, cudaStream_t s)
{
  _global_vg_kernel<<<1, 32, 0, s>>> (U, d, scale, Vg);

  return cudaGetLastError ();
}

/* c_i = ln w_i - lnnorm_i (VKDE) or ln w_i (KDE); marks wcum stale */
__global__ void
_weights_c_kernel (const double *w, const double *lnnorm, int n, int kind, double *c)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;

  if (i < n)
    c[i] = (kind == NCG_VKDE) ? log (w[i]) - lnnorm[i] : log (w[i]);
}

extern "C" cudaError_t
ncg_launch_weights_c (const double *w, const double *lnnorm, int n, int kind, double *c,
                      double *wcum_dirty, cudaStream_t s)
{
  (void) wcum_dirty;
  _weights_c_kernel<<<(n + 255) / 256, 256, 0, s>>> (w, lnnorm, n, kind, c);

  return cudaGetLastError ();
}

__global__ void
_fill_kernel (double *p, double v, int64_t n)
{
  for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x)
    p[i] = v;
}

extern "C" cudaError_t
ncg_launch_fill (double *p, double v, int64_t n, cudaStream_t s)
{
  int64_t g = (n + 255) / 256;

  if (g > 152 * 8)
    g = 152 * 8;

  if (g < 1)
    g = 1;

  _fill_kernel<<<(int) g, 256, 0, s>>> (p, v, n);

  return cudaGetLastError ();
}
