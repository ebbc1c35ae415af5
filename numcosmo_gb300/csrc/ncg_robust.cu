/*
 * ncg_robust.cu -- the robust covariance types of NcmStatsDistKDE/VKDE
 * (cov-type ROBUST_DIAG and ROBUST): ncm_stats_vec_compute_cov_robust_diag
 * and ncm_stats_vec_compute_cov_robust_ogk
 * (numcosmo/ncm/stats/ncm_stats_vec.c:1833-1884, 1898-2077), used for the
 * global covariance (ncm_stats_dist_kde.c:423-440) and for each VKDE kernel's
 * neighbourhood (ncm_stats_dist_vkde.c:467-472).
 *
 * Both rest on the Qn scale estimator (GSL gsl_stats_Qn_from_sorted_data;
 * Rousseeuw & Croux 1993, Croux & Rousseeuw 1992):
 *   Qn = 2.21914 d_m {|x_a - x_b|; a < b}_(k),  k = C(h, 2),  h = floor(m/2) + 1,
 * d_m the small-sample factor (tabulated for m <= 9, m/(m+1.4) for odd and
 * m/(m+3.8) for even m above).  One CTA (large sets) or one warp (the VKDE
 * neighbourhoods) computes one Qn: a bitonic sort of the m values in shared
 * memory on order-preserving integer keys, then the k-th smallest pairwise
 * difference found exactly by bisection over the bit patterns of
 * non-negative doubles (their order is the integer order):
 * count(t) = #{a < b : x_b - x_a <= t}, and the smallest t with
 * count(t) >= k is the order statistic itself (a difference of two sample
 * values, computed as the reference computes it).
 *
 * Each test fl64(x_b - x_a) <= t of the count is first decided on FP32
 * copies of the sorted values less their median c (FP64 runs at 1/64 of the
 * FP32 rate on this part): with y = fl32(x - c), b = y_a, tf = fl32(t) and
 * e = 2^-19 (|b| + tf) + 2^-100, y_b <= b + tf - e proves the test true and
 * y_b > b + tf + e proves it false (the shift, the conversions, the float
 * sums and the FP64 rounding of the difference stay below
 * 2^-21.4 (|b| + tf) + 10 2^-126 for sets with every |x - c| < 2^100); the
 * band between, and every test of a set with larger values, is decided in
 * FP64.  The decisions, and so the selected difference, are those of the
 * FP64 count.
 *
 * Sets.  A set is m rows of the sample X (n x d): the whole sample (global
 * covariance) or the k nearest neighbours of one kernel (rows from the kNN
 * list).  The OGK estimate of a set runs in five launches over all sets:
 *   1. sigma_i = Qn(x_i) per coordinate (ROBUST_DIAG ends here: cov = diag sigma^2);
 *   2. per pair i < j with y = x / sigma (times the reciprocal, as the
 *      reference scales its columns): C_ij = (Qn(y_i + y_j)^2 - Qn(y_i - y_j)^2) / 4,
 *      C_ii = 1;
 *   3. eigenvectors E of C (cyclic Jacobi in place of dsyevr), ascending;
 *   4. sigma_z_i = Qn(z_i), z_i = E_i . y (the projections on eigenvector i);
 *   5. cov = sum_i (sigma_z_i E_i o sigma)(sigma_z_i E_i o sigma)^T.
 * The covariance goes where the sample covariance would (the VKDE factor
 * slot, or the global covariance) and is factorised there.
 */
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "ncg_internal.h"
#include "ncg_jacobi.cuh"

#define RQ_TH 256

/* -------------------------------------------------------------- Qn on a CTA */

__device__ __forceinline__ double
_qn_dn (int m)
{
  /* small-sample factors for m = 2..9, Croux & Rousseeuw (1992) */
  switch (m)
  {
    case 2: return 0.399;
    case 3: return 0.994;
    case 4: return 0.512;
    case 5: return 0.844;
    case 6: return 0.611;
    case 7: return 0.857;
    case 8: return 0.669;
    case 9: return 0.872;
    default: break;
  }

  return (m & 1) ? m / (m + 1.4) : m / (m + 3.8);
}

__device__ __forceinline__ long long
_rq_block_sum (long long v, long long *red)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync (0xffffffffu, v, o);

  __syncthreads ();

  if (lane == 0)
    red[wid] = v;

  __syncthreads ();

  long long t = 0;

#pragma unroll
  for (int w = 0; w < RQ_TH / 32; w++)
    t += red[w];

  return t;
}

/* order-preserving map of a double's bits to a signed integer (its own
 * inverse): non-negative values keep their bits, negative ones flip all
 * but the sign; the orders agree for every non-NaN value (-0 < +0 only
 * separates equal values) */
__device__ __forceinline__ long long
_qn_key (long long b)
{
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

/* sort v[0..mpad) ascending (slots from m on padded with +inf) by a bitonic
 * network on the keys, by nt threads t = 0..nt-1 synchronised by sync; then
 * f[a] = fl32(v[a] - v[m/2]) (the median taken out, so that the FP32 copies
 * keep the spread of a set far from zero) */
template <typename Sync>
__device__ __forceinline__ void
_qn_sort (double *v, float *f, int m, int mpad, int t0, int nt, Sync sync)
{
  long long *kv = (long long *) v;

  for (int t = t0; t < mpad; t += nt)
    kv[t] = (t < m) ? _qn_key (kv[t]) : __double_as_longlong (CUDART_INF);

  sync ();

  for (int k = 2; k <= mpad; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1)
    {
      for (int t = t0; t < mpad; t += nt)
      {
        const int u = t ^ j;

        if (u > t)
        {
          const long long a = kv[t], b = kv[u];
          const bool up     = (t & k) == 0;

          if ((a > b) == up)
          {
            kv[t] = b;
            kv[u] = a;
          }
        }
      }

      sync ();
    }

  for (int t = t0; t < mpad; t += nt)
    kv[t] = _qn_key (kv[t]);

  sync ();

  const double c = v[m >> 1];

  for (int t = t0; t < mpad; t += nt)
    f[t] = __double2float_rn (v[t] - c);

  sync ();
}

/* the row x_a of a count and its FP32 decision band (NaN bounds: every
 * test goes to FP64) */
struct QnRow
{
  double x;
  float lo, hi;
};

__device__ __forceinline__ QnRow
_qn_row (const double *v, const float *f, int a, float tf, bool fast)
{
  QnRow r;

  r.x = v[a];

  if (fast)
  {
    const float b = f[a], c = b + tf, e = 0x1p-19f * (fabsf (b) + tf) + 0x1p-100f;

    r.lo = c - e;
    r.hi = c + e;
  }
  else
  {
    r.lo = CUDART_NAN_F;
    r.hi = CUDART_NAN_F;
  }

  return r;
}

/* fl64(v[j] - r.x) <= t, for j past the row (v[j] >= r.x) */
__device__ __forceinline__ bool
_qn_le (const double *v, const float *f, int j, const QnRow &r, double t)
{
  const float y = f[j];

  if (y <= r.lo)
    return true;

  if (y > r.hi)
    return false;

  return v[j] - r.x <= t;
}

/* the FP32 band holds for the set: every |v - v[m/2]| < 2^100 (v sorted) */
__device__ __forceinline__ bool
_qn_fast (const double *v, int m)
{
  const double c = v[m >> 1];

  return fabs (v[0] - c) < 0x1p100 && fabs (v[m - 1] - c) < 0x1p100;
}

/* Qn of v[0..m) (v holds mpad >= m slots, mpad a power of two; sorted on
 * return; f holds mpad floats); every thread gets the value */
__device__ double
_qn_cta (double *v, float *f, int m, int mpad, long long *red)
{
  const int tid = threadIdx.x;

  _qn_sort (v, f, m, mpad, tid, RQ_TH, [] () { __syncthreads (); });

  const long long h = m / 2 + 1, kk = h * (h - 1) / 2;
  const double span = v[m - 1] - v[0];
  const bool fast   = _qn_fast (v, m);
  unsigned long long lo = 0ull, hi = (unsigned long long) __double_as_longlong (span > 0.0 ? span : 0.0);

  while (lo < hi)
  {
    const unsigned long long mid = lo + ((hi - lo) >> 1);
    const double t = __longlong_as_double ((long long) mid);
    const float tf = __double2float_rn (t);
    long long c    = 0;

    for (int i = tid; i < m - 1; i += RQ_TH)
    {
      const QnRow r = _qn_row (v, f, i, tf, fast);
      int a = i, b = m - 1;

      /* largest j in [i, m) with v[j] - v[i] <= t (monotone in j) */
      while (a < b)
      {
        const int md = (a + b + 1) >> 1;

        if (_qn_le (v, f, md, r, t))
          a = md;
        else
          b = md - 1;
      }

      c += a - i;
    }

    c = _rq_block_sum (c, red);

    if (c >= kk)
      hi = mid;
    else
      lo = mid + 1;
  }

  return 2.21914 * _qn_dn (m) * __longlong_as_double ((long long) lo);
}

/* row a of set s; an index outside [0, n) is counted in *bad and replaced by 0 */
__device__ __forceinline__ int
_rq_row (const int32_t *idx, int s, int m, int a, int n, int32_t *bad)
{
  if (idx == NULL)
    return a;

  const int r = idx[(size_t) s * m + a];

  if (r < 0 || r >= n)
  {
    atomicAdd (bad, 1);

    return 0;
  }

  return r;
}

/* Qn of v[0..m) by one warp (sets of at most RQ_WARP_MPAD values): the
 * same sort and bisection as _qn_cta, each lane counting a contiguous run of
 * rows; a row's pointer a_i(t) = max{j : fl(v[j] - v[i]) <= t} is bounded by
 * its values at the bracket's ends, kept per row in bnd (L = a_i below lo,
 * H = a_i(hi), and a_i at the last step, 10 bits each), and by the previous
 * row's pointer (a_i >= a_{i-1}); a row whose bounds meet costs no test, so
 * once the bracket holds few differences a count is nearly free */
#define RQ_WARP_MPAD 1024

__device__ double
_qn_warp (double *v, float *f, uint32_t *bnd, int m, int mpad)
{
  const int lane = threadIdx.x & 31;

  _qn_sort (v, f, m, mpad, lane, 32, [] () { __syncwarp (); });

  const long long h = m / 2 + 1, kk = h * (h - 1) / 2;
  const double span = v[m - 1] - v[0];
  const bool fast   = _qn_fast (v, m);
  const int chunk = (m - 1 + 31) / 32, r0 = lane * chunk, r1 = min (m - 1, r0 + chunk);
  unsigned long long lo = 0ull, hi = (unsigned long long) __double_as_longlong (span > 0.0 ? span : 0.0);
  int pend = 0;   /* the last step's verdict, applied as each row is read: 1 L := a, 2 H := a */

  for (int i = r0; i < r1; i++)
    bnd[i] = (uint32_t) i | ((uint32_t) (m - 1) << 10);

  while (lo < hi)
  {
    const unsigned long long mid = lo + ((hi - lo) >> 1);
    const double t = __longlong_as_double ((long long) mid);
    const float tf = __double2float_rn (t);
    long long c    = 0;
    int a          = -1;

    for (int i = r0; i < r1; i++)
    {
      const uint32_t wd = bnd[i];
      int L = (int) (wd & 1023u), H = (int) ((wd >> 10) & 1023u);

      if (pend == 1)
        L = (int) (wd >> 20);
      else if (pend == 2)
        H = (int) (wd >> 20);

      int l = (a > L) ? a : L;

      if (l < H)
      {
        const QnRow r = _qn_row (v, f, i, tf, fast);

        if (i == r0)
        {
          int b = H;

          while (l < b)
          {
            const int md = (l + b + 1) >> 1;

            if (_qn_le (v, f, md, r, t))
              l = md;
            else
              b = md - 1;
          }
        }
        else
          while (l < H && _qn_le (v, f, l + 1, r, t))
            l++;
      }

      a = l;
      c += a - i;
      bnd[i] = (uint32_t) L | ((uint32_t) H << 10) | ((uint32_t) a << 20);
    }

#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      c += __shfl_xor_sync (0xffffffffu, c, o);

    if (c >= kk)
    {
      hi   = mid;
      pend = 2;
    }
    else
    {
      lo   = mid + 1;
      pend = 1;
    }
  }

  return 2.21914 * _qn_dn (m) * __longlong_as_double ((long long) lo);
}

/* ------------------------------------------------------------------ stages */

/* A worker computes one Qn task: the whole CTA (W = false, large sets) or
 * one warp with its own slice of the shared values (W = true; CTAs of 2 to
 * RQ_WPB such warps, as many as keep the most warps resident). */
#define RQ_WPB (RQ_TH / 32)

template <bool W>
struct RqWorker
{
  int id, t, nt;
  double *v;      /* the set's values (mpad slots) */
  float *f;       /* their FP32 copies, after every worker's values */
  uint32_t *bnd;  /* W: the rows' pointer bounds, after every worker's copies */

  __device__ RqWorker (double *smem, int mpad)
  {
    const int warp = threadIdx.x >> 5, wpb = W ? (int) (blockDim.x >> 5) : 1;

    id  = W ? blockIdx.x * wpb + warp : blockIdx.x;
    t   = W ? (threadIdx.x & 31) : threadIdx.x;
    nt  = W ? 32 : RQ_TH;
    v   = W ? smem + (size_t) warp * mpad : smem;
    f   = (float *) (smem + (size_t) mpad * wpb) + (W ? (size_t) warp * mpad : 0);
    bnd = W ? (uint32_t *) ((float *) (smem + (size_t) mpad * wpb) + (size_t) mpad * wpb) + (size_t) warp * mpad
            : NULL;
  }

  __device__ void sync () const
  {
    if (W)
      __syncwarp ();
    else
      __syncthreads ();
  }

  __device__ double qn (int m, int mpad, long long *red) const
  {
    return W ? _qn_warp (v, f, bnd, m, mpad) : _qn_cta (v, f, m, mpad, red);
  }
};

/* 1. sigma[s][i] = Qn of coordinate i over the set; with diag the covariance
 * row i is written (sigma^2 on the diagonal), else C's row i (1 on the
 * diagonal) */
template <bool W>
__global__ void __launch_bounds__ (RQ_TH)
_rq_sigma_kernel (const double *__restrict__ X, int n, int d, int32_t *__restrict__ bad,
                  const int32_t *__restrict__ idx, int m, int mpad, int ntasks, double *__restrict__ sig,
                  double *__restrict__ out, int diag)
{
  extern __shared__ double rq_v[];
  __shared__ long long red[RQ_TH / 32];
  const RqWorker<W> w (rq_v, mpad);

  if (w.id >= ntasks)   /* whole warps (W) or the whole CTA leave together */
    return;

  const int s = w.id / d, i = w.id % d;

  for (int a = w.t; a < m; a += w.nt)
    w.v[a] = X[(size_t) _rq_row (idx, s, m, a, n, bad) * d + i];

  w.sync ();

  const double q = w.qn (m, mpad, red);

  if (w.t == 0)
    sig[(size_t) s * d + i] = q;

  if (w.t < d)
    out[(size_t) s * d * d + i * d + w.t] = (w.t == i) ? (diag ? q * q : 1.0) : 0.0;
}

/* 2. C[s][i][j] = C[s][j][i] = (Qn(y_i + y_j)^2 - Qn(y_i - y_j)^2) / 4 */
template <bool W>
__global__ void __launch_bounds__ (RQ_TH)
_rq_pair_kernel (const double *__restrict__ X, int n, int d, int32_t *__restrict__ bad,
                 const int32_t *__restrict__ idx, int m, int mpad, int ntasks, const double *__restrict__ sig,
                 double *__restrict__ C)
{
  extern __shared__ double rq_v[];
  __shared__ long long red[RQ_TH / 32];
  const RqWorker<W> w (rq_v, mpad);

  if (w.id >= ntasks)
    return;

  const int np = d * (d - 1) / 2;
  const int s  = w.id / np;
  int p = w.id % np, i = 0;

  while (p >= d - 1 - i)
  {
    p -= d - 1 - i;
    i++;
  }

  const int j = i + 1 + p;
  const double ri = 1.0 / sig[(size_t) s * d + i], rj = 1.0 / sig[(size_t) s * d + j];
  double sq0 = 0.0, sq1 = 0.0;

  for (int pass = 0; pass < 2; pass++)
  {
    for (int a = w.t; a < m; a += w.nt)
    {
      const double *x = X + (size_t) _rq_row (idx, s, m, a, n, bad) * d;
      const double yi = x[i] * ri, yj = x[j] * rj;

      w.v[a] = pass ? yi - yj : yi + yj;
    }

    w.sync ();

    const double q = w.qn (m, mpad, red);

    if (pass)
      sq1 = q * q;
    else
      sq0 = q * q;

    w.sync ();
  }

  if (w.t == 0)
  {
    const double c = 0.25 * (sq0 - sq1);

    C[(size_t) s * d * d + i * d + j] = c;
    C[(size_t) s * d * d + j * d + i] = c;
  }
}

/* 3. E[s] rows = eigenvectors of C[s], eigenvalues ascending */
__global__ void __launch_bounds__ (NPD_THREADS)
_rq_eig_kernel (const double *__restrict__ C, int d, double *__restrict__ E)
{
  __shared__ double W[NCG_DMAX][NPD_LD];
  __shared__ double V[NCG_DMAX][NPD_LD];
  __shared__ double eva[NCG_DMAX];
  __shared__ double2 cs[NCG_DMAX / 2 + 1];
  __shared__ double red[NPD_THREADS / 32];
  __shared__ int perm[NCG_DMAX];
  const int s = blockIdx.x, tid = threadIdx.x;

  for (int e = tid; e < d * d; e += NPD_THREADS)
    W[e / d][e % d] = C[(size_t) s * d * d + e];

  __syncthreads ();

  _npd_jacobi (W, V, d, eva, cs, red);

  if (tid == 0)
  {
    for (int a = 0; a < d; a++)
      perm[a] = a;

    /* ascending eigenvalues (ties keep their index order) */
    for (int a = 1; a < d; a++)
    {
      const int pa = perm[a];
      int b        = a - 1;

      while (b >= 0 && eva[perm[b]] > eva[pa])
      {
        perm[b + 1] = perm[b];
        b--;
      }

      perm[b + 1] = pa;
    }
  }

  __syncthreads ();

  for (int e = tid; e < d * d; e += NPD_THREADS)
  {
    const int r = e / d, c = e % d;

    E[(size_t) s * d * d + e] = V[c][perm[r]];
  }
}

/* 4. sigz[s][i] = Qn of z_i = E_i . y over the set */
template <bool W>
__global__ void __launch_bounds__ (RQ_TH)
_rq_z_kernel (const double *__restrict__ X, int n, int d, int32_t *__restrict__ bad,
              const int32_t *__restrict__ idx, int m, int mpad, int ntasks, const double *__restrict__ sig,
              const double *__restrict__ E, double *__restrict__ sigz)
{
  extern __shared__ double rq_v[];
  __shared__ long long red[RQ_TH / 32];
  __shared__ double eis[RQ_WPB][NCG_DMAX], rss[RQ_WPB][NCG_DMAX];
  const RqWorker<W> w (rq_v, mpad);

  if (w.id >= ntasks)
    return;

  const int s = w.id / d, i = w.id % d, slot = W ? (threadIdx.x >> 5) : 0;
  double *ei = eis[slot], *rs = rss[slot];

  if (w.t < d)
  {
    ei[w.t] = E[(size_t) s * d * d + i * d + w.t];
    rs[w.t] = 1.0 / sig[(size_t) s * d + w.t];
  }

  w.sync ();

  for (int a = w.t; a < m; a += w.nt)
  {
    const double *x = X + (size_t) _rq_row (idx, s, m, a, n, bad) * d;
    double z        = 0.0;

    for (int r = 0; r < d; r++)
      z += ei[r] * (x[r] * rs[r]);

    w.v[a] = z;
  }

  w.sync ();

  const double q = w.qn (m, mpad, red);

  if (w.t == 0)
    sigz[(size_t) s * d + i] = q;
}

/* 5. cov[s] = V^T V with V_ij = sigz_i E_ij sig_j, full symmetric storage */
__global__ void
_rq_final_kernel (const double *__restrict__ E, int d, const double *__restrict__ sig,
                  const double *__restrict__ sigz, double *__restrict__ out)
{
  const int s = blockIdx.x;
  const double *Es = E + (size_t) s * d * d, *sg = sig + (size_t) s * d, *sz = sigz + (size_t) s * d;

  for (int e = threadIdx.x; e < d * d; e += blockDim.x)
  {
    const int p = e / d, q = e % d;
    const int a = (p <= q) ? p : q, b = (p <= q) ? q : p;
    double c = 0.0;

    for (int i = 0; i < d; i++)
      c += (sz[i] * Es[i * d + a] * sg[a]) * (sz[i] * Es[i * d + b] * sg[b]);

    out[(size_t) s * d * d + e] = c;
  }
}

/* ------------------------------------------------------------------- host */

static int
_pow2_at_least (int m)
{
  int p = 1;

  while (p < m)
    p <<= 1;

  return p;
}

extern "C" size_t
ncg_robust_work_doubles (int nsets, int d)
{
  return (size_t) nsets * (2 * (size_t) d + 2 * (size_t) d * d);
}

/* warps per CTA of a warp-per-Qn kernel: of RQ_WPB, RQ_WPB/2, .., 2 the one
 * with the most warps resident per SM under its shared memory (ties: the
 * larger CTA) */
static int
_rq_wpb (const void *fn, size_t per_warp)
{
  int best = RQ_WPB, best_warps = -1;

  for (int w = RQ_WPB; w >= 2; w >>= 1)
  {
    int nb = 0;

    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor (&nb, fn, 32 * w, per_warp * w) != cudaSuccess)
    {
      (void) cudaGetLastError ();
      continue;
    }

    if (nb * w > best_warps)
    {
      best_warps = nb * w;
      best       = w;
    }
  }

  return best;
}

template <bool W>
static cudaError_t
_robust_launch (const double *X, int n, int d, const int32_t *idx, int m, int nsets, int ogk, double *sig,
                double *sigz, double *C, double *E, double *out, int32_t *bad, cudaStream_t s)
{
  const int mpad        = _pow2_at_least (m);
  const size_t per_warp = (W ? sizeof (double) + sizeof (float) + sizeof (uint32_t) : sizeof (double) + sizeof (float)) *
                          (size_t) mpad;
  const size_t smax     = per_warp * (W ? RQ_WPB : 1);
  const int t1 = nsets * d, t2 = nsets * (d * (d - 1) / 2);
  cudaError_t e;

  /* raised whatever the size: the kernels' static arrays (up to 4 KiB) count
   * against the 48 KiB default too */
  static int lim_sigma[NCG_MAX_DEVICES], lim_pair[NCG_MAX_DEVICES], lim_z[NCG_MAX_DEVICES];

  if ((e = ncg_raise_smem_limit ((const void *) _rq_sigma_kernel<W>, smax, lim_sigma)) != cudaSuccess ||
      (e = ncg_raise_smem_limit ((const void *) _rq_pair_kernel<W>, smax, lim_pair)) != cudaSuccess ||
      (e = ncg_raise_smem_limit ((const void *) _rq_z_kernel<W>, smax, lim_z)) != cudaSuccess)
    return e;

  const int w1 = W ? _rq_wpb ((const void *) _rq_sigma_kernel<W>, per_warp) : 1;
  const int w2 = W ? _rq_wpb ((const void *) _rq_pair_kernel<W>, per_warp) : 1;
  const int w3 = W ? _rq_wpb ((const void *) _rq_z_kernel<W>, per_warp) : 1;

  _rq_sigma_kernel<W><<<(t1 + w1 - 1) / w1, W ? 32 * w1 : RQ_TH, per_warp * w1, s>>> (X, n, d, bad, idx, m, mpad, t1,
                                                                                      sig, ogk ? C : out, !ogk);

  if (ogk)
  {
    if (d > 1)
      _rq_pair_kernel<W><<<(t2 + w2 - 1) / w2, W ? 32 * w2 : RQ_TH, per_warp * w2, s>>> (X, n, d, bad, idx, m, mpad,
                                                                                         t2, sig, C);

    _rq_eig_kernel<<<nsets, NPD_THREADS, 0, s>>> (C, d, E);
    _rq_z_kernel<W><<<(t1 + w3 - 1) / w3, W ? 32 * w3 : RQ_TH, per_warp * w3, s>>> (X, n, d, bad, idx, m, mpad, t1,
                                                                                    sig, E, sigz);
    _rq_final_kernel<<<nsets, 128, 0, s>>> (E, d, sig, sigz, out);
  }

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_robust_cov (const double *X, int n, int d, const int32_t *idx, int m, int nsets, int ogk,
                       double *work, double *out, int32_t *bad, cudaStream_t s)
{
  if (nsets <= 0 || m < 4 || m > NCG_ROBUST_MAX_ROWS || d < 1 || d > NCG_DMAX)
    return cudaErrorInvalidValue;

  double *sig  = work;
  double *sigz = sig + (size_t) nsets * d;
  double *C    = sigz + (size_t) nsets * d;
  double *E    = C + (size_t) nsets * d * d;

  /* a warp per Qn for small sets (the VKDE neighbourhoods), the CTA for large ones */
  if (_pow2_at_least (m) <= RQ_WARP_MPAD)
    return _robust_launch<true> (X, n, d, idx, m, nsets, ogk, sig, sigz, C, E, out, bad, s);

  return _robust_launch<false> (X, n, d, idx, m, nsets, ogk, sig, sigz, C, E, out, bad, s);
}
