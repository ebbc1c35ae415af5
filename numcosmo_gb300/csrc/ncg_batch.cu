/*
 * ncg_batch.cu -- eval_m2lnp of many independent problems (any mix of
 * dimension, kernel count, KDE/VKDE, Gaussian/Student-t, FP64/mixed) in one
 * persistent launch.
 *
 * The grid is sized to the GPU (SMs x resident CTAs); each CTA takes work
 * items from a list with an atomic counter.  An item is one tile of
 * ncg_eval_tiles.cuh -- EV_THREADS points of one problem against one slice
 * of its kernels -- so a problem's arithmetic is the one of its one-problem
 * launch.  The CTA that finishes the last slice of a point tile (counted with
 * an atomic per tile, after a fence) merges the tile's slices in slice order
 * and writes -2 ln p; no CTA ever waits for another.
 *
 * A problem's class (tile arithmetic, padded dimension, kind, kernel) picks
 * the tile code through a switch.  The register budget of the launch is the
 * one of its largest class, so the host may split the classes over two
 * launches (dp <= 16 and dp > 16) that run as two branches of one graph.
 */
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "ncg_internal.h"
#include "ncg_eval_tiles.cuh"

template <int MIXED, int DP, int KIND>
struct BTile
{
  static constexpr int KC = MIXED ? NcgEvMx<DP, KIND>::KCB : NcgEv64<DP, KIND>::KC;
  static constexpr size_t smem = MIXED ? (size_t) NcgEvMx<DP, KIND>::KCB * NcgEvMx<DP, KIND>::S * sizeof (float)
                                       : (size_t) NcgEv64<DP, KIND>::KC * (NcgEv64<DP, KIND>::S + 1) * sizeof (double);
};

template <int MODE, int SET, int MIXED, int DP>
__host__ __device__ constexpr bool
_in_set ()
{
  return (MIXED == 0 || MODE == 1) &&
         (SET == NCG_BSET_ALL || (SET == NCG_BSET_SMALL && DP <= NCG_BSET_SPLIT_DP) ||
          (SET == NCG_BSET_LARGE && DP > NCG_BSET_SPLIT_DP));
}

template <int MIXED, int DP, int KIND, int KERN>
__device__ __forceinline__ void
_tile (const ncg_bprob_t &p, const double *__restrict__ Xq, int bx, int sy, unsigned char *smem)
{
  if constexpr (MIXED)
  {
    constexpr int KC = NcgEvMx<DP, KIND>::KCB;

    ncg_tile_evalmx<DP, KIND, KERN, KC> (p.a, Xq + p.x_off, p.packmx, p.Vg, p.mu, (float2 *) p.part, p.kper, bx, sy,
                                         (float *) smem);
  }
  else
  {
    constexpr int KC = NcgEv64<DP, KIND>::KC;
    constexpr int S  = NcgEv64<DP, KIND>::S;

    ncg_tile_eval64<DP, KIND, KERN, KC> (p.a, Xq + p.x_off, p.pack64, p.c, p.Vg, (double2 *) p.part, p.kper, bx, sy,
                                         (double *) smem, (double *) smem + KC * S);
  }
}

#define NCG_BCASE(M, DP, KIND, KERN)                           \
  case NCG_BCLS (M, DP, KIND, KERN):                           \
    if constexpr (_in_set<MODE, SET, M, DP> ())                \
      _tile<M, DP, KIND, KERN> (p, Xq, bx, sy, smem);          \
    break;
#define NCG_BCASE4(M, DP) \
  NCG_BCASE (M, DP, 0, 0) NCG_BCASE (M, DP, 0, 1) NCG_BCASE (M, DP, 1, 0) NCG_BCASE (M, DP, 1, 1)
#define NCG_BCASES(M)                                                                          \
  NCG_BCASE4 (M, 4) NCG_BCASE4 (M, 8) NCG_BCASE4 (M, 12) NCG_BCASE4 (M, 16) NCG_BCASE4 (M, 20) \
  NCG_BCASE4 (M, 24) NCG_BCASE4 (M, 28) NCG_BCASE4 (M, 32)

template <int MODE, int SET>
__device__ __forceinline__ void
_dispatch (const ncg_bprob_t &p, const double *__restrict__ Xq, int bx, int sy, unsigned char *smem)
{
  switch (p.cls)
  {
    NCG_BCASES (0)
    NCG_BCASES (1)
    default:
      break;
  }
}

/* the slices of point tile bx in slice order, then -2 (gamma + log1p(lambda)
 * - d ln h), the same expression as the one-problem merge kernel.  The pairs
 * were written by other CTAs of this launch: read them past L1 (__ldcg). */
__device__ __forceinline__ void
_merge_tile (const ncg_bprob_t &p, int bx, double *__restrict__ out)
{
  const int64_t j = (int64_t) bx * EV_THREADS + threadIdx.x;

  if (j >= p.a.m)
    return;

  const bool mixed = p.cls >= NCG_BCLS (1, 4, 0, 0);
  double G = -CUDART_INF, L = 0.0;

  for (int s = 0; s < p.ns; s++)
  {
    double ms, ls;

    if (mixed)
    {
      const float2 q = __ldcg ((const float2 *) p.part + (size_t) s * p.a.m + j);

      ms = (double) q.x;
      ls = (double) q.y;
    }
    else
    {
      const double2 q = __ldcg ((const double2 *) p.part + (size_t) s * p.a.m + j);

      ms = q.x;
      ls = q.y;
    }

    if (ms > G)
    {
      L = (L + 1.0) * exp (G - ms) + ls;
      G = ms;
    }
    else if (ms > -CUDART_INF)
    {
      L += (ls + 1.0) * exp (ms - G);
    }
  }

  const double gamma = G - p.a.final_shift + (p.dshift ? *p.dshift : 0.0);
  const double lnp   = gamma + log1p (L) - p.a.d_ln_href;

  out[p.out_off + j] = -2.0 * lnp;
}

/* MODE 0: FP64 tiles only; MODE 1: mixed and FP64 tiles (a mixed batch serves
 * a problem whose FP32 whitening is ill-conditioned with FP64 tiles) */
template <int MODE, int SET>
__global__ void __launch_bounds__ (EV_THREADS)
_batch_eval_kernel (const ncg_bprob_t *__restrict__ probs, const int2 *__restrict__ items, int nitems,
                    int32_t *counter, const double *__restrict__ Xq, double *__restrict__ out)
{
  extern __shared__ __align__ (16) unsigned char smem[];
  __shared__ ncg_bprob_t sp;
  __shared__ int s_item, s_last;
  constexpr int NW = (int) (sizeof (ncg_bprob_t) / sizeof (int));

  static_assert (sizeof (ncg_bprob_t) % sizeof (int) == 0, "descriptor copy by words");
  static_assert (NW <= EV_THREADS, "descriptor copy by one pass");

  for (;;)
  {
    __syncthreads ();

    if (threadIdx.x == 0)
      s_item = atomicAdd (counter, 1);

    __syncthreads ();

    const int it = s_item;

    if (it >= nitems)
      return;

    const int2 w = items[it];

    if (threadIdx.x < NW)
      ((int *) &sp)[threadIdx.x] = ((const int *) (probs + w.x))[threadIdx.x];

    __syncthreads ();

    const int bx = w.y % sp.bx, sy = w.y / sp.bx;

    _dispatch<MODE, SET> (sp, Xq, bx, sy, smem);

    __threadfence ();
    __syncthreads ();

    if (threadIdx.x == 0)
    {
      const int done = atomicAdd (sp.tile_cnt + bx, 1) + 1;

      s_last = (done == sp.ns);

      if (s_last)
        sp.tile_cnt[bx] = 0;
    }

    __syncthreads ();

    if (s_last)
    {
      __threadfence ();
      _merge_tile (sp, bx, out);
    }
  }
}

/* per-class tables (index NCG_BCLS) */
#define NCG_BROW(M, DP, KIND, KERN) BTile<M, DP, KIND>::KC,
#define NCG_BROW4(M, DP) NCG_BROW (M, DP, 0, 0) NCG_BROW (M, DP, 0, 1) NCG_BROW (M, DP, 1, 0) NCG_BROW (M, DP, 1, 1)
#define NCG_BROWS(M) NCG_BROW4 (M, 4) NCG_BROW4 (M, 8) NCG_BROW4 (M, 12) NCG_BROW4 (M, 16) NCG_BROW4 (M, 20) \
  NCG_BROW4 (M, 24) NCG_BROW4 (M, 28) NCG_BROW4 (M, 32)

static const int g_kc[NCG_BATCH_NCLS] = { NCG_BROWS (0) NCG_BROWS (1) };

#undef NCG_BROW
#define NCG_BROW(M, DP, KIND, KERN) BTile<M, DP, KIND>::smem,

static const size_t g_smem[NCG_BATCH_NCLS] = { NCG_BROWS (0) NCG_BROWS (1) };

extern "C" int
ncg_batch_chunk (int cls)
{
  return (cls >= 0 && cls < NCG_BATCH_NCLS) ? g_kc[cls] : 0;
}

/* the largest tile shared memory over the classes a launch may carry */
extern "C" size_t
ncg_batch_smem_bytes (int mixed, int set)
{
  size_t mx = 0;

  for (int c = 0; c < NCG_BATCH_NCLS; c++)
  {
    const int m  = c / 32;
    const int dp = ((c / 4) % 8 + 1) * 4;

    if (m > mixed)
      continue;

    if ((set == NCG_BSET_SMALL && dp > NCG_BSET_SPLIT_DP) || (set == NCG_BSET_LARGE && dp <= NCG_BSET_SPLIT_DP))
      continue;

    if (g_smem[c] > mx)
      mx = g_smem[c];
  }

  return mx;
}

typedef void (*bk_fn) (const ncg_bprob_t *, const int2 *, int, int32_t *, const double *, double *);

static bk_fn
_pick (int mixed, int set)
{
  if (mixed)
  {
    switch (set)
    {
      case NCG_BSET_SMALL: return _batch_eval_kernel<1, NCG_BSET_SMALL>;
      case NCG_BSET_LARGE: return _batch_eval_kernel<1, NCG_BSET_LARGE>;
      default:             return _batch_eval_kernel<1, NCG_BSET_ALL>;
    }
  }

  switch (set)
  {
    case NCG_BSET_SMALL: return _batch_eval_kernel<0, NCG_BSET_SMALL>;
    case NCG_BSET_LARGE: return _batch_eval_kernel<0, NCG_BSET_LARGE>;
    default:             return _batch_eval_kernel<0, NCG_BSET_ALL>;
  }
}

extern "C" int
ncg_batch_ctas_per_sm (int mixed, int set)
{
  int nb = 0;

  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor (&nb, _pick (mixed, set), EV_THREADS,
                                                     ncg_batch_smem_bytes (mixed, set)) != cudaSuccess)
    return 1;

  return nb > 0 ? nb : 1;
}

extern "C" cudaError_t
ncg_launch_batch_eval (int mixed, int set, const ncg_bprob_t *probs, const int32_t *items, int nitems,
                       int32_t *counter, const double *Xq, double *out, int grid, cudaStream_t s)
{
  if (nitems <= 0)
    return cudaSuccess;

  cudaError_t e = cudaMemsetAsync (counter, 0, sizeof (int32_t), s);

  if (e != cudaSuccess)
    return e;

  _pick (mixed, set)<<<grid, EV_THREADS, ncg_batch_smem_bytes (mixed, set), s>>> (probs, (const int2 *) items, nitems,
                                                                               counter, Xq, out);

  return cudaGetLastError ();
}
