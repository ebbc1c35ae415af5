/*
 * ncg_syrk_tc.cu -- symmetric rank-K products C (+|-)= A^T A on the tcgen05
 * tensor cores, TF32x3 split products with FP32 accumulation: the mixed NNLS
 * builds its FP32 A^T A with it and its FP32 blocked Cholesky takes its
 * trailing updates from it (ncm_nnls.c solves these normal equations with a
 * dense FP64 factorisation; here the factor is only the preconditioner of an
 * FP64 conjugate-gradient refinement, so FP32-level accuracy is enough).
 *
 * Operands.  A is K x nn (rows are the contraction index).  A pack of it holds,
 * for each 128-column tile t and each 32-row K-chunk c, a 32 KB block at
 * ((t * nkc) + c) * 32 KB: the TF32 hi part of the 128 x 32 sub-matrix in the
 * K-major core-matrix layout of ncg_tc_ptx.cuh (LBO 2048), then the lo part
 * (a - hi, rounded to TF32).  The same pack serves as the A and the B operand
 * (the product is symmetric).  Rows of a tile past nn may hold anything: they
 * only reach outputs past nn, which are not stored.
 *
 * Kernel.  One output tile is 128 x 128 (upper tiles ti <= tj only); per
 * K-chunk the MMA warp issues 4 k-steps x 3 products (hi.hi, hi.lo, lo.hi) of
 * tcgen05.mma.kind::tf32 M=128 N=128 K=8 into a TMEM accumulator.  Persistent
 * CTAs, one per SM: warp 0 copies the two 32 KB operand blocks of a K-chunk
 * with the bulk-copy engine into one of two 64 KB stages, warp 1 allocates
 * TMEM (two 128-column accumulators) and issues the MMAs, warps 2-9 are two
 * epilogue warpgroups, warpgroup e taking the CTA's tiles of parity e: each
 * warp reads its 32 TMEM lanes (rows), transposes them 32 x 32 at a time
 * through shared memory and updates C row by row with coalesced accesses,
 * only the elements with i <= j inside the nn x nn block.  Every mbarrier
 * wait is bounded; on timeout the CTA sets *err = -1, drains its copies,
 * waits for its MMAs and frees TMEM.  A launch that finds *err != 0 (the
 * Cholesky's info word: a failed or timed-out factorisation) does nothing.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "ncg_internal.h"
#include "ncg_tc_ptx.cuh"
#include "ncg_syrk_tc.cuh"

#define SK_STAGES 2
#define SK_EPI_WARP0 2
#define SK_EPI_WARPS 8
#define SK_THREADS ((SK_EPI_WARP0 + SK_EPI_WARPS) * 32)

struct SkSmem
{
  uint8_t stage[SK_STAGES][SK_STAGE];
  float tr[SK_EPI_WARPS][32][33];
  uint64_t full[SK_STAGES], empty[SK_STAGES], t_full[2], t_empty[2], done;
  uint32_t tmem_base;
  int err;
};

#define SK_SMEM_BYTES (sizeof (SkSmem) + 1024)

/* D(f32) (+)= A(tf32, K-major, 128 x 8) . B(tf32, K-major, 128 x 8)^T */
__device__ __forceinline__ void
_mma_tf32_128 (uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t) (SK_T >> 3) << 17) |
                         ((uint32_t) (SK_T >> 4) << 24);

  asm volatile ("{\n\t.reg .pred p;\n\t"
                "setp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
                ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
                : "memory");
}

__device__ __forceinline__ void
_tile_of (int u, int T_, int *ti, int *tj)
{
  int b = u, i = 0;

  while (b >= T_ - i)
  {
    b -= T_ - i;
    i++;
  }

  *ti = i;
  *tj = i + b;
}

/* pack rows [r0, r1) x columns [c0, c0 + nn) of A (FP64, leading dimension
 * lda): one CTA per (tile, chunk), thread = (row, quad pair) */
__global__ void __launch_bounds__ (256)
_pack_f64_kernel (const double *__restrict__ A, int lda, int r0, int r1, int c0, int nn, int nkc,
                  float *__restrict__ pk)
{
  const int t = blockIdx.x / nkc, c = blockIdx.x % nkc;
  const int row = threadIdx.x & 127, q0 = threadIdx.x >> 7;
  const int col = t * SK_T + row;
  float *blk    = pk + (size_t) blockIdx.x * (SK_BLOCK / 4);

#pragma unroll
  for (int m = 0; m < 4; m++)
  {
    const int q = q0 + 2 * m, k = r0 + c * SK_KC + 4 * q;
    double v[4];

#pragma unroll
    for (int e = 0; e < 4; e++)
      v[e] = (col < nn && k + e < r1) ? A[(size_t) (k + e) * lda + c0 + col] : 0.0;

    _put_split4 (blk, row, 4 * q, v[0], v[1], v[2], v[3]);
  }
}

/* mode: 0 C = A^T A, 1 C -= A^T A, 2 C += A^T A (upper, i <= j) */
__global__ void __launch_bounds__ (SK_THREADS, 1)
_syrk_tc_kernel (const uint8_t *__restrict__ pk, int nkc, int nn, float *__restrict__ C, int ldc, int mode,
                 int *__restrict__ err_out)
{
  extern __shared__ uint8_t smem_raw[];
  SkSmem &sm = *(SkSmem *) (((uintptr_t) smem_raw + 1023) & ~(uintptr_t) 1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int T_ = (nn + SK_T - 1) / SK_T, ntiles = T_ * (T_ + 1) / 2;
  volatile int *err = &sm.err;
  /* a factorisation that already failed (or timed out) needs no more updates */
  const bool skip = *(volatile int *) err_out != 0;

  if (threadIdx.x == 0)
  {
    sm.err = skip ? 1 : 0;

    for (int s = 0; s < SK_STAGES; s++)
    {
      _mbar_init (&sm.full[s], 1);
      _mbar_init (&sm.empty[s], 1);
    }

    for (int b = 0; b < 2; b++)
    {
      _mbar_init (&sm.t_full[b], 1);
      _mbar_init (&sm.t_empty[b], 4);
    }

    _mbar_init (&sm.done, 1);
    asm volatile ("fence.mbarrier_init.release.cluster;" ::: "memory");
  }

  if (warp == 1)
  {
    asm volatile ("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                  ::"r"(_smem_u32 (&sm.tmem_base)), "r"(2 * SK_T)
                  : "memory");
    asm volatile ("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }

  _tc_fence_before ();
  __syncthreads ();
  _tc_fence_after ();

  const uint32_t tmem = sm.tmem_base;

  if (warp == 0)
  {
    /* ---------------- producer ---------------- */
    if (lane == 0)
    {
      int stage = 0;
      uint32_t phase = 0;
      int armed[SK_STAGES];

      for (int s = 0; s < SK_STAGES; s++)
        armed[s] = -1;

      for (int u = blockIdx.x; u < ntiles && !*err; u += gridDim.x)
      {
        int ti, tj;

        _tile_of (u, T_, &ti, &tj);

        for (int c = 0; c < nkc; c++)
        {
          if (!_mbar_wait (&sm.empty[stage], phase ^ 1, err))
            break;

          _mbar_arrive_tx (&sm.full[stage], SK_STAGE);
          _bulk_g2s (sm.stage[stage], pk + ((size_t) ti * nkc + c) * SK_BLOCK, SK_BLOCK, &sm.full[stage]);
          _bulk_g2s (sm.stage[stage] + SK_BLOCK, pk + ((size_t) tj * nkc + c) * SK_BLOCK, SK_BLOCK, &sm.full[stage]);
          armed[stage] = (int) phase;

          if (++stage == SK_STAGES)
          {
            stage = 0;
            phase ^= 1;
          }
        }
      }

      for (int s = 0; s < SK_STAGES; s++)
        if (armed[s] >= 0)
          _mbar_wait (&sm.full[s], (uint32_t) armed[s], err, false);
    }
  }
  else if (warp == 1)
  {
    /* ---------------- MMA issuer ---------------- */
    if (lane == 0)
    {
      int stage = 0, tc = 0;
      uint32_t phase = 0;

      for (int u = blockIdx.x; u < ntiles && !*err; u += gridDim.x, tc++)
      {
        const int tb = tc & 1;

        if (!_mbar_wait (&sm.t_empty[tb], ((tc >> 1) & 1) ^ 1, err))
          break;

        _tc_fence_after ();

        const uint32_t d = tmem + (uint32_t) (tb * SK_T);
        bool ok = true;

        for (int c = 0; c < nkc; c++)
        {
          if (!_mbar_wait (&sm.full[stage], phase, err))
          {
            ok = false;
            break;
          }

          _tc_fence_after ();

          const uint8_t *Ah = sm.stage[stage], *Al = Ah + SK_HALF, *Bh = Ah + SK_BLOCK, *Bl = Bh + SK_HALF;

#pragma unroll
          for (int ks = 0; ks < SK_KC / 8; ks++)
          {
            const uint32_t o = (uint32_t) ks * 2 * SK_LBO;

            _mma_tf32_128 (d, _sdesc (Ah + o, SK_LBO), _sdesc (Bh + o, SK_LBO), (c > 0 || ks > 0) ? 1u : 0u);
            _mma_tf32_128 (d, _sdesc (Ah + o, SK_LBO), _sdesc (Bl + o, SK_LBO), 1u);
            _mma_tf32_128 (d, _sdesc (Al + o, SK_LBO), _sdesc (Bh + o, SK_LBO), 1u);
          }

          _mma_commit (&sm.empty[stage]);

          if (++stage == SK_STAGES)
          {
            stage = 0;
            phase ^= 1;
          }
        }

        if (!ok)
          break;

        _mma_commit (&sm.t_full[tb]);
      }

      /* every MMA this thread issued completes before TMEM is freed */
      _mma_commit (&sm.done);
      _mbar_wait (&sm.done, 0, err, false);
    }
  }
  else
  {
    /* ---------------- epilogue warpgroups ---------------- */
    const int ew = warp - SK_EPI_WARP0, e = ew >> 2;
    const int q  = warp & 3;   /* TMEM lane quarter (hardware: warp id mod 4) */
    const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16) + (uint32_t) (e * SK_T);
    float (*tr)[33] = sm.tr[ew];
    int k = e;

    for (int u = blockIdx.x + e * gridDim.x; u < ntiles && !*err; u += 2 * gridDim.x, k += 2)
    {
      int ti, tj;

      _tile_of (u, T_, &ti, &tj);

      const int i0 = ti * SK_T + q * 32, j0 = tj * SK_T;

      /* C element (i0 + r, column of block b = 32-column slice b of the tile) */
#define SK_CJ(b_) (j0 + (b_) * 32 + lane)
#define SK_IN(r_, j_) (i0 + (r_) < nn && (j_) < nn && (j_) >= i0 + (r_))

      /* the C values of slice b are loaded one slice ahead (the first before
       * the accumulator is ready), so their latency overlaps the TMEM reads,
       * the transposes and the stores of the previous slice */
      float cv[32];

      {
        const int j = SK_CJ (0);

#pragma unroll
        for (int r = 0; r < 32; r++)
          cv[r] = (mode != 0 && SK_IN (r, j)) ? C[(size_t) (i0 + r) * ldc + j] : 0.0f;
      }

      const bool got = _mbar_wait (&sm.t_full[e], (k >> 1) & 1, err);

      /* the TMEM loads below are warp-collective: agree before issuing them */
      if (!__all_sync (0xffffffffu, got))
        break;

      _tc_fence_after ();

      for (int h = 0; h < 2; h++)
      {
        float v[64];

        _tmem_ld64 (lane_base + (uint32_t) (h * 64), lane_base + (uint32_t) (h * 64 + 32), v);

        if (h == 1)
        {
          _tc_fence_before ();
          __syncwarp ();

          if (lane == 0)
            _mbar_arrive (&sm.t_empty[e]);
        }

#pragma unroll
        for (int sb = 0; sb < 2; sb++)
        {
          const int bl = h * 2 + sb, j = SK_CJ (bl);
          float nv[32];

#pragma unroll
          for (int cc = 0; cc < 32; cc++)
            tr[lane][cc] = v[sb * 32 + cc];

          __syncwarp ();

#pragma unroll
          for (int r = 0; r < 32; r++)
          {
            const float t = tr[r][lane];

            nv[r] = (mode == 0) ? t : ((mode == 1) ? cv[r] - t : cv[r] + t);
          }

          __syncwarp ();

          if (bl < 3)
          {
            const int jn = SK_CJ (bl + 1);

#pragma unroll
            for (int r = 0; r < 32; r++)
              cv[r] = (mode != 0 && SK_IN (r, jn)) ? C[(size_t) (i0 + r) * ldc + jn] : 0.0f;
          }

#pragma unroll
          for (int r = 0; r < 32; r++)
            if (SK_IN (r, j))
              C[(size_t) (i0 + r) * ldc + j] = nv[r];
        }
      }

#undef SK_IN
#undef SK_CJ
    }
  }

  _tc_fence_before ();
  __syncthreads ();

  if (warp == 1)
  {
    _tc_fence_after ();
    asm volatile ("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * SK_T) : "memory");
  }

  if (threadIdx.x == 0 && sm.err && !skip)
    atomicExch (err_out, -1);
}

/* ------------------------------------------------------------------- host side */

/* SM count of the current device and the kernel's shared-memory opt-in there
 * (once per device, under the shared lock of ncg_raise_smem_limit: serving
 * workers call in parallel, and no launch may precede the opt-in) */
static cudaError_t
_sk_grid (int *nsm)
{
  static int limit[NCG_MAX_DEVICES];
  int dev = 0;
  cudaError_t e = cudaGetDevice (&dev);

  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute (nsm, cudaDevAttrMultiProcessorCount, dev);

  if (e == cudaSuccess)
    e = ncg_raise_smem_limit ((const void *) _syrk_tc_kernel, SK_SMEM_BYTES, limit);

  return e;
}

extern "C" size_t
ncg_syrk_tc_pack_bytes (int nn, int K)
{
  const size_t T_ = (size_t) ((nn + SK_T - 1) / SK_T), nkc = (size_t) ((K + SK_KC - 1) / SK_KC);

  return T_ * nkc * SK_BLOCK;
}

extern "C" cudaError_t
ncg_launch_syrk_tc (const void *pk, int K, int nn, float *C, int ldc, int mode, int *err, cudaStream_t s)
{
  if (nn <= 0 || K <= 0)
    return cudaSuccess;

  int nsm = 0;
  cudaError_t e    = _sk_grid (&nsm);

  if (e != cudaSuccess)
    return e;

  const int T_     = (nn + SK_T - 1) / SK_T;
  const int ntiles = T_ * (T_ + 1) / 2;
  const int grid   = (ntiles < nsm) ? ntiles : nsm;

  _syrk_tc_kernel<<<grid, SK_THREADS, SK_SMEM_BYTES, s>>> ((const uint8_t *) pk, (K + SK_KC - 1) / SK_KC, nn, C,
                                                           ldc, mode, err);

  return cudaGetLastError ();
}

/* C = A^T A over the ncols x ncols upper triangle (A FP64, nrows x ncols,
 * row-major), in K slabs that fit the pack scratch of `cap` bytes; the first
 * slab writes C, the others add to it */
extern "C" cudaError_t
ncg_launch_syrk_upper_tc_f64 (const double *A, int nrows, int ncols, float *C, void *scratch, size_t cap, int *err,
                              cudaStream_t s)
{
  const size_t per_chunk = (size_t) ((ncols + SK_T - 1) / SK_T) * SK_BLOCK;
  int kslab              = (int) (cap / per_chunk) * SK_KC;

  if (kslab <= 0)
    return cudaErrorInvalidValue;

  if (kslab > nrows)
    kslab = nrows;

  for (int r0 = 0; r0 < nrows; r0 += kslab)
  {
    const int r1  = (r0 + kslab < nrows) ? r0 + kslab : nrows;
    const int nkc = (r1 - r0 + SK_KC - 1) / SK_KC;
    const int T_  = (ncols + SK_T - 1) / SK_T;

    _pack_f64_kernel<<<T_ * nkc, 256, 0, s>>> (A, ncols, r0, r1, 0, ncols, nkc, (float *) scratch);

    cudaError_t e = ncg_launch_syrk_tc (scratch, r1 - r0, ncols, C, ncols, (r0 == 0) ? 0 : 2, err, s);

    if (e != cudaSuccess)
      return e;
  }

  return cudaGetLastError ();
}
