/*
 * ncg_eval_tc.cu -- VKDE eval_m2lnp on the 5th-generation tensor cores
 * (tcgen05, TMEM accumulators), TF32x3 split products, FP32 log-sum-exp.
 *
 * The per-pair whitening of _ncm_stats_dist_vkde_eval_weights_m2lnp
 * (numcosmo/ncm/stats/ncm_stats_dist_vkde.c:682-723), y_i = U_i^{-T}(x - theta_i)/h,
 * is rewritten in globally whitened coordinates as y_i = W'_i x' - b_i with
 * x' = U_g^{-T}(x - mu), W'_i = U_i^{-T} U_g^T / h and b_i = W'_i theta'_i, so that
 * for a tile of 128 points and 16 kernels the products W'_i x' form ONE GEMM:
 *     D[128 points x (16 kernels x 16 coords)] = X'[128 x 16] . W'^T[16 x 256]
 * issued as tcgen05.mma.kind::tf32 (M=128, N=256, K=8) with the operands split
 * into TF32 hi + lo parts: D = Xh Wh^T + Xh Wl^T + Xl Wh^T (FP32 accumulation).
 * The epilogue reads D from TMEM (tcgen05.ld), subtracts b_i, squares and sums
 * over the 16 coordinates (chi^2 never reaches memory) and keeps an online
 * log-sum-exp per point in base 2.  Partials (max, sum) per kernel slice are
 * merged by the FP64 merge kernel of ncg_eval.cu.
 *
 * CTA roles (persistent, one CTA per SM): warp 0 copies operand tiles with the
 * bulk-copy engine (cp.async.bulk + mbarrier complete_tx), warp 1 allocates
 * TMEM and issues the MMAs, warps 4-7 and 8-11 are two epilogue warpgroups that
 * take the two TMEM accumulator buffers in turn.  Every mbarrier wait is bounded;
 * on timeout the CTA records an error flag, drains its copies and frees TMEM.
 *
 * Operand layout (K-major, no swizzle, 8x16-byte core matrices; LBO = 128 B
 * between K-adjacent core matrices, SBO = 512 B between 8-row groups):
 *   A tile  (128 points):  [hi 8 KiB][lo 8 KiB]                       16 KiB
 *   B tile  (16 kernels):  [hi 16 KiB][lo 16 KiB][consts 16 x 20 f32]  33 KiB + 1280 B
 */
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "ncg_internal.h"

#define TC_M 128
#define TC_KT 16
#define TC_DP 16
#define TC_N (TC_KT * TC_DP)
#define TC_STAGES 4
#define TC_A_MAT 8192
#define TC_A_BYTES (2 * TC_A_MAT)
#define TC_B_MAT 16384
#define TC_CONST_F 20
#define TC_B_BYTES (2 * TC_B_MAT + TC_KT * TC_CONST_F * 4)
#define TC_B_STRIDE 34816          /* TC_B_BYTES rounded up to 1 KiB */
#define TC_THREADS 384
#define TC_LBO 128
#define TC_SBO 512


#define LOG2E_F 1.4426950408889634f
#define LN2_D 0.69314718055994530942

/* ---------------------------------------------------------------- PTX helpers */

__device__ __forceinline__ uint32_t
_smem_u32 (const void *p)
{
  return (uint32_t) __cvta_generic_to_shared (p);
}

__device__ __forceinline__ void
_mbar_init (uint64_t *bar, uint32_t count)
{
  asm volatile ("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(_smem_u32 (bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void
_mbar_arrive (uint64_t *bar)
{
  asm volatile ("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(_smem_u32 (bar)) : "memory");
}

__device__ __forceinline__ void
_mbar_arrive_tx (uint64_t *bar, uint32_t bytes)
{
  asm volatile ("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(_smem_u32 (bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool
_mbar_try (uint64_t *bar, uint32_t parity)
{
  uint32_t ok;

  asm volatile ("{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.b32 %0, 1, 0, p;\n\t}"
                : "=r"(ok)
                : "r"(_smem_u32 (bar)), "r"(parity)
                : "memory");

  return ok != 0;
}

__device__ __forceinline__ uint64_t
_globaltimer (void)
{
  uint64_t t;

  asm volatile ("mov.u64 %0, %%globaltimer;" : "=l"(t));

  return t;
}

/* Bounded wait: gives up after TC_WAIT_NS of wall time (setting the CTA error
 * flag) and, with bail set, as soon as another role has raised the flag. */
#define TC_WAIT_NS 1500000000ull

__device__ __forceinline__ bool
_mbar_wait (uint64_t *bar, uint32_t parity, volatile int *err, bool bail = true)
{
  if (_mbar_try (bar, parity))
    return true;

  const uint64_t t0 = _globaltimer ();

  for (uint32_t i = 1;; i++)
  {
    if (_mbar_try (bar, parity))
      return true;

    if ((i & 63u) == 0u)
    {
      if (bail && *err)
        return false;

      if (_globaltimer () - t0 > TC_WAIT_NS)
        break;
    }
  }

  *err = 1;

  return false;
}

__device__ __forceinline__ void
_bulk_g2s (void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
  asm volatile ("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                ::"r"(_smem_u32 (dst)), "l"(src), "r"(bytes), "r"(_smem_u32 (bar))
                : "memory");
}

__device__ __forceinline__ uint64_t
_sdesc (const void *p)
{
  const uint64_t a = (uint64_t) _smem_u32 (p);

  return ((a & 0x3FFFFull) >> 4) | ((uint64_t) (TC_LBO >> 4) << 16) | ((uint64_t) (TC_SBO >> 4) << 32) |
         (1ull << 46);
}

/* D(f32) += A(tf32, K-major) x B(tf32, K-major)^T, M=128 N=256 */
__device__ __forceinline__ void
_mma_tf32 (uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t) (TC_N >> 3) << 17) |
                         ((uint32_t) (TC_M >> 4) << 24);

  asm volatile ("{\n\t.reg .pred p;\n\t"
                "setp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
                ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
                : "memory");
}

__device__ __forceinline__ void
_mma_commit (uint64_t *bar)
{
  asm volatile ("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                ::"r"(_smem_u32 (bar))
                : "memory");
}

__device__ __forceinline__ void
_tc_fence_before (void)
{
  asm volatile ("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void
_tc_fence_after (void)
{
  asm volatile ("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void
_tmem_ld32 (uint32_t taddr, float *v)
{
  uint32_t r[32];

  asm volatile ("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(taddr));
  asm volatile ("tcgen05.wait::ld.sync.aligned;" ::: "memory");

#pragma unroll
  for (int i = 0; i < 32; i++)
    v[i] = __uint_as_float (r[i]);
}

__device__ __forceinline__ float
_ex2 (float x)
{
  float y;

  asm ("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));

  return y;
}

__device__ __forceinline__ float
_lg2 (float x)
{
  float y;

  asm ("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));

  return y;
}

__device__ __forceinline__ float
_tf32 (float x)
{
  uint32_t r;

  asm ("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));

  return __uint_as_float (r);
}

/* byte offset of element (row, k) in a K-major no-swizzle tile with K = 16 */
__host__ __device__ __forceinline__ uint32_t
_cm_off (int row, int k)
{
  return (uint32_t) ((row >> 3) * TC_SBO + (k >> 2) * TC_LBO + (row & 7) * 16 + (k & 3) * 4);
}

/* ------------------------------------------------------------- operand packs */

/* A tiles: x' = Vg (x - mu) in FP64, split into TF32 hi + lo (one thread per row,
 * rows past m are zero) */
__global__ void
_build_tc_A_kernel (const double *__restrict__ Xq, int64_t m, int d, const double *__restrict__ mu,
                    const double *__restrict__ Vg, uint8_t *__restrict__ A, int64_t rows)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;

  if (j >= rows)
    return;

  double x[TC_DP], v[TC_DP];

#pragma unroll
  for (int c = 0; c < TC_DP; c++)
    x[c] = (j < m && c < d) ? Xq[j * d + c] - mu[c] : 0.0;

  int p = 0;

#pragma unroll
  for (int r = 0; r < TC_DP; r++)
  {
    double s = 0.0;

#pragma unroll
    for (int c = 0; c <= r; c++)
      s = fma (Vg[p++], x[c], s);

    v[r] = s;
  }

  uint8_t *tile = A + (j / TC_M) * (int64_t) TC_A_BYTES;
  const int row = (int) (j % TC_M);

#pragma unroll
  for (int k = 0; k < TC_DP; k++)
  {
    const float hi = _tf32 ((float) v[k]);
    const float lo = _tf32 ((float) (v[k] - (double) hi));

    *(float *) (tile + _cm_off (row, k))            = hi;
    *(float *) (tile + TC_A_MAT + _cm_off (row, k)) = lo;
  }
}

/* B tiles from the mixed float pack (theta'_hi, theta'_lo, W' packed lower, c'):
 * rows n = kk*16 + r hold prescale * W'_kk[r][:], consts hold prescale * b and
 * c2 = c' log2(e).  Padding kernels get W = 0, b = 0 and c2 = -1e30. */
__global__ void __launch_bounds__ (TC_N)
_build_tc_B_kernel (const float *__restrict__ pk, int n, int smx, float prescale, uint8_t *__restrict__ B)
{
  const int t   = blockIdx.x;
  const int row = threadIdx.x;
  const int kk  = row / TC_DP, r = row % TC_DP;
  const int i   = t * TC_KT + kk;
  uint8_t *tile = B + (size_t) t * TC_B_STRIDE;
  float *cst    = (float *) (tile + 2 * TC_B_MAT) + kk * TC_CONST_F;
  double bsum   = 0.0;

#pragma unroll
  for (int k = 0; k < TC_DP; k++)
  {
    float w = 0.0f;
    const float *src = pk + (size_t) (i < n ? i : 0) * smx;

    if (i < n && k <= r)
      w = src[2 * TC_DP + r * (r + 1) / 2 + k] * prescale;

    const float hi = _tf32 (w);
    const float lo = _tf32 (w - hi);

    /* b from the split weights the MMA sees, so y = W'(x' - theta') exactly in them */
    if (i < n && k <= r)
      bsum += ((double) hi + (double) lo) * ((double) src[k] + (double) src[TC_DP + k]);

    *(float *) (tile + _cm_off (row, k))            = hi;
    *(float *) (tile + TC_B_MAT + _cm_off (row, k)) = lo;
  }

  cst[r] = (float) bsum;

  if (r == 0)
  {
    const float *src = pk + (size_t) (i < n ? i : 0) * smx;

    cst[TC_DP]     = (i < n) ? src[2 * TC_DP + TC_DP * (TC_DP + 1) / 2] * LOG2E_F : -1.0e30f;
    cst[TC_DP + 1] = 0.0f;
    cst[TC_DP + 2] = 0.0f;
    cst[TC_DP + 3] = 0.0f;
  }
}

/* ------------------------------------------------------------------ the kernel */

struct TcParams
{
  const uint8_t *A;      /* point tiles  */
  const uint8_t *B;      /* kernel tiles */
  float2 *part;          /* [2*nslices][m] */
  int *err;              /* device error flag */
  int64_t m;
  int npt, nkt, nslices, tps;
  float kappa;           /* ST: -(nu + d)/2 */
};

struct TcSmem
{
  uint8_t A[2][TC_A_BYTES];
  uint8_t B[TC_STAGES][TC_B_STRIDE];
  uint64_t a_full[2], a_empty[2], b_full[TC_STAGES], b_empty[TC_STAGES], t_full[2], t_empty[2], done;
  uint32_t tmem_base;
  int err;
};

template <int KERN>
__global__ void __launch_bounds__ (TC_THREADS, 1)
_eval_tc_kernel (const TcParams p)
{
  extern __shared__ __align__ (1024) uint8_t tc_raw[];
  TcSmem &sm = *(TcSmem *) (((uintptr_t) tc_raw + 1023) & ~(uintptr_t) 1023);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nunits = p.npt * p.nslices;
  volatile int *err = &sm.err;

  if (threadIdx.x == 0)
  {
    sm.err = 0;

    for (int b = 0; b < 2; b++)
    {
      _mbar_init (&sm.a_full[b], 1);
      _mbar_init (&sm.a_empty[b], 1);
      _mbar_init (&sm.t_full[b], 1);
      _mbar_init (&sm.t_empty[b], 4);
    }

    for (int s = 0; s < TC_STAGES; s++)
    {
      _mbar_init (&sm.b_full[s], 1);
      _mbar_init (&sm.b_empty[s], 1 + 4);
    }

    _mbar_init (&sm.done, 1);

    asm volatile ("fence.mbarrier_init.release.cluster;" ::: "memory");
  }

  if (warp == 1)
  {
    asm volatile ("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                  ::"r"(_smem_u32 (&sm.tmem_base)), "r"(512)
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
      int stage = 0, lu = 0;
      uint32_t bphase = 0;
      int armed_b[TC_STAGES], armed_a[2];   /* parity of the last armed phase, -1 none */

      for (int s = 0; s < TC_STAGES; s++)
        armed_b[s] = -1;

      armed_a[0] = armed_a[1] = -1;

      for (int u = blockIdx.x; u < nunits && !*err; u += gridDim.x, lu++)
      {
        const int pt = u / p.nslices, sl = u % p.nslices;
        const int t0 = sl * p.tps, t1 = min (p.nkt, t0 + p.tps);
        const int ab = lu & 1;

        if (!_mbar_wait (&sm.a_empty[ab], ((lu >> 1) & 1) ^ 1, err))
          break;

        _mbar_arrive_tx (&sm.a_full[ab], TC_A_BYTES);
        _bulk_g2s (sm.A[ab], p.A + (size_t) pt * TC_A_BYTES, TC_A_BYTES, &sm.a_full[ab]);
        armed_a[ab] = (lu >> 1) & 1;

        for (int t = t0; t < t1; t++)
        {
          if (!_mbar_wait (&sm.b_empty[stage], bphase ^ 1, err))
            break;

          _mbar_arrive_tx (&sm.b_full[stage], TC_B_BYTES);
          _bulk_g2s (sm.B[stage], p.B + (size_t) t * TC_B_STRIDE, TC_B_BYTES, &sm.b_full[stage]);
          armed_b[stage] = (int) bphase;

          if (++stage == TC_STAGES)
          {
            stage  = 0;
            bphase ^= 1;
          }
        }
      }

      /* drain: every copy this thread armed must land before the CTA may exit
       * (a no-op in the normal flow, where the consumers waited on them) */
      for (int s = 0; s < TC_STAGES; s++)
        if (armed_b[s] >= 0)
          _mbar_wait (&sm.b_full[s], (uint32_t) armed_b[s], err, false);

      for (int b = 0; b < 2; b++)
        if (armed_a[b] >= 0)
          _mbar_wait (&sm.a_full[b], (uint32_t) armed_a[b], err, false);
    }
  }
  else if (warp == 1)
  {
    /* ---------------- MMA issuer ---------------- */
    if (lane == 0)
    {
      int stage = 0, lu = 0, tc = 0;
      uint32_t bphase = 0;

      for (int u = blockIdx.x; u < nunits && !*err; u += gridDim.x, lu++)
      {
        const int sl = u % p.nslices;
        const int t0 = sl * p.tps, t1 = min (p.nkt, t0 + p.tps);
        const int ab = lu & 1;

        if (!_mbar_wait (&sm.a_full[ab], (lu >> 1) & 1, err))
          break;

        const uint8_t *Ah = sm.A[ab], *Al = sm.A[ab] + TC_A_MAT;

        for (int t = t0; t < t1; t++, tc++)
        {
          const int tb = tc & 1;

          if (!_mbar_wait (&sm.b_full[stage], bphase, err))
            break;

          if (!_mbar_wait (&sm.t_empty[tb], ((tc >> 1) & 1) ^ 1, err))
            break;

          _tc_fence_after ();

          const uint8_t *Bh = sm.B[stage], *Bl = sm.B[stage] + TC_B_MAT;
          const uint32_t d  = tmem + (uint32_t) (tb * TC_N);

#pragma unroll
          for (int ks = 0; ks < 2; ks++)
          {
            _mma_tf32 (d, _sdesc (Ah + ks * 256), _sdesc (Bh + ks * 256), ks > 0);
            _mma_tf32 (d, _sdesc (Ah + ks * 256), _sdesc (Bl + ks * 256), 1);
            _mma_tf32 (d, _sdesc (Al + ks * 256), _sdesc (Bh + ks * 256), 1);
          }

          _mma_commit (&sm.t_full[tb]);
          _mma_commit (&sm.b_empty[stage]);

          if (++stage == TC_STAGES)
          {
            stage  = 0;
            bphase ^= 1;
          }
        }

        _mma_commit (&sm.a_empty[ab]);
      }

      /* every MMA this thread issued completes before TMEM is freed */
      _mma_commit (&sm.done);
      _mbar_wait (&sm.done, 0, err, false);
    }
  }
  else if (warp >= 4)
  {
    /* ---------------- epilogue warpgroups ---------------- */
    const int wg   = (warp - 4) >> 2;           /* 0 takes even tiles, 1 odd */
    const int q    = warp & 3;                  /* TMEM lane quarter          */
    const int row  = q * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
    int stage = 0, tc = 0;
    uint32_t bphase = 0;

    for (int u = blockIdx.x; u < nunits && !*err; u += gridDim.x)
    {
      const int pt = u / p.nslices, sl = u % p.nslices;
      const int t0 = sl * p.tps, t1 = min (p.nkt, t0 + p.tps);
      float m2 = -CUDART_INF_F, S = 0.0f;
      bool ok = true;

      for (int t = t0; t < t1; t++, tc++)
      {
        const int tb = tc & 1;
        const int my = (tb == wg);

        if (my)
        {
          bool got = _mbar_wait (&sm.t_full[tb], (tc >> 1) & 1, err) && _mbar_wait (&sm.b_full[stage], bphase, err);

          /* the TMEM loads below are warp-collective: agree before issuing them */
          if (!__all_sync (0xffffffffu, got))
          {
            ok = false;
            break;
          }

          _tc_fence_after ();

          const float *cst = (const float *) (sm.B[stage] + 2 * TC_B_MAT);
          float tv[TC_KT];
          float tmax = -CUDART_INF_F;

#pragma unroll
          for (int pr = 0; pr < TC_KT / 2; pr++)
          {
            float v[32];

            _tmem_ld32 (lane_base + (uint32_t) (tb * TC_N + pr * 32), v);

#pragma unroll
            for (int h = 0; h < 2; h++)
            {
              const int kk    = 2 * pr + h;
              const float *bk = cst + kk * TC_CONST_F;
              float s         = 0.0f;

#pragma unroll
              for (int r = 0; r < TC_DP; r++)
              {
                const float dl = v[h * 16 + r] - bk[r];

                s = fmaf (dl, dl, s);
              }

              const float c2 = bk[TC_DP];
              const float tt = (KERN == NCG_KERNEL_ST) ? fmaf (p.kappa, _lg2 (1.0f + s), c2) : c2 - s;

              tv[kk] = tt;
              tmax   = fmaxf (tmax, tt);
            }
          }

          _tc_fence_before ();
          __syncwarp ();

          if (lane == 0)
          {
            _mbar_arrive (&sm.t_empty[tb]);
            _mbar_arrive (&sm.b_empty[stage]);
          }

          const float mn = fmaxf (m2, tmax);
          float acc      = S * _ex2 (m2 - mn);

#pragma unroll
          for (int kk = 0; kk < TC_KT; kk++)
            acc += _ex2 (tv[kk] - mn);

          S  = acc;
          m2 = mn;
        }

        if (++stage == TC_STAGES)
        {
          stage  = 0;
          bphase ^= 1;
        }
      }

      if (!ok)
        break;

      const int64_t j = (int64_t) pt * TC_M + row;

      if (j < p.m)
        p.part[(size_t) (2 * sl + wg) * p.m + j] = make_float2 ((float) (m2 * LN2_D), S - 1.0f);
    }
  }

  _tc_fence_before ();
  __syncthreads ();

  if (warp == 1)
  {
    _tc_fence_after ();
    asm volatile ("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
  }

  if (threadIdx.x == 0 && sm.err)
    atomicExch (p.err, 1);
}

/* ------------------------------------------------------------------- host side */

static void
_tc_slicing (int npt, int nkt, int nsm, int *nslices, int *tps)
{
  long best = -1;
  int bs = 1;

  for (int s = 1; s <= nkt && s <= 64; s++)
  {
    const int tp     = (nkt + s - 1) / s;
    const int units  = npt * s;
    const long waves = (units + nsm - 1) / nsm;
    const long cost  = waves * tp;

    if (best < 0 || cost < best)
    {
      best = cost;
      bs   = s;
    }
  }

  *nslices = bs;
  *tps     = (nkt + bs - 1) / bs;
  *nslices = (nkt + *tps - 1) / *tps;
}

extern "C" int
ncg_tc_supported (int kind, int dp)
{
  return kind == NCG_VKDE && dp == TC_DP;
}

extern "C" size_t
ncg_tc_B_bytes (int n)
{
  return (size_t) ((n + TC_KT - 1) / TC_KT) * TC_B_STRIDE;
}

extern "C" size_t
ncg_tc_scratch_bytes (int64_t m, int n)
{
  int ns, tps;
  const int npt = (int) ((m + TC_M - 1) / TC_M), nkt = (n + TC_KT - 1) / TC_KT;

  _tc_slicing (npt, nkt, 152, &ns, &tps);

  /* A tiles | partials | error flag */
  return (size_t) npt * TC_A_BYTES + (size_t) 2 * ns * (size_t) m * sizeof (float2) + 256;
}

extern "C" cudaError_t
ncg_launch_build_tc_B (const float *packmx, int n, int dp, int kernel, double nu, uint8_t *B, cudaStream_t s)
{
  const int nkt       = (n + TC_KT - 1) / TC_KT;
  const int smx       = ((2 * dp + dp * (dp + 1) / 2 + 1) + 3) / 4 * 4;
  const float prescale = (kernel == NCG_KERNEL_ST) ? (float) (1.0 / sqrt (nu)) : (float) sqrt (0.5 * 1.4426950408889634);

  _build_tc_B_kernel<<<nkt, TC_N, 0, s>>> (packmx, n, smx, prescale, B);

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_eval_tc (const ncg_eval_args_t *a, const double *Xq, const uint8_t *B, const double *mu,
                    const double *Vg, void *scratch, int **err_out, int *nparts_out, float2 **part_out,
                    cudaStream_t s)
{
  const int npt = (int) ((a->m + TC_M - 1) / TC_M), nkt = (a->n + TC_KT - 1) / TC_KT;
  int ns, tps, dev, nsm;
  cudaError_t e;

  if ((e = cudaGetDevice (&dev)) != cudaSuccess)
    return e;

  if ((e = cudaDeviceGetAttribute (&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return e;

  _tc_slicing (npt, nkt, 152, &ns, &tps);

  uint8_t *A    = (uint8_t *) scratch;
  float2 *part  = (float2 *) (A + (size_t) npt * TC_A_BYTES);
  int *err      = (int *) (part + (size_t) 2 * ns * a->m);
  const int64_t rows = (int64_t) npt * TC_M;

  if ((e = cudaMemsetAsync (err, 0, sizeof (int), s)) != cudaSuccess)
    return e;

  _build_tc_A_kernel<<<(unsigned) ((rows + 127) / 128), 128, 0, s>>> (Xq, a->m, a->d, mu, Vg, A, rows);

  TcParams p;

  p.A       = A;
  p.B       = B;
  p.part    = part;
  p.err     = err;
  p.m       = a->m;
  p.npt     = npt;
  p.nkt     = nkt;
  p.nslices = ns;
  p.tps     = tps;
  p.kappa   = (float) a->kappa;

  const size_t smem = sizeof (TcSmem) + 1024;
  void (*fn) (const TcParams) = (a->kernel == NCG_KERNEL_ST) ? _eval_tc_kernel<NCG_KERNEL_ST>
                                                              : _eval_tc_kernel<NCG_KERNEL_GAUSS>;

  if ((e = cudaFuncSetAttribute (fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)) != cudaSuccess)
    return e;

  const int units = npt * ns;
  const int grid  = units < nsm ? units : nsm;

  fn<<<grid, TC_THREADS, smem, s>>> (p);

  *err_out    = err;
  *nparts_out = 2 * ns;
  *part_out   = part;

  return cudaGetLastError ();
}
