/*
 * ncg_eval_tc.cu -- VKDE eval_m2lnp on the 5th-generation tensor cores
 * (tcgen05, TMEM accumulators), TF32x3 split products, FP32 log-sum-exp.
 *
 * The per-pair whitening of _ncm_stats_dist_vkde_eval_weights_m2lnp
 * (numcosmo/ncm/stats/ncm_stats_dist_vkde.c:682-723), y_i = U_i^{-T}(x - theta_i)/h,
 * is rewritten in globally whitened coordinates as y_i = W'_i x' - b_i with
 * x' = U_g^{-T}(x - mu), W'_i = U_i^{-T} U_g^T / h and b_i = W'_i theta'_i.  For a
 * tile of 128 points and 16 kernels, y for all pairs is ONE GEMM with the
 * subtraction folded in by a constant column: with x'' = [x', 1, 1] and
 * w''_{i,r} = [W'_i[r,:], -b_hi, -b_lo],
 *     D[128 points x (16 kernels x 16 coords)] = X''[128 x 24] . W''^T[24 x 256]
 * issued as tcgen05.mma.kind::tf32 (M=128, N=256, K=8) with the operands split
 * into TF32 hi + lo parts: D = Xh Wh^T (3 k-steps, incl. the -b column pair)
 * + Xh Wl^T + Xl Wh^T (2 k-steps each), FP32 accumulation: 7 MMAs per tile.
 * The epilogue reads y from TMEM (tcgen05.ld), squares and sums it over the 16
 * coordinates with packed FP32x2 FMAs (chi^2 never reaches memory) and keeps an
 * online log-sum-exp per point in base 2.  Partials (max, sum) per (kernel
 * slice, warpgroup) are merged by a warp-per-point FP32 reduction with an FP64
 * finish.
 *
 * CTA roles (persistent, one CTA per SM): warp 0 copies operand tiles with the
 * bulk-copy engine (cp.async.bulk + mbarrier complete_tx), warp 1 allocates
 * TMEM and issues the MMAs into a double-buffered accumulator (2 x 256
 * columns), warps 2-17 are four epilogue warpgroups that each take 4 of the 16
 * kernels of every tile.  Every mbarrier wait is bounded; on timeout the CTA
 * records an error flag, drains its copies, waits for its MMAs and frees TMEM.
 *
 * Operand layout: K-major, no swizzle, 8-row x 16-byte core matrices, K-chunk
 * outermost: element (row, k) of a tile with R rows sits at byte
 *     (k / 4) * LBO + (row / 8) * 128 + (row % 8) * 16 + (k % 4) * 4,
 * LBO = R / 8 * 128 (the descriptor's leading byte offset), SBO = 128.
 *   A tile (128 points): Xh chunks 0-5 (k 16,17 = 1, k 18-23 = 0) 12 KiB | Xl chunks 0-3 8 KiB
 *   B tile (16 kernels): Wh chunks 0-4 (k 16,17 = -b_hi,-b_lo) 20 KiB | Wl chunks 0-3 16 KiB | c2[16]
 * The all-zero chunk 5 of Wh is not stored in memory: it is zeroed once per
 * pipeline stage in shared memory.
 */
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "ncg_internal.h"

#define TC_M 128                         /* points per tile (MMA M)            */
#define TC_KT 16                         /* kernels per tile                   */
#define TC_DP 16                         /* coordinates per kernel             */
#define TC_N (TC_KT * TC_DP)             /* MMA N                              */
#define TC_STAGES 4
#define TC_CHUNK_A (TC_M / 8 * 128)      /* 2048: A LBO                        */
#define TC_CHUNK_B (TC_N / 8 * 128)      /* 4096: B LBO                        */
#define TC_XH_BYTES (6 * TC_CHUNK_A)     /* 12 KiB */
#define TC_XL_BYTES (4 * TC_CHUNK_A)     /* 8 KiB  */
#define TC_A_BYTES (TC_XH_BYTES + TC_XL_BYTES)
#define TC_WH_GLOBAL (5 * TC_CHUNK_B)    /* 20 KiB: chunks 0-4 of Wh           */
#define TC_WH_SMEM (6 * TC_CHUNK_B)      /* 24 KiB: + the zero chunk 5         */
#define TC_WL_BYTES (4 * TC_CHUNK_B)     /* 16 KiB */
#define TC_C2_BYTES (TC_KT * 4)
#define TC_B_BYTES (TC_WH_GLOBAL + TC_WL_BYTES + TC_C2_BYTES)    /* copied per tile */
#define TC_B_GSTRIDE 37888               /* global tile stride (1 KiB multiple) */
#define TC_B_SSTRIDE 41984               /* shared stage stride                 */
#define TC_EPI_WARP0 2                   /* warps 0,1: copies, MMA; then the epilogue */
#define TC_EPI_WG 4
#define TC_THREADS ((TC_EPI_WARP0 + 4 * TC_EPI_WG) * 32)
#define TC_SBO 128

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

/* shared-memory matrix descriptor: K-major, no swizzle, version 1 (bit 46) */
__device__ __forceinline__ uint64_t
_sdesc (const void *p, uint32_t lbo)
{
  const uint64_t a = (uint64_t) _smem_u32 (p);

  return ((a & 0x3FFFFull) >> 4) | ((uint64_t) (lbo >> 4) << 16) | ((uint64_t) (TC_SBO >> 4) << 32) | (1ull << 46);
}

/* D(f32) (+)= A(tf32, K-major, 128 x 8) . B(tf32, K-major, 256 x 8)^T */
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

/* two 32-column TMEM loads in flight and their wait in one asm statement, so
 * no register the loads write is touched before the wait */
__device__ __forceinline__ void
_tmem_ld64 (uint32_t t0, uint32_t t1, float *v)
{
  uint32_t r[64];

  asm volatile ("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%64];\n\t"
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                "{%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
                "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%65];\n\t"
                "tcgen05.wait::ld.sync.aligned;"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]),
                  "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]),
                  "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]),
                  "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]),
                  "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
                : "r"(t0), "r"(t1)
                : "memory");

#pragma unroll
  for (int i = 0; i < 64; i++)
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

/* byte offset of element (row, k) in a chunk-outer K-major tile with lbo = R/8*128 */
__device__ __forceinline__ uint32_t
_cm_off (int row, int k, uint32_t lbo)
{
  return (uint32_t) ((k >> 2) * lbo + (row >> 3) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

/* ------------------------------------------------------------- operand packs */

/* A tiles: x' = Vg (x - mu) in FP64, split into TF32 hi + lo, with the two
 * constant-1 columns that carry -b.  One thread per (point, coordinate),
 * 16 points per block; rows past m are zero.  Also clears the error word. */
#define TC_APB 16

__global__ void __launch_bounds__ (TC_APB * TC_DP)
_build_tc_A_kernel (const double *__restrict__ Xq, int64_t m, int d, const double *__restrict__ mu,
                    const double *__restrict__ Vg, uint8_t *__restrict__ A, int64_t rows, int *err)
{
  __shared__ double xs[TC_APB][TC_DP + 1];
  const int pl = threadIdx.x / TC_DP, r = threadIdx.x % TC_DP;
  const int64_t j = (int64_t) blockIdx.x * TC_APB + pl;

  if (blockIdx.x == 0 && threadIdx.x == 0)
    *err = 0;

  {
    /* coalesced staging of the block's points: element e = (point, coordinate) */
    const int64_t j0 = (int64_t) blockIdx.x * TC_APB;
    const int e = threadIdx.x;
    const int ep = e / TC_DP, ec = e % TC_DP;
    const int64_t je = j0 + ep;

    xs[ep][ec] = (je < m && ec < d) ? Xq[je * d + ec] - mu[ec] : 0.0;
  }

  __syncthreads ();

  if (j >= rows)
    return;

  double v = 0.0;
  const int off = r * (r + 1) / 2;

  for (int c = 0; c <= r; c++)
    v = fma (Vg[off + c], xs[pl][c], v);

  uint8_t *tile = A + (j / TC_M) * (int64_t) TC_A_BYTES;
  const int row = (int) (j % TC_M);
  const float hi = _tf32 ((float) v);
  const float lo = _tf32 ((float) (v - (double) hi));

  *(float *) (tile + _cm_off (row, r, TC_CHUNK_A))               = hi;
  *(float *) (tile + TC_XH_BYTES + _cm_off (row, r, TC_CHUNK_A)) = lo;

  if (r < 24 - TC_DP)
    *(float *) (tile + _cm_off (row, TC_DP + r, TC_CHUNK_A)) = (r < 2 && j < m) ? 1.0f : 0.0f;
}

/* B tiles from the mixed float pack (theta'_hi, theta'_lo, W' packed lower, c'):
 * row n = kk*16 + r holds prescale * W'_kk[r][:] (hi, lo) and, in Wh columns
 * 16, 17, -b_r split hi + lo with b = prescale * W'_kk theta'_kk (FP64); c2 =
 * c' log2(e).  Padding kernels get W = 0, b = 0 and c2 = -1e30. */
__global__ void __launch_bounds__ (TC_N)
_build_tc_B_kernel (const float *__restrict__ pk, int n, int smx, float prescale, uint8_t *__restrict__ B)
{
  const int t   = blockIdx.x;
  const int row = threadIdx.x;
  const int kk  = row / TC_DP, r = row % TC_DP;
  const int i   = t * TC_KT + kk;
  uint8_t *tile = B + (size_t) t * TC_B_GSTRIDE;
  const float *src = pk + (size_t) (i < n ? i : 0) * smx;
  double bsum   = 0.0;

#pragma unroll
  for (int k = 0; k < TC_DP; k++)
  {
    float w = 0.0f;

    if (i < n && k <= r)
      w = src[2 * TC_DP + r * (r + 1) / 2 + k] * prescale;

    const float hi = _tf32 (w);
    const float lo = _tf32 (w - hi);

    /* b from the split weights the MMA sees, so y = W'(x' - theta') exactly in them */
    if (i < n && k <= r)
      bsum += ((double) hi + (double) lo) * ((double) src[k] + (double) src[TC_DP + k]);

    *(float *) (tile + _cm_off (row, k, TC_CHUNK_B))                = hi;
    *(float *) (tile + TC_WH_GLOBAL + _cm_off (row, k, TC_CHUNK_B)) = lo;
  }

  {
    const float nbh = _tf32 ((float) -bsum);
    const float nbl = _tf32 ((float) (-bsum - (double) nbh));

    *(float *) (tile + _cm_off (row, TC_DP + 0, TC_CHUNK_B)) = nbh;
    *(float *) (tile + _cm_off (row, TC_DP + 1, TC_CHUNK_B)) = nbl;
    *(float *) (tile + _cm_off (row, TC_DP + 2, TC_CHUNK_B)) = 0.0f;
    *(float *) (tile + _cm_off (row, TC_DP + 3, TC_CHUNK_B)) = 0.0f;
  }

  if (r == 0)
  {
    float *c2 = (float *) (tile + TC_WH_GLOBAL + TC_WL_BYTES);

    c2[kk] = (i < n) ? src[2 * TC_DP + TC_DP * (TC_DP + 1) / 2] * LOG2E_F : -1.0e30f;
  }
}

/* ------------------------------------------------------------------ the kernel */

struct TcParams
{
  const uint8_t *A;      /* point tiles  */
  const uint8_t *B;      /* kernel tiles */
  float2 *part;          /* [m][TC_EPI_WG * nslices] */
  int *err;              /* device error flag */
  int64_t m;
  int npt, nkt, nslices, tps;
  float kappa;           /* ST: -(nu + d)/2 */
};

struct TcSmem
{
  uint8_t A[2][TC_A_BYTES];
  uint8_t B[TC_STAGES][TC_B_SSTRIDE];
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
      _mbar_init (&sm.t_empty[b], 4 * TC_EPI_WG);
    }

    for (int s = 0; s < TC_STAGES; s++)
    {
      _mbar_init (&sm.b_full[s], 1);
      _mbar_init (&sm.b_empty[s], 1 + 4 * TC_EPI_WG);
    }

    _mbar_init (&sm.done, 1);
    asm volatile ("fence.mbarrier_init.release.cluster;" ::: "memory");
  }

  /* the zero chunk 5 of every stage's Wh: written once here, never copied over */
  for (int s = 0; s < TC_STAGES; s++)
    for (int e = threadIdx.x; e < TC_CHUNK_B / 16; e += TC_THREADS)
      ((uint4 *) (sm.B[s] + TC_WH_GLOBAL))[e] = make_uint4 (0u, 0u, 0u, 0u);

  /* generic-proxy writes read later by the tensor core (async proxy) */
  asm volatile ("fence.proxy.async.shared::cta;" ::: "memory");

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

          const uint8_t *g = p.B + (size_t) t * TC_B_GSTRIDE;

          _mbar_arrive_tx (&sm.b_full[stage], TC_B_BYTES);
          _bulk_g2s (sm.B[stage], g, TC_WH_GLOBAL, &sm.b_full[stage]);
          _bulk_g2s (sm.B[stage] + TC_WH_SMEM, g + TC_WH_GLOBAL, TC_WL_BYTES + TC_C2_BYTES, &sm.b_full[stage]);
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

        const uint8_t *Xh = sm.A[ab], *Xl = sm.A[ab] + TC_XH_BYTES;

        for (int t = t0; t < t1; t++, tc++)
        {
          const int tb = tc & 1;

          if (!_mbar_wait (&sm.b_full[stage], bphase, err))
            break;

          if (!_mbar_wait (&sm.t_empty[tb], ((tc >> 1) & 1) ^ 1, err))
            break;

          _tc_fence_after ();

          const uint8_t *Wh = sm.B[stage], *Wl = sm.B[stage] + TC_WH_SMEM;
          const uint32_t d  = tmem + (uint32_t) (tb * TC_N);

          /* Xh.Wh over k 0-23 (k 16,17: 1 x -b_hi, 1 x -b_lo), then the cross terms over k 0-15 */
          _mma_tf32 (d, _sdesc (Xh, TC_CHUNK_A), _sdesc (Wh, TC_CHUNK_B), 0);
          _mma_tf32 (d, _sdesc (Xh + 2 * TC_CHUNK_A, TC_CHUNK_A), _sdesc (Wh + 2 * TC_CHUNK_B, TC_CHUNK_B), 1);
          _mma_tf32 (d, _sdesc (Xh + 4 * TC_CHUNK_A, TC_CHUNK_A), _sdesc (Wh + 4 * TC_CHUNK_B, TC_CHUNK_B), 1);
          _mma_tf32 (d, _sdesc (Xh, TC_CHUNK_A), _sdesc (Wl, TC_CHUNK_B), 1);
          _mma_tf32 (d, _sdesc (Xh + 2 * TC_CHUNK_A, TC_CHUNK_A), _sdesc (Wl + 2 * TC_CHUNK_B, TC_CHUNK_B), 1);
          _mma_tf32 (d, _sdesc (Xl, TC_CHUNK_A), _sdesc (Wh, TC_CHUNK_B), 1);
          _mma_tf32 (d, _sdesc (Xl + 2 * TC_CHUNK_A, TC_CHUNK_A), _sdesc (Wh + 2 * TC_CHUNK_B, TC_CHUNK_B), 1);

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
  else
  {
    /* ---------------- epilogue warpgroups ---------------- */
    /* Every warpgroup works on every tile: warpgroup wg takes the 4 kernels
     * [4 wg, 4 wg + 4) of it (64 TMEM columns), each warp the 32 points of
     * its TMEM lane quarter, so four independent warps share each SMSP. */
    const int ew   = warp - TC_EPI_WARP0;
    const int wg   = ew >> 2;
    const int q    = warp & 3;                  /* TMEM lane quarter (hardware: warp id mod 4) */
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
        bool got = _mbar_wait (&sm.t_full[tb], (tc >> 1) & 1, err) && _mbar_wait (&sm.b_full[stage], bphase, err);

        /* the TMEM loads below are warp-collective: agree before issuing them */
        if (!__all_sync (0xffffffffu, got))
        {
          ok = false;
          break;
        }

        _tc_fence_after ();

        const float4 c2v = *(const float4 *) (sm.B[stage] + TC_WH_SMEM + TC_WL_BYTES + 16 * wg);
        const float c2[4] = { c2v.x, c2v.y, c2v.z, c2v.w };
        float tv[4];
        float v[64];

        _tmem_ld64 (lane_base + (uint32_t) (tb * TC_N + wg * 64), lane_base + (uint32_t) (tb * TC_N + wg * 64 + 32), v);

        _tc_fence_before ();
        __syncwarp ();

        if (lane == 0)
        {
          _mbar_arrive (&sm.t_empty[tb]);
          _mbar_arrive (&sm.b_empty[stage]);
        }

#pragma unroll
        for (int h = 0; h < 4; h++)
        {
          /* chi^2 = |y|^2 with packed FP32x2 FMAs, two chains */
          float2 a0 = make_float2 (0.0f, 0.0f), a1 = make_float2 (0.0f, 0.0f);

#pragma unroll
          for (int q4 = 0; q4 < TC_DP; q4 += 4)
          {
            const float2 y0 = make_float2 (v[h * 16 + q4 + 0], v[h * 16 + q4 + 1]);
            const float2 y1 = make_float2 (v[h * 16 + q4 + 2], v[h * 16 + q4 + 3]);

            a0 = __ffma2_rn (y0, y0, a0);
            a1 = __ffma2_rn (y1, y1, a1);
          }

          const float s = (a0.x + a0.y) + (a1.x + a1.y);

          tv[h] = (KERN == NCG_KERNEL_ST) ? fmaf (p.kappa, _lg2 (1.0f + s), c2[h]) : c2[h] - s;
        }

        const float mn = fmaxf (fmaxf (m2, fmaxf (tv[0], tv[1])), fmaxf (tv[2], tv[3]));

        S  = S * _ex2 (m2 - mn) + ((_ex2 (tv[0] - mn) + _ex2 (tv[1] - mn)) + (_ex2 (tv[2] - mn) + _ex2 (tv[3] - mn)));
        m2 = mn;

        if (++stage == TC_STAGES)
        {
          stage  = 0;
          bphase ^= 1;
        }
      }

      if (!ok)
        break;

      const int64_t j = (int64_t) pt * TC_M + row;

      /* point-major partials: (base-2 max, sum of 2^(t - max) incl. the max) */
      if (j < p.m)
        p.part[(size_t) j * (TC_EPI_WG * p.nslices) + TC_EPI_WG * sl + wg] = make_float2 (m2, S);
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

/* one warp per point combines its base-2 partials in FP32 (lanes stride the
 * slices, then a shuffle tree), the final value in FP64:
 * -2 ( ln2 (M + log2 S) + C0 - d ln h ) */
__global__ void
_merge_tc_kernel (const float2 *__restrict__ part, int nparts, int64_t m, const double *__restrict__ cshift,
                  double d_ln_href, double *__restrict__ out, const int *__restrict__ err, int *flag_host)
{
  const int64_t j = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane  = threadIdx.x & 31;

  /* forward the eval kernel's error word to the caller's mapped host flag */
  if (blockIdx.x == 0 && threadIdx.x == 0 && flag_host != NULL)
    *(volatile int *) flag_host = *err;

  if (j >= m)
    return;

  float M = -CUDART_INF_F, S = 0.0f;
  const float2 *row = part + (size_t) j * nparts;

  for (int q = lane; q < nparts; q += 32)
  {
    const float2 v = row[q];
    const float mn = fmaxf (M, v.x);

    S = ((M > -CUDART_INF_F) ? S * _ex2 (M - mn) : 0.0f) + ((v.x > -CUDART_INF_F) ? v.y * _ex2 (v.x - mn) : 0.0f);
    M = mn;
  }

#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    const float Mo = __shfl_xor_sync (0xffffffffu, M, o);
    const float So = __shfl_xor_sync (0xffffffffu, S, o);
    const float mn = fmaxf (M, Mo);

    S = ((M > -CUDART_INF_F) ? S * _ex2 (M - mn) : 0.0f) + ((Mo > -CUDART_INF_F) ? So * _ex2 (Mo - mn) : 0.0f);
    M = mn;
  }

  if (lane == 0)
    out[j] = -2.0 * (LN2_D * ((double) M + log2 ((double) S)) + *cshift - d_ln_href);
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
  return (size_t) ((n + TC_KT - 1) / TC_KT) * TC_B_GSTRIDE;
}

extern "C" size_t
ncg_tc_scratch_bytes (int64_t m, int n)
{
  int ns, tps;
  const int npt = (int) ((m + TC_M - 1) / TC_M), nkt = (n + TC_KT - 1) / TC_KT;

  _tc_slicing (npt, nkt, 152, &ns, &tps);

  /* A tiles | partials | error flag */
  return (size_t) npt * TC_A_BYTES + (size_t) TC_EPI_WG * ns * (size_t) m * sizeof (float2) + 256;
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
                    const double *Vg, const double *cshift, void *scratch, double *out, int *flag_host,
                    cudaEvent_t *ev, cudaStream_t s)
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
  int *err      = (int *) (part + (size_t) TC_EPI_WG * ns * a->m);
  const int64_t rows = (int64_t) npt * TC_M;

  _build_tc_A_kernel<<<(unsigned) ((rows + TC_APB - 1) / TC_APB), TC_APB * TC_DP, 0, s>>> (Xq, a->m, a->d, mu, Vg, A,
                                                                                          rows, err);

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

  if (ev != NULL && (e = cudaEventRecord (ev[0], s)) != cudaSuccess)
    return e;

  fn<<<grid, TC_THREADS, smem, s>>> (p);

  if ((e = cudaGetLastError ()) != cudaSuccess)
    return e;

  if (ev != NULL && (e = cudaEventRecord (ev[1], s)) != cudaSuccess)
    return e;

  _merge_tc_kernel<<<(unsigned) ((a->m * 32 + 255) / 256), 256, 0, s>>> (part, TC_EPI_WG * ns, a->m, cshift,
                                                                         a->d_ln_href, out, err, flag_host);

  return cudaGetLastError ();
}
