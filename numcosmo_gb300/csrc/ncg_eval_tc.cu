/*
 * ncg_eval_tc.cu -- KDE / VKDE eval_m2lnp on the 5th-generation tensor cores
 * (tcgen05, TMEM accumulators), TF32x3 split products, FP32 log-sum-exp.
 *
 * The per-pair whitening of _ncm_stats_dist_vkde_eval_weights_m2lnp
 * (numcosmo/ncm/stats/ncm_stats_dist_vkde.c:682-723), y_i = U_i^{-T}(x - theta_i)/h,
 * is rewritten in globally whitened coordinates as y_i = W'_i x' - b_i with
 * x' = U_g^{-T}(x - mu), W'_i = U_i^{-T} U_g^T / h and b_i = W'_i theta'_i; the
 * KDE form (numcosmo/ncm/stats/ncm_stats_dist_kde.c:640-681) would be the same
 * with W'_i = I (the operand builder handles it) but is not routed here (see
 * ncg_tc_supported).  The folded subtraction costs FP32 cancellation of the
 * size of |W'_i theta'_i|; the host checks each operand on the kernel centres
 * against the FP64 form before using it (ncg_sd_get_tc_check).  For a tile
 * of 128 points and KT kernels, y for all pairs is ONE GEMM with the
 * subtraction folded in by a constant column: with x'' = [x', 1, 1] and
 * w''_{i,r} = [W'_i[r,:], -b_hi, -b_lo],
 *     D[128 points x 256] = X''[128 x KA] . W''^T[KA x 256]
 * issued as tcgen05.mma.kind::tf32 (M=128, N=256, K=8) with the operands split
 * into TF32 hi + lo parts: D = Xh Wh^T (KA/8 k-steps, incl. the -b column
 * pair) + Xh Wl^T + Xl Wh^T (KD/8 k-steps each), FP32 accumulation.  The 256
 * columns are four 64-column bands, one per epilogue warpgroup; a band holds
 * KPW = floor(64/dp) kernels of dp coordinates (the rest of the band is zero),
 * so a tile carries KT = 4 KPW kernels.  The epilogue reads y from TMEM
 * (tcgen05.ld), squares and sums it over the dp coordinates with packed
 * FP32x2 FMAs (chi^2 never reaches memory) and keeps an online log-sum-exp per
 * point in base 2.  Partials (max, sum) per (kernel slice, warpgroup) are
 * merged by a warp-per-point FP32 reduction with an FP64 finish.
 *
 *   dp          4   8  12  16  20  24  28  32
 *   KPW        16   8   5   4   3   2   2   2
 *   KA (K hi)   8  16  16  24  24  32  32  40
 *   KD (K x)    8   8  16  16  24  24  32  32
 *   MMAs/tile   3   4   6   7   9  10  12  13
 *   stages      4   4   4   4   3   2   2   2
 *
 * CTA roles (persistent, one CTA per SM): warp 0 copies operand tiles with the
 * bulk-copy engine (cp.async.bulk + mbarrier complete_tx), warp 1 allocates
 * TMEM and issues the MMAs into a double-buffered accumulator (2 x 256
 * columns), warps 2-17 are the four epilogue warpgroups.  Every mbarrier wait
 * is bounded; on timeout the CTA records an error flag, drains its copies,
 * waits for its MMAs and frees TMEM.
 *
 * Operand layout (ncg_tc_ptx.cuh): K-major, no swizzle, core matrices of
 * 8 rows x 16 bytes, K-chunk outermost.
 *   A tile (128 points): Xh chunks 0..KA/4-1 (k dp, dp+1 = 1) | Xl chunks 0..KD/4-1
 *   B tile (256 rows): Wh chunks 0..NWH-1 (k dp, dp+1 = -b_hi, -b_lo) | Wl chunks
 *   0..KD/4-1 | c2[KT]; the all-zero trailing Wh chunks (NWH = ceil((dp+2)/4)
 *   up to KA/4) are not stored in memory: they are zeroed once per pipeline
 *   stage in shared memory.
 */
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "ncg_internal.h"
#include "ncg_tc_ptx.cuh"

#define TC_M 128                         /* points per tile (MMA M)            */
#define TC_N 256                         /* MMA N: four 64-column bands        */
#define TC_CHUNK_A (TC_M / 8 * 128)      /* 2048: A LBO                        */
#define TC_CHUNK_B (TC_N / 8 * 128)      /* 4096: B LBO                        */
#define TC_EPI_WARP0 2                   /* warps 0,1: copies, MMA; then the epilogue */
#define TC_EPI_WG 4
#define TC_THREADS ((TC_EPI_WARP0 + 4 * TC_EPI_WG) * 32)

template <int DP>
struct TcShape
{
  static constexpr int KPW       = 64 / DP;                 /* kernels per band          */
  static constexpr int KT        = 4 * KPW;                 /* kernels per tile          */
  static constexpr int KA        = (DP + 2 + 7) / 8 * 8;    /* K of Xh.Wh (with -b)      */
  static constexpr int KD        = (DP + 7) / 8 * 8;        /* K of the cross terms      */
  static constexpr int NWH       = (DP + 2 + 3) / 4;        /* Wh chunks stored          */
  static constexpr int XH_BYTES  = KA / 4 * TC_CHUNK_A;
  static constexpr int A_BYTES   = XH_BYTES + KD / 4 * TC_CHUNK_A;
  static constexpr int WH_GLOBAL = NWH * TC_CHUNK_B;
  static constexpr int WH_SMEM   = KA / 4 * TC_CHUNK_B;
  static constexpr int WL_BYTES  = KD / 4 * TC_CHUNK_B;
  static constexpr int C2_BYTES  = KT * 4;
  static constexpr int B_BYTES   = WH_GLOBAL + WL_BYTES + C2_BYTES;           /* copied per tile */
  static constexpr int B_GSTRIDE = (B_BYTES + 1023) / 1024 * 1024;
  static constexpr int B_SSTRIDE = (WH_SMEM + WL_BYTES + C2_BYTES + 1023) / 1024 * 1024;
  static constexpr int STAGES    = DP <= 16 ? 4 : (DP <= 20 ? 3 : 2);
};

#define LOG2E_F 1.4426950408889634f
#define LN2_D 0.69314718055994530942

/* ---------------------------------------------------------------- PTX helpers */

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

/* ------------------------------------------------------------- operand packs */

/* A tiles: x' = Vg (x - mu) in FP64 (KDE: mu = NULL), split into TF32 hi + lo,
 * with the two constant-1 columns that carry -b and zero padding up to KA / KD.
 * One thread per (point, coordinate), 16 points per block; rows past m are
 * zero.  Also clears the error word. */
#define TC_APB 16

template <int DP>
__global__ void __launch_bounds__ (TC_APB * DP)
_build_tc_A_kernel (const double *__restrict__ Xq, int64_t m, int d, const double *__restrict__ mu,
                    const double *__restrict__ Vg, uint8_t *__restrict__ A, int64_t rows, int *err)
{
  using S = TcShape<DP>;
  __shared__ double xs[TC_APB][DP + 1];
  const int pl = threadIdx.x / DP, r = threadIdx.x % DP;
  const int64_t j = (int64_t) blockIdx.x * TC_APB + pl;

  if (blockIdx.x == 0 && threadIdx.x == 0)
    *err = 0;

  {
    /* coalesced staging of the block's points: element e = (point, coordinate) */
    const int64_t je = (int64_t) blockIdx.x * TC_APB + pl;

    xs[pl][r] = (je < m && r < d) ? Xq[je * d + r] - (mu ? mu[r] : 0.0) : 0.0;
  }

  __syncthreads ();

  if (j >= rows)
    return;

  double v = 0.0;
  const int off = r * (r + 1) / 2;

  for (int c = 0; c <= r; c++)
    v = fma (Vg[off + c], xs[pl][c], v);

  uint8_t *tile = A + (j / TC_M) * (int64_t) S::A_BYTES;
  const int row = (int) (j % TC_M);
  const float hi = _tf32 ((float) v);
  const float lo = _tf32 ((float) (v - (double) hi));

  *(float *) (tile + _cm_off (row, r, TC_CHUNK_A))               = hi;
  *(float *) (tile + S::XH_BYTES + _cm_off (row, r, TC_CHUNK_A)) = lo;

  if (r < S::KA - DP)
    *(float *) (tile + _cm_off (row, DP + r, TC_CHUNK_A)) = (r < 2 && j < m) ? 1.0f : 0.0f;

  if (r < S::KD - DP)
    *(float *) (tile + S::XH_BYTES + _cm_off (row, DP + r, TC_CHUNK_A)) = 0.0f;
}

/* B tiles from the mixed float pack (VKDE: theta'_hi, theta'_lo, W' packed
 * lower, c'; KDE: theta'_hi, theta'_lo, c').  Row = band * 64 + kk * DP + r
 * holds prescale * W'_kk[r][:] (hi, lo; KDE: prescale on the diagonal) and,
 * in Wh columns DP, DP+1, -b_r split hi + lo with b = prescale * W'_kk
 * theta'_kk (FP64); c2 = c' log2(e).  Padding kernels and the rest of a band
 * get W = 0, b = 0 and (kernels) c2 = -1e30. */
template <int DP, int KIND>
__global__ void __launch_bounds__ (TC_N)
_build_tc_B_kernel (const float *__restrict__ pk, int n, int smx, float prescale, uint8_t *__restrict__ B)
{
  using S = TcShape<DP>;
  const int t      = blockIdx.x;
  const int row    = threadIdx.x;
  const int band   = row / 64, within = row % 64;
  const int kk     = within / DP, r = within % DP;
  const bool inb   = kk < S::KPW;
  const int i      = t * S::KT + band * S::KPW + kk;
  const bool valid = inb && i < n;
  uint8_t *tile    = B + (size_t) t * S::B_GSTRIDE;
  const float *src = pk + (size_t) (valid ? i : 0) * smx;
  double bsum      = 0.0;

#pragma unroll
  for (int k = 0; k < DP; k++)
  {
    float w = 0.0f;

    if (valid && k <= r)
      w = (KIND == NCG_VKDE) ? src[2 * DP + r * (r + 1) / 2 + k] * prescale : ((k == r) ? prescale : 0.0f);

    const float hi = _tf32 (w);
    const float lo = _tf32 (w - hi);

    /* b from the split weights the MMA sees, so y = W'(x' - theta') exactly in them */
    if (valid && k <= r)
      bsum += ((double) hi + (double) lo) * ((double) src[k] + (double) src[DP + k]);

    *(float *) (tile + _cm_off (row, k, TC_CHUNK_B))                   = hi;
    *(float *) (tile + S::WH_GLOBAL + _cm_off (row, k, TC_CHUNK_B)) = lo;
  }

  {
    const float nbh = _tf32 ((float) -bsum);
    const float nbl = _tf32 ((float) (-bsum - (double) nbh));

    for (int k = DP; k < 4 * S::NWH; k++)
      *(float *) (tile + _cm_off (row, k, TC_CHUNK_B)) = (k == DP) ? nbh : ((k == DP + 1) ? nbl : 0.0f);

    for (int k = DP; k < S::KD; k++)
      *(float *) (tile + S::WH_GLOBAL + _cm_off (row, k, TC_CHUNK_B)) = 0.0f;
  }

  if (inb && r == 0)
  {
    float *c2 = (float *) (tile + S::WH_GLOBAL + S::WL_BYTES);
    const int coff = (KIND == NCG_VKDE) ? 2 * DP + DP * (DP + 1) / 2 : 2 * DP;

    c2[band * S::KPW + kk] = (i < n) ? src[coff] * LOG2E_F : -1.0e30f;
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

template <int DP>
struct TcSmem
{
  uint8_t A[2][TcShape<DP>::A_BYTES];
  uint8_t B[TcShape<DP>::STAGES][TcShape<DP>::B_SSTRIDE];
  uint64_t a_full[2], a_empty[2], b_full[TcShape<DP>::STAGES], b_empty[TcShape<DP>::STAGES], t_full[2], t_empty[2],
           done;
  uint32_t tmem_base;
  int err;
};

template <int DP, int KERN>
__global__ void __launch_bounds__ (TC_THREADS, 1)
_eval_tc_kernel (const TcParams p)
{
  using S = TcShape<DP>;
  constexpr int STAGES = S::STAGES;
  extern __shared__ __align__ (1024) uint8_t tc_raw[];
  TcSmem<DP> &sm = *(TcSmem<DP> *) (((uintptr_t) tc_raw + 1023) & ~(uintptr_t) 1023);

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

    for (int s = 0; s < STAGES; s++)
    {
      _mbar_init (&sm.b_full[s], 1);
      _mbar_init (&sm.b_empty[s], 1 + 4 * TC_EPI_WG);
    }

    _mbar_init (&sm.done, 1);
    asm volatile ("fence.mbarrier_init.release.cluster;" ::: "memory");
  }

  /* the zero trailing Wh chunks of every stage: written once here, never copied over */
  if (S::WH_SMEM > S::WH_GLOBAL)
    for (int s = 0; s < STAGES; s++)
      for (int e = threadIdx.x; e < (S::WH_SMEM - S::WH_GLOBAL) / 16; e += TC_THREADS)
        ((uint4 *) (sm.B[s] + S::WH_GLOBAL))[e] = make_uint4 (0u, 0u, 0u, 0u);

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
      int armed_b[STAGES], armed_a[2];   /* parity of the last armed phase, -1 none */

      for (int s = 0; s < STAGES; s++)
        armed_b[s] = -1;

      armed_a[0] = armed_a[1] = -1;

      for (int u = blockIdx.x; u < nunits && !*err; u += gridDim.x, lu++)
      {
        const int pt = u / p.nslices, sl = u % p.nslices;
        const int t0 = sl * p.tps, t1 = min (p.nkt, t0 + p.tps);
        const int ab = lu & 1;

        if (!_mbar_wait (&sm.a_empty[ab], ((lu >> 1) & 1) ^ 1, err))
          break;

        _mbar_arrive_tx (&sm.a_full[ab], S::A_BYTES);
        _bulk_g2s (sm.A[ab], p.A + (size_t) pt * S::A_BYTES, S::A_BYTES, &sm.a_full[ab]);
        armed_a[ab] = (lu >> 1) & 1;

        for (int t = t0; t < t1; t++)
        {
          if (!_mbar_wait (&sm.b_empty[stage], bphase ^ 1, err))
            break;

          const uint8_t *g = p.B + (size_t) t * S::B_GSTRIDE;

          _mbar_arrive_tx (&sm.b_full[stage], S::B_BYTES);
          _bulk_g2s (sm.B[stage], g, S::WH_GLOBAL, &sm.b_full[stage]);
          _bulk_g2s (sm.B[stage] + S::WH_SMEM, g + S::WH_GLOBAL, S::WL_BYTES + S::C2_BYTES, &sm.b_full[stage]);
          armed_b[stage] = (int) bphase;

          if (++stage == STAGES)
          {
            stage  = 0;
            bphase ^= 1;
          }
        }
      }

      /* drain: every copy this thread armed must land before the CTA may exit
       * (a no-op in the normal flow, where the consumers waited on them) */
      for (int s = 0; s < STAGES; s++)
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

        const uint8_t *Xh = sm.A[ab], *Xl = sm.A[ab] + S::XH_BYTES;

        for (int t = t0; t < t1; t++, tc++)
        {
          const int tb = tc & 1;

          if (!_mbar_wait (&sm.b_full[stage], bphase, err))
            break;

          if (!_mbar_wait (&sm.t_empty[tb], ((tc >> 1) & 1) ^ 1, err))
            break;

          _tc_fence_after ();

          const uint8_t *Wh = sm.B[stage], *Wl = sm.B[stage] + S::WH_SMEM;
          const uint32_t d  = tmem + (uint32_t) (tb * TC_N);

          /* Xh.Wh over k 0..KA-1 (k DP, DP+1: 1 x -b_hi, 1 x -b_lo), then the cross terms over k 0..KD-1 */
#pragma unroll
          for (int ks = 0; ks < S::KA / 8; ks++)
            _mma_tf32 (d, _sdesc (Xh + 2 * ks * TC_CHUNK_A, TC_CHUNK_A), _sdesc (Wh + 2 * ks * TC_CHUNK_B, TC_CHUNK_B),
                       ks > 0 ? 1u : 0u);

#pragma unroll
          for (int ks = 0; ks < S::KD / 8; ks++)
            _mma_tf32 (d, _sdesc (Xh + 2 * ks * TC_CHUNK_A, TC_CHUNK_A), _sdesc (Wl + 2 * ks * TC_CHUNK_B, TC_CHUNK_B), 1u);

#pragma unroll
          for (int ks = 0; ks < S::KD / 8; ks++)
            _mma_tf32 (d, _sdesc (Xl + 2 * ks * TC_CHUNK_A, TC_CHUNK_A), _sdesc (Wh + 2 * ks * TC_CHUNK_B, TC_CHUNK_B), 1u);

          _mma_commit (&sm.t_full[tb]);
          _mma_commit (&sm.b_empty[stage]);

          if (++stage == STAGES)
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
    /* Every warpgroup works on every tile: warpgroup wg takes the KPW kernels
     * of band wg (64 TMEM columns), each warp the 32 points of its TMEM lane
     * quarter, so four independent warps share each SMSP. */
    constexpr int KPW = S::KPW;
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
      float m2 = -CUDART_INF_F, S2 = 0.0f;
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

        const float *c2s = (const float *) (sm.B[stage] + S::WH_SMEM + S::WL_BYTES) + KPW * wg;
        float c2[KPW], tv[KPW];
        float v[64];

#pragma unroll
        for (int h = 0; h < KPW; h++)
          c2[h] = c2s[h];

        _tmem_ld64 (lane_base + (uint32_t) (tb * TC_N + wg * 64), lane_base + (uint32_t) (tb * TC_N + wg * 64 + 32), v);

        _tc_fence_before ();
        __syncwarp ();

        if (lane == 0)
        {
          _mbar_arrive (&sm.t_empty[tb]);
          _mbar_arrive (&sm.b_empty[stage]);
        }

#pragma unroll
        for (int h = 0; h < KPW; h++)
        {
          /* chi^2 = |y|^2 with packed FP32x2 FMAs, two chains */
          float2 a0 = make_float2 (0.0f, 0.0f), a1 = make_float2 (0.0f, 0.0f);

#pragma unroll
          for (int q4 = 0; q4 < DP; q4 += 4)
          {
            const float2 y0 = make_float2 (v[h * DP + q4 + 0], v[h * DP + q4 + 1]);
            const float2 y1 = make_float2 (v[h * DP + q4 + 2], v[h * DP + q4 + 3]);

            a0 = __ffma2_rn (y0, y0, a0);
            a1 = __ffma2_rn (y1, y1, a1);
          }

          const float s = (a0.x + a0.y) + (a1.x + a1.y);

          tv[h] = (KERN == NCG_KERNEL_ST) ? fmaf (p.kappa, _lg2 (1.0f + s), c2[h]) : c2[h] - s;
        }

        float mx = tv[0];

#pragma unroll
        for (int h = 1; h < KPW; h++)
          mx = fmaxf (mx, tv[h]);

        const float mn = fmaxf (m2, mx);
        float acc = 0.0f;

#pragma unroll
        for (int h = 0; h < KPW; h += 2)
          acc = acc + ((h + 1 < KPW) ? (_ex2 (tv[h] - mn) + _ex2 (tv[h + 1] - mn)) : _ex2 (tv[h] - mn));

        S2 = S2 * _ex2 (m2 - mn) + acc;
        m2 = mn;

        if (++stage == STAGES)
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
        p.part[(size_t) j * (TC_EPI_WG * p.nslices) + TC_EPI_WG * sl + wg] = make_float2 (m2, S2);
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
 * -2 ( ln2 (M + log2 S) + C0 - shift - d ln h ), shift = the KDE kernel lnnorm */
__global__ void
_merge_tc_kernel (const float2 *__restrict__ part, int nparts, int64_t m, const double *__restrict__ cshift,
                  double shift, double d_ln_href, double *__restrict__ out, const int *__restrict__ err,
                  int *flag_host)
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
    out[j] = -2.0 * (LN2_D * ((double) M + log2 ((double) S)) + *cshift - shift - d_ln_href);
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

/* compile-time shape of a runtime dp (dp in {4, 8, ..., 32}) */
#define TC_DISPATCH(dp, F)  \
  switch (dp)               \
  {                         \
    case 4:  F (4);  break; \
    case 8:  F (8);  break; \
    case 12: F (12); break; \
    case 16: F (16); break; \
    case 20: F (20); break; \
    case 24: F (24); break; \
    case 28: F (28); break; \
    case 32: F (32); break; \
    default: break;         \
  }

typedef struct { int kt, a_bytes, b_gstride; size_t smem; } tc_dims_t;

static int
_tc_dims (int dp, tc_dims_t *t)
{
  int ok = 0;

#define TC_DIMS(D)                                                            \
  do {                                                                        \
    t->kt = TcShape<D>::KT;                                                   \
    t->a_bytes = TcShape<D>::A_BYTES;                                         \
    t->b_gstride = TcShape<D>::B_GSTRIDE;                                     \
    t->smem = sizeof (TcSmem<D>) + 1024;                                      \
    ok = 1;                                                                   \
  } while (0)

  TC_DISPATCH (dp, TC_DIMS);
#undef TC_DIMS

  return ok;
}

/* VKDE only: the KDE operand (identity whitening, centres theta'/h far from
 * the origin) loses more than the 1e-6 budget to the folded subtraction, and
 * its SIMT form costs about 2 dp flops per pair anyway */
extern "C" int
ncg_tc_supported (int kind, int dp)
{
  tc_dims_t t;

  return kind == NCG_VKDE && _tc_dims (dp, &t);
}

extern "C" size_t
ncg_tc_B_bytes (int n, int dp)
{
  tc_dims_t t;

  if (!_tc_dims (dp, &t))
    return 0;

  return (size_t) ((n + t.kt - 1) / t.kt) * (size_t) t.b_gstride;
}

extern "C" size_t
ncg_tc_scratch_bytes (int64_t m, int n, int dp)
{
  tc_dims_t t;
  int ns, tps;

  if (!_tc_dims (dp, &t))
    return 0;

  const int npt = (int) ((m + TC_M - 1) / TC_M), nkt = (n + t.kt - 1) / t.kt;

  _tc_slicing (npt, nkt, 152, &ns, &tps);

  /* A tiles | partials | error flag */
  return (size_t) npt * t.a_bytes + (size_t) TC_EPI_WG * ns * (size_t) m * sizeof (float2) + 256;
}

extern "C" cudaError_t
ncg_launch_build_tc_B (const float *packmx, int kind, int n, int dp, int kernel, double nu, uint8_t *B,
                       cudaStream_t s)
{
  tc_dims_t t;

  if (!_tc_dims (dp, &t))
    return cudaErrorInvalidValue;

  const int nkt        = (n + t.kt - 1) / t.kt;
  const int raw        = (kind == NCG_VKDE) ? 2 * dp + dp * (dp + 1) / 2 + 1 : 2 * dp + 1;
  const int smx        = (raw + 3) / 4 * 4;
  const float prescale = (kernel == NCG_KERNEL_ST) ? (float) (1.0 / sqrt (nu)) : (float) sqrt (0.5 * 1.4426950408889634);

#define TC_BUILD_B(D)                                                                                         \
  do {                                                                                                        \
    if (kind == NCG_VKDE)                                                                                     \
      _build_tc_B_kernel<D, NCG_VKDE><<<nkt, TC_N, 0, s>>> (packmx, n, smx, prescale, B);                      \
    else                                                                                                      \
      _build_tc_B_kernel<D, NCG_KDE><<<nkt, TC_N, 0, s>>> (packmx, n, smx, prescale, B);                       \
  } while (0)

  TC_DISPATCH (dp, TC_BUILD_B);
#undef TC_BUILD_B

  return cudaGetLastError ();
}

template <int DP>
static cudaError_t
_launch_tc (const ncg_eval_args_t *a, const double *Xq, const uint8_t *B, const double *mu, const double *Vg,
            const double *cshift, void *scratch, double *out, int *flag_host, cudaEvent_t *ev, cudaStream_t s)
{
  using S = TcShape<DP>;
  const int npt = (int) ((a->m + TC_M - 1) / TC_M), nkt = (a->n + S::KT - 1) / S::KT;
  int ns, tps, dev, nsm;
  cudaError_t e;

  if ((e = cudaGetDevice (&dev)) != cudaSuccess)
    return e;

  if ((e = cudaDeviceGetAttribute (&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return e;

  _tc_slicing (npt, nkt, 152, &ns, &tps);

  uint8_t *A    = (uint8_t *) scratch;
  float2 *part  = (float2 *) (A + (size_t) npt * S::A_BYTES);
  int *err      = (int *) (part + (size_t) TC_EPI_WG * ns * a->m);
  const int64_t rows = (int64_t) npt * TC_M;

  _build_tc_A_kernel<DP><<<(unsigned) ((rows + TC_APB - 1) / TC_APB), TC_APB * DP, 0, s>>> (
    Xq, a->m, a->d, (a->kind == NCG_VKDE) ? mu : NULL, Vg, A, rows, err);

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

  const size_t smem = sizeof (TcSmem<DP>) + 1024;
  void (*fn) (const TcParams) = (a->kernel == NCG_KERNEL_ST) ? _eval_tc_kernel<DP, NCG_KERNEL_ST>
                                                              : _eval_tc_kernel<DP, NCG_KERNEL_GAUSS>;

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
                                                                         a->final_shift, a->d_ln_href, out, err,
                                                                         flag_host);

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_eval_tc (const ncg_eval_args_t *a, const double *Xq, const uint8_t *B, const double *mu,
                    const double *Vg, const double *cshift, void *scratch, double *out, int *flag_host,
                    cudaEvent_t *ev, cudaStream_t s)
{
  cudaError_t e = cudaErrorInvalidValue;

#define TC_LAUNCH(D) e = _launch_tc<D> (a, Xq, B, mu, Vg, cshift, scratch, out, flag_host, ev, s)

  TC_DISPATCH (a->dp, TC_LAUNCH);
#undef TC_LAUNCH

  return e;
}
