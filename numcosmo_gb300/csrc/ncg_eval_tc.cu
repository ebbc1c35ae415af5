/*
 * ncg_eval_tc.cu -- KDE / VKDE eval_m2lnp on the 5th-generation tensor cores
 * (tcgen05, TMEM accumulators): FP16x3 split products on kind::f16 with FP32
 * accumulation, FP32 log-sum-exp, the slice merge fused into the kernel.
 *
 * The per-pair whitening of _ncm_stats_dist_vkde_eval_weights_m2lnp
 * (numcosmo/ncm/stats/ncm_stats_dist_vkde.c:682-723), y_i = U_i^{-T}(x - theta_i)/h,
 * is rewritten in globally whitened coordinates as y_i = W'_i x' - b_i with
 * x' = U_g^{-T}(x - mu), W'_i = U_i^{-T} U_g^T / h and b_i = W'_i theta'_i; the
 * KDE form (numcosmo/ncm/stats/ncm_stats_dist_kde.c:640-681) would be the same
 * with W'_i = I (the operand builder handles it) but is not routed here (see
 * ncg_tc_supported).  The folded subtraction costs FP32 cancellation of the
 * size of |W'_i theta'_i|; the host checks each operand on the kernel centres
 * against the FP64 form before using it (ncg_sd_get_tc_check).
 *
 * Split precision.  Every operand value v is held as two FP16 numbers,
 * v = hi + lo with hi = fp16(v) and lo = fp16(v - hi): 22 significant bits,
 * the budget of a TF32 hi/lo pair, at twice the TF32 tensor rate.  The three
 * products that carry it, Wh.xh + Wh.xl + Wl.xh, are exact in the FP32
 * accumulator (11 x 11 bits); Wl.xl (2^-22 relative) is dropped.  FP16 has a
 * narrow exponent range, so operands are scaled by powers of two (exact):
 * a point by 2^sx (its largest coordinate lands in [2^11, 2^12)), a tile of
 * kernels by 2^sw (its largest weight below 2^12 and its largest bias below
 * 2^14 after the 2^-f of the constant column).  The accumulator then holds
 * 2^(sx + sw) y, and the epilogue multiplies chi^2 by 2^(-2 sx - 2 sw), one
 * factor per (point, tile) folded into an FMA it already issues.
 *
 * The GEMM.  For a tile of 128 points and KT kernels,
 *     D[128 points x 256] = sum over MMA windows of A_w[128 x 16] . B_w[16 x 256]^T
 * issued as tcgen05.mma.kind::f16 (M=128, N=256, K=16): each window covers two
 * 8-wide K chunks.  B (per kernel tile, stored once) is the chunk sequence
 *     [bias | Wh_0 .. Wh_{C-1} | Wl_0 .. Wl_{C-1}],  C = ceil(dp / 8),
 * the bias chunk holding (-b_hi, -b_lo) 2^(sw - f); window w reads B chunks
 * (b_w, b_w + 1).  A (per point tile) stores, for every window, the two
 * chunks that multiply them: the constant chunk (2^(sx + f) twice, then 0), xh_k,
 * xl_k or zeros.  Windows 0..C slide over [bias, Wh_0 .. Wh_{C-1}, Wl_0]
 * (A: [1, xl_0], [xh_0, xl_1], ..., [xh_{C-1}, xh_0]), the rest pair up
 * Wl_1 .. Wl_{C-1} with xh_1 .. xh_{C-1}; C + 1 + floor(C/2) MMAs a tile:
 *
 *   dp          4   8  12  16  20  24  28  32
 *   KPW        16   8   5   4   3   2   2   2     kernels per 64-column band
 *   MMAs/tile   2   2   4   4   5   5   7   7     (the TF32x3 form: 3..13)
 *
 * The 256 columns are four 64-column bands, one per epilogue warpgroup; a
 * band holds KPW = floor(64 / dp) kernels of dp coordinates.  The epilogue
 * reads y from TMEM (tcgen05.ld), squares and sums it over the dp
 * coordinates with packed FP32x2 FMAs (chi^2 never reaches memory) and keeps
 * an online base-2 log-sum-exp per point.  Each (kernel slice, warpgroup)
 * partial (max, sum) goes to global memory; the warp that completes the last
 * partial of a 32-point quarter of a point tile (a counter per quarter)
 * merges that quarter in FP32, finishing in FP64, so no merge launch follows.
 *
 * CTA roles (persistent, one CTA per SM): warp 0 copies operand tiles with the
 * bulk-copy engine (cp.async.bulk + mbarrier complete_tx), warp 1 allocates
 * TMEM and issues the MMAs into a double-buffered accumulator (2 x 256
 * columns), warps 2-17 are the four epilogue warpgroups.  Units (point tile,
 * kernel slice) run slice-major, so the CTAs working at one time read the same
 * kernel tiles (once from DRAM, then from L2) for different point tiles.
 * Every mbarrier wait is bounded; on timeout the CTA records an error flag,
 * drains its copies, waits for its MMAs and frees TMEM.
 *
 * Operand layout (ncg_tc_ptx.cuh): K-major, no swizzle, core matrices of
 * 8 rows x 16 bytes (8 FP16 values), K-chunk outermost: element (row, k) of
 * chunk q sits at byte q * LBO + (row / 8) * 128 + (row % 8) * 16 + (k % 8) * 2.
 */
#include <cuda_fp16.h>
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
#define TC_MAX_THREADS ((TC_EPI_WARP0 + 16) * 32)
#define TC_BIAS_F 1                      /* constant column 2^(sx + f), bias 2^(sw - f) (-b) */
#define TC_SMEM_CAP (212 * 1024)

/* A chunk contents of the MMA windows */
#define TCA_ZERO 0
#define TCA_ONE 1
#define TCA_XH 8                         /* + k: xh chunk k */
#define TCA_XL 16                        /* + k: xl chunk k */

__host__ __device__ constexpr int
tc_nwin (int c)
{
  return c + 1 + c / 2;
}

/* first B chunk of window w */
__host__ __device__ constexpr int
tc_win_b0 (int c, int w)
{
  return (w <= c) ? w : ((w - (c + 1) < (c - 1) / 2) ? c + 2 + 2 * (w - (c + 1)) : 2 * c - 1);
}

/* A chunk e (0, 1) of window w */
__host__ __device__ constexpr int
tc_win_a (int c, int w, int e)
{
  return (w <= c) ? ((e == 0) ? ((w == 0) ? TCA_ONE : TCA_XH + w - 1) : ((w < c) ? TCA_XL + w : TCA_XH))
                  : ((w - (c + 1) < (c - 1) / 2) ? TCA_XH + 1 + 2 * (w - (c + 1)) + e
                                                 : ((e == 0) ? TCA_ZERO : TCA_XH + c - 1));
}

template <int DP>
struct TcShape
{
  static constexpr int KPW      = 64 / DP;                 /* kernels per band          */
  static constexpr int KT       = 4 * KPW;                 /* kernels per tile          */
  static constexpr int C        = (DP + 7) / 8;            /* 8-wide K chunks per operand */
  static constexpr int NW       = tc_nwin (C);             /* MMAs per tile             */
  static constexpr int A_BYTES  = 2 * NW * TC_CHUNK_A;
  static constexpr int NCB      = 2 * C + 1;               /* B chunks: bias | Wh | Wl  */
  static constexpr int C2_OFF   = NCB * TC_CHUNK_B;
  static constexpr int C2_BYTES = (KT * 4 + 4 + 15) / 16 * 16;   /* c2[KT], 2^(-2 sw) */
  static constexpr int B_BYTES  = C2_OFF + C2_BYTES;
  static constexpr int B_STRIDE = (B_BYTES + 1023) / 1024 * 1024;
  static constexpr int STAGES   = (2 * A_BYTES + 4 * B_STRIDE <= TC_SMEM_CAP) ? 4 : 3;
  /* epilogue warpgroups: each takes BPW of the four 64-column bands of every
   * tile; two bands a warp (dp >= 8) halve the per-tile overhead per pair
   * (measured: dp 8 0.122 vs 0.134 ms, dp 16 0.122 vs 0.131 ms at N = M = 8192) */
  static constexpr int EPI_WG   = (DP >= 8) ? 2 : 4;
  static constexpr int BPW      = 4 / EPI_WG;
  static constexpr int KPWW     = KPW * BPW;               /* kernels per warp and tile */
  static constexpr int THREADS  = (TC_EPI_WARP0 + 4 * EPI_WG) * 32;
};

#define LOG2E_F 1.4426950408889634f
#define LN2_D 0.69314718055994530942

/* ---------------------------------------------------------------- PTX helpers */

/* D(f32) (+)= A(f16, K-major, 128 x 16) . B(f16, K-major, 256 x 16)^T */
__device__ __forceinline__ void
_mma_f16 (uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
  /* dtype F32 (bit 4), atype = btype = F16 (0), both K-major, N >> 3, M >> 4 */
  const uint32_t idesc = (1u << 4) | ((uint32_t) (TC_N >> 3) << 17) | ((uint32_t) (TC_M >> 4) << 24);

  asm volatile ("{\n\t.reg .pred p;\n\t"
                "setp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
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

/* 32 TMEM columns of this warp's lane quarter into r[0..31]; no wait */
__device__ __forceinline__ void
_tmem_ld32_async (uint32_t t, uint32_t *r)
{
  asm volatile ("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(t)
                : "memory");
}

/* wait for this thread's TMEM loads; r[0..31] are tied to the wait so that no
 * use of a loaded register can be scheduled before it */
__device__ __forceinline__ void
_tmem_wait32 (uint32_t *r)
{
  asm volatile ("tcgen05.wait::ld.sync.aligned;"
                : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                  "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                  "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                  "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                  "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
                :
                : "memory");
}

/* hi + lo FP16 split of an FP64 value (both halves as raw bits).  hi goes
 * through FP32 (hardware conversions only); whichever FP16 neighbour it lands
 * on, lo = fp16(v - hi) is formed from the exact FP64 remainder, so the pair
 * carries v to the rounding of lo. */
__device__ __forceinline__ void
_split16 (double v, uint16_t *hi, uint16_t *lo)
{
  const __half h = __float2half_rn ((float) v);
  const __half l = __float2half_rn ((float) (v - (double) __half2float (h)));

  *hi = __half_as_ushort (h);
  *lo = __half_as_ushort (l);
}

/* 2^e as FP64 / FP32 for the small exponents used here (normal range) */
__device__ __forceinline__ double
_pow2d (int e)
{
  return __longlong_as_double ((long long) (1023 + e) << 52);
}

__device__ __forceinline__ float
_pow2f (int e)
{
  return __int_as_float ((127 + e) << 23);
}

/* floor(log2 |x|) of a finite nonzero FP64 (subnormals read as -1023) */
__device__ __forceinline__ int
_exp2i (double x)
{
  return (int) ((__double_as_longlong (x) >> 52) & 0x7ff) - 1023;
}

__device__ __forceinline__ uint32_t
_pack2 (uint16_t a, uint16_t b)
{
  return (uint32_t) a | ((uint32_t) b << 16);
}

/* byte offset of row `row` of chunk q in a tile whose chunks are lbo bytes */
__device__ __forceinline__ uint32_t
_row_off (int q, int row, uint32_t lbo)
{
  return (uint32_t) (q * lbo + (row >> 3) * 128 + (row & 7) * 16);
}

/* ------------------------------------------------------------- operand packs */

/* A tiles: x' = Vg (x - mu) in FP64 (KDE: mu = NULL), scaled by 2^sx and split
 * into FP16 hi + lo, laid out as the windows' chunk pairs; xinv = 2^(-2 sx)
 * per point (-1: a point too far out for the FP16 range, reported as
 * -2 ln p = +inf).  A point takes a group of DPW lanes (dp rounded up to a
 * power of two), so a warp whitens 32 / DPW points at once: FP64 is a narrow
 * pipe on this part, and the triangular product runs as a fixed, unrolled
 * loop over the zero-padded matrix in shared memory (adding exact zeros, the
 * sum is the triangular one).  Rows past m are zero.  Also clears the merge
 * counters and the error word. */
#define TC_A_WARPS 8

template <int DP>
struct TcAShape
{
  static constexpr int DPW = DP <= 4 ? 4 : (DP <= 8 ? 8 : (DP <= 16 ? 16 : 32));   /* lanes per point  */
  static constexpr int PPW = 32 / DPW;                                            /* points per warp  */
  static constexpr int PB  = TC_A_WARPS * PPW;                                    /* points per block */
};

template <int DP>
__global__ void __launch_bounds__ (TC_A_WARPS * 32)
_build_tc_A_kernel (const double *__restrict__ Xq, int64_t m, int d, const double *__restrict__ mu,
                    const double *__restrict__ Vg, uint8_t *__restrict__ A, float *__restrict__ xinv, int64_t rows,
                    int *__restrict__ cnt, int ncnt, int *err)
{
  using S  = TcShape<DP>;
  using SA = TcAShape<DP>;
  constexpr int DPW = SA::DPW;
  __shared__ double V[DP][DP + 1];
  __shared__ double xs[SA::PB][DP];
  const int lane = threadIdx.x & 31, ps = lane / DPW, r = lane % DPW;
  const int pl   = (threadIdx.x >> 5) * SA::PPW + ps;
  const int64_t j = (int64_t) blockIdx.x * SA::PB + pl;

  for (int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; e < ncnt; e += (int64_t) gridDim.x * blockDim.x)
    cnt[e] = 0;

  if (blockIdx.x == 0 && threadIdx.x == 0)
    *err = 0;

  /* the packed lower factor, zero padded to a full matrix */
  for (int e = threadIdx.x; e < DP * DP; e += blockDim.x)
  {
    const int a = e / DP, c = e % DP;

    V[a][c] = (c <= a) ? Vg[a * (a + 1) / 2 + c] : 0.0;
  }

  /* coalesced staging of the block's points: element e = (point, coordinate) */
  for (int e = threadIdx.x; e < SA::PB * DP; e += blockDim.x)
  {
    const int p = e / DP, c = e % DP;
    const int64_t jj = (int64_t) blockIdx.x * SA::PB + p;

    xs[p][c] = (jj < m && c < d) ? Xq[jj * d + c] - (mu ? mu[c] : 0.0) : 0.0;
  }

  __syncthreads ();

  if (j >= rows)
    return;

  double v = 0.0;

  if (r < DP)
  {
#pragma unroll
    for (int c = 0; c < DP; c++)
      v = fma (V[r][c], xs[pl][c], v);
  }

  double mx = fabs (v);

#pragma unroll
  for (int o = DPW / 2; o > 0; o >>= 1)
    mx = fmax (mx, __shfl_xor_sync (0xffffffffu, mx, o));

  /* 2^sx puts the largest coordinate in [2^11, 2^12) */
  int sx     = (mx > 0.0) ? 11 - _exp2i (mx) : 14;
  bool far   = false;

  if (sx > 14)
    sx = 14;

  if (sx < -24)
  {
    sx  = -24;
    far = mx * _pow2d (sx) >= 16384.0;
  }

  uint16_t hi, lo;

  _split16 (far ? 0.0 : v * _pow2d (sx), &hi, &lo);

  const uint32_t hl = _pack2 (hi, lo);
  const uint16_t one = (j < m && !far) ? __half_as_ushort (__float2half_rn (_pow2f (sx + TC_BIAS_F))) : 0;

  /* lane r < 2 NW of the point's group writes row j of A chunk slot r (window
   * r / 2, half r % 2); the whole warp takes part in the shuffles that gather
   * the chunk's values from the group's coordinate lanes */
  const int slot = (r < 2 * S::NW) ? r : 0;
  const int code = tc_win_a (S::C, slot >> 1, slot & 1);
  const int src0 = (code >= TCA_XL) ? 8 * (code - TCA_XL) : ((code >= TCA_XH) ? 8 * (code - TCA_XH) : 0);
  uint16_t h[8];

#pragma unroll
  for (int e = 0; e < 8; e++)
  {
    const uint32_t w = __shfl_sync (0xffffffffu, hl, (ps * DPW + src0 + e) & 31);

    h[e] = (code >= TCA_XL) ? (uint16_t) (w >> 16) : ((code >= TCA_XH) ? (uint16_t) (w & 0xffffu) : 0);

    if (src0 + e >= DP)
      h[e] = 0;
  }

  if (code == TCA_ONE)
    h[0] = h[1] = one;                 /* times -b_hi and -b_lo */

  if (r < 2 * S::NW)
  {
    uint8_t *tile = A + (j / TC_M) * (int64_t) S::A_BYTES;
    const uint4 q = make_uint4 (_pack2 (h[0], h[1]), _pack2 (h[2], h[3]), _pack2 (h[4], h[5]), _pack2 (h[6], h[7]));

    *(uint4 *) (tile + _row_off (r, (int) (j % TC_M), TC_CHUNK_A)) = q;
  }

  if (r == 0)
    xinv[j] = (j >= m) ? 0.0f : (far ? -1.0f : _pow2f (-2 * sx));
}

/* B tiles from the mixed float pack (VKDE: theta'_hi, theta'_lo, W' packed
 * lower, c'; KDE: theta'_hi, theta'_lo, c').  Row = band * 64 + kk * DP + r
 * holds prescale * W'_kk[r][:] and the bias -b_r = -prescale W'_kk theta'_kk,
 * scaled by the tile's 2^sw and split into FP16 hi + lo (b from the split
 * weights the MMA sees, so y = W'(x' - theta') exactly in them); c2 = c'
 * log2(e), then 2^(-2 sw).  Padding kernels and the rest of a band get W = 0,
 * b = 0 and (kernels) c2 = -1e30. */
template <int DP, int KIND>
__global__ void __launch_bounds__ (TC_N)
_build_tc_B_kernel (const float *__restrict__ pk, int n, int smx, float prescale, uint8_t *__restrict__ B)
{
  using S = TcShape<DP>;
  __shared__ double red[2][TC_N / 32];
  const int t      = blockIdx.x;
  const int row    = threadIdx.x, lane = row & 31, wid = row >> 5;
  const int band   = row / 64, within = row % 64;
  const int kk     = within / DP, r = within % DP;
  const bool inb   = kk < S::KPW;
  const int i      = t * S::KT + band * S::KPW + kk;
  const bool valid = inb && i < n;
  uint8_t *tile    = B + (size_t) t * S::B_STRIDE;
  const float *src = pk + (size_t) (valid ? i : 0) * smx;
  float w[DP];
  double th[DP];
  double mw = 0.0, b0 = 0.0;

#pragma unroll
  for (int k = 0; k < DP; k++)
  {
    w[k]  = 0.0f;
    th[k] = valid ? (double) src[k] + (double) src[DP + k] : 0.0;

    if (valid && k <= r)
      w[k] = (KIND == NCG_VKDE) ? src[2 * DP + r * (r + 1) / 2 + k] * prescale : ((k == r) ? prescale : 0.0f);

    mw = fmax (mw, fabs ((double) w[k]));
    b0 += (double) w[k] * th[k];
  }

  /* the tile's largest weight and bias */
  double mb = fabs (b0);

#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    mw = fmax (mw, __shfl_xor_sync (0xffffffffu, mw, o));
    mb = fmax (mb, __shfl_xor_sync (0xffffffffu, mb, o));
  }

  if (lane == 0)
  {
    red[0][wid] = mw;
    red[1][wid] = mb;
  }

  __syncthreads ();

  mw = red[0][0];
  mb = red[1][0];

#pragma unroll
  for (int q = 1; q < TC_N / 32; q++)
  {
    mw = fmax (mw, red[0][q]);
    mb = fmax (mb, red[1][q]);
  }

  int sw = 0;

  if (mw > 0.0)
  {
    sw = 11 - _exp2i (mw);

    if (mb > 0.0 && 14 - _exp2i (mb) < sw)
      sw = 14 - _exp2i (mb);

    sw = sw < -60 ? -60 : (sw > 60 ? 60 : sw);
  }

  uint16_t wh[DP], wl[DP];
  double bsum = 0.0;

#pragma unroll
  for (int k = 0; k < DP; k++)
  {
    _split16 ((double) w[k] * _pow2d (sw), &wh[k], &wl[k]);
    bsum += ((double) __half2float (__ushort_as_half (wh[k])) + (double) __half2float (__ushort_as_half (wl[k]))) * th[k];
  }

  uint16_t bh, bl;

  _split16 (-bsum * _pow2d (-TC_BIAS_F), &bh, &bl);

  *(uint4 *) (tile + _row_off (0, row, TC_CHUNK_B)) = make_uint4 (_pack2 (bh, bl), 0u, 0u, 0u);

#pragma unroll
  for (int q = 0; q < S::C; q++)
  {
    uint16_t h[8], l[8];

#pragma unroll
    for (int e = 0; e < 8; e++)
    {
      h[e] = (8 * q + e < DP) ? wh[8 * q + e] : 0;
      l[e] = (8 * q + e < DP) ? wl[8 * q + e] : 0;
    }

    *(uint4 *) (tile + _row_off (1 + q, row, TC_CHUNK_B)) =
      make_uint4 (_pack2 (h[0], h[1]), _pack2 (h[2], h[3]), _pack2 (h[4], h[5]), _pack2 (h[6], h[7]));
    *(uint4 *) (tile + _row_off (1 + S::C + q, row, TC_CHUNK_B)) =
      make_uint4 (_pack2 (l[0], l[1]), _pack2 (l[2], l[3]), _pack2 (l[4], l[5]), _pack2 (l[6], l[7]));
  }

  float *c2 = (float *) (tile + S::C2_OFF);

  if (inb && r == 0)
  {
    const int coff = (KIND == NCG_VKDE) ? 2 * DP + DP * (DP + 1) / 2 : 2 * DP;

    c2[band * S::KPW + kk] = (i < n) ? src[coff] * LOG2E_F : -1.0e30f;
  }

  if (row == 0)
    c2[S::KT] = _pow2f (-2 * sw);
}

/* ------------------------------------------------------------------ the kernel */

struct TcParams
{
  const uint8_t *A;      /* point tiles  */
  const uint8_t *B;      /* kernel tiles */
  const float *xinv;     /* per point 2^(-2 sx), -1 for a point out of range */
  float2 *part;          /* [m][nparts]: EPI_WG partials per kernel slice */
  int *cnt;              /* [npt][4] partials written per 32-point quarter */
  int *err;              /* device error flag */
  int *flag_host;        /* mapped host word raised on error (may be NULL) */
  double *out;
  const double *cshift;  /* C0: the constant taken out of the log-weights */
  double final_shift, d_ln_href;
  int64_t m;
  int npt, nkt, nslices, tps, nparts;
  float kappa;           /* ST: -(nu + d)/2 */
  int fault;             /* wait-fault test hook: the copy warp issues nothing */
};

template <int DP>
struct TcSmem
{
  uint8_t A[2][TcShape<DP>::A_BYTES];
  uint8_t B[TcShape<DP>::STAGES][TcShape<DP>::B_STRIDE];
  uint64_t a_full[2], a_empty[2], b_full[TcShape<DP>::STAGES], b_empty[TcShape<DP>::STAGES], t_full[2], t_empty[2],
           done;
  uint32_t tmem_base;
  int err;
};

/* merge the 4 nslices partials of the 32 points of quarter q of point tile pt
 * (one point per lane): -2 ( ln2 (M + log2 S) + C0 - shift - d ln h ) */
__device__ __forceinline__ void
_merge_quarter (const TcParams &p, int pt, int q, int lane)
{
  const int64_t j = (int64_t) pt * TC_M + q * 32 + lane;

  if (j >= p.m)
    return;

  const int np       = p.nparts;
  const float2 *row  = p.part + (size_t) j * np;
  float M = -CUDART_INF_F, S = 0.0f;

  for (int s = 0; s < np; s++)
  {
    const float2 v = __ldcg (row + s);
    const float mn = fmaxf (M, v.x);

    S = ((M > -CUDART_INF_F) ? S * _ex2 (M - mn) : 0.0f) + ((v.x > -CUDART_INF_F) ? v.y * _ex2 (v.x - mn) : 0.0f);
    M = mn;
  }

  const float xi = __ldcg (p.xinv + j);

  p.out[j] = (xi < 0.0f) ? CUDART_INF
                         : -2.0 * (LN2_D * ((double) M + log2 ((double) S)) + *p.cshift - p.final_shift - p.d_ln_href);
}

template <int DP, int KERN>
__global__ void __launch_bounds__ (TcShape<DP>::THREADS, 1)
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
      _mbar_init (&sm.t_empty[b], 4 * S::EPI_WG);
    }

    for (int s = 0; s < STAGES; s++)
    {
      _mbar_init (&sm.b_full[s], 1);
      _mbar_init (&sm.b_empty[s], 1);         /* released by the MMA commit alone */
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
    if (lane == 0 && !p.fault)
    {
      int stage = 0, lu = 0;
      uint32_t bphase = 0;
      int armed_b[STAGES], armed_a[2];   /* parity of the last armed phase, -1 none */

      for (int s = 0; s < STAGES; s++)
        armed_b[s] = -1;

      armed_a[0] = armed_a[1] = -1;

      for (int u = blockIdx.x; u < nunits && !*err; u += gridDim.x, lu++)
      {
        const int pt = u % p.npt, sl = u / p.npt;
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

          _mbar_arrive_tx (&sm.b_full[stage], S::B_BYTES);
          _bulk_g2s (sm.B[stage], p.B + (size_t) t * S::B_STRIDE, S::B_BYTES, &sm.b_full[stage]);
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
        const int sl = u / p.npt;
        const int t0 = sl * p.tps, t1 = min (p.nkt, t0 + p.tps);
        const int ab = lu & 1;

        if (!_mbar_wait (&sm.a_full[ab], (lu >> 1) & 1, err))
          break;

        for (int t = t0; t < t1; t++, tc++)
        {
          const int tb = tc & 1;

          if (!_mbar_wait (&sm.b_full[stage], bphase, err))
            break;

          if (!_mbar_wait (&sm.t_empty[tb], ((tc >> 1) & 1) ^ 1, err))
            break;

          _tc_fence_after ();

          const uint32_t d = tmem + (uint32_t) (tb * TC_N);

#pragma unroll
          for (int w = 0; w < S::NW; w++)
            _mma_f16 (d, _sdesc (sm.A[ab] + 2 * w * TC_CHUNK_A, TC_CHUNK_A),
                      _sdesc (sm.B[stage] + tc_win_b0 (S::C, w) * TC_CHUNK_B, TC_CHUNK_B), w > 0 ? 1u : 0u);

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
    /* Every warpgroup works on every tile: warpgroup wg takes the KPWW
     * kernels of bands wg * BPW .. wg * BPW + BPW - 1 (64 TMEM columns each),
     * each warp the 32 points of its TMEM lane quarter. */
    constexpr int KPW  = S::KPW;
    constexpr int BPW  = S::BPW;
    constexpr int KPWW = S::KPWW;
    const int ew   = warp - TC_EPI_WARP0;
    const int wg   = ew >> 2;
    const int q    = warp & 3;                  /* TMEM lane quarter (hardware: warp id mod 4) */
    const int row  = q * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16) + (uint32_t) (wg * BPW * 64);
    int tc = 0;

    for (int u = blockIdx.x; u < nunits && !*err; u += gridDim.x)
    {
      const int pt = u % p.npt, sl = u / p.npt;
      const int t0 = sl * p.tps, t1 = min (p.nkt, t0 + p.tps);
      const float xi = p.xinv[(size_t) pt * TC_M + row];
      float m2 = -CUDART_INF_F, S2 = 0.0f;
      bool ok = true;

      /* the tile constants (c2 of this warp's kernels, 2^(-2 sw)) come from
       * the kernel tile in global memory (L1/L2), one tile ahead of their use */
      float c2n[KPWW], swn;

      {
        const float *g = (const float *) (p.B + (size_t) t0 * S::B_STRIDE + S::C2_OFF);

#pragma unroll
        for (int h = 0; h < KPWW; h++)
          c2n[h] = __ldg (g + KPWW * wg + h);

        swn = __ldg (g + S::KT);
      }

      for (int t = t0; t < t1; t++, tc++)
      {
        const int tb = tc & 1;
        float c2[KPWW], tv[KPWW];

#pragma unroll
        for (int h = 0; h < KPWW; h++)
          c2[h] = c2n[h];

        const float sc = xi * swn;              /* 2^(-2 sx - 2 sw) */

        /* prefetch the next tile's constants */
        if (t + 1 < t1)
        {
          const float *g = (const float *) (p.B + (size_t) (t + 1) * S::B_STRIDE + S::C2_OFF);

#pragma unroll
          for (int h = 0; h < KPWW; h++)
            c2n[h] = __ldg (g + KPWW * wg + h);

          swn = __ldg (g + S::KT);
        }

        /* the TMEM loads below are warp-collective: agree before issuing them */
        if (!__all_sync (0xffffffffu, _mbar_wait (&sm.t_full[tb], (tc >> 1) & 1, err)))
        {
          ok = false;
          break;
        }

        _tc_fence_after ();

        /* the warp's 64 BPW columns in two halves: the second half's loads
         * are in flight while the first half's kernels are computed */
        constexpr int HC = 32 * BPW;                 /* columns a half      */
        constexpr int KH = (BPW == 2) ? KPW : KPW / 2;   /* kernels in the first */
        uint32_t r[64 * BPW];

#pragma unroll
        for (int c = 0; c < HC; c += 32)
          _tmem_ld32_async (lane_base + (uint32_t) (tb * TC_N + c), r + c);

#pragma unroll
        for (int c = 0; c < HC; c += 32)
          _tmem_wait32 (r + c);

#pragma unroll
        for (int c = HC; c < 2 * HC; c += 32)
          _tmem_ld32_async (lane_base + (uint32_t) (tb * TC_N + c), r + c);

        auto kern = [&] (int h) {
          /* kernel h of the warp: band h / KPW, slot h % KPW of that band */
          const uint32_t *y = r + (h / KPW) * 64 + (h % KPW) * DP;
          /* 2^(2 sx + 2 sw) chi^2 (prescaled) = |y|^2, one packed FP32x2 FMA chain */
          float2 a = make_float2 (0.0f, 0.0f);

#pragma unroll
          for (int q2 = 0; q2 < DP; q2 += 2)
          {
            const float2 yy = make_float2 (__uint_as_float (y[q2]), __uint_as_float (y[q2 + 1]));

            a = __ffma2_rn (yy, yy, a);
          }

          const float s = a.x + a.y;

          tv[h] = (KERN == NCG_KERNEL_ST) ? fmaf (p.kappa, _lg2 (fmaf (s, sc, 1.0f)), c2[h]) : fmaf (-sc, s, c2[h]);
        };

#pragma unroll
        for (int h = 0; h < KH; h++)
          kern (h);

#pragma unroll
        for (int c = HC; c < 2 * HC; c += 32)
          _tmem_wait32 (r + c);

        _tc_fence_before ();
        __syncwarp ();

        if (lane == 0)
          _mbar_arrive (&sm.t_empty[tb]);

#pragma unroll
        for (int h = KH; h < KPWW; h++)
          kern (h);

        float mx = tv[0];

#pragma unroll
        for (int h = 1; h < KPWW; h++)
          mx = fmaxf (mx, tv[h]);

        const float mn = fmaxf (m2, mx);
        float acc = 0.0f;

#pragma unroll
        for (int h = 0; h < KPWW; h += 2)
          acc = acc + ((h + 1 < KPWW) ? (_ex2 (tv[h] - mn) + _ex2 (tv[h + 1] - mn)) : _ex2 (tv[h] - mn));

        S2 = S2 * _ex2 (m2 - mn) + acc;
        m2 = mn;
      }

      if (!ok)
        break;

      const int64_t j = (int64_t) pt * TC_M + row;

      /* point-major partials: (base-2 max, sum of 2^(t - max) incl. the max) */
      if (j < p.m)
        p.part[(size_t) j * p.nparts + S::EPI_WG * sl + wg] = make_float2 (m2, S2);

      /* the warp that writes the last partial of this quarter merges it: the
       * warp barrier orders its lanes' stores before lane 0's release fence
       * and count; the merging warp fences after seeing the final count */
      __syncwarp ();

      int last = 0;

      if (lane == 0)
      {
        asm volatile ("fence.acq_rel.gpu;" ::: "memory");
        last = atomicAdd (p.cnt + pt * 4 + q, 1) == p.nparts - 1;
      }

      if (__shfl_sync (0xffffffffu, last, 0))
      {
        asm volatile ("fence.acq_rel.gpu;" ::: "memory");
        _merge_quarter (p, pt, q, lane);

        if (lane == 0)
          p.cnt[pt * 4 + q] = 0;
      }
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
  {
    atomicExch (p.err, 1);

    if (p.flag_host != NULL)
      *(volatile int *) p.flag_host = 1;
  }
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

typedef struct { int kt, a_bytes, b_stride, epi_wg, threads; size_t smem; } tc_dims_t;

static int
_tc_dims (int dp, tc_dims_t *t)
{
  int ok = 0;

#define TC_DIMS(D)                                                            \
  do {                                                                        \
    t->kt = TcShape<D>::KT;                                                   \
    t->a_bytes = TcShape<D>::A_BYTES;                                         \
    t->b_stride = TcShape<D>::B_STRIDE;                                       \
    t->epi_wg = TcShape<D>::EPI_WG;                                           \
    t->threads = TcShape<D>::THREADS;                                         \
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

  return (size_t) ((n + t.kt - 1) / t.kt) * (size_t) t.b_stride;
}

#define TC_ALIGN(x) (((x) + 255) / 256 * 256)

/* scratch of one call: A tiles | partials | xinv | merge counters | error word */
typedef struct { size_t part, xinv, cnt, err, total; } tc_scratch_t;

static int
_tc_scratch (int64_t m, int n, int dp, tc_scratch_t *o, int *npt_out, int *ns_out, int *tps_out)
{
  tc_dims_t t;
  int ns, tps;

  if (!_tc_dims (dp, &t))
    return 0;

  const int npt = (int) ((m + TC_M - 1) / TC_M), nkt = (n + t.kt - 1) / t.kt;

  _tc_slicing (npt, nkt, 152, &ns, &tps);

  o->part  = TC_ALIGN ((size_t) npt * t.a_bytes);
  o->xinv  = o->part + TC_ALIGN ((size_t) t.epi_wg * ns * (size_t) m * sizeof (float2));
  o->cnt   = o->xinv + TC_ALIGN ((size_t) npt * TC_M * sizeof (float));
  o->err   = o->cnt + TC_ALIGN ((size_t) npt * 4 * sizeof (int));
  o->total = o->err + 256;

  if (npt_out)
  {
    *npt_out = npt;
    *ns_out  = ns;
    *tps_out = tps;
  }

  return 1;
}

extern "C" size_t
ncg_tc_scratch_bytes (int64_t m, int n, int dp)
{
  tc_scratch_t o;

  return _tc_scratch (m, n, dp, &o, NULL, NULL, NULL) ? o.total : 0;
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
  tc_scratch_t o;
  int npt, ns, tps, dev, nsm;
  cudaError_t e;

  if ((e = cudaGetDevice (&dev)) != cudaSuccess)
    return e;

  if ((e = cudaDeviceGetAttribute (&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return e;

  _tc_scratch (a->m, a->n, DP, &o, &npt, &ns, &tps);

  uint8_t *A         = (uint8_t *) scratch;
  float2 *part       = (float2 *) (A + o.part);
  float *xinv        = (float *) (A + o.xinv);
  int *cnt           = (int *) (A + o.cnt);
  int *err           = (int *) (A + o.err);
  const int64_t rows = (int64_t) npt * TC_M;

  _build_tc_A_kernel<DP><<<(unsigned) (rows / TcAShape<DP>::PB), TC_A_WARPS * 32, 0, s>>> (
    Xq, a->m, a->d, (a->kind == NCG_VKDE) ? mu : NULL, Vg, A, xinv, rows, cnt, npt * 4, err);

  TcParams p;

  p.A           = A;
  p.B           = B;
  p.xinv        = xinv;
  p.part        = part;
  p.cnt         = cnt;
  p.err         = err;
  p.flag_host   = flag_host;
  p.out         = out;
  p.cshift      = cshift;
  p.final_shift = a->final_shift;
  p.d_ln_href   = a->d_ln_href;
  p.m           = a->m;
  p.npt         = npt;
  p.nkt         = (a->n + S::KT - 1) / S::KT;
  p.nslices     = ns;
  p.tps         = tps;
  p.nparts      = S::EPI_WG * ns;
  p.kappa       = (float) a->kappa;
  p.fault       = ncg_fault_take (NCG_FAULT_EVAL_TC_WAIT);

  const size_t smem = sizeof (TcSmem<DP>) + 1024;
  void (*fn) (const TcParams) = (a->kernel == NCG_KERNEL_ST) ? _eval_tc_kernel<DP, NCG_KERNEL_ST>
                                                              : _eval_tc_kernel<DP, NCG_KERNEL_GAUSS>;

  /* the shared-memory opt-in, once per device and kernel variant */
  static int attr_done[64][2];
  const int kv = (a->kernel == NCG_KERNEL_ST) ? 1 : 0;

  if (dev >= 64 || !__atomic_load_n (&attr_done[dev][kv], __ATOMIC_ACQUIRE))
  {
    if ((e = cudaFuncSetAttribute (fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)) != cudaSuccess)
      return e;

    if (dev < 64)
      __atomic_store_n (&attr_done[dev][kv], 1, __ATOMIC_RELEASE);
  }

  const int units = npt * ns;
  const int grid  = units < nsm ? units : nsm;

  if (ev != NULL && (e = cudaEventRecord (ev[0], s)) != cudaSuccess)
    return e;

  fn<<<grid, S::THREADS, smem, s>>> (p);

  if ((e = cudaGetLastError ()) != cudaSuccess)
    return e;

  if (ev != NULL && (e = cudaEventRecord (ev[1], s)) != cudaSuccess)
    return e;

  return cudaSuccess;
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
