/*
 * ncg_syrk_tc.cuh -- the operand pack of the tensor-core symmetric rank-K
 * update (ncg_syrk_tc.cu): layout constants and the writers shared with the
 * FP32 Cholesky's panel solve (ncg_linalg.cu), which packs its panel as it
 * finishes it.
 *
 * For each 128-column tile t and 32-row K-chunk c the pack holds a 32 KB block
 * at ((t * nkc) + c) * 32 KB: the TF32 hi part of the 128 x 32 sub-matrix in
 * the K-major core-matrix layout of ncg_tc_ptx.cuh (LBO 2048), then the lo
 * part (value - hi, rounded to TF32).
 */
#ifndef NCG_SYRK_TC_CUH
#define NCG_SYRK_TC_CUH

#include "ncg_tc_ptx.cuh"

#define SK_T 128                     /* output tile edge (MMA M and N)       */
#define SK_KC 32                     /* K rows per chunk                     */
#define SK_LBO (SK_T / 8 * 128)      /* 2048: K-adjacent core matrices       */
#define SK_HALF (SK_KC / 4 * SK_LBO) /* 16 KB: hi (or lo) of a 128 x 32 block */
#define SK_BLOCK (2 * SK_HALF)       /* 32 KB per tile and chunk             */
#define SK_STAGE (2 * SK_BLOCK)      /* A block + B block                    */
/* one float4 of four consecutive k of column-row `row`, split hi / lo */
static __device__ __forceinline__ void
_put_split4 (float *blk, int row, int k4, double v0, double v1, double v2, double v3)
{
  const uint32_t off = _cm_off (row, k4, SK_LBO) >> 2;
  const float h0 = _tf32 ((float) v0), h1 = _tf32 ((float) v1), h2 = _tf32 ((float) v2), h3 = _tf32 ((float) v3);

  *(float4 *) (blk + off) = make_float4 (h0, h1, h2, h3);
  *(float4 *) (blk + SK_HALF / 4 + off) =
    make_float4 (_tf32 ((float) (v0 - (double) h0)), _tf32 ((float) (v1 - (double) h1)),
                 _tf32 ((float) (v2 - (double) h2)), _tf32 ((float) (v3 - (double) h3)));
}

/* column rel (0-based past the panel's diagonal block) of a 64-row panel
 * (nkc = 2) whose values are a[0..nb), into the pack pk */
static __device__ __forceinline__ void
_sk_pack_column (float *pk, int rel, const float *a, int nb)
{
  const int t = rel >> 7, row = rel & 127;

#pragma unroll
  for (int c = 0; c < 2; c++)
  {
    float *blk = pk + (size_t) (t * 2 + c) * (SK_BLOCK / 4);

#pragma unroll
    for (int q = 0; q < 8; q++)
    {
      const int k = c * SK_KC + 4 * q;

      _put_split4 (blk, row, 4 * q, (k + 0 < nb) ? a[k + 0] : 0.0f, (k + 1 < nb) ? a[k + 1] : 0.0f,
                   (k + 2 < nb) ? a[k + 2] : 0.0f, (k + 3 < nb) ? a[k + 3] : 0.0f);
    }
  }
}

#endif /* NCG_SYRK_TC_CUH */
