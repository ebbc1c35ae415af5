/*
 * ncg_linalg.cu -- dense kernels behind prepare_interp's NNLS
 * (ncm_nnls_solve, numcosmo/ncm/algebra/ncm_nnls.c:767-871, NORMAL umethod):
 *
 *   syrk_upper    M = A^T A, upper triangle (ncm_matrix_square_to_sym,
 *                 numcosmo/ncm/algebra/ncm_matrix.c:1548-1572); FP64, and an
 *                 FP32 copy for the mixed solver's preconditioner
 *   gemv          y = alpha op(A) x + beta y, deterministic reductions
 *   gather_sub    M[P,P], b[P] for an active set P (ncm_iset_get_submatrix)
 *   potrf         blocked right-looking Cholesky, upper, row-major (dpotrf),
 *                 FP64 and FP32
 *   potrs         U^T U x = b (dposv's solve), blocked over many CTAs
 *   residual_norm res = f - A x and |res|^2 (ncm_nnls.c:700-711)
 *   pcg_*         the FP64 conjugate-gradient refinement of the mixed solver
 *
 * Every reduction has a fixed order, so two runs give identical bits.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "ncg_internal.h"
#include "ncg_syrk_tc.cuh"

#define TB 64     /* output tile */
#define KB 16     /* rows per smem stage */

/* C[i][j] = (or -=) sum_{r in [r0, r1)} A[r][i] A[r][j] for off <= i <= j < off + nn.
 * TI is the storage type of A, T the arithmetic and output type. */
template <typename TI, typename T>
__global__ void __launch_bounds__ (256)
_syrk_tile_kernel (const TI *__restrict__ A, int lda, int r0, int r1, int off, int nn,
                   T *__restrict__ C, int ldc, int minus)
{
  __shared__ T As[KB][TB];
  __shared__ T Bs[KB][TB];

  /* map the linear block id onto the upper tiles (ti <= tj) */
  const int T_ = (nn + TB - 1) / TB;
  int b = blockIdx.x, ti = 0;

  while (b >= T_ - ti)
  {
    b -= T_ - ti;
    ti++;
  }

  const int tj  = ti + b;
  const int i0  = off + ti * TB, j0 = off + tj * TB;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int end = off + nn;
  T acc[4][4];

#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++)
      acc[a][c] = (T) 0;

  for (int rb = r0; rb < r1; rb += KB)
  {
    for (int e = tid; e < KB * TB; e += 256)
    {
      const int rr = e / TB, cc = e - rr * TB;
      const int r  = rb + rr;

      As[rr][cc] = (r < r1 && i0 + cc < end) ? (T) A[(size_t) r * lda + i0 + cc] : (T) 0;
      Bs[rr][cc] = (r < r1 && j0 + cc < end) ? (T) A[(size_t) r * lda + j0 + cc] : (T) 0;
    }

    __syncthreads ();

#pragma unroll
    for (int rr = 0; rr < KB; rr++)
    {
      T a[4], bb[4];

#pragma unroll
      for (int q = 0; q < 4; q++)
      {
        a[q]  = As[rr][ty * 4 + q];
        bb[q] = Bs[rr][tx * 4 + q];
      }

#pragma unroll
      for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++)
          acc[p][q] = fma (a[p], bb[q], acc[p][q]);
    }

    __syncthreads ();
  }

#pragma unroll
  for (int p = 0; p < 4; p++)
#pragma unroll
    for (int q = 0; q < 4; q++)
    {
      const int i = i0 + ty * 4 + p, j = j0 + tx * 4 + q;

      if (i < end && j < end && j >= i)
      {
        T *dst = C + (size_t) i * ldc + j;

        *dst = minus ? (*dst - acc[p][q]) : acc[p][q];
      }
    }
}

template <typename TI, typename T>
static cudaError_t
_syrk (const TI *A, int lda, int r0, int r1, int off, int nn, T *C, int ldc, int minus, cudaStream_t s)
{
  if (nn <= 0)
    return cudaSuccess;

  const int T_      = (nn + TB - 1) / TB;
  const int nblocks = T_ * (T_ + 1) / 2;

  _syrk_tile_kernel<TI, T><<<nblocks, 256, 0, s>>> (A, lda, r0, r1, off, nn, C, ldc, minus);

  return cudaGetLastError ();
}

/* FP32 products (the mixed solver's A^T A and its factor's trailing updates):
 * 128 x 128 upper tiles, 256 threads of 8 x 8 outputs (rows ty*4 + {0..3} and
 * 64 + ty*4 + {0..3}, columns likewise by tx), contraction rows staged 8 at a
 * time in double-buffered shared memory (the next chunk is loaded into
 * registers while the current one is used).  Each output is still one FMA
 * chain over the rows in ascending order, as in _syrk_tile_kernel. */
#define SY_T 128
#define SY_KB 8

template <typename TI>
__global__ void __launch_bounds__ (256)
_syrk128_f32_kernel (const TI *__restrict__ A, int lda, int r0, int r1, int off, int nn, float *__restrict__ C,
                     int ldc, int minus)
{
  __shared__ __align__ (16) float As[2][SY_KB][SY_T];
  __shared__ __align__ (16) float Bs[2][SY_KB][SY_T];

  const int T_ = (nn + SY_T - 1) / SY_T;
  int b = blockIdx.x, ti = 0;

  while (b >= T_ - ti)
  {
    b -= T_ - ti;
    ti++;
  }

  const int tj  = ti + b;
  const int i0  = off + ti * SY_T, j0 = off + tj * SY_T, end = off + nn;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int lr  = tid >> 5, lc = (tid & 31) * 4;      /* loader: row of the chunk, 4 columns */
  float acc[8][8];
  float ra[4], rb[4];

#pragma unroll
  for (int p = 0; p < 8; p++)
#pragma unroll
    for (int q = 0; q < 8; q++)
      acc[p][q] = 0.0f;

  /* chunk rows [rb0, rb0 + 8): this thread's row lr, columns lc..lc+3 */
#define SY_LOAD(rb0)                                                                          \
  do {                                                                                        \
    const int r_ = (rb0) + lr;                                                                \
    _Pragma ("unroll") for (int q = 0; q < 4; q++)                                            \
    {                                                                                         \
      ra[q] = (r_ < r1 && i0 + lc + q < end) ? (float) A[(size_t) r_ * lda + i0 + lc + q] : 0.0f; \
      rb[q] = (r_ < r1 && j0 + lc + q < end) ? (float) A[(size_t) r_ * lda + j0 + lc + q] : 0.0f; \
    }                                                                                         \
  } while (0)

  int buf = 0;

  SY_LOAD (r0);
  *(float4 *) &As[0][lr][lc] = make_float4 (ra[0], ra[1], ra[2], ra[3]);
  *(float4 *) &Bs[0][lr][lc] = make_float4 (rb[0], rb[1], rb[2], rb[3]);
  __syncthreads ();

  for (int rb0 = r0; rb0 < r1; rb0 += SY_KB)
  {
    const bool more = rb0 + SY_KB < r1;

    if (more)
      SY_LOAD (rb0 + SY_KB);

#pragma unroll
    for (int k = 0; k < SY_KB; k++)
    {
      const float4 a0 = *(const float4 *) &As[buf][k][ty * 4], a1 = *(const float4 *) &As[buf][k][64 + ty * 4];
      const float4 b0 = *(const float4 *) &Bs[buf][k][tx * 4], b1 = *(const float4 *) &Bs[buf][k][64 + tx * 4];
      const float a[8]  = { a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w };
      const float bb[8] = { b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w };

#pragma unroll
      for (int p = 0; p < 8; p++)
#pragma unroll
        for (int q = 0; q < 8; q++)
          acc[p][q] = fmaf (a[p], bb[q], acc[p][q]);
    }

    if (more)
    {
      *(float4 *) &As[buf ^ 1][lr][lc] = make_float4 (ra[0], ra[1], ra[2], ra[3]);
      *(float4 *) &Bs[buf ^ 1][lr][lc] = make_float4 (rb[0], rb[1], rb[2], rb[3]);
    }

    __syncthreads ();
    buf ^= 1;
  }

#undef SY_LOAD

#pragma unroll
  for (int p = 0; p < 8; p++)
  {
    const int i = i0 + ((p < 4) ? ty * 4 + p : 64 + ty * 4 + p - 4);

#pragma unroll
    for (int q = 0; q < 8; q++)
    {
      const int j = j0 + ((q < 4) ? tx * 4 + q : 64 + tx * 4 + q - 4);

      if (i < end && j < end && j >= i)
      {
        float *dst = C + (size_t) i * ldc + j;

        *dst = minus ? (*dst - acc[p][q]) : acc[p][q];
      }
    }
  }
}

template <typename TI>
static cudaError_t
_syrk128 (const TI *A, int lda, int r0, int r1, int off, int nn, float *C, int ldc, int minus, cudaStream_t s)
{
  if (nn <= 0 || r1 <= r0)
    return cudaSuccess;

  const int T_ = (nn + SY_T - 1) / SY_T;

  _syrk128_f32_kernel<TI><<<T_ * (T_ + 1) / 2, 256, 0, s>>> (A, lda, r0, r1, off, nn, C, ldc, minus);

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_syrk_upper (const double *A, int nrows, int ncols, double *M, cudaStream_t s)
{
  return _syrk<double, double> (A, ncols, 0, nrows, 0, ncols, M, ncols, 0, s);
}

extern "C" cudaError_t
ncg_launch_syrk_upper_f32 (const double *A, int nrows, int ncols, float *M, cudaStream_t s)
{
  return _syrk128<double> (A, ncols, 0, nrows, 0, ncols, M, ncols, 0, s);
}

/* ---- gemv --------------------------------------------------------------- */

/* y[r] = alpha sum_c A[r][c] x[c] + beta y[r]; one warp per row */
__global__ void
_gemv_n_kernel (const double *__restrict__ A, int nrows, int ncols, double alpha, const double *__restrict__ x,
                double beta, double *__restrict__ y)
{
  const int lane = threadIdx.x & 31;
  const int r    = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;

  if (r >= nrows)
    return;

  const double *a = A + (size_t) r * ncols;
  double s        = 0.0;

  for (int c = lane; c < ncols; c += 32)
    s = fma (a[c], x[c], s);

#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    s += __shfl_xor_sync (0xffffffffu, s, o);

  if (lane == 0)
    y[r] = (beta == 0.0) ? alpha * s : fma (beta, y[r], alpha * s);
}

#define GT_ROWS 256

/* part[rb][c] = sum over rows of block rb of A[r][c] x[r] */
__global__ void
_gemv_t_partial_kernel (const double *__restrict__ A, int nrows, int ncols, const double *__restrict__ x,
                        double *__restrict__ part)
{
  const int c  = blockIdx.x * blockDim.x + threadIdx.x;
  const int rb = blockIdx.y;

  if (c >= ncols)
    return;

  const int r0 = rb * GT_ROWS, r1 = min (nrows, r0 + GT_ROWS);
  double s     = 0.0;

  for (int r = r0; r < r1; r++)
    s = fma (A[(size_t) r * ncols + c], x[r], s);

  part[(size_t) rb * ncols + c] = s;
}

__global__ void
_gemv_t_final_kernel (const double *__restrict__ part, int nrb, int ncols, double alpha, double beta,
                      double *__restrict__ y)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;

  if (c >= ncols)
    return;

  double s = 0.0;

  for (int rb = 0; rb < nrb; rb++)
    s += part[(size_t) rb * ncols + c];

  y[c] = (beta == 0.0) ? alpha * s : fma (beta, y[c], alpha * s);
}

extern "C" size_t
ncg_gemv_t_scratch (int nrows, int ncols)
{
  return (size_t) ((nrows + GT_ROWS - 1) / GT_ROWS) * (size_t) ncols * sizeof (double);
}

extern "C" cudaError_t
ncg_launch_gemv_ex (const double *A, int nrows, int ncols, int trans, double alpha, const double *x, double beta,
                    double *y, double *part, cudaStream_t s)
{
  if (!trans)
  {
    const int th = 256;

    _gemv_n_kernel<<<(unsigned) (((size_t) nrows * 32 + th - 1) / th), th, 0, s>>> (A, nrows, ncols, alpha, x, beta, y);
  }
  else
  {
    const int nrb = (nrows + GT_ROWS - 1) / GT_ROWS;
    dim3 g ((ncols + 127) / 128, nrb);

    _gemv_t_partial_kernel<<<g, 128, 0, s>>> (A, nrows, ncols, x, part);
    _gemv_t_final_kernel<<<(ncols + 255) / 256, 256, 0, s>>> (part, nrb, ncols, alpha, beta, y);
  }

  return cudaGetLastError ();
}

/* ---- active-set gather / scatter ----------------------------------------- */

__global__ void
_gather_kernel (const double *__restrict__ M, int n, const int32_t *__restrict__ P, int np,
                double *__restrict__ Msub, const double *__restrict__ b, double *__restrict__ bsub)
{
  const int a = blockIdx.y;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;

  if (a >= np)
    return;

  const size_t ra = (size_t) P[a] * n;

  for (int bb = c; bb < np; bb += gridDim.x * blockDim.x)
    Msub[(size_t) a * np + bb] = (bb >= a) ? M[ra + P[bb]] : 0.0;

  if (c == 0)
    bsub[a] = b[P[a]];
}

extern "C" cudaError_t
ncg_launch_gather_sub (const double *M, int n, const int32_t *P, int np, double *Msub, const double *b,
                       double *bsub, cudaStream_t s)
{
  if (np <= 0)
    return cudaSuccess;

  dim3 g ((np + 255) / 256 < 8 ? (np + 255) / 256 : 8, np);

  _gather_kernel<<<g, 256, 0, s>>> (M, n, P, np, Msub, b, bsub);

  return cudaGetLastError ();
}

/* The mixed solver's preconditioner operand, in two launches: Dsub[a] =
 * 1/sqrt(diagM[P_a]) (Jacobi scaling, FP64) and bsub[a] = b[P_a]; then
 * Msub[a][b] = D_a M32[P_a][P_b] D_b in FP32, upper triangle only, with the
 * unit diagonal raised by `shift`. */
__global__ void
_scale_vec_kernel (const int32_t *__restrict__ P, int np, const double *__restrict__ diagM,
                   double *__restrict__ Dsub, const double *__restrict__ b, double *__restrict__ bsub)
{
  const int a = blockIdx.x * blockDim.x + threadIdx.x;

  if (a < np)
  {
    const int pa = P[a];

    Dsub[a] = 1.0 / sqrt (diagM[pa]);
    bsub[a] = b[pa];
  }
}

__global__ void
_gather_scaled_kernel (const float *__restrict__ M32, int n, const int32_t *__restrict__ P, int np,
                       const double *__restrict__ Dsub, float shift, float *__restrict__ Msub)
{
  const int a = blockIdx.y;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;

  if (a >= np)
    return;

  const float *row = M32 + (size_t) P[a] * n;
  const float Da   = (float) Dsub[a];

  for (int bb = c; bb < np; bb += gridDim.x * blockDim.x)
  {
    float v = 0.0f;

    if (bb > a)
      v = (Da * row[P[bb]]) * (float) Dsub[bb];
    else if (bb == a)
      v = (Da * row[P[bb]]) * Da * (1.0f + shift);

    Msub[(size_t) a * np + bb] = v;
  }
}

extern "C" cudaError_t
ncg_launch_gather_scaled_f32 (const float *M32, int n, const int32_t *P, int np, const double *diagM, double shift,
                              float *Msub, double *Dsub, const double *b, double *bsub, cudaStream_t s)
{
  if (np <= 0)
    return cudaSuccess;

  dim3 g ((np + 255) / 256 < 8 ? (np + 255) / 256 : 8, np);

  _scale_vec_kernel<<<(np + 255) / 256, 256, 0, s>>> (P, np, diagM, Dsub, b, bsub);
  _gather_scaled_kernel<<<g, 256, 0, s>>> (M32, n, P, np, Dsub, (float) shift, Msub);

  return cudaGetLastError ();
}

/* diagM[c] = sum_r A[r][c]^2, the FP64 diagonal of A^T A */
__global__ void
_colsumsq_kernel (const double *__restrict__ A, int nrows, int ncols, double *__restrict__ out)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;

  if (c >= ncols)
    return;

  double s = 0.0;

  for (int r = 0; r < nrows; r++)
  {
    const double v = A[(size_t) r * ncols + c];

    s = fma (v, v, s);
  }

  out[c] = s;
}

extern "C" cudaError_t
ncg_launch_colsumsq (const double *A, int nrows, int ncols, double *out, cudaStream_t s)
{
  _colsumsq_kernel<<<(ncols + 127) / 128, 128, 0, s>>> (A, nrows, ncols, out);

  return cudaGetLastError ();
}

__global__ void
_scatter_kernel (const double *__restrict__ xsub, const int32_t *__restrict__ P, int np, int n, double *__restrict__ x)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;

  if (i < n)
    x[i] = 0.0;
}

__global__ void
_scatter2_kernel (const double *__restrict__ xsub, const int32_t *__restrict__ P, int np, double *__restrict__ x)
{
  const int a = blockIdx.x * blockDim.x + threadIdx.x;

  if (a < np)
    x[P[a]] = xsub[a];
}

extern "C" cudaError_t
ncg_launch_scatter_x (const double *xsub, const int32_t *P, int np, int n, double *x, cudaStream_t s)
{
  _scatter_kernel<<<(n + 255) / 256, 256, 0, s>>> (xsub, P, np, n, x);

  if (np > 0)
    _scatter2_kernel<<<(np + 255) / 256, 256, 0, s>>> (xsub, P, np, x);

  return cudaGetLastError ();
}

__global__ void
_gather_vec_kernel (const double *__restrict__ xf, const int32_t *__restrict__ P, int np, double *__restrict__ xs)
{
  const int a = blockIdx.x * blockDim.x + threadIdx.x;

  if (a < np)
    xs[a] = xf[P[a]];
}

/* ---- blocked Cholesky ------------------------------------------------------ */

#define PB 64

/* S[r][c] = A[(r0 + r) ld + c0 + c] for r, c < nb (zero elsewhere), B x B
 * block, NT threads; the loads go out in batches of up to 32 per thread so
 * that they overlap instead of waiting for one another */
template <typename T, int NT, int B>
__device__ __forceinline__ void
_stage_block (T (*S)[B + 1], const T *__restrict__ A, int ld, int r0, int c0, int nb, int tid)
{
  constexpr int PER = (B * B + NT - 1) / NT;
  constexpr int CH  = (PER < 32) ? PER : 32;

#pragma unroll
  for (int k0 = 0; k0 < PER; k0 += CH)
  {
    T v[CH];

#pragma unroll
    for (int k = 0; k < CH; k++)
    {
      const int e = tid + (k0 + k) * NT;
      const int r = e / B, c = e % B;

      v[k] = (e < B * B && r < nb && c < nb) ? A[(size_t) (r0 + r) * ld + c0 + c] : (T) 0;
    }

#pragma unroll
    for (int k = 0; k < CH; k++)
    {
      const int e = tid + (k0 + k) * NT;

      if (e < B * B)
        S[e / B][e % B] = v[k];
    }
  }
}

/* factor the nb x nb diagonal block at (kb, kb) in place (upper), right-looking
 * inside shared memory: at step j the row j is final, scaled by 1/U_jj, and
 * the trailing block takes the rank-1 update in ascending j order.  Thread
 * (ty, tx) of the 16 x 16 block owns the elements (ty + 16p, tx + 16q), which
 * spreads the shrinking trailing triangle over all threads.  Two barriers a
 * step: the diagonal read and the row scaling, then the update (which also
 * stores U_jj, read by nobody in that phase). */
template <typename T>
__global__ void __launch_bounds__ (256)
_potrf_diag_kernel (T *A, int ld, int kb, int nb, int32_t *info)
{
  __shared__ T S[PB][PB + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  int fail      = 0;

  if (*info)
    return;

  _stage_block<T, 256, PB> (S, A, ld, kb, kb, nb, tid);

  __syncthreads ();

  for (int j = 0; j < nb; j++)
  {
    const T ajj = S[j][j];

    if (!(ajj > (T) 0))
    {
      fail = j + 1;
      break;
    }

    const T ujj = sqrt (ajj);

    /* FP32 (the preconditioner's factor): one reciprocal, then products,
     * within an ulp of the quotients; FP64 keeps the quotients */
    if constexpr (sizeof (T) == sizeof (float))
    {
      const float ri = __frcp_rn (ujj);

      if (tid > j && tid < nb)
        S[j][tid] = S[j][tid] * ri;
    }
    else if (tid > j && tid < nb)
      S[j][tid] = S[j][tid] / ujj;

    __syncthreads ();

    if (tid == 0)
      S[j][j] = ujj;

#pragma unroll
    for (int p = 0; p < PB / 16; p++)
    {
      const int r = ty + 16 * p;

      if (r > j && r < nb)
      {
        const T sjr = S[j][r];

#pragma unroll
        for (int q = 0; q < PB / 16; q++)
        {
          const int c = tx + 16 * q;

          if (c >= r && c < nb)
            S[r][c] = fma (-sjr, S[j][c], S[r][c]);
        }
      }
    }

    __syncthreads ();
  }

  if (fail)
  {
    if (tid == 0)
      atomicCAS (info, 0, kb + fail);

    return;
  }

  for (int e = tid; e < nb * nb; e += 256)
  {
    const int r = e / nb, c = e - r * nb;

    if (c >= r)
      A[(size_t) (kb + r) * ld + kb + c] = S[r][c];
  }
}

/* rows kb..kb+nb of the columns right of the block: X = U_kk^{-T} A_panel,
 * one column per thread held in registers (column sweep in ascending row
 * order) */
#define TRSM_TH 128

template <typename T>
__global__ void __launch_bounds__ (TRSM_TH)
_potrf_trsm_kernel (T *A, int ld, int kb, int nb, int n, const int32_t *info, float *pk)
{
  __shared__ T S[PB][PB + 1];
  const int tid = threadIdx.x;

  if (*info)
    return;

  _stage_block<T, TRSM_TH, PB> (S, A, ld, kb, kb, nb, tid);

  __syncthreads ();

  const int col = kb + nb + blockIdx.x * TRSM_TH + tid;

  if (col >= n)
    return;

  T a[PB];

#pragma unroll
  for (int r = 0; r < PB; r++)
    a[r] = (r < nb) ? A[(size_t) (kb + r) * ld + col] : (T) 0;

#pragma unroll
  for (int r = 0; r < PB; r++)
  {
    if (r < nb)
    {
      if constexpr (sizeof (T) == sizeof (float))
        a[r] = a[r] * __frcp_rn (S[r][r]);   /* FP32: reciprocal products, as the diagonal factor */
      else
        a[r] = a[r] / S[r][r];

#pragma unroll
      for (int m = r + 1; m < PB; m++)
        a[m] = fma (-S[r][m], a[r], a[m]);
    }
  }

#pragma unroll
  for (int r = 0; r < PB; r++)
    if (r < nb)
      A[(size_t) (kb + r) * ld + col] = a[r];

  /* the panel as the tensor-core trailing update's operand */
  if constexpr (sizeof (T) == sizeof (float))
    if (pk != NULL)
      _sk_pack_column (pk, col - kb - nb, (const float *) a, nb);
}

__global__ void
_zero_int_kernel (int32_t *p)
{
  *p = 0;
}

/* trailing blocks at least this wide take the tensor-core update (FP32 with a pack) */
#define POTRF_TC_MIN 1024

template <typename T>
static cudaError_t
_potrf (T *A, int n, int32_t *info, float *pk, cudaStream_t s)
{
  _zero_int_kernel<<<1, 1, 0, s>>> (info);

  for (int kb = 0; kb < n; kb += PB)
  {
    const int nb = (n - kb < PB) ? n - kb : PB;

    _potrf_diag_kernel<T><<<1, 256, 0, s>>> (A, n, kb, nb, info);

    if (kb + nb < n)
    {
      const int rest = n - kb - nb;
      const bool tc  = sizeof (T) == sizeof (float) && pk != NULL && rest >= POTRF_TC_MIN;

      _potrf_trsm_kernel<T><<<(rest + TRSM_TH - 1) / TRSM_TH, TRSM_TH, 0, s>>> (A, n, kb, nb, n, info,
                                                                                tc ? pk : NULL);

      cudaError_t e;

      /* FP32: TF32x3 tensor-core tiles for the large updates (pack written by
       * the panel solve), else 128-wide then 64-wide CUDA-core tiles */
      if constexpr (sizeof (T) == sizeof (float))
        e = tc ? ncg_launch_syrk_tc (pk, nb, rest, (float *) A + (size_t) (kb + nb) * n + kb + nb, n, 1, info, s)
               : (rest >= 2048) ? _syrk128<float> ((const float *) A, n, kb, kb + nb, kb + nb, rest, (float *) A, n, 1, s)
                                : _syrk<T, T> (A, n, kb, kb + nb, kb + nb, rest, A, n, 1, s);
      else
        e = _syrk<T, T> (A, n, kb, kb + nb, kb + nb, rest, A, n, 1, s);

      if (e != cudaSuccess)
        return e;
    }
  }

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_potrf (double *A, int n, int32_t *info, double *work, cudaStream_t s)
{
  (void) work;

  return _potrf<double> (A, n, info, NULL, s);
}

extern "C" cudaError_t
ncg_launch_potrf_f32 (float *A, int n, int32_t *info, float *pk, cudaStream_t s)
{
  return _potrf<float> (A, n, info, pk, s);
}

/* ---- blocked triangular solves ------------------------------------------- */

#define SB 64     /* diagonal block of the solves */
#define SV_TH 128

/* U^T y = b, block [kb, kb+nb): every CTA stages the diagonal block in shared
 * memory and solves it from the (final) b_k with one warp (lanes own y_l and
 * y_{l+32}), CTA 0 stores y_k into y, and each CTA subtracts the block's
 * contribution from its slice of b past the block, in ascending row order
 * (the operation order of a plain column sweep).  b_k is read by every CTA
 * and written by none, so the launch has no race. */
template <typename T>
__global__ void __launch_bounds__ (SV_TH)
_trsv_t_kernel (const T *__restrict__ U, int n, int kb, int nb, T *__restrict__ b, T *__restrict__ yout)
{
  __shared__ T S[SB][SB + 1];
  __shared__ T y[SB];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

  _stage_block<T, SV_TH, SB> (S, U, n, kb, kb, nb, tid);

  __syncthreads ();

  if (wid == 0)
  {
    T y0 = (lane < nb) ? b[kb + lane] : (T) 0;
    T y1 = (lane + 32 < nb) ? b[kb + lane + 32] : (T) 0;

    for (int r = 0; r < nb; r++)
    {
      const T yraw = __shfl_sync (0xffffffffu, (r < 32) ? y0 : y1, r & 31);
      const T yr   = yraw / S[r][r];

      if (r < 32)
      {
        if (lane == r)
          y0 = yr;
      }
      else if (lane == r - 32)
      {
        y1 = yr;
      }

      if (lane > r && lane < nb)
        y0 = fma (-S[r][lane], yr, y0);

      if (lane + 32 > r && lane + 32 < nb)
        y1 = fma (-S[r][lane + 32], yr, y1);
    }

    y[lane] = y0;

    if (lane + 32 < SB)
      y[lane + 32] = y1;
  }

  __syncthreads ();

  if (blockIdx.x == 0 && tid < nb)
    yout[kb + tid] = y[tid];

  const int i = kb + nb + blockIdx.x * SV_TH + tid;

  if (i < n)
  {
    T bi = b[i];

#pragma unroll 16
    for (int r = 0; r < nb; r++)
      bi = fma (-U[(size_t) (kb + r) * n + i], y[r], bi);

    b[i] = bi;
  }
}

/* U x = y, block [kb, kb+nb) (blocks taken from the last): every CTA stages
 * the diagonal block and solves it by back substitution from the (final)
 * y_k with one warp, CTA 0 stores x_k into x, and the rows of y before the
 * block take the block's contribution, one warp per row. */
template <typename T>
__global__ void __launch_bounds__ (SV_TH)
_trsv_n_kernel (const T *__restrict__ U, int n, int kb, int nb, T *__restrict__ yv, T *__restrict__ xout)
{
  __shared__ T S[SB][SB + 1];
  __shared__ T x[SB];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

  _stage_block<T, SV_TH, SB> (S, U, n, kb, kb, nb, tid);

  __syncthreads ();

  if (wid == 0)
  {
    T x0 = (lane < nb) ? yv[kb + lane] : (T) 0;
    T x1 = (lane + 32 < nb) ? yv[kb + lane + 32] : (T) 0;

    for (int r = nb - 1; r >= 0; r--)
    {
      const T xraw = __shfl_sync (0xffffffffu, (r < 32) ? x0 : x1, r & 31);
      const T xr   = xraw / S[r][r];

      if (r < 32)
      {
        if (lane == r)
          x0 = xr;
      }
      else if (lane == r - 32)
      {
        x1 = xr;
      }

      if (lane < r)
        x0 = fma (-S[lane][r], xr, x0);

      if (lane + 32 < r)
        x1 = fma (-S[lane + 32][r], xr, x1);
    }

    x[lane] = x0;

    if (lane + 32 < SB)
      x[lane + 32] = x1;
  }

  __syncthreads ();

  if (blockIdx.x == 0 && tid < nb)
    xout[kb + tid] = x[tid];

  const int row = blockIdx.x * (SV_TH / 32) + wid;

  if (row < kb)
  {
    const T *u = U + (size_t) row * n + kb;
    T s        = (T) 0;

    for (int c = lane; c < nb; c += 32)
      s = fma (u[c], x[c], s);

#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      s += __shfl_xor_sync (0xffffffffu, s, o);

    if (lane == 0)
      yv[row] -= s;
  }
}

/* U^T U x = b: b is the right-hand side on entry and the solution on exit,
 * work an n-long scratch vector */
template <typename T>
static cudaError_t
_potrs (const T *U, int n, T *b, T *work, cudaStream_t s)
{
  for (int kb = 0; kb < n; kb += SB)
  {
    const int nb   = (n - kb < SB) ? n - kb : SB;
    const int rest = n - kb - nb;
    const int g    = (rest + SV_TH - 1) / SV_TH;

    _trsv_t_kernel<T><<<g > 0 ? g : 1, SV_TH, 0, s>>> (U, n, kb, nb, b, work);
  }

  const int last = ((n - 1) / SB) * SB;

  for (int kb = last; kb >= 0; kb -= SB)
  {
    const int nb = (n - kb < SB) ? n - kb : SB;
    const int g  = (kb + SV_TH / 32 - 1) / (SV_TH / 32);

    _trsv_n_kernel<T><<<g > 0 ? g : 1, SV_TH, 0, s>>> (U, n, kb, nb, work, b);
  }

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_potrs (const double *U, int n, double *b, double *work, cudaStream_t s)
{
  if (n <= 0)
    return cudaSuccess;

  return _potrs<double> (U, n, b, work, s);
}

/* ---- residuals --------------------------------------------------------- */

__global__ void
_sumsq_kernel (const double *__restrict__ v, int n, double *__restrict__ out)
{
  __shared__ double red[1024];
  double s = 0.0;

  for (int i = threadIdx.x; i < n; i += blockDim.x)
    s = fma (v[i], v[i], s);

  red[threadIdx.x] = s;
  __syncthreads ();

  for (int st = blockDim.x / 2; st > 0; st >>= 1)
  {
    if (threadIdx.x < st)
      red[threadIdx.x] += red[threadIdx.x + st];

    __syncthreads ();
  }

  if (threadIdx.x == 0)
    *out = red[0];
}

extern "C" cudaError_t
ncg_launch_residual_norm (const double *A, int nrows, int ncols, const double *x, const double *f, double *res,
                          double *rnorm2, cudaStream_t s)
{
  cudaError_t e = cudaMemcpyAsync (res, f, sizeof (double) * nrows, cudaMemcpyDeviceToDevice, s);

  if (e != cudaSuccess)
    return e;

  e = ncg_launch_gemv_ex (A, nrows, ncols, 0, -1.0, x, 1.0, res, NULL, s);

  if (e != cudaSuccess)
    return e;

  _sumsq_kernel<<<1, 1024, 0, s>>> (res, nrows, rnorm2);

  return cudaGetLastError ();
}

/* ---- weight normalisation (ncm_stats_dist.c:1086-1093) ------------------- */

__global__ void
_normalize_weights_kernel (double *w, int n, double shrink, int32_t *bad)
{
  __shared__ double sc, ad;

  if (threadIdx.x == 0)
  {
    double total = 0.0;

    for (int i = 0; i < n; i++)
      total += w[i];

    *bad = !(total > 0.0);
    sc   = (1.0 - shrink) / total;
    ad   = shrink / n;
  }

  __syncthreads ();

  for (int i = threadIdx.x; i < n; i += blockDim.x)
    w[i] = __dadd_rn (__dmul_rn (w[i], sc), ad);
}

extern "C" cudaError_t
ncg_launch_normalize_weights (double *w, int n, double shrink, int32_t *bad, cudaStream_t s)
{
  _normalize_weights_kernel<<<1, 1024, 0, s>>> (w, n, shrink, bad);

  return cudaGetLastError ();
}

/* ---- mixed solver: FP32 preconditioned FP64 conjugate gradients ----------
 *
 * Solves the active-set normal equations A_P^T A_P x = A_P^T 1 with the
 * products taken from A in FP64 (so the residual is an FP64 residual of the
 * reference's own system) and the preconditioner D R^{-1} R^{-T} D from the
 * FP32 Cholesky factor R of the Jacobi-scaled D (A^T A)_P D.  The conjugate
 * direction uses the flexible (Polak-Ribiere) beta, which stays robust when
 * the FP32 preconditioner is not exactly linear.  The scalars live on the
 * device (sc[]), so an iteration needs no host round trip; the host reads
 * sc[PCG_RR] to decide when to stop.
 */

#define PCG_THREADS 1024

/* sc[out0] = <u0, v0> (and sc[out1] = <u1, v1> when u1 != NULL); one CTA,
 * fixed reduction order */
__global__ void __launch_bounds__ (PCG_THREADS)
_dot2_kernel (const double *__restrict__ u0, const double *__restrict__ v0, const double *__restrict__ u1,
              const double *__restrict__ v1, const double *__restrict__ w, int n, double *sc, int out0, int out1)
{
  __shared__ double r0[PCG_THREADS / 32], r1[PCG_THREADS / 32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  double s0 = 0.0, s1 = 0.0;

  for (int i = tid; i < n; i += PCG_THREADS)
  {
    const double wi = (w != NULL) ? w[i] * w[i] : 1.0;

    s0 = fma (u0[i] * wi, v0[i], s0);

    if (u1 != NULL)
      s1 = fma (u1[i], v1[i], s1);
  }

#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    s0 += __shfl_xor_sync (0xffffffffu, s0, o);
    s1 += __shfl_xor_sync (0xffffffffu, s1, o);
  }

  if (lane == 0)
  {
    r0[wid] = s0;
    r1[wid] = s1;
  }

  __syncthreads ();

  if (tid == 0)
  {
    double t0 = 0.0, t1 = 0.0;

    for (int k = 0; k < PCG_THREADS / 32; k++)
    {
      t0 += r0[k];
      t1 += r1[k];
    }

    sc[out0] = t0;

    if (u1 != NULL)
      sc[out1] = t1;
  }
}

/* x += alpha p, r_prev = r, r -= alpha q with alpha = sc[RZ] / sc[PQ] */
__global__ void
_pcg_step_kernel (double *__restrict__ x, double *__restrict__ r, double *__restrict__ rprev,
                  const double *__restrict__ p, const double *__restrict__ q, int n, const double *sc)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;

  if (i >= n)
    return;

  const double al = sc[NCG_PCG_RZ] / sc[NCG_PCG_PQ];
  const double ri = r[i];

  x[i]     = fma (al, p[i], x[i]);
  rprev[i] = ri;
  r[i]     = fma (-al, q[i], ri);
}

/* p = z + beta p with beta = (sc[RZN] - sc[ZRP]) / sc[RZ]; the following
 * _pcg_shift_kernel launch then sets sc[RZ] = sc[RZN] */
__global__ void
_pcg_dir_kernel (double *__restrict__ p, const double *__restrict__ z, int n, const double *sc)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;

  if (i >= n)
    return;

  const double be = (sc[NCG_PCG_RZN] - sc[NCG_PCG_ZRP]) / sc[NCG_PCG_RZ];

  p[i] = fma (be, p[i], z[i]);
}

__global__ void
_pcg_shift_kernel (double *sc)
{
  sc[NCG_PCG_RZ] = sc[NCG_PCG_RZN];
}

/* r = b - r (turns r = A_P^T A_P x into the residual) */
__global__ void
_rsub_kernel (const double *__restrict__ b, double *__restrict__ r, int n)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;

  if (i < n)
    r[i] = b[i] - r[i];
}

#define VB(n) (((n) + 255) / 256), 256

/* q = A_P^T (A_P v) for a compact v on the set P (np entries), A nrows x n;
 * vf and qf are n-long work vectors, yf nrows-long, part the transposed-gemv
 * scratch */
extern "C" cudaError_t
ncg_launch_pcg_matvec (const double *A, int nrows, int n, const int32_t *P, int np, const double *v, double *vf,
                       double *yf, double *qf, double *part, double *q, cudaStream_t s)
{
  cudaError_t e = ncg_launch_scatter_x (v, P, np, n, vf, s);

  if (e == cudaSuccess)
    e = ncg_launch_gemv_ex (A, nrows, n, 0, 1.0, vf, 0.0, yf, NULL, s);

  if (e == cudaSuccess)
    e = ncg_launch_gemv_ex (A, nrows, n, 1, 1.0, yf, 0.0, qf, part, s);

  if (e != cudaSuccess)
    return e;

  _gather_vec_kernel<<<VB (np), 0, s>>> (qf, P, np, q);

  return cudaGetLastError ();
}

/* ---- chained triangular solves of the FP32 preconditioner ----------------
 *
 * z = D (R^T R)^{-1} D r, one launch per triangular solve instead of one per
 * 64-row block.  Each CTA takes the next block from a ticket counter, so every
 * block it waits for belongs to a CTA that is already running and the launch
 * cannot deadlock whatever the residency.  While the blocks before its own
 * finish, a CTA streams its off-diagonal 64 x 64 tiles of R (the loads do not
 * depend on the waits), then applies the inverse of its diagonal block
 * (ncg_launch_trinv_diag_f32, once per factorisation).  A block publishes
 * each of its 64 values as one 64-bit word (value, epoch): a single-copy
 * atomic store that carries its own validity, so a reader polls the value
 * itself (one memory round trip, no flag and no fence).  The epoch is unique
 * to the launch (the host counts launches; the words are zeroed when the
 * buffer is set up, and epochs start at 1).  Every block's arithmetic runs in
 * a fixed order, so results do not depend on timing.
 *
 * sync: [0] ticket, [1] finished CTAs, [2] timeout seen; zero between
 * launches (the last CTA to finish clears them).  A wait gives up after
 * CS_SPIN polls, sets *err = 1 and sync[2], and the launch goes on with what
 * it has, so it always ends; a later wait that sees sync[2] does not spin. */
#define CS_TH 128
#define CS_SPIN (1 << 21)

__device__ __forceinline__ unsigned long long
_ld_relaxed64 (const unsigned long long *p)
{
  unsigned long long v;

  asm volatile ("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");

  return v;
}

__device__ __forceinline__ int
_ld_relaxed32 (const int32_t *p)
{
  int v;

  asm volatile ("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");

  return v;
}

/* publish value v of this launch */
__device__ __forceinline__ void
_cs_put (unsigned long long *w, float v, uint32_t epoch)
{
  const unsigned long long x = ((unsigned long long) epoch << 32) | __float_as_uint (v);

  asm volatile ("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(w), "l"(x) : "memory");
}

/* the value of word w once this launch has published it */
__device__ __forceinline__ float
_cs_get (const unsigned long long *w, uint32_t epoch, int32_t *sync, double *err)
{
  unsigned long long x = _ld_relaxed64 (w);
  int k = 0;

  while ((uint32_t) (x >> 32) != epoch)
  {
    if (++k > CS_SPIN || ((k & 255) == 0 && _ld_relaxed32 (sync + 2) != 0))
    {
      atomicExch (sync + 2, 1);
      *err = 1.0;
      break;
    }

    x = _ld_relaxed64 (w);
  }

  return __uint_as_float ((uint32_t) x);
}

/* count the CTA as finished; the last one clears the ticket and the counters */
__device__ __forceinline__ void
_cs_finish (int32_t *sync, int tid)
{
  __syncthreads ();

  if (tid == 0 && atomicAdd (sync + 1, 1) == (int) gridDim.x - 1)
  {
    sync[0] = 0;
    sync[1] = 0;
    sync[2] = 0;
  }
}

/* V_i = (U_ii^T)^{-1}, lower triangular, for each 64 x 64 diagonal block of the
 * upper factor U (zero outside the nb x nb triangle of a partial last block);
 * thread c computes column c by forward substitution */
__global__ void __launch_bounds__ (SB)
_trinv_diag_kernel (const float *__restrict__ U, int n, float *__restrict__ V)
{
  __shared__ float S[SB][SB + 1];
  __shared__ float X[SB][SB + 1];
  const int i = blockIdx.x, kb = i * SB, nb = (n - kb < SB) ? n - kb : SB, c = threadIdx.x;

  _stage_block<float, SB, SB> (S, U, n, kb, kb, nb, c);

  __syncthreads ();

  for (int r = 0; r < SB; r++)
  {
    float v = 0.0f;

    if (c < nb && r < nb && r >= c)
    {
      float acc = (r == c) ? 1.0f : 0.0f;

      for (int k = c; k < r; k++)
        acc = fmaf (-S[k][r], X[k][c], acc);

      v = acc / S[r][r];
    }

    X[r][c] = v;
  }

  __syncthreads ();

  for (int e = c; e < SB * SB; e += SB)
    V[(size_t) i * SB * SB + e] = X[e / SB][e % SB];
}

/* U^T y = (float) (D r): block i, y_i = V_i ((D r)_i - sum_{j<i} U_ji^T y_j);
 * warp w owns rows 16w..16w+15 of each tile, lanes its two columns */
__global__ void __launch_bounds__ (CS_TH)
_fsolve_chain_kernel (const float *__restrict__ U, const float *__restrict__ V, const double *__restrict__ D,
                      const double *__restrict__ r, int n, unsigned long long *__restrict__ y, uint32_t epoch,
                      uint32_t pepoch, int32_t *__restrict__ sync, double *__restrict__ err)
{
  __shared__ float Vs[SB][SB + 1];
  __shared__ float part[CS_TH / 32][SB];
  __shared__ float sv[SB];
  __shared__ int blk;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

  if (tid == 0)
    blk = atomicAdd (sync, 1);

  __syncthreads ();

  const int i = blk, kb = i * SB, nb = (n - kb < SB) ? n - kb : SB;

  for (int e = tid; e < SB * SB; e += CS_TH)
    Vs[e / SB][e % SB] = V[(size_t) i * SB * SB + e];

  const bool v0 = lane < nb, v1 = lane + 32 < nb;
  float a0 = 0.0f, a1 = 0.0f;

  for (int j = 0; j < i; j++)
  {
    const float *row = U + (size_t) (j * SB + wid * 16) * n + kb + lane;
    float u0[16], u1[16];

#pragma unroll
    for (int rr = 0; rr < 16; rr++)
    {
      u0[rr] = v0 ? row[(size_t) rr * n] : 0.0f;
      u1[rr] = v1 ? row[(size_t) rr * n + 32] : 0.0f;
    }

    /* y_j of this warp's 16 rows: lane rr waits for row rr, then shares it */
    const float ym = (lane < 16) ? _cs_get (y + j * SB + wid * 16 + lane, epoch, sync, err) : 0.0f;

#pragma unroll
    for (int rr = 0; rr < 16; rr++)
    {
      const float yv = __shfl_sync (0xffffffffu, ym, rr);

      a0 = fmaf (u0[rr], yv, a0);
      a1 = fmaf (u1[rr], yv, a1);
    }
  }

  part[wid][lane]      = a0;
  part[wid][lane + 32] = a1;

  __syncthreads ();

  if (tid < SB)
  {
    float b = 0.0f;

    if (tid < nb)
      b = (float) (D[kb + tid] * r[kb + tid]) - (((part[0][tid] + part[1][tid]) + part[2][tid]) + part[3][tid]);

    sv[tid] = b;
  }

  __syncthreads ();

  {
    const int row = tid >> 1, h = (tid & 1) * 32;
    float acc = 0.0f;

#pragma unroll 8
    for (int c = 0; c < 32; c++)
      acc = fmaf (Vs[row][h + c], sv[h + c], acc);

    acc += __shfl_xor_sync (0xffffffffu, acc, 1);

    if (h == 0 && row < nb)
      _cs_put (y + kb + row, acc, pepoch);
  }

  _cs_finish (sync, tid);
}

/* U x = y, z = D x: block i (from the last), x_i = V_i^T (y_i - sum_{j>i} U_ij x_j) */
__global__ void __launch_bounds__ (CS_TH)
_bsolve_chain_kernel (const float *__restrict__ U, const float *__restrict__ V, const double *__restrict__ D,
                      const unsigned long long *__restrict__ y, int n, unsigned long long *__restrict__ x,
                      uint32_t epoch, uint32_t pepoch, double *__restrict__ z, int32_t *__restrict__ sync,
                      double *__restrict__ err)
{
  __shared__ float Vs[SB][SB + 1];
  __shared__ float sv[SB];
  __shared__ int blk;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int nbk = (n + SB - 1) / SB;

  if (tid == 0)
    blk = nbk - 1 - atomicAdd (sync, 1);

  __syncthreads ();

  const int i = blk, kb = i * SB, nb = (n - kb < SB) ? n - kb : SB, r0 = wid * 16;

  for (int e = tid; e < SB * SB; e += CS_TH)
    Vs[e / SB][e % SB] = V[(size_t) i * SB * SB + e];

  float p[16];

#pragma unroll
  for (int rr = 0; rr < 16; rr++)
    p[rr] = 0.0f;

  for (int j = nbk - 1; j > i; j--)
  {
    const int jb = j * SB, nbj = (n - jb < SB) ? n - jb : SB;
    const bool v0 = lane < nbj, v1 = lane + 32 < nbj;
    const float *row = U + (size_t) (kb + r0) * n + jb + lane;
    float u0[16], u1[16];

#pragma unroll
    for (int rr = 0; rr < 16; rr++)
    {
      const bool ok = r0 + rr < nb;

      u0[rr] = (ok && v0) ? row[(size_t) rr * n] : 0.0f;
      u1[rr] = (ok && v1) ? row[(size_t) rr * n + 32] : 0.0f;
    }

    const float x0 = v0 ? _cs_get (x + jb + lane, epoch, sync, err) : 0.0f;
    const float x1 = v1 ? _cs_get (x + jb + lane + 32, epoch, sync, err) : 0.0f;

#pragma unroll
    for (int rr = 0; rr < 16; rr++)
      p[rr] = fmaf (u1[rr], x1, fmaf (u0[rr], x0, p[rr]));
  }

#pragma unroll
  for (int rr = 0; rr < 16; rr++)
  {
    float v = p[rr];

#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      v += __shfl_xor_sync (0xffffffffu, v, o);

    if (lane == 0)
      sv[r0 + rr] = (r0 + rr < nb) ? __uint_as_float ((uint32_t) y[kb + r0 + rr]) - v : 0.0f;
  }

  __syncthreads ();

  {
    const int row = tid >> 1, h = (tid & 1) * 32;
    float acc = 0.0f;

#pragma unroll 8
    for (int c = 0; c < 32; c++)
      acc = fmaf (Vs[h + c][row], sv[h + c], acc);

    acc += __shfl_xor_sync (0xffffffffu, acc, 1);

    if (h == 0 && row < nb)
    {
      _cs_put (x + kb + row, acc, pepoch);
      z[kb + row] = D[kb + row] * (double) acc;
    }
  }

  _cs_finish (sync, tid);
}

extern "C" size_t
ncg_pcg_trinv_bytes (int n)
{
  return sizeof (float) * SB * SB * (size_t) ((n + SB - 1) / SB);
}

extern "C" size_t
ncg_pcg_sync_bytes (int n)
{
  (void) n;

  return sizeof (int32_t) * 4;
}

extern "C" size_t
ncg_pcg_chain_bytes (int n)
{
  return sizeof (unsigned long long) * 2 * (size_t) n;
}

extern "C" cudaError_t
ncg_launch_trinv_diag_f32 (const float *U, int n, float *V, cudaStream_t s)
{
  if (n <= 0)
    return cudaSuccess;

  _trinv_diag_kernel<<<(n + SB - 1) / SB, SB, 0, s>>> (U, n, V);

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_pcg_precond (const float *R, const float *V, const double *D, int np, const double *r, void *chain,
                        uint32_t *epoch, double *z, int32_t *sync, double *err, cudaStream_t s)
{
  if (np <= 0)
    return cudaSuccess;

  const int nbk = (np + SB - 1) / SB;
  unsigned long long *y = (unsigned long long *) chain, *x = y + np;
  const uint32_t ey = ++*epoch, ex = ++*epoch;
  /* values are published under the launch's own epoch; the wait-fault test
   * hook publishes the forward solve's under one that no reader waits for,
   * so its first dependent wait runs out (CS_SPIN polls) and reports */
  const uint32_t py = ncg_fault_take (NCG_FAULT_CHAIN_WAIT) ? ey ^ 0x80000000u : ey;

  _fsolve_chain_kernel<<<nbk, CS_TH, 0, s>>> (R, V, D, r, np, y, ey, py, sync, err);
  _bsolve_chain_kernel<<<nbk, CS_TH, 0, s>>> (R, V, D, y, np, x, ex, ex, z, sync, err);

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_pcg_dot (const double *u0, const double *v0, const double *u1, const double *v1, const double *w, int n,
                    double *sc, int out0, int out1, cudaStream_t s)
{
  _dot2_kernel<<<1, PCG_THREADS, 0, s>>> (u0, v0, u1, v1, w, n, sc, out0, out1);

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_pcg_step (double *x, double *r, double *rprev, const double *p, const double *q, int n, const double *sc,
                     cudaStream_t s)
{
  _pcg_step_kernel<<<VB (n), 0, s>>> (x, r, rprev, p, q, n, sc);

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_pcg_dir (double *p, const double *z, int n, double *sc, cudaStream_t s)
{
  _pcg_dir_kernel<<<VB (n), 0, s>>> (p, z, n, sc);
  _pcg_shift_kernel<<<1, 1, 0, s>>> (sc);

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_rsub (const double *b, double *r, int n, cudaStream_t s)
{
  _rsub_kernel<<<VB (n), 0, s>>> (b, r, n);

  return cudaGetLastError ();
}

/* ------------------------------------------------------------------------ */
/* The FP64 NNLS solve's fallbacks when the normal equations of a set are    */
/* not positive definite (ncm_nnls.c:573-638, dispatch :655-666): a general  */
/* symmetric solve (the dsysv step; here Gaussian elimination with partial  */
/* pivoting on the full symmetric matrix) and, when that meets an exactly    */
/* zero pivot, the least-squares solve of A_P x = f by Householder QR (the  */
/* dgels step).  Both follow the oracle's operation order with explicitly   */
/* rounded operations (no FMA contraction), so the same inputs give the same */
/* bits: pivots are chosen by exact comparisons (the lowest row among equal  */
/* magnitudes), each reduction is one thread's sequential sum.  One launch  */
/* per elimination or reflection step; these are rare paths, sized for      */
/* correctness, not speed.                                                   */
/* ------------------------------------------------------------------------ */

/* the lower triangle of an upper-stored symmetric n x n matrix, in place */
__global__ void
_sym_mirror_kernel (double *A, int n)
{
  const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;

  if (e >= (int64_t) n * n)
    return;

  const int r = (int) (e / n), c = (int) (e % n);

  if (c < r)
    A[e] = A[(size_t) c * n + r];
}

#define GE_PIV_TH 256

/* step k: the pivot row (largest |A[r][k]|, r >= k, lowest r among equals),
 * then the swap of rows k and p and of b[k], b[p]; *info = k + 1 when the
 * column is exactly zero */
__global__ void __launch_bounds__ (GE_PIV_TH)
_ge_pivot_kernel (double *A, int n, int k, double *b, int32_t *info)
{
  __shared__ double sv[GE_PIV_TH];
  __shared__ int si[GE_PIV_TH];
  const int t = threadIdx.x;

  if (*info)
    return;

  double amax = -1.0;
  int p       = n;

  for (int r = k + t; r < n; r += GE_PIV_TH)
  {
    const double v = fabs (A[(size_t) r * n + k]);

    if (v > amax)
    {
      amax = v;
      p    = r;
    }
  }

  sv[t] = amax;
  si[t] = p;
  __syncthreads ();

  for (int o = GE_PIV_TH / 2; o > 0; o >>= 1)
  {
    if (t < o && (sv[t + o] > sv[t] || (sv[t + o] == sv[t] && si[t + o] < si[t])))
    {
      sv[t] = sv[t + o];
      si[t] = si[t + o];
    }

    __syncthreads ();
  }

  amax = sv[0];
  p    = si[0];

  if (amax == 0.0)
  {
    if (t == 0)
      *info = k + 1;

    return;
  }

  if (p != k)
  {
    for (int c = t; c < n; c += GE_PIV_TH)
    {
      const double x = A[(size_t) k * n + c];

      A[(size_t) k * n + c] = A[(size_t) p * n + c];
      A[(size_t) p * n + c] = x;
    }

    if (t == 0)
    {
      const double x = b[k];

      b[k] = b[p];
      b[p] = x;
    }
  }
}

#define GE_UP_RX 32
#define GE_UP_RY 8

/* step k: rows r > k minus f_r times row k over the columns c > k (column k
 * below the diagonal is never read again), b[r] minus f_r b[k];
 * f_r = A[r][k] / A[k][k], rows with f_r = 0 untouched */
__global__ void __launch_bounds__ (GE_UP_RX * GE_UP_RY)
_ge_update_kernel (double *A, int n, int k, double *b, const int32_t *info)
{
  __shared__ double f[GE_UP_RY];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int r  = k + 1 + blockIdx.y * GE_UP_RY + ty;

  if (*info)
    return;

  if (tx == 0)
    f[ty] = (r < n) ? __ddiv_rn (A[(size_t) r * n + k], A[(size_t) k * n + k]) : 0.0;

  __syncthreads ();

  if (r >= n || f[ty] == 0.0)
    return;

  const double fr = f[ty];

  for (int c = k + 1 + blockIdx.x * GE_UP_RX + tx; c < n; c += gridDim.x * GE_UP_RX)
    A[(size_t) r * n + c] = __dsub_rn (A[(size_t) r * n + c], __dmul_rn (fr, A[(size_t) k * n + c]));

  if (blockIdx.x == 0 && tx == 0)
    b[r] = __dsub_rn (b[r], __dmul_rn (fr, b[k]));
}

/* back substitution of the eliminated system, one thread, the oracle's order */
__global__ void
_ge_backsub_kernel (const double *A, int n, double *b, const int32_t *info)
{
  if (*info || threadIdx.x != 0 || blockIdx.x != 0)
    return;

  for (int r = n - 1; r >= 0; r--)
  {
    double s = b[r];

    for (int c = r + 1; c < n; c++)
      s = __dsub_rn (s, __dmul_rn (A[(size_t) r * n + c], b[c]));

    b[r] = __ddiv_rn (s, A[(size_t) r * n + r]);
  }
}

extern "C" cudaError_t
ncg_launch_sysv (double *A, int n, double *b, int32_t *info, cudaStream_t s)
{
  if (n <= 0)
    return cudaSuccess;

  cudaError_t e = cudaMemsetAsync (info, 0, sizeof (int32_t), s);

  if (e != cudaSuccess)
    return e;

  _sym_mirror_kernel<<<(unsigned) (((int64_t) n * n + 255) / 256), 256, 0, s>>> (A, n);

  for (int k = 0; k < n; k++)
  {
    _ge_pivot_kernel<<<1, GE_PIV_TH, 0, s>>> (A, n, k, b, info);

    const int rows = n - k - 1;

    if (rows > 0)
    {
      const int gx = ((rows + GE_UP_RX - 1) / GE_UP_RX < 8) ? (rows + GE_UP_RX - 1) / GE_UP_RX : 8;
      dim3 grid ((unsigned) gx, (unsigned) ((rows + GE_UP_RY - 1) / GE_UP_RY));

      _ge_update_kernel<<<grid, dim3 (GE_UP_RX, GE_UP_RY), 0, s>>> (A, n, k, b, info);
    }
  }

  _ge_backsub_kernel<<<1, 32, 0, s>>> (A, n, b, info);

  return cudaGetLastError ();
}

/* Q = A[:, P] (nrows x np, row-major), y = f */
__global__ void
_qr_gather_kernel (const double *__restrict__ A, int nrows, int ncols, const int32_t *__restrict__ P, int np,
                   const double *__restrict__ f, double *__restrict__ Q, double *__restrict__ y)
{
  const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;

  if (e < (int64_t) nrows * np)
  {
    const int r = (int) (e / np), c = (int) (e % np);

    Q[e] = A[(size_t) r * ncols + P[c]];
  }

  if (e < nrows)
    y[e] = f[e];
}

/* reflection k, part 1 (one thread): restore the diagonal of step k - 1,
 * then nrm = |Q[k:, k]|, alpha = -sign(Q[k][k]) nrm, Q[k][k] -= alpha and
 * vtv = |Q[k:, k]|^2; sc = {alpha, vtv, skip} (skip when the column is zero) */
__global__ void
_qr_house_kernel (double *Q, int nrows, int np, int k, double *sc)
{
  if (threadIdx.x != 0 || blockIdx.x != 0)
    return;

  if (k > 0 && sc[2] == 0.0)
    Q[(size_t) (k - 1) * np + (k - 1)] = sc[0];

  double nrm = 0.0;

  for (int r = k; r < nrows; r++)
    nrm = __dadd_rn (nrm, __dmul_rn (Q[(size_t) r * np + k], Q[(size_t) r * np + k]));

  nrm = __dsqrt_rn (nrm);

  const double alpha = (Q[(size_t) k * np + k] > 0.0) ? -nrm : nrm;

  if (nrm == 0.0)
  {
    sc[2] = 1.0;

    return;
  }

  Q[(size_t) k * np + k] = __dsub_rn (Q[(size_t) k * np + k], alpha);

  double vtv = 0.0;

  for (int r = k; r < nrows; r++)
    vtv = __dadd_rn (vtv, __dmul_rn (Q[(size_t) r * np + k], Q[(size_t) r * np + k]));

  sc[0] = alpha;
  sc[1] = vtv;
  sc[2] = 0.0;
}

/* reflection k, part 2: one thread per column c > k (c = np: the right-hand
 * side y), s = 2 (v . q_c) / vtv with the sum in row order, q_c -= s v */
__global__ void
_qr_apply_kernel (double *Q, int nrows, int np, int k, double *y, const double *sc)
{
  const int c = k + 1 + blockIdx.x * blockDim.x + threadIdx.x;

  if (sc[2] != 0.0 || c > np)
    return;

  const double vtv = sc[1];
  double s         = 0.0;

  if (c < np)
  {
    for (int r = k; r < nrows; r++)
      s = __dadd_rn (s, __dmul_rn (Q[(size_t) r * np + k], Q[(size_t) r * np + c]));

    s = __ddiv_rn (__dmul_rn (2.0, s), vtv);

    for (int r = k; r < nrows; r++)
      Q[(size_t) r * np + c] = __dsub_rn (Q[(size_t) r * np + c], __dmul_rn (s, Q[(size_t) r * np + k]));
  }
  else
  {
    for (int r = k; r < nrows; r++)
      s = __dadd_rn (s, __dmul_rn (Q[(size_t) r * np + k], y[r]));

    s = __ddiv_rn (__dmul_rn (2.0, s), vtv);

    for (int r = k; r < nrows; r++)
      y[r] = __dsub_rn (y[r], __dmul_rn (s, Q[(size_t) r * np + k]));
  }
}

/* the last diagonal, then R x = y by back substitution (one thread); a zero
 * diagonal gives x = 0 for that variable */
__global__ void
_qr_backsub_kernel (double *Q, int np, int kmax, const double *y, const double *sc, double *x)
{
  if (threadIdx.x != 0 || blockIdx.x != 0)
    return;

  if (kmax > 0 && sc[2] == 0.0)
    Q[(size_t) (kmax - 1) * np + (kmax - 1)] = sc[0];

  for (int k = np - 1; k >= 0; k--)
  {
    double s = y[k];

    for (int c = k + 1; c < np; c++)
      s = __dsub_rn (s, __dmul_rn (Q[(size_t) k * np + c], x[c]));

    x[k] = (Q[(size_t) k * np + k] != 0.0) ? __ddiv_rn (s, Q[(size_t) k * np + k]) : 0.0;
  }
}

extern "C" cudaError_t
ncg_launch_gels (const double *A, int nrows, int ncols, const int32_t *P, int np, const double *f, double *Q,
                 double *y, double *sc, double *x, cudaStream_t s)
{
  if (np <= 0)
    return cudaSuccess;

  const int64_t tot = (int64_t) nrows * np > nrows ? (int64_t) nrows * np : nrows;
  const int kmax    = np < nrows ? np : nrows;
  cudaError_t e;

  _qr_gather_kernel<<<(unsigned) ((tot + 255) / 256), 256, 0, s>>> (A, nrows, ncols, P, np, f, Q, y);

  if ((e = cudaMemsetAsync (sc, 0, 3 * sizeof (double), s)) != cudaSuccess)
    return e;

  for (int k = 0; k < kmax; k++)
  {
    _qr_house_kernel<<<1, 32, 0, s>>> (Q, nrows, np, k, sc);
    _qr_apply_kernel<<<(unsigned) ((np - k + 127) / 128), 128, 0, s>>> (Q, nrows, np, k, y, sc);
  }

  _qr_backsub_kernel<<<1, 32, 0, s>>> (Q, np, kmax, y, sc, x);

  return cudaGetLastError ();
}

/* ---- row sums of a square interpolation matrix (the AMISE of the LOO fit,
 * ncm_stats_dist.c:581-598): rowx[i] = sum_{j != i} IM[i][j] in column order
 * per lane, diag[i] = IM[i][i]; one warp per row */
__global__ void
_im_rowsums_kernel (const double *__restrict__ IM, int n, double *__restrict__ rowx, double *__restrict__ diag)
{
  const int warp = (int) ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;

  if (warp >= n)
    return;

  const double *row = IM + (size_t) warp * n;
  double s = 0.0;

  for (int j = lane; j < n; j += 32)
    if (j != warp)
      s += row[j];

  for (int o = 16; o > 0; o >>= 1)
    s += __shfl_xor_sync (0xffffffffu, s, o);

  if (lane == 0)
  {
    rowx[warp] = s;
    diag[warp] = row[warp];
  }
}

extern "C" cudaError_t
ncg_launch_im_rowsums (const double *IM, int n, double *rowx, double *diag, cudaStream_t s)
{
  if (n <= 0)
    return cudaSuccess;

  _im_rowsums_kernel<<<(unsigned) ((n + 7) / 8), 256, 0, s>>> (IM, n, rowx, diag);

  return cudaGetLastError ();
}
