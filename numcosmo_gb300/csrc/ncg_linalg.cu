/*
 * ncg_linalg.cu -- FP64 dense kernels behind prepare_interp's NNLS
 * (ncm_nnls_solve, numcosmo/ncm/algebra/ncm_nnls.c:767-871, NORMAL umethod):
 *
 *   syrk_upper    M = A^T A, upper triangle (ncm_matrix_square_to_sym,
 *                 numcosmo/ncm/algebra/ncm_matrix.c:1548-1572)
 *   gemv          y = alpha op(A) x + beta y, deterministic reductions
 *   gather_sub    M[P,P], b[P] for an active set P (ncm_iset_get_submatrix)
 *   potrf         blocked right-looking Cholesky, upper, row-major (dpotrf)
 *   potrs         U^T U x = b (dposv's solve)
 *   residual_norm res = f - A x and |res|^2 (ncm_nnls.c:700-711)
 *
 * Every reduction has a fixed order, so two runs give identical bits.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "ncg_internal.h"

#define TB 64     /* output tile */
#define KB 16     /* rows per smem stage */

/* C[i][j] = (or -=) sum_{r in [r0, r1)} A[r][i] A[r][j] for off <= i <= j < off + nn */
__global__ void __launch_bounds__ (256)
_syrk_tile_kernel (const double *__restrict__ A, int lda, int r0, int r1, int off, int nn,
                   double *__restrict__ C, int ldc, int minus)
{
  __shared__ double As[KB][TB];
  __shared__ double Bs[KB][TB];

  /* map the linear block id onto the upper tiles (ti <= tj) */
  const int T = (nn + TB - 1) / TB;
  int b = blockIdx.x, ti = 0;

  while (b >= T - ti)
  {
    b -= T - ti;
    ti++;
  }

  const int tj  = ti + b;
  const int i0  = off + ti * TB, j0 = off + tj * TB;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int end = off + nn;
  double acc[4][4];

#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++)
      acc[a][c] = 0.0;

  for (int rb = r0; rb < r1; rb += KB)
  {
    for (int e = tid; e < KB * TB; e += 256)
    {
      const int rr = e / TB, cc = e - rr * TB;
      const int r  = rb + rr;

      As[rr][cc] = (r < r1 && i0 + cc < end) ? A[(size_t) r * lda + i0 + cc] : 0.0;
      Bs[rr][cc] = (r < r1 && j0 + cc < end) ? A[(size_t) r * lda + j0 + cc] : 0.0;
    }

    __syncthreads ();

#pragma unroll
    for (int rr = 0; rr < KB; rr++)
    {
      double a[4], bb[4];

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
        double *dst = C + (size_t) i * ldc + j;

        *dst = minus ? (*dst - acc[p][q]) : acc[p][q];
      }
    }
}

static cudaError_t
_syrk (const double *A, int lda, int r0, int r1, int off, int nn, double *C, int ldc, int minus, cudaStream_t s)
{
  if (nn <= 0)
    return cudaSuccess;

  const int T       = (nn + TB - 1) / TB;
  const int nblocks = T * (T + 1) / 2;

  _syrk_tile_kernel<<<nblocks, 256, 0, s>>> (A, lda, r0, r1, off, nn, C, ldc, minus);

  return cudaGetLastError ();
}

extern "C" cudaError_t
ncg_launch_syrk_upper (const double *A, int nrows, int ncols, double *M, cudaStream_t s)
{
  return _syrk (A, ncols, 0, nrows, 0, ncols, M, ncols, 0, s);
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

/* ---- blocked Cholesky ------------------------------------------------------ */

#define PB 64

/* factor the nb x nb diagonal block at (kb, kb) in place (upper) */
__global__ void __launch_bounds__ (256)
_potrf_diag_kernel (double *A, int ld, int kb, int nb, int32_t *info)
{
  __shared__ double S[PB][PB + 1];
  __shared__ int fail;
  const int tid = threadIdx.x;

  for (int e = tid; e < nb * nb; e += 256)
  {
    const int r = e / nb, c = e - r * nb;

    S[r][c] = A[(size_t) (kb + r) * ld + kb + c];
  }

  if (tid == 0)
    fail = 0;

  __syncthreads ();

  for (int j = 0; j < nb; j++)
  {
    if (tid == 0)
    {
      double ajj = S[j][j];

      for (int k = 0; k < j; k++)
        ajj -= S[k][j] * S[k][j];

      if (!(ajj > 0.0))
      {
        fail = j + 1;
        S[j][j] = ajj;
      }
      else
      {
        S[j][j] = sqrt (ajj);
      }
    }

    __syncthreads ();

    if (fail)
      break;

    const double ajj = S[j][j];

    for (int i = j + 1 + tid; i < nb; i += 256)
    {
      double aji = S[j][i];

      for (int k = 0; k < j; k++)
        aji -= S[k][j] * S[k][i];

      S[j][i] = aji / ajj;
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

/* rows kb..kb+nb of the columns right of the block: X = U_kk^{-T} A_panel */
__global__ void __launch_bounds__ (128)
_potrf_trsm_kernel (double *A, int ld, int kb, int nb, int n, const int32_t *info)
{
  __shared__ double S[PB][PB + 1];
  const int tid = threadIdx.x;

  if (*info)
    return;

  for (int e = tid; e < nb * nb; e += 128)
  {
    const int r = e / nb, c = e - r * nb;

    S[r][c] = A[(size_t) (kb + r) * ld + kb + c];
  }

  __syncthreads ();

  const int col = kb + nb + blockIdx.x * 128 + tid;

  if (col >= n)
    return;

  double y[PB];

  for (int r = 0; r < nb; r++)
  {
    double s = A[(size_t) (kb + r) * ld + col];

    for (int m = 0; m < r; m++)
      s -= S[m][r] * y[m];

    y[r] = s / S[r][r];
    A[(size_t) (kb + r) * ld + col] = y[r];
  }
}

__global__ void
_zero_int_kernel (int32_t *p)
{
  *p = 0;
}

extern "C" cudaError_t
ncg_launch_potrf (double *A, int n, int32_t *info, double *work, cudaStream_t s)
{
  (void) work;
  _zero_int_kernel<<<1, 1, 0, s>>> (info);

  for (int kb = 0; kb < n; kb += PB)
  {
    const int nb = (n - kb < PB) ? n - kb : PB;

    _potrf_diag_kernel<<<1, 256, 0, s>>> (A, n, kb, nb, info);

    if (kb + nb < n)
    {
      const int rest = n - kb - nb;

      _potrf_trsm_kernel<<<(rest + 127) / 128, 128, 0, s>>> (A, n, kb, nb, n, info);

      cudaError_t e = _syrk (A, n, kb, kb + nb, kb + nb, rest, A, n, 1, s);

      if (e != cudaSuccess)
        return e;
    }
  }

  return cudaGetLastError ();
}

/* U^T y = b (column sweeps over rows of U), then U x = y (row dots); one CTA */
__global__ void __launch_bounds__ (1024)
_potrs_kernel (const double *__restrict__ U, int n, double *__restrict__ b)
{
  __shared__ double red[32];
  __shared__ double yj;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;

  for (int j = 0; j < n; j++)
  {
    if (tid == 0)
      yj = b[j] / U[(size_t) j * n + j];

    __syncthreads ();

    const double y = yj;

    for (int i = j + 1 + tid; i < n; i += blockDim.x)
      b[i] -= U[(size_t) j * n + i] * y;

    if (tid == 0)
      b[j] = y;

    __syncthreads ();
  }

  for (int j = n - 1; j >= 0; j--)
  {
    double s = 0.0;

    for (int k = j + 1 + tid; k < n; k += blockDim.x)
      s = fma (U[(size_t) j * n + k], b[k], s);

#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      s += __shfl_xor_sync (0xffffffffu, s, o);

    if (lane == 0)
      red[wid] = s;

    __syncthreads ();

    if (tid == 0)
    {
      double t = 0.0;

      for (int w = 0; w < nw; w++)
        t += red[w];

      b[j] = (b[j] - t) / U[(size_t) j * n + j];
    }

    __syncthreads ();
  }
}

extern "C" cudaError_t
ncg_launch_potrs (const double *U, int n, double *b, cudaStream_t s)
{
  if (n <= 0)
    return cudaSuccess;

  _potrs_kernel<<<1, 1024, 0, s>>> (U, n, b);

  return cudaGetLastError ();
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
