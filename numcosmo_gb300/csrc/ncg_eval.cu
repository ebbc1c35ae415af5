/*
 * ncg_eval.cu -- eval_m2lnp / eval / compute_IM over (points x kernels) for
 * one problem.
 *
 * Grid: x = tiles of EV_THREADS points (one point per thread), y = slices of
 * the kernel range; each CTA runs one tile of ncg_eval_tiles.cuh and keeps,
 * per point, the reference's (gamma, lambda) pair online: gamma = running
 * maximum of lnt_i, lambda = sum over the other kernels of exp(lnt_i -
 * gamma).  A merge kernel combines the slices in slice order and applies
 * -2 (gamma + log1p(lambda) - d ln h), in FP64 for both forms.
 */
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "ncg_internal.h"
#include "ncg_eval_tiles.cuh"

/* ------------------------------------------------------------------------ */
/* FP64                                                                     */
/* ------------------------------------------------------------------------ */

template <int DP, int KIND, int KERN>
__global__ void __launch_bounds__ (EV_THREADS)
_eval64_kernel (const ncg_eval_args_t a, const double *__restrict__ Xq, const double *__restrict__ pack,
                const double *__restrict__ cvec, const double *__restrict__ Vg, double2 *__restrict__ part,
                int kper)
{
  constexpr int S  = NcgEv64<DP, KIND>::S;
  constexpr int KC = NcgEv64<DP, KIND>::KC;
  __shared__ double sm[KC * S];
  __shared__ double sc[KC];

  ncg_tile_eval64<DP, KIND, KERN, KC> (a, Xq, pack, cvec, Vg, part, kper, blockIdx.x, blockIdx.y, sm, sc);
}

/* combine the slices in order; out = -2 (gamma + log1p(lambda) - d ln h) or
 * the linear density exp(gamma + log1p(lambda) - d ln h) */
template <typename T2>
__global__ void
_merge_kernel (const T2 *__restrict__ part, int nslices, int64_t m, double shift, const double *dshift,
               double d_ln_href, int linear, double *__restrict__ out)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;

  if (j >= m)
    return;

  double G = -CUDART_INF, L = 0.0;

  for (int s = 0; s < nslices; s++)
  {
    const T2 p      = part[(size_t) s * m + j];
    const double ms = (double) p.x, ls = (double) p.y;

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

  const double gamma = G - shift + (dshift ? *dshift : 0.0);
  const double lnp   = gamma + log1p (L) - d_ln_href;

  out[j] = linear ? exp (lnp) : -2.0 * lnp;
}

typedef void (*ev64_fn) (const ncg_eval_args_t, const double *, const double *, const double *,
                         const double *, double2 *, int);

template <int KIND, int KERN>
static ev64_fn
_pick64 (int dp)
{
  switch (dp)
  {
    case 4:  return _eval64_kernel<4, KIND, KERN>;
    case 8:  return _eval64_kernel<8, KIND, KERN>;
    case 12: return _eval64_kernel<12, KIND, KERN>;
    case 16: return _eval64_kernel<16, KIND, KERN>;
    case 20: return _eval64_kernel<20, KIND, KERN>;
    case 24: return _eval64_kernel<24, KIND, KERN>;
    case 28: return _eval64_kernel<28, KIND, KERN>;
    case 32: return _eval64_kernel<32, KIND, KERN>;
    default: return NULL;
  }
}

static int
_kc64 (int kind, int dp)
{
  const int P = dp * (dp + 1) / 2;
  const int S = (kind == NCG_VKDE) ? dp + P : dp;
  int kc      = 32768 / ((S + 1) * 8);

  return kc < 4 ? 4 : (kc > 256 ? 256 : kc);
}

/* slices of the kernel range so that the grid fills the GPU several times */
static void
_slicing (int64_t m, int n, int kc, int *nslices, int *kper)
{
  const int64_t bx = (m + EV_THREADS - 1) / EV_THREADS;
  const int64_t target = 152 * 10;
  int64_t s = (target + bx - 1) / bx;
  const int64_t smax = (n + kc - 1) / kc;

  if (s > smax)
    s = smax;

  if (s < 1)
    s = 1;

  if (s > 4096)
    s = 4096;

  int kp = (int) ((n + s - 1) / s);

  kp = ((kp + kc - 1) / kc) * kc;

  *kper    = kp;
  *nslices = (n + kp - 1) / kp;
}

extern "C" size_t
ncg_eval_scratch_bytes (const ncg_eval_args_t *a, int precision)
{
  int ns, kp;

  _slicing (a->m, a->n, (precision == NCG_PREC_FP64) ? _kc64 (a->kind, a->dp) : 64, &ns, &kp);

  return (size_t) ns * (size_t) a->m * ((precision == NCG_PREC_FP64) ? sizeof (double2) : sizeof (float2));
}

extern "C" cudaError_t
ncg_launch_eval_m2lnp_fp64 (const ncg_eval_args_t *a, const double *Xq, const double *pack64, const double *c,
                            const double *Vg, double *out, void *scratch, int linear, cudaStream_t s)
{
  ev64_fn fn;

  if (a->kind == NCG_VKDE)
    fn = (a->kernel == NCG_KERNEL_ST) ? _pick64<NCG_VKDE, NCG_KERNEL_ST> (a->dp) : _pick64<NCG_VKDE, NCG_KERNEL_GAUSS> (a->dp);
  else
    fn = (a->kernel == NCG_KERNEL_ST) ? _pick64<NCG_KDE, NCG_KERNEL_ST> (a->dp) : _pick64<NCG_KDE, NCG_KERNEL_GAUSS> (a->dp);

  if (fn == NULL || a->m <= 0 || a->n <= 0)
    return cudaErrorInvalidValue;

  int ns, kp;

  _slicing (a->m, a->n, _kc64 (a->kind, a->dp), &ns, &kp);

  const int64_t bx = (a->m + EV_THREADS - 1) / EV_THREADS;
  dim3 grid ((unsigned) bx, (unsigned) ns);

  fn<<<grid, EV_THREADS, 0, s>>> (*a, Xq, pack64, c, Vg, (double2 *) scratch, kp);

  cudaError_t e = cudaGetLastError ();

  if (e != cudaSuccess)
    return e;

  _merge_kernel<double2><<<(unsigned) ((a->m + 255) / 256), 256, 0, s>>> (
    (const double2 *) scratch, ns, a->m, a->final_shift, NULL, a->d_ln_href, linear, out);

  return cudaGetLastError ();
}

/* ------------------------------------------------------------------------ */
/* Mixed precision (SIMT FP32 with hi/lo differences)                       */
/* ------------------------------------------------------------------------ */

/* per-kernel float operand:
 *  VKDE: theta_hi[dp] theta_lo[dp] W[dp(dp+1)/2] c'   padded to a multiple of 4
 *  KDE : yhat_hi[dp]  yhat_lo[dp]  c'                   padded to a multiple of 4 */
__host__ __device__ static inline int
_smx (int kind, int dp)
{
  const int raw = (kind == NCG_VKDE) ? 2 * dp + dp * (dp + 1) / 2 + 1 : 2 * dp + 1;

  return (raw + 3) / 4 * 4;
}

/* packmx = [n x smx floats][C0 (double) | kappa_max (double) | pad to 64 B][kappa_i, n doubles] */
extern "C" size_t
ncg_packmx_bytes (int kind, int n, int dp)
{
  return (size_t) n * _smx (kind, dp) * sizeof (float) + 64 + (size_t) n * sizeof (double);
}

__global__ void
_cmax_kernel (const double *c, int n, double *out)
{
  __shared__ double red[256];
  double v = -CUDART_INF;

  for (int i = threadIdx.x; i < n; i += blockDim.x)
    v = fmax (v, c[i]);

  red[threadIdx.x] = v;
  __syncthreads ();

  for (int st = blockDim.x / 2; st > 0; st >>= 1)
  {
    if (threadIdx.x < st)
      red[threadIdx.x] = fmax (red[threadIdx.x], red[threadIdx.x + st]);

    __syncthreads ();
  }

  if (threadIdx.x == 0)
    *out = red[0];
}

__global__ void
_build_packmx_kernel (int kind, int n, int dp, const double *__restrict__ pack64, const double *__restrict__ c,
                      const double *__restrict__ cshift, float *__restrict__ pk)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;

  if (i >= n)
    return;

  const int S64  = ncg_pack64_stride (kind, dp);
  const int Smx  = _smx (kind, dp);
  const double *src = pack64 + (size_t) i * S64;
  float *dst        = pk + (size_t) i * Smx;
  const double C0   = *cshift;

  for (int e = 0; e < dp; e++)
  {
    const double v = src[e];
    const float hi = __double2float_rn (v);

    dst[e]      = hi;
    dst[dp + e] = __double2float_rn (v - (double) hi);
  }

  int o = 2 * dp;

  if (kind == NCG_VKDE)
  {
    const int P = dp * (dp + 1) / 2;

    for (int e = 0; e < P; e++)
      dst[o + e] = __double2float_rn (src[dp + e]);

    o += P;
  }

  dst[o++] = __double2float_rn (c[i] - C0);

  for (; o < Smx; o++)
    dst[o] = 0.0f;
}

/* VKDE mixed operand in globally whitened coordinates: with Vg = U_g^{-T} and
 * mu the centre mean, y_i = U_i^{-T}(x - theta_i)/h = W'_i (x' - theta'_i) where
 * x' = Vg (x - mu), theta'_i = Vg (theta_i - mu) and W'_i = U_i^{-T} U_g^T / h
 * (lower triangular).  When the local covariances share the global shape,
 * W'_i is well conditioned, so the FP32 whitening keeps its accuracy.  One warp
 * per kernel; lane c owns column c. */
#define PMX_WARPS 2

__global__ void __launch_bounds__ (PMX_WARPS * 32)
_build_packmx_vkde_kernel (int n, int d, int dp, const double *__restrict__ X, const double *__restrict__ Ui,
                           const double *__restrict__ Ug, const double *__restrict__ Vg,
                           const double *__restrict__ mu, double inv_href, const double *__restrict__ c,
                           const double *__restrict__ cshift, float *__restrict__ pk, double *__restrict__ kappa)
{
  __shared__ double sG[NCG_DMAX * NCG_DMAX];
  __shared__ double sU[PMX_WARPS][NCG_DMAX * NCG_DMAX];
  __shared__ double sW[PMX_WARPS][NCG_DMAX * NCG_DMAX];
  __shared__ double sT[PMX_WARPS][NCG_DMAX];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int P = dp * (dp + 1) / 2, Smx = _smx (NCG_VKDE, dp);

  for (int e = threadIdx.x; e < d * d; e += blockDim.x)
    sG[e] = Ug[e];

  __syncthreads ();

  const double C0 = *cshift;

  for (int i = blockIdx.x * PMX_WARPS + w; i < n; i += gridDim.x * PMX_WARPS)
  {
    const double *U = Ui + (size_t) i * d * d;
    float *dst      = pk + (size_t) i * Smx;

    for (int e = lane; e < d * d; e += 32)
      sU[w][e] = U[e];

    if (lane < d)
      sT[w][lane] = X[(size_t) i * d + lane] - mu[lane];

    __syncwarp ();

    if (lane < d)
    {
      const int cc = lane;

      sW[w][cc * d + cc] = 1.0 / sU[w][cc * d + cc];

      for (int r = cc + 1; r < d; r++)
      {
        double s = 0.0;

        for (int m = cc; m < r; m++)
          s += sU[w][m * d + r] * sW[w][m * d + cc];

        sW[w][r * d + cc] = -s / sU[w][r * d + r];
      }
    }

    __syncwarp ();

    /* theta' (lane r) */
    if (lane < dp)
    {
      double t = 0.0;

      if (lane < d)
      {
        const int r   = lane;
        const int off = r * (r + 1) / 2;

        for (int m = 0; m <= r; m++)
          t += Vg[off + m] * sT[w][m];
      }

      const float hi = __double2float_rn (t);

      dst[lane]      = hi;
      dst[dp + lane] = __double2float_rn (t - (double) hi);
    }

    /* W'[r][cc] = sum_{m=cc}^{r} W[r][m] Ug[cc][m] / h (lane cc) */
    for (int e = lane; e < P; e += 32)
    {
      int r = (int) ((sqrt (8.0 * e + 1.0) - 1.0) * 0.5);

      while (r * (r + 1) / 2 > e)
        r--;

      while ((r + 1) * (r + 2) / 2 <= e)
        r++;

      const int cc = e - r * (r + 1) / 2;
      double v     = 0.0;

      if (r < d && cc < d)
      {
        for (int m = cc; m <= r; m++)
          v += sW[w][r * d + m] * sG[cc * d + m];

        v *= inv_href;
      }

      dst[2 * dp + e] = __double2float_rn (v);
    }

    if (lane == 0)
    {
      dst[2 * dp + P] = __double2float_rn (c[i] - C0);

      for (int o = 2 * dp + P + 1; o < Smx; o++)
        dst[o] = 0.0f;
    }

    /* infinity-norm condition number of W'_i = U_i^{-T} U_g^T / h, with
     * W'_i^{-1} = h U_g^{-T} U_i^T: the accuracy of the FP32 whitening */
    {
      double n1 = 0.0, n2 = 0.0;

      for (int r = 0; r < d; r++)
      {
        double a1 = 0.0, a2 = 0.0;

        if (lane <= r)
        {
          for (int m = lane; m <= r; m++)
          {
            a1 += sW[w][r * d + m] * sG[lane * d + m];
            a2 += Vg[r * (r + 1) / 2 + m] * sU[w][lane * d + m];
          }

          a1 = fabs (a1 * inv_href);
          a2 = fabs (a2 / inv_href);
        }

#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
          a1 += __shfl_xor_sync (0xffffffffu, a1, o);
          a2 += __shfl_xor_sync (0xffffffffu, a2, o);
        }

        n1 = fmax (n1, a1);
        n2 = fmax (n2, a2);
      }

      if (lane == 0)
        kappa[i] = n1 * n2;
    }

    __syncwarp ();
  }
}

extern "C" cudaError_t
ncg_launch_build_packmx (const ncg_eval_args_t *a, const double *X, const double *pack64, const double *c,
                         const double *Ui, const double *Ug, const double *Vg, const double *mu, float *packmx,
                         cudaStream_t s)
{
  /* the shift C0 = max_i c_i lives in the trailing 64 bytes of packmx */
  double *cshift = (double *) ((char *) packmx + (size_t) a->n * _smx (a->kind, a->dp) * sizeof (float));

  _cmax_kernel<<<1, 256, 0, s>>> (c, a->n, cshift);

  double *kappa_max = cshift + 1;
  double *kappa     = (double *) ((char *) cshift + 64);

  if (a->kind == NCG_VKDE)
  {
    int grid = (a->n + PMX_WARPS - 1) / PMX_WARPS;

    if (grid > 152 * 16)
      grid = 152 * 16;

    _build_packmx_vkde_kernel<<<grid, PMX_WARPS * 32, 0, s>>> (a->n, a->d, a->dp, X, Ui, Ug, Vg, mu, a->inv_href, c,
                                                                cshift, packmx, kappa);
  }
  else
  {
    /* KDE: differences of hi/lo-split whitened coordinates, no per-kernel
     * whitening, so no conditioning loss */
    _build_packmx_kernel<<<(a->n + 127) / 128, 128, 0, s>>> (a->kind, a->n, a->dp, pack64, c, cshift, packmx);
    ncg_launch_fill (kappa, 1.0, a->n, s);
  }

  _cmax_kernel<<<1, 256, 0, s>>> (kappa, a->n, kappa_max);

  return cudaGetLastError ();
}

/* device address of kappa_max = max_i cond(W'_i), stored behind the mixed pack */
extern "C" const double *
ncg_packmx_kappa_max (const float *packmx, int kind, int n, int dp)
{
  return (const double *) ((const char *) packmx + (size_t) n * _smx (kind, dp) * sizeof (float)) + 1;
}

template <int DP, int KIND, int KERN>
__global__ void __launch_bounds__ (EV_THREADS)
_evalmx_kernel (const ncg_eval_args_t a, const double *__restrict__ Xq, const float *__restrict__ pack,
                const double *__restrict__ Vg, const double *__restrict__ mu, float2 *__restrict__ part, int kper)
{
  constexpr int S  = NcgEvMx<DP, KIND>::S;
  constexpr int KC = NcgEvMx<DP, KIND>::KC;
  __shared__ __align__ (16) float sm[KC * S];

  ncg_tile_evalmx<DP, KIND, KERN, KC> (a, Xq, pack, Vg, mu, part, kper, blockIdx.x, blockIdx.y, sm);
}

typedef void (*evmx_fn) (const ncg_eval_args_t, const double *, const float *, const double *, const double *,
                         float2 *, int);

template <int KIND, int KERN>
static evmx_fn
_pickmx (int dp)
{
  switch (dp)
  {
    case 4:  return _evalmx_kernel<4, KIND, KERN>;
    case 8:  return _evalmx_kernel<8, KIND, KERN>;
    case 12: return _evalmx_kernel<12, KIND, KERN>;
    case 16: return _evalmx_kernel<16, KIND, KERN>;
    case 20: return _evalmx_kernel<20, KIND, KERN>;
    case 24: return _evalmx_kernel<24, KIND, KERN>;
    case 28: return _evalmx_kernel<28, KIND, KERN>;
    case 32: return _evalmx_kernel<32, KIND, KERN>;
    default: return NULL;
  }
}

extern "C" cudaError_t
ncg_launch_eval_m2lnp_mixed (const ncg_eval_args_t *a, const double *Xq, const float *packmx, const double *mu,
                             const double *Vg, double *out, void *scratch, cudaStream_t s)
{
  evmx_fn fn;

  if (a->kind == NCG_VKDE)
    fn = (a->kernel == NCG_KERNEL_ST) ? _pickmx<NCG_VKDE, NCG_KERNEL_ST> (a->dp) : _pickmx<NCG_VKDE, NCG_KERNEL_GAUSS> (a->dp);
  else
    fn = (a->kernel == NCG_KERNEL_ST) ? _pickmx<NCG_KDE, NCG_KERNEL_ST> (a->dp) : _pickmx<NCG_KDE, NCG_KERNEL_GAUSS> (a->dp);

  if (fn == NULL || a->m <= 0 || a->n <= 0)
    return cudaErrorInvalidValue;

  int ns, kp;

  _slicing (a->m, a->n, 64, &ns, &kp);

  const int64_t bx = (a->m + EV_THREADS - 1) / EV_THREADS;
  dim3 grid ((unsigned) bx, (unsigned) ns);
  const double *cshift = (const double *) ((const char *) packmx + (size_t) a->n * _smx (a->kind, a->dp) * sizeof (float));

  fn<<<grid, EV_THREADS, 0, s>>> (*a, Xq, packmx, Vg, (a->kind == NCG_VKDE) ? mu : NULL, (float2 *) scratch, kp);

  cudaError_t e = cudaGetLastError ();

  if (e != cudaSuccess)
    return e;

  _merge_kernel<float2><<<(unsigned) ((a->m + 255) / 256), 256, 0, s>>> (
    (const float2 *) scratch, ns, a->m, a->final_shift, cshift, a->d_ln_href, 0, out);

  return cudaGetLastError ();
}

/* ------------------------------------------------------------------------ */
/* compute_IM (FP64): IM[j][i] = K(chi2_ji) / exp(lnnorm_i + d ln h) / f_j     */
/* VKDE: ncm_stats_dist_vkde.c:518-606; KDE: ncm_stats_dist_kde.c:493-557;     */
/* row scaling: ncm_stats_dist.c:791-804.  One thread per observation row;   */
/* n_obs rows (a.m at the launcher) by n_kernels columns (a.n), row-major.    */
/* ------------------------------------------------------------------------ */

template <int DP, int KIND, int KERN>
__global__ void __launch_bounds__ (EV_THREADS)
_im64_kernel (const ncg_eval_args_t a, const double *__restrict__ X, const double *__restrict__ pack,
              const double *__restrict__ lnnorm, double kde_scale, const double *__restrict__ f,
              double *__restrict__ IM, int nrows)
{
  constexpr int S  = NcgEv64<DP, KIND>::S;
  constexpr int KC = NcgEv64<DP, KIND>::KC;
  __shared__ double sm[KC * S];
  __shared__ double sn[KC];

  const int n      = a.n;
  const int j      = blockIdx.x * EV_THREADS + threadIdx.x;
  const bool valid = j < nrows;
  double x[DP];

  if (KIND == NCG_VKDE)
  {
#pragma unroll
    for (int c = 0; c < DP; c++)
      x[c] = (valid && c < a.d) ? X[(size_t) j * a.d + c] : 0.0;
  }
  else
  {
    /* whitened observation / h is the kernel operand itself */
#pragma unroll
    for (int c = 0; c < DP; c++)
      x[c] = valid ? pack[(size_t) j * S + c] : 0.0;
  }

  const double inv_f = valid ? 1.0 / f[j] : 0.0;
  const int i0 = blockIdx.y * a.m;   /* a.m carries the per-slice kernel count here */
  const int i1 = min (n, i0 + (int) a.m);

  for (int ic = i0; ic < i1; ic += KC)
  {
    const int kc = min (KC, i1 - ic);

    __syncthreads ();

    for (int e = threadIdx.x; e < kc * S; e += EV_THREADS)
      sm[e] = pack[(size_t) ic * S + e];

    for (int e = threadIdx.x; e < kc; e += EV_THREADS)
      sn[e] = (KIND == NCG_VKDE) ? 1.0 / exp (lnnorm[ic + e] + a.d_ln_href) : kde_scale;

    __syncthreads ();

    if (!valid)
      continue;

    for (int kk = 0; kk < kc; kk++)
    {
      const double *pk = sm + kk * S;
      double chi2      = 0.0;

      if (KIND == NCG_VKDE)
      {
        double dl[DP];

#pragma unroll
        for (int c = 0; c < DP; c++)
          dl[c] = x[c] - pk[c];

        const double *W = pk + DP;
        int p           = 0;

#pragma unroll
        for (int r = 0; r < DP; r++)
        {
          double y = 0.0;

#pragma unroll
          for (int c = 0; c <= r; c++)
            y = fma (W[p++], dl[c], y);

          chi2 = fma (y, y, chi2);
        }
      }
      else
      {
#pragma unroll
        for (int c = 0; c < DP; c++)
        {
          const double t = pk[c] - x[c];

          chi2 = fma (t, t, chi2);
        }
      }

      const double K = (KERN == NCG_KERNEL_ST) ? pow (1.0 + chi2 / a.nu, -0.5 * (a.nu + a.d)) : exp (-0.5 * chi2);

      IM[(size_t) j * n + ic + kk] = (K * sn[kk]) * inv_f;
    }
  }
}

typedef void (*im64_fn) (const ncg_eval_args_t, const double *, const double *, const double *, double,
                         const double *, double *, int);

template <int KIND, int KERN>
static im64_fn
_pickim (int dp)
{
  switch (dp)
  {
    case 4:  return _im64_kernel<4, KIND, KERN>;
    case 8:  return _im64_kernel<8, KIND, KERN>;
    case 12: return _im64_kernel<12, KIND, KERN>;
    case 16: return _im64_kernel<16, KIND, KERN>;
    case 20: return _im64_kernel<20, KIND, KERN>;
    case 24: return _im64_kernel<24, KIND, KERN>;
    case 28: return _im64_kernel<28, KIND, KERN>;
    case 32: return _im64_kernel<32, KIND, KERN>;
    default: return NULL;
  }
}

extern "C" cudaError_t
ncg_launch_compute_IM (const ncg_eval_args_t *a, const double *X, const double *pack64, const double *lnnorm,
                       double kernel_lnnorm, const double *f, double *IM, cudaStream_t s)
{
  im64_fn fn;

  if (a->kind == NCG_VKDE)
    fn = (a->kernel == NCG_KERNEL_ST) ? _pickim<NCG_VKDE, NCG_KERNEL_ST> (a->dp) : _pickim<NCG_VKDE, NCG_KERNEL_GAUSS> (a->dp);
  else
    fn = (a->kernel == NCG_KERNEL_ST) ? _pickim<NCG_KDE, NCG_KERNEL_ST> (a->dp) : _pickim<NCG_KDE, NCG_KERNEL_GAUSS> (a->dp);

  if (fn == NULL || a->n <= 0 || a->m < a->n || a->m > INT32_MAX)
    return cudaErrorInvalidValue;

  int ns, kp;

  _slicing (a->m, a->n, _kc64 (a->kind, a->dp), &ns, &kp);

  ncg_eval_args_t b = *a;

  b.m = kp;

  const double kde_scale = exp (-(kernel_lnnorm + a->d_ln_href));
  dim3 grid ((unsigned) ((a->m + EV_THREADS - 1) / EV_THREADS), (unsigned) ns);

  fn<<<grid, EV_THREADS, 0, s>>> (b, X, pack64, lnnorm, kde_scale, f, IM, (int) a->m);

  return cudaGetLastError ();
}

/* merge of float2 (max, lambda) partials written by the tensor-core kernel */
extern "C" cudaError_t
ncg_launch_merge_f2 (const void *part, int nparts, int64_t m, double shift, const double *dshift, double d_ln_href,
                     double *out, cudaStream_t s)
{
  _merge_kernel<float2><<<(unsigned) ((m + 255) / 256), 256, 0, s>>> ((const float2 *) part, nparts, m, shift, dshift,
                                                                     d_ln_href, 0, out);

  return cudaGetLastError ();
}

/* device address of the constant C0 = max_i c_i stored behind the mixed pack */
extern "C" const double *
ncg_packmx_cshift (const float *packmx, int kind, int n, int dp)
{
  return (const double *) ((const char *) packmx + (size_t) n * _smx (kind, dp) * sizeof (float));
}

/* ------------------------------------------------------------------------ */
/* FP64 eval with a static scratch: the launcher behind                       */
/* ncg_sd_eval_m2lnp_device_noalloc.                                          */
/*                                                                           */
/* The FP64 eval writes one (gamma, lambda) pair per (kernel slice, point)    */
/* before the merge reads it; the regular entry points keep that buffer in    */
/* device memory the handle allocates on demand.  Callers that must not       */
/* allocate during evaluation use this variant instead: the pairs live in     */
/* the file-scope array below, 4 MiB per device, resident on every GPU that  */
/* loads the library until the process exits.  Every entry of the array a   */
/* call reads is written earlier in the same call, so nothing needs clearing; */
/* two calls whose kernels overlap on the GPU (e.g. on two streams) share the */
/* array and race.                                                           */
/* ------------------------------------------------------------------------ */

#define NCG_NOALLOC_SCRATCH_BYTES ((size_t) 4 << 20)
#define NCG_NOALLOC_MAX_DEVICES 64

static __device__ __align__ (256) unsigned char ncg_noalloc_scratch[NCG_NOALLOC_SCRATCH_BYTES];

/* device address of ncg_noalloc_scratch per device, set up on the first call
 * on that device (with that device current) */
static void *g_noalloc_addr[NCG_NOALLOC_MAX_DEVICES];

extern "C" size_t
ncg_noalloc_scratch_bytes (void)
{
  return NCG_NOALLOC_SCRATCH_BYTES;
}

/* the largest point count one call can take (one slice: m pairs of doubles) */
extern "C" int64_t
ncg_noalloc_max_points (void)
{
  return (int64_t) (NCG_NOALLOC_SCRATCH_BYTES / sizeof (double2));
}

extern "C" cudaError_t
ncg_launch_eval_m2lnp_fp64_noalloc (const ncg_eval_args_t *a, const double *Xq, const double *pack64, const double *c,
                                    const double *Vg, double *out, cudaStream_t s)
{
  ev64_fn fn;
  int dev = 0;
  cudaError_t e;

  if (a->kind == NCG_VKDE)
    fn = (a->kernel == NCG_KERNEL_ST) ? _pick64<NCG_VKDE, NCG_KERNEL_ST> (a->dp) : _pick64<NCG_VKDE, NCG_KERNEL_GAUSS> (a->dp);
  else
    fn = (a->kernel == NCG_KERNEL_ST) ? _pick64<NCG_KDE, NCG_KERNEL_ST> (a->dp) : _pick64<NCG_KDE, NCG_KERNEL_GAUSS> (a->dp);

  if (fn == NULL || a->m <= 0 || a->n <= 0 || a->m > ncg_noalloc_max_points ())
    return cudaErrorInvalidValue;

  if ((e = cudaGetDevice (&dev)) != cudaSuccess)
    return e;

  if (dev < 0 || dev >= NCG_NOALLOC_MAX_DEVICES)
    return cudaErrorInvalidDevice;

  void *addr = __atomic_load_n (&g_noalloc_addr[dev], __ATOMIC_ACQUIRE);

  if (addr == NULL)
  {
    /* set-up, once per device: the host-side name of the array is not a
     * device address, the runtime gives the address on the current device
     * (concurrent first calls store the same value) */
    if ((e = cudaGetSymbolAddress (&addr, ncg_noalloc_scratch)) != cudaSuccess)
      return e;

    __atomic_store_n (&g_noalloc_addr[dev], addr, __ATOMIC_RELEASE);
  }

  /* the regular slicing, with the slice count capped by the static size */
  const int kc = _kc64 (a->kind, a->dp);
  int ns, kp;

  _slicing (a->m, a->n, kc, &ns, &kp);

  const int64_t ns_max = (int64_t) (NCG_NOALLOC_SCRATCH_BYTES / ((size_t) a->m * sizeof (double2)));

  if (ns > ns_max)
  {
    kp = (int) ((a->n + ns_max - 1) / ns_max);
    kp = ((kp + kc - 1) / kc) * kc;
    ns = (a->n + kp - 1) / kp;
  }

  double2 *part    = (double2 *) addr;
  const int64_t bx = (a->m + EV_THREADS - 1) / EV_THREADS;
  dim3 grid ((unsigned) bx, (unsigned) ns);

  fn<<<grid, EV_THREADS, 0, s>>> (*a, Xq, pack64, c, Vg, part, kp);

  if ((e = cudaGetLastError ()) != cudaSuccess)
    return e;

  _merge_kernel<double2><<<(unsigned) ((a->m + 255) / 256), 256, 0, s>>> (part, ns, a->m, a->final_shift, NULL,
                                                                          a->d_ln_href, 0, out);

  return cudaGetLastError ();
}

/* ------------------------------------------------- FP64 pipe measurement */

/* Eight independent FMA chains per thread, x <- x * b + c with |b| < 1 (the
 * chains converge to c / (1 - b), no overflow or subnormals); one store per
 * thread keeps the work live.  2 * 8 * iters flops per thread. */
__global__ void __launch_bounds__ (256)
_dfma_peak_kernel (double *out, int iters, double b, double c)
{
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1.0, x2 = x0 + 2.0, x3 = x0 + 3.0;
  double x4 = x0 + 4.0, x5 = x0 + 5.0, x6 = x0 + 6.0, x7 = x0 + 7.0;

  for (int i = 0; i < iters; i++)
  {
#pragma unroll
    for (int u = 0; u < 16; u++)
    {
      x0 = fma (x0, b, c);
      x1 = fma (x1, b, c);
      x2 = fma (x2, b, c);
      x3 = fma (x3, b, c);
      x4 = fma (x4, b, c);
      x5 = fma (x5, b, c);
      x6 = fma (x6, b, c);
      x7 = fma (x7, b, c);
    }
  }

  out[(size_t) blockIdx.x * blockDim.x + threadIdx.x] = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
}

extern "C" cudaError_t
ncg_launch_dfma_peak (double *out, int blocks, int iters, cudaStream_t s)
{
  _dfma_peak_kernel<<<blocks, 256, 0, s>>> (out, iters, 0.9999999, 1e-3);

  return cudaGetLastError ();
}

/* ------------------------------------------------- non-finite inputs */

/* flag = 1 when any of the n values is NaN or infinite (a plain store of 1:
 * every writer writes the same value) */
__global__ void __launch_bounds__ (256)
_nonfinite_kernel (const double *__restrict__ X, int64_t n, int32_t *flag)
{
  int bad = 0;

  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x)
    bad |= !isfinite (X[i]);

  if (__syncthreads_or (bad) && threadIdx.x == 0)
    *(volatile int32_t *) flag = 1;
}

extern "C" cudaError_t
ncg_launch_nonfinite (const double *X, int64_t n, int32_t *flag, cudaStream_t s)
{
  if (n <= 0)
    return cudaSuccess;

  const int64_t b = (n + 255) / 256;

  _nonfinite_kernel<<<(unsigned) (b < 608 ? b : 608), 256, 0, s>>> (X, n, flag);

  return cudaGetLastError ();
}
