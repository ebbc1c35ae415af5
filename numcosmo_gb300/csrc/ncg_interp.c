/*
 * ncg_interp.c -- prepare_interp and its NNLS weight fit (n_obs x n_kernels).
 *
 * Control flow of _ncm_stats_dist_prepare_interp
 * (numcosmo/ncm/stats/ncm_stats_dist.c:878-1094): range cut and heuristic
 * weights, recursion on the cut sample, f_i = exp(-(m2lnp_i - min)/2), the
 * interpolation matrix with rows scaled by 1/f_i, NNLS on IM w = 1, and the
 * shrink normalisation.  The NNLS is the active-set method of ncm_nnls_solve
 * (numcosmo/ncm/algebra/ncm_nnls.c:728-871) with the index-set rules of
 * numcosmo/ncm/core/ncm_iset.c:853-1078: the set bookkeeping (a few integer
 * decisions per iteration) runs here, every O(n^2) and O(n^3) step runs on
 * the device (ncg_linalg.cu).
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "ncg_internal.h"
#include "ncg_host.h"

#define CK(call, where)                                   \
  do {                                                    \
    ncg_status_t _s = ncg_cuda_status ((call), (where));  \
    if (_s != NCG_OK)                                     \
      return _s;                                          \
  } while (0)

#define NRES(ptr, cap, bytes) \
  do { ncg_status_t _r = ncg_sd_reserve (sd, (void **) &sd->nn.ptr, &sd->nn.cap, (bytes)); if (_r != NCG_OK) return _r; } while (0)

/* GSL_LOG_DBL_EPSILON */
#define NCG_LOG_DBL_EPSILON (-3.6043653389117154e+01)

static int
_in_ws (const ncg_sd_t *sd, const void *p)
{
  return sd->ws_base != NULL && p != NULL && (const char *) p >= (const char *) sd->ws_base &&
         (const char *) p < (const char *) sd->ws_base + sd->ws_size;
}

void
ncg_nnls_free (ncg_sd_t *sd)
{
  void **bufs[] = {
    (void **) &sd->nn.IM, (void **) &sd->nn.M, (void **) &sd->nn.b, (void **) &sd->nn.f1, (void **) &sd->nn.x,
    (void **) &sd->nn.xsub, (void **) &sd->nn.Msub, (void **) &sd->nn.bsub, (void **) &sd->nn.res,
    (void **) &sd->nn.mg, (void **) &sd->nn.part, (void **) &sd->nn.red, (void **) &sd->nn.P, (void **) &sd->nn.info,
    (void **) &sd->nn.M32, (void **) &sd->nn.R32, (void **) &sd->nn.t32, (void **) &sd->nn.diagM,
    (void **) &sd->nn.D, (void **) &sd->nn.xv, (void **) &sd->nn.pv, (void **) &sd->nn.qv, (void **) &sd->nn.zv,
    (void **) &sd->nn.rv, (void **) &sd->nn.rp, (void **) &sd->nn.vf, (void **) &sd->nn.yf, (void **) &sd->nn.qf,
    (void **) &sd->nn.sc, (void **) &sd->nn.Vi, (void **) &sd->nn.csync, (void **) &sd->nn.pk32,
    (void **) &sd->nn.Q, (void **) &sd->nn.qy,
  };

  for (size_t i = 0; i < sizeof (bufs) / sizeof (bufs[0]); i++)
  {
    if (*bufs[i] && !_in_ws (sd, *bufs[i]))
      ncg_sd_release (sd, *bufs[i]);

    *bufs[i] = NULL;
  }

  memset (&sd->nn, 0, sizeof (sd->nn));
}

/* forget the arena's carving (a new prepare_interp / compute_IM carves it
 * again from the start, in the same order) */
static void
_ws_reset (ncg_sd_t *sd)
{
  void **big[]   = { (void **) &sd->nn.IM, (void **) &sd->nn.M, (void **) &sd->nn.Msub, (void **) &sd->nn.M32,
                     (void **) &sd->nn.R32 };
  size_t *caps[] = { &sd->nn.cIM, &sd->nn.cM, &sd->nn.cMsub, &sd->nn.cM32, &sd->nn.cR32 };

  sd->ws_off = 0;

  for (size_t i = 0; i < sizeof (big) / sizeof (big[0]); i++)
    if (_in_ws (sd, *big[i]))
    {
      *big[i]  = NULL;
      *caps[i] = 0;
    }
}

/* The O(n^2) matrices (IM, M, Msub, M32, R32): carved from the caller's
 * arena when one is set, else owned by the handle.  `arena_ok` = 0 for the
 * mixed solver's rare FP64 fallback, which always allocates. */
static ncg_status_t
_big_reserve (ncg_sd_t *sd, void **ptr, size_t *cap, size_t bytes, int arena_ok)
{
  if (sd->ws_base == NULL || !arena_ok)
  {
    if (_in_ws (sd, *ptr))
    {
      *ptr = NULL;
      *cap = 0;
    }

    return ncg_sd_reserve (sd, ptr, cap, bytes);
  }

  if (*ptr != NULL && _in_ws (sd, *ptr) && *cap >= bytes)
    return NCG_OK;

  if (*ptr != NULL && !_in_ws (sd, *ptr))
    ncg_sd_release (sd, *ptr);

  {
    const size_t off = (sd->ws_off + 255) & ~(size_t) 255;

    if (off + bytes > sd->ws_size)
    {
      ncg_set_error ("prepare_interp: workspace of %zu bytes too small (needs more than %zu)", sd->ws_size,
                     off + bytes);
      *ptr = NULL;
      *cap = 0;

      return NCG_ERR_OUT_OF_MEMORY;
    }

    *ptr       = (char *) sd->ws_base + off;
    *cap       = bytes;
    sd->ws_off = off + bytes;
  }

  return NCG_OK;
}

#define BRES(ptr, cap, bytes, arena_ok) \
  do { ncg_status_t _r = _big_reserve (sd, (void **) &sd->nn.ptr, &sd->nn.cap, (bytes), (arena_ok)); if (_r != NCG_OK) return _r; } while (0)

size_t
ncg_sd_workspace_bytes_for (uint64_t n, int mixed)
{
  return ncg_sd_workspace_bytes_rect (n, n, mixed);
}

/* the interpolation matrix (n_obs x n_kernels) and the n_kernels^2 normal-
 * equation matrices: M32 and R32 (mixed) or M and Msub (FP64) */
size_t
ncg_sd_workspace_bytes_rect (uint64_t nobs, uint64_t nk, int mixed)
{
  const size_t im = 8 * (size_t) nobs * (size_t) nk, k2 = (size_t) nk * (size_t) nk;

  return im + (mixed ? 8 * k2 : 16 * k2) + 4 * 256;
}

/* n_kernels of a sample of n observations under the handle's CV type
 * (ncm_stats_dist.c:714-740) */
uint64_t
ncg_sd_kernels_for (const ncg_sd_t *sd, uint64_t n)
{
  if (sd->cfg.cv_type == NCG_CV_SPLIT || sd->cfg.cv_type == NCG_CV_SPLIT_NOFIT)
    return (uint64_t) ceil ((double) n * sd->split_frac);

  return n;
}

ncg_status_t
ncg_sd_workspace_bytes (ncg_sd_t *sd, uint64_t n, size_t *bytes)
{
  if (sd == NULL || bytes == NULL)
    return NCG_ERR_INVALID_ARG;

  {
    const uint64_t nobs = n ? n : sd->n;

    *bytes = ncg_sd_workspace_bytes_rect (nobs, ncg_sd_kernels_for (sd, nobs), sd->cfg.precision != NCG_PREC_FP64);
  }

  return NCG_OK;
}

ncg_status_t
ncg_sd_set_workspace (ncg_sd_t *sd, void *d_ws, size_t bytes)
{
  if (sd == NULL || (d_ws == NULL && bytes != 0) || (d_ws != NULL && ((uintptr_t) d_ws & 255) != 0))
    return NCG_ERR_INVALID_ARG;

  cudaSetDevice (sd->cfg.device);
  cudaStreamSynchronize (sd->stream);

  {
    void **big[]   = { (void **) &sd->nn.IM, (void **) &sd->nn.M, (void **) &sd->nn.Msub, (void **) &sd->nn.M32,
                       (void **) &sd->nn.R32 };
    size_t *caps[] = { &sd->nn.cIM, &sd->nn.cM, &sd->nn.cMsub, &sd->nn.cM32, &sd->nn.cR32 };

    for (size_t i = 0; i < sizeof (big) / sizeof (big[0]); i++)
    {
      if (*big[i] && !_in_ws (sd, *big[i]))
        ncg_sd_release (sd, *big[i]);

      *big[i]  = NULL;
      *caps[i] = 0;
    }
  }

  sd->ws_base = d_ws;
  sd->ws_size = d_ws ? bytes : 0;
  sd->ws_off  = 0;

  return NCG_OK;
}

typedef struct
{
  ncg_sd_t *sd;
  int n, mixed;           /* n: columns (kernels) */
  int nr;                 /* rows (observations) of the interpolation matrix */
  char *P, *Ptry;
  int32_t *Pidx;
  double *x, *xtry, *mg;
  double rnorm;
} nnls_t;

/* FP64 A^T A (upper), made on first use by the mixed solver's fallback */
static ncg_status_t
_ensure_M64 (nnls_t *s)
{
  ncg_sd_t *sd = s->sd;

  if (sd->nn.M64_ready)
    return NCG_OK;

  BRES (M, cM, sizeof (double) * (size_t) s->n * s->n, 0);
  CK (ncg_launch_syrk_upper (sd->nn.IM, s->nr, s->n, sd->nn.M, sd->stream), "syrk");
  sd->nn.M64_ready = 1;

  return NCG_OK;
}

/* dposv on the set P (Pidx[0..np) already on the device): FP64 Cholesky of
 * the gathered normal equations; when they are not positive definite, the
 * fallbacks of _ncm_nnls_solve_normal_cholesky (ncm_nnls.c:640-652): the
 * symmetric solve of the regathered system (LU, :573-606) and, at an exactly
 * zero pivot, least squares on the columns P of A itself (QR, :608-638) */
static ncg_status_t
_solve_fp64 (nnls_t *s, int np, double *dx)
{
  ncg_sd_t *sd = s->sd;
  cudaStream_t st = sd->stream;
  int info = 0;

  BRES (Msub, cMsub, sizeof (double) * (size_t) np * np, !s->mixed);
  CK (ncg_launch_gather_sub (sd->nn.M, s->n, sd->nn.P, np, sd->nn.Msub, sd->nn.b, sd->nn.bsub, st), "gather");
  CK (ncg_launch_potrf (sd->nn.Msub, np, sd->nn.info, NULL, st), "potrf");
  CK (cudaMemcpyAsync (&info, sd->nn.info, sizeof (int32_t), cudaMemcpyDeviceToHost, st), "D2H info");
  CK (cudaStreamSynchronize (st), "sync");
  sd->istats.n_fp64++;

  if (info == 0)
  {
    CK (ncg_launch_potrs (sd->nn.Msub, np, sd->nn.bsub, sd->nn.xsub, st), "potrs");
    CK (ncg_launch_scatter_x (sd->nn.bsub, sd->nn.P, np, s->n, dx, st), "scatter");

    return NCG_OK;
  }

  sd->istats.n_lu++;
  CK (ncg_launch_gather_sub (sd->nn.M, s->n, sd->nn.P, np, sd->nn.Msub, sd->nn.b, sd->nn.bsub, st), "gather");
  CK (ncg_launch_sysv (sd->nn.Msub, np, sd->nn.bsub, sd->nn.info, st), "sysv");
  CK (cudaMemcpyAsync (&info, sd->nn.info, sizeof (int32_t), cudaMemcpyDeviceToHost, st), "D2H info");
  CK (cudaStreamSynchronize (st), "sync");

  if (info == 0)
  {
    CK (ncg_launch_scatter_x (sd->nn.bsub, sd->nn.P, np, s->n, dx, st), "scatter");

    return NCG_OK;
  }

  sd->istats.n_qr++;
  NRES (Q, cQ, sizeof (double) * (size_t) s->nr * np);
  NRES (qy, cqy, sizeof (double) * ((size_t) s->nr + 4));
  CK (ncg_launch_gels (sd->nn.IM, s->nr, s->n, sd->nn.P, np, sd->nn.f1, sd->nn.Q, sd->nn.qy, sd->nn.qy + s->nr,
                       sd->nn.bsub, st), "gels");
  CK (ncg_launch_scatter_x (sd->nn.bsub, sd->nn.P, np, s->n, dx, st), "scatter");

  return NCG_OK;
}

/* Iteration limits of the mixed solver.  The scaled residual |D r| / |D b|
 * reaches the FP64 rounding floor (a few 1e-15) in a handful of iterations
 * when the FP32 factor is a good preconditioner; the loop stops there, or
 * when the residual has stopped halving for NCG_PCG_STALL iterations. */
#define NCG_PCG_MAXIT 60
#define NCG_PCG_TOL 1.0e-14
#define NCG_PCG_STALL 3
#define NCG_PCG_ACCEPT 1.0e-9
#define NCG_PCG_RESTART 8

/* The mixed solve on the set P: FP32 Cholesky of the Jacobi-scaled
 * (A^T A)_P as the preconditioner of FP64 conjugate gradients whose products
 * are taken from A itself.  A factorisation that breaks down is retried with
 * a diagonal shift; a preconditioner that does not bring the residual below
 * NCG_PCG_ACCEPT hands the set to the FP64 Cholesky. */
static ncg_status_t
_solve_mixed (nnls_t *s, int np, double *dx)
{
  static const double shifts[] = { 0.0, 1.0e-6, 1.0e-3 };
  ncg_sd_t *sd = s->sd;
  ncg_nnls_dev_t *nn = &sd->nn;
  cudaStream_t st = sd->stream;
  const int n = s->n, nr = s->nr;
  int32_t info[2] = { 1, 0 };
  double hs[NCG_PCG_NSC];

  for (int a = 0; a < 3 && info[0] != 0; a++)
  {
    if (a > 0)
      sd->istats.n_shifted++;

    CK (ncg_launch_gather_scaled_f32 (nn->M32, n, nn->P, np, nn->diagM, shifts[a], nn->R32, nn->D, nn->b, nn->bsub,
                                      st), "gather scaled");
    CK (ncg_launch_potrf_f32 (nn->R32, np, nn->info, nn->pk32, st), "potrf f32");
    CK (ncg_launch_trinv_diag_f32 (nn->R32, np, nn->Vi, st), "diagonal inverses");
    CK (cudaMemcpyAsync (info, nn->info, sizeof (info), cudaMemcpyDeviceToHost, st), "D2H info");
    CK (cudaStreamSynchronize (st), "sync");

    /* info[0] < 0: a wait of the tensor-core update gave up (in A^T A: info[1]) */
    if (info[0] < 0 || info[1] != 0)
    {
      ncg_set_error ("prepare_interp: a wait of the tensor-core rank-K update gave up");

      return NCG_ERR_TIMEOUT;
    }
  }

  if (info[0] == 0)
  {
    double best = INFINITY;
    int stall = 0, it;

    /* x0 = B^{-1} b (the FP32 factor makes it accurate to about its own
     * precision), r = b - A_P^T A_P x0, z = B^{-1} r, p = z */
    CK (ncg_launch_pcg_precond (nn->R32, nn->Vi, nn->D, np, nn->bsub, nn->t32, &nn->cs_epoch, nn->xv, nn->csync,
                                 nn->sc + NCG_PCG_ERR, st), "precond");
    CK (ncg_launch_pcg_matvec (nn->IM, nr, n, nn->P, np, nn->xv, nn->vf, nn->yf, nn->qf, nn->part, nn->rv, st), "matvec");
    CK (ncg_launch_rsub (nn->bsub, nn->rv, np, st), "rsub");
    CK (ncg_launch_pcg_precond (nn->R32, nn->Vi, nn->D, np, nn->rv, nn->t32, &nn->cs_epoch, nn->zv, nn->csync,
                                 nn->sc + NCG_PCG_ERR, st), "precond");
    CK (cudaMemcpyAsync (nn->pv, nn->zv, sizeof (double) * np, cudaMemcpyDeviceToDevice, st), "D2D p");
    CK (ncg_launch_pcg_dot (nn->rv, nn->zv, NULL, NULL, NULL, np, nn->sc, NCG_PCG_RZ, 0, st), "dot");
    CK (ncg_launch_pcg_dot (nn->bsub, nn->bsub, NULL, NULL, nn->D, np, nn->sc, NCG_PCG_BB, 0, st), "dot");
    CK (ncg_launch_pcg_dot (nn->rv, nn->rv, NULL, NULL, nn->D, np, nn->sc, NCG_PCG_RR, 0, st), "dot");

    for (it = 0;; it++)
    {
      double rel;

      CK (cudaMemcpyAsync (hs, nn->sc, sizeof (hs), cudaMemcpyDeviceToHost, st), "D2H sc");
      CK (cudaStreamSynchronize (st), "sync");

      if (hs[NCG_PCG_ERR] != 0.0)
      {
        ncg_set_error ("prepare_interp: a wait of the preconditioner's triangular solve gave up");

        return NCG_ERR_TIMEOUT;
      }

      rel = (hs[NCG_PCG_BB] > 0.0) ? sqrt (hs[NCG_PCG_RR] / hs[NCG_PCG_BB]) : 0.0;

      if (!isfinite (rel))
        break;

      if (rel < 0.5 * best)
      {
        best  = rel;
        stall = 0;
      }
      else
      {
        stall++;
      }

      if (rel <= NCG_PCG_TOL || it >= NCG_PCG_MAXIT || (stall >= NCG_PCG_STALL && best < NCG_PCG_ACCEPT) ||
          !(hs[NCG_PCG_RZ] > 0.0))
        break;

      CK (ncg_launch_pcg_matvec (nn->IM, nr, n, nn->P, np, nn->pv, nn->vf, nn->yf, nn->qf, nn->part, nn->qv, st),
          "matvec");
      CK (ncg_launch_pcg_dot (nn->pv, nn->qv, NULL, NULL, NULL, np, nn->sc, NCG_PCG_PQ, 0, st), "dot");
      CK (ncg_launch_pcg_step (nn->xv, nn->rv, nn->rp, nn->pv, nn->qv, np, nn->sc, st), "step");

      if ((it + 1) % NCG_PCG_RESTART == 0)
      {
        /* replace the recurred residual by the true one */
        CK (ncg_launch_pcg_matvec (nn->IM, nr, n, nn->P, np, nn->xv, nn->vf, nn->yf, nn->qf, nn->part, nn->rv, st),
            "matvec");
        CK (ncg_launch_rsub (nn->bsub, nn->rv, np, st), "rsub");
      }

      CK (ncg_launch_pcg_precond (nn->R32, nn->Vi, nn->D, np, nn->rv, nn->t32, &nn->cs_epoch, nn->zv, nn->csync,
                                 nn->sc + NCG_PCG_ERR, st), "precond");
      CK (ncg_launch_pcg_dot (nn->rv, nn->zv, nn->zv, nn->rp, NULL, np, nn->sc, NCG_PCG_RZN, NCG_PCG_ZRP, st), "dot");
      CK (ncg_launch_pcg_dir (nn->pv, nn->zv, np, nn->sc, st), "dir");
      CK (ncg_launch_pcg_dot (nn->rv, nn->rv, NULL, NULL, nn->D, np, nn->sc, NCG_PCG_RR, 0, st), "dot");
    }

    sd->istats.n_cg_iters += it;

    if (best <= NCG_PCG_ACCEPT)
    {
      CK (ncg_launch_scatter_x (nn->xv, nn->P, np, n, dx, st), "scatter");

      return NCG_OK;
    }
  }

  {
    ncg_status_t r = _ensure_M64 (s);

    if (r != NCG_OK)
      return r;
  }

  return _solve_fp64 (s, np, dx);
}

/* solve the normal equations on the set P into the device vector dx */
static ncg_status_t
_solve_unconstrained (nnls_t *s, const char *inP, double *dx)
{
  ncg_sd_t *sd = s->sd;
  cudaStream_t st = sd->stream;
  int np = 0;

  for (int i = 0; i < s->n; i++)
    if (inP[i])
      s->Pidx[np++] = i;

  sd->istats.n_solves++;

  if (np == 0)
  {
    CK (cudaMemsetAsync (dx, 0, sizeof (double) * s->n, st), "memset");

    return NCG_OK;
  }

  CK (cudaMemcpyAsync (sd->nn.P, s->Pidx, sizeof (int32_t) * np, cudaMemcpyHostToDevice, st), "H2D P");

  return s->mixed ? _solve_mixed (s, np, dx) : _solve_fp64 (s, np, dx);
}

typedef struct { double v; int pos; } _vi_t;

static int
_vi_asc (const void *a, const void *b)
{
  const _vi_t *pa = a, *pb = b;

  if (pa->v < pb->v) return -1;
  if (pa->v > pb->v) return 1;
  return (pa->pos < pb->pos) ? -1 : (pa->pos > pb->pos);
}

static int
_vi_desc (const void *a, const void *b)
{
  const _vi_t *pa = a, *pb = b;

  if (pa->v > pb->v) return -1;
  if (pa->v < pb->v) return 1;
  return (pa->pos < pb->pos) ? -1 : (pa->pos > pb->pos);
}

/* _ncm_nnls_solve_feasible (ncm_nnls.c:728-751); leaves the solution in dx
 * and its host copy in hx */
static ncg_status_t
_solve_feasible (nnls_t *s, char *inP, double *dx, double *hx, int max_remove)
{
  ncg_sd_t *sd = s->sd;
  _vi_t *inv   = malloc (sizeof (_vi_t) * s->n);
  ncg_status_t r;

  if (inv == NULL)
    return NCG_ERR_OUT_OF_MEMORY;

  r = _solve_unconstrained (s, inP, dx);

  while (r == NCG_OK)
  {
    int ninv = 0;

    r = ncg_cuda_status (cudaMemcpyAsync (hx, dx, sizeof (double) * s->n, cudaMemcpyDeviceToHost, sd->stream), "D2H x");

    if (r == NCG_OK)
      r = ncg_cuda_status (cudaStreamSynchronize (sd->stream), "sync");

    if (r != NCG_OK)
      break;

    /* ncm_iset_get_subset_vec_lt (ncm_iset.c:853-875) */
    for (int i = 0; i < s->n; i++)
      if (inP[i] && hx[i] < 1.0e-300)
      {
        inv[ninv].v   = hx[i];
        inv[ninv].pos = i;
        ninv++;
      }

    if (ninv == 0)
      break;

    /* ncm_iset_remove_smallest_subset (ncm_iset.c:920-975) */
    if (max_remove >= ninv)
    {
      for (int i = 0; i < ninv; i++)
        inP[inv[i].pos] = 0;
    }
    else
    {
      qsort (inv, ninv, sizeof (_vi_t), _vi_asc);

      for (int i = 0; i < max_remove; i++)
        inP[inv[i].pos] = 0;
    }

    r = _solve_unconstrained (s, inP, dx);
  }

  free (inv);

  return r;
}

static ncg_status_t
_residuals (nnls_t *s, const double *dx, double *dres, double *rnorm)
{
  ncg_sd_t *sd = s->sd;
  double r2    = 0.0;

  CK (ncg_launch_residual_norm (sd->nn.IM, s->nr, s->n, dx, sd->nn.f1, dres, sd->nn.red, sd->stream), "residual");
  CK (cudaMemcpyAsync (&r2, sd->nn.red, sizeof (double), cudaMemcpyDeviceToHost, sd->stream), "D2H rnorm");
  CK (cudaStreamSynchronize (sd->stream), "sync");
  *rnorm = sqrt (r2);

  return NCG_OK;
}

static ncg_status_t
_mgrad (nnls_t *s, const double *dres)
{
  ncg_sd_t *sd = s->sd;

  CK (ncg_launch_gemv_ex (sd->nn.IM, s->nr, s->n, 1, 1.0, dres, 0.0, sd->nn.mg, sd->nn.part, sd->stream), "mgrad");
  CK (cudaMemcpyAsync (s->mg, sd->nn.mg, sizeof (double) * s->n, cudaMemcpyDeviceToHost, sd->stream), "D2H mgrad");
  CK (cudaStreamSynchronize (sd->stream), "sync");

  return NCG_OK;
}

/* ncm_iset_add_largest_subset (ncm_iset.c:994-1078) */
static int
_add_largest (char *inP, int n, const double *v, double vmin, double add_frac)
{
  _vi_t *cand = malloc (sizeof (_vi_t) * n);
  int k = 0, adds, csize = 0;

  for (int i = 0; i < n; i++)
    if (!inP[i])
    {
      csize++;

      if (v[i] > vmin)
      {
        cand[k].v   = v[i];
        cand[k].pos = i;
        k++;
      }
    }

  if (csize == 0)
  {
    free (cand);

    return 0;
  }

  {
    const double kf = k * add_frac;
    const double mx = (kf > 1.0) ? kf : 1.0;

    adds = (int) ((k < mx) ? (double) k : mx);
  }

  if (adds > 0)
  {
    qsort (cand, k, sizeof (_vi_t), _vi_desc);

    for (int i = 0; i < adds; i++)
      inP[cand[i].pos] = 1;
  }

  free (cand);

  return adds;
}

/* every device buffer the NNLS of an nr x n system reserves (the large
 * matrices from the caller's arena when one is set, after the interpolation
 * matrix) */
static ncg_status_t
_nnls_reserve (ncg_sd_t *sd, int nr, int n, int mixed)
{
  NRES (b, cb, sizeof (double) * n);
  NRES (f1, cf1, sizeof (double) * nr);
  NRES (x, cx, sizeof (double) * n);
  NRES (xsub, cxsub, sizeof (double) * n);
  NRES (bsub, cbsub, sizeof (double) * n);
  NRES (res, cres, sizeof (double) * nr * 2);
  NRES (mg, cmg, sizeof (double) * n);
  NRES (part, cpart, ncg_gemv_t_scratch (nr, n));
  NRES (red, cred, sizeof (double) * 4);
  NRES (P, cP, sizeof (int32_t) * n);
  NRES (info, cinfo, sizeof (int32_t) * 4);

  if (mixed)
  {
    BRES (M32, cM32, sizeof (float) * (size_t) n * n, 1);
    BRES (R32, cR32, sizeof (float) * (size_t) n * n, 1);
    NRES (t32, ct32, ncg_pcg_chain_bytes (n));
    NRES (diagM, cdiagM, sizeof (double) * n);
    NRES (D, cD, sizeof (double) * n);
    NRES (xv, cxv, sizeof (double) * n);
    NRES (pv, cpv, sizeof (double) * n);
    NRES (qv, cqv, sizeof (double) * n);
    NRES (zv, czv, sizeof (double) * n);
    NRES (rv, crv, sizeof (double) * n);
    NRES (rp, crp, sizeof (double) * n);
    NRES (vf, cvf, sizeof (double) * n);
    NRES (yf, cyf, sizeof (double) * nr);
    NRES (qf, cqf, sizeof (double) * n);
    NRES (sc, csc, sizeof (double) * NCG_PCG_NSC);
    NRES (Vi, cVi, ncg_pcg_trinv_bytes (n));
    NRES (csync, ccsync, ncg_pcg_sync_bytes (n));
    NRES (pk32, cpk32, ncg_syrk_tc_pack_bytes (n, 64));
  }
  else
  {
    BRES (M, cM, sizeof (double) * (size_t) n * n, 1);
    BRES (Msub, cMsub, sizeof (double) * (size_t) n * n, 1);
  }

  return NCG_OK;
}

/* Every buffer a weight fit of the current sample reserves -- the prepare's,
 * the interpolation matrix and the NNLS's -- reserved now (before several
 * handles' fits run at once from host threads, where a cudaMalloc would
 * synchronise the device under all of them).  What the fit would reject is
 * left for the fit to report; a range cut only shrinks the sizes. */
void
ncg_sd_interp_reserve (ncg_sd_t *sd)
{
  const uint64_t n = sd ? sd->n : 0, nk = sd ? ncg_sd_kernels_for (sd, n) : 0;

  ncg_sd_prepare_reserve (sd);

  if (n == 0 || nk == 0 || n > 0x7fffffffULL)
    return;

  if (ncg_sd_reserve (sd, (void **) &sd->df, &sd->cap.f, sizeof (double) * n) != NCG_OK)
    return;

  _ws_reset (sd);

  if (_big_reserve (sd, (void **) &sd->nn.IM, &sd->nn.cIM, sizeof (double) * (size_t) n * nk, 1) != NCG_OK)
    return;

  (void) _nnls_reserve (sd, (int) n, (int) nk, sd->cfg.precision != NCG_PREC_FP64);
}

/* ncm_nnls_solve (ncm_nnls.c:767-871), reltol = DBL_EPSILON; the solution is
 * left in sd->dw.  With mixed = 1 every active-set solve goes through
 * _solve_mixed (the O(n^3) work in FP32, FP64 refinement); the set logic,
 * residuals and gradients are the same FP64 computations in both forms. */
static ncg_status_t
_nnls (ncg_sd_t *sd, int nr, int n, int mixed, double *rnorm_out)
{
  const double reltol = DBL_EPSILON;
  cudaStream_t st     = sd->stream;
  nnls_t s;
  ncg_status_t r = NCG_OK;
  double rnorm;

  if ((r = _nnls_reserve (sd, nr, n, mixed)) != NCG_OK)
    return r;

  sd->nn.M64_ready = 0;
  memset (&sd->istats, 0, sizeof (sd->istats));

  CK (ncg_launch_fill (sd->nn.f1, 1.0, nr, st), "fill");
  CK (ncg_launch_gemv_ex (sd->nn.IM, nr, n, 1, 1.0, sd->nn.f1, 0.0, sd->nn.b, sd->nn.part, st), "gemv b");

  if (mixed)
  {
    CK (cudaMemsetAsync (sd->nn.sc, 0, sizeof (double) * NCG_PCG_NSC, st), "memset sc");
    CK (cudaMemsetAsync (sd->nn.csync, 0, ncg_pcg_sync_bytes (n), st), "memset sync");
    /* the chained solves' words: epoch 0 matches no launch */
    CK (cudaMemsetAsync (sd->nn.t32, 0, ncg_pcg_chain_bytes (n), st), "memset chain");
    CK (cudaMemsetAsync (sd->nn.info, 0, sizeof (int32_t) * 4, st), "memset info");

    /* A^T A on the tensor cores (TF32x3; packed K slabs in the factor's
     * buffer, which is free until the first solve), small n on CUDA cores */
    if (n >= 1024)
      CK (ncg_launch_syrk_upper_tc_f64 (sd->nn.IM, nr, n, sd->nn.M32, sd->nn.R32, sizeof (float) * (size_t) n * n,
                                        sd->nn.info + 1, st), "syrk tc");
    else
      CK (ncg_launch_syrk_upper_f32 (sd->nn.IM, nr, n, sd->nn.M32, st), "syrk f32");
    CK (ncg_launch_colsumsq (sd->nn.IM, nr, n, sd->nn.diagM, st), "colsumsq");
  }
  else
  {
    CK (ncg_launch_syrk_upper (sd->nn.IM, nr, n, sd->nn.M, st), "syrk");
    sd->nn.M64_ready = 1;
  }

  memset (&s, 0, sizeof (s));
  s.sd    = sd;
  s.n     = n;
  s.nr    = nr;
  s.mixed = mixed;
  s.P    = malloc (n);
  s.Ptry = malloc (n);
  s.Pidx = malloc (sizeof (int32_t) * n);
  s.x    = malloc (sizeof (double) * n);
  s.xtry = malloc (sizeof (double) * n);
  s.mg   = malloc (sizeof (double) * n);

  if (!s.P || !s.Ptry || !s.Pidx || !s.x || !s.xtry || !s.mg)
  {
    r = NCG_ERR_OUT_OF_MEMORY;
    goto out;
  }

  {
    double *dres = sd->nn.res, *drtr = sd->nn.res + nr;
    double *dxtr = sd->nn.x;      /* trial solution */
    double *dxac = sd->dw;        /* accepted solution */

    memset (s.P, 1, n);

    if ((r = _solve_feasible (&s, s.P, dxac, s.x, n)) != NCG_OK)
      goto out;

    if ((r = _residuals (&s, dxac, dres, &rnorm)) != NCG_OK)
      goto out;

    if ((r = _mgrad (&s, dres)) != NCG_OK)
      goto out;

    while (1)
    {
      double add_frac = 1.0;
      int finish      = 0;

      while (1)
      {
        double lrnorm;
        int added;

        memcpy (s.Ptry, s.P, n);
        added     = _add_largest (s.Ptry, n, s.mg, rnorm * reltol, add_frac);
        add_frac *= 0.5;

        if (added == 0)
        {
          finish = 1;
          break;
        }

        if ((r = _solve_feasible (&s, s.Ptry, dxtr, s.xtry, added)) != NCG_OK)
          goto out;

        if ((r = _residuals (&s, dxtr, drtr, &lrnorm)) != NCG_OK)
          goto out;

        if (rnorm - lrnorm > rnorm * reltol)
        {
          memcpy (s.P, s.Ptry, n);
          memcpy (s.x, s.xtry, sizeof (double) * n);
          CK (cudaMemcpyAsync (dxac, dxtr, sizeof (double) * n, cudaMemcpyDeviceToDevice, st), "D2D x");
          CK (cudaMemcpyAsync (dres, drtr, sizeof (double) * nr, cudaMemcpyDeviceToDevice, st), "D2D res");
          rnorm = lrnorm;
          break;
        }

        if (added == 1)
        {
          finish = 1;
          break;
        }
      }

      if (finish)
        break;

      if ((r = _mgrad (&s, dres)) != NCG_OK)
        goto out;
    }

    *rnorm_out = rnorm;
  }

out:
  free (s.P);
  free (s.Ptry);
  free (s.Pidx);
  free (s.x);
  free (s.xtry);
  free (s.mg);

  return r;
}

typedef struct { double v; int idx; } _sv_t;

static int
_sv_cmp (const void *a, const void *b)
{
  const _sv_t *pa = a, *pb = b;

  if (pa->v < pb->v) return -1;
  if (pa->v > pb->v) return 1;
  return (pa->idx < pb->idx) ? -1 : (pa->idx > pb->idx);
}

static ncg_status_t
_upload_weights (ncg_sd_t *sd, const double *w)
{
  CK (cudaMemcpyAsync (sd->dw, w, sizeof (double) * sd->nk, cudaMemcpyHostToDevice, sd->stream), "H2D weights");
  CK (ncg_launch_weights_c (sd->dw, sd->dlnnorm, (int) sd->nk, sd->kind, sd->dc, NULL, sd->stream), "weights_c");
  CK (cudaStreamSynchronize (sd->stream), "sync");
  sd->wcum_ready   = 0;
  sd->packmx_ready = 0;
  sd->gen++;

  return NCG_OK;
}

/* _ncm_stats_dist_compute_IM_full (ncm_stats_dist.c:791-804) at the current
 * href (rows scaled by the 1/f already on the device), then the NNLS fit */
static ncg_status_t
_im_full_nnls (ncg_sd_t *sd, int n, int nk, double *rnorm)
{
  ncg_eval_args_t a;

  a.kind        = sd->kind;
  a.kernel      = sd->kernel;
  a.d           = (int32_t) sd->d;
  a.dp          = sd->dp;
  a.n           = nk;
  a.m           = n;
  a.nu          = (sd->kernel == NCG_KERNEL_ST) ? sd->nu : 1.0;
  a.kappa       = -0.5 * (sd->nu + sd->d);
  a.final_shift = 0.0;
  a.d_ln_href   = sd->d * log (sd->href);
  a.inv_href    = 1.0 / sd->href;
  a.c_shift     = 0.0;

  CK (ncg_launch_compute_IM (&a, sd->dX, sd->dpack64, sd->dlnnorm, sd->kernel_lnnorm, sd->df, sd->nn.IM,
                             sd->stream), "compute_IM");

  return _nnls (sd, n, nk, sd->cfg.precision != NCG_PREC_FP64, rnorm);
}

/* the weight fit at over_smooth = exp(lnos) */
static ncg_status_t
_fit_at (ncg_sd_t *sd, int n, int nk, double lnos, double *rnorm)
{
  ncg_status_t r;

  sd->cfg.over_smooth = exp (lnos);
  sd->href            = ncg_sd_href_for (sd);

  if ((r = ncg_sd_href_operand (sd)) != NCG_OK)
    return r;

  return _im_full_nnls (sd, n, nk, rnorm);
}

typedef struct
{
  ncg_sd_t *sd;
  int n, nk;
  const double *m2lnp;
  double min_m2lnp;
  double *m2;             /* host, n: -2 ln p at the observations */
} _split_lm_t;

/* _ncm_stats_dist_prepare_interp_fit_nnls_f (ncm_stats_dist.c:815-846): the
 * weight fit at exp(p), then per observation
 * hx_i = expm1(-(m2lnp_fit(x_i) - (m2lnp_i - min))/2) with the fit's raw
 * (unnormalised) NNLS weights */
static ncg_status_t
_split_f (_split_lm_t *c, double p, double *hx)
{
  ncg_sd_t *sd = c->sd;
  ncg_eval_args_t a;
  double rnorm = 0.0;
  ncg_status_t r;

  if ((r = _fit_at (sd, c->n, c->nk, p, &rnorm)) != NCG_OK)
    return r;

  CK (ncg_launch_weights_c (sd->dw, sd->dlnnorm, c->nk, sd->kind, sd->dc, NULL, sd->stream), "weights_c");
  ncg_sd_fill_args (sd, (uint64_t) c->n, &a);
  NRES (res, cres, sizeof (double) * 2 * (size_t) c->n);
  {
    const size_t need = ncg_eval_scratch_bytes (&a, NCG_PREC_FP64);

    if ((r = ncg_sd_reserve (sd, (void **) &sd->dscratch, &sd->cap.scratch, need)) != NCG_OK)
      return r;
  }
  CK (ncg_launch_eval_m2lnp_fp64 (&a, sd->dX, sd->dpack64, sd->dc, sd->dVg, sd->nn.res, sd->dscratch, 0, sd->stream),
      "eval_fp64");
  CK (cudaMemcpyAsync (c->m2, sd->nn.res, sizeof (double) * c->n, cudaMemcpyDeviceToHost, sd->stream), "D2H m2lnp");
  CK (cudaStreamSynchronize (sd->stream), "sync");

  for (int i = 0; i < c->n; i++)
    hx[i] = expm1 (-0.5 * (c->m2[i] - (c->m2lnp[i] - c->min_m2lnp)));

  return NCG_OK;
}

/* |y|^2 in levmar's accumulation order (LEVMAR_L2NRMXMY, lm misc_core.c):
 * blocks of eight from the last full block downwards into four partial sums
 * (sum0..sum3 by position mod 4 within the block, counting down), the
 * remainder upwards continuing the pattern, then sum0 + sum1 + sum2 + sum3 */
static double
_l2_lm (const double *y, int n)
{
  const int blockn = (n >> 3) << 3;
  double s[4] = { 0.0, 0.0, 0.0, 0.0 };

  for (int i = blockn - 1; i > 0; i -= 8)
    for (int j = 0; j < 8; j++)
      s[j & 3] += y[i - j] * y[i - j];

  for (int i = blockn, t = 7 - (n - blockn); i < n; i++, t++)
    s[t & 3] += y[i] * y[i];

  return ((s[0] + s[1]) + s[2]) + s[3];
}

/* The Levenberg-Marquardt fit of dlevmar_dif (the levmar library vendored by
 * the reference, numcosmo/external/levmar/lm_core.c:439-830, Lourakis 2004:
 * damping by Nielsen's rule, forward-difference Jacobian refreshed by Broyden
 * rank-one updates) restated for the one parameter p = ln over_smooth and a
 * zero measurement vector: minimise |f(p)|^2.  opts = (tau, eps1, eps2,
 * eps3, delta) as the reference passes them (ncm_stats_dist.c:1034-1038).
 * The one-by-one normal equation is solved by division; the squared norms
 * follow levmar's summation order, J^T J and J^T e its order for n <= 1024
 * (descending; above that levmar calls BLAS, here ascending). */
static ncg_status_t
_lm1 (_split_lm_t *c, double *p, int itmax, const double *opts)
{
  const int n = c->n;
  const double tau = opts[0], eps1 = opts[1], eps2 = opts[2], eps2_sq = opts[2] * opts[2], eps3 = opts[3];
  const double delta = opts[4];
  const double one_third = 0.3333333334, lm_eps = 1.0e-12;
  double *hx   = malloc (sizeof (double) * n), *wrk = malloc (sizeof (double) * n);
  double *jac  = malloc (sizeof (double) * n), *e = malloc (sizeof (double) * n);
  double p_eL2 = 0.0, mu = 0.0, jacTe = 0.0, jacTjac = 0.0, jacTe_inf = 0.0, p_L2 = 0.0;
  int nu = 20, updjac = 0, updp = 1, newjac = 0, k;
  const int K = 10;
  ncg_status_t r = NCG_OK;

  if (!hx || !wrk || !jac || !e)
  {
    r = NCG_ERR_OUT_OF_MEMORY;
    goto out;
  }

  if ((r = _split_f (c, *p, hx)) != NCG_OK)
    goto out;

  for (int i = 0; i < n; i++)
    e[i] = -hx[i];

  p_eL2 = _l2_lm (e, n);

  if (!isfinite (p_eL2))
    goto out;

  for (k = 0; k < itmax; k++)
  {
    if (p_eL2 <= eps3)
      break;

    if ((updp && nu > 16) || updjac == K)
    {
      /* forward difference, step max(1e-4 |p|, delta) */
      double d = fabs (1.0e-4 * *p);
      const double p0 = *p;

      if (d < delta)
        d = delta;

      if ((r = _split_f (c, p0 + d, wrk)) != NCG_OK)
        goto out;

      d = 1.0 / d;

      for (int i = 0; i < n; i++)
        jac[i] = (wrk[i] - hx[i]) * d;

      nu     = 2;
      updjac = 0;
      updp   = 0;
      newjac = 1;
    }

    if (newjac)
    {
      newjac  = 0;
      jacTjac = 0.0;
      jacTe   = 0.0;

      if (n <= 1024)
        for (int i = n - 1; i >= 0; i--)
        {
          jacTjac += jac[i] * jac[i];
          jacTe   += jac[i] * e[i];
        }
      else
        for (int i = 0; i < n; i++)
        {
          jacTjac += jac[i] * jac[i];
          jacTe   += jac[i] * e[i];
        }

      jacTe_inf = fabs (jacTe);
      p_L2      = *p * *p;
    }

    if (jacTe_inf <= eps1)
      break;

    if (k == 0)
      mu = tau * ((jacTjac > -DBL_MAX) ? jacTjac : -DBL_MAX);

    {
      const double A = jacTjac + mu;

      if (A != 0.0)
      {
        const double Dp   = jacTe / A;
        const double pDp  = *p + Dp;
        const double Dp_L2 = Dp * Dp;
        double pDp_eL2 = 0.0, dF, dL;

        if (Dp_L2 <= eps2_sq * p_L2)
          break;

        if (Dp_L2 >= (p_L2 + eps2) / (lm_eps * lm_eps))
          break;

        if ((r = _split_f (c, pDp, wrk)) != NCG_OK)
          goto out;

        pDp_eL2 = _l2_lm (wrk, n);

        if (!isfinite (pDp_eL2))
          break;

        dF = p_eL2 - pDp_eL2;

        if (updp || dF > 0.0)
        {
          /* Broyden rank-one update of the Jacobian */
          for (int i = 0; i < n; i++)
          {
            const double t = (wrk[i] - hx[i] - jac[i] * Dp) / Dp_L2;

            jac[i] += t * Dp;
          }

          updjac++;
          newjac = 1;
        }

        dL = Dp * (mu * Dp + jacTe);

        if (dL > 0.0 && dF > 0.0)
        {
          double t = 2.0 * dF / dL - 1.0;

          t   = 1.0 - t * t * t;
          mu  = mu * ((t >= one_third) ? t : one_third);
          nu  = 2;
          *p  = pDp;

          for (int i = 0; i < n; i++)
          {
            e[i]  = -wrk[i];
            hx[i] = wrk[i];
          }

          p_eL2 = pDp_eL2;
          updp  = 1;
          continue;
        }
      }
    }

    mu *= nu;

    {
      const int nu2 = nu << 1;

      if (nu2 <= nu)
        break;

      nu = nu2;
    }
  }

out:
  free (hx);
  free (wrk);
  free (jac);
  free (e);

  return r;
}

/* CV_SPLIT (ncm_stats_dist.c:1018-1066): the weight fit at the current
 * bandwidth, ten restarts at ln over_smooth drawn N(ln_os, 0.5) from the
 * handle's generator (kept when they lower the NNLS residual), the
 * Levenberg-Marquardt fit of ln over_smooth to the observations' -2 ln p, and
 * the weight fit at its result */
static ncg_status_t
_split_fit (ncg_sd_t *sd, int n, int nk, const double *m2lnp, double min_m2lnp, double *rnorm)
{
  static const double opts[5] = { 1.0e-3, 1.0e-7, 1.0e-7, 1.0e-10, 1.0e-6 };
  _split_lm_t c;
  double ln_os = log (sd->cfg.over_smooth), rnorm0 = 0.0;
  ncg_status_t r;

  if (sd->cv_rng == NULL && (r = ncg_rng_new (4357u, &sd->cv_rng)) != NCG_OK)
    return r;

  if ((r = _im_full_nnls (sd, n, nk, &rnorm0)) != NCG_OK)
    return r;

  for (int i = 0; i < 10; i++)
  {
    const double ln_os_try = ncg_rng_ugaussian (sd->cv_rng) * 0.5 + ln_os;
    double rnorm_try = 0.0;

    if ((r = _fit_at (sd, n, nk, ln_os_try, &rnorm_try)) != NCG_OK)
      return r;

    if (rnorm_try < rnorm0)
    {
      ln_os  = ln_os_try;
      rnorm0 = rnorm_try;
    }
  }

  c.sd        = sd;
  c.n         = n;
  c.nk        = nk;
  c.m2lnp     = m2lnp;
  c.min_m2lnp = min_m2lnp;
  c.m2        = malloc (sizeof (double) * n);

  if (c.m2 == NULL)
    return NCG_ERR_OUT_OF_MEMORY;

  r = _lm1 (&c, &ln_os, 10000, opts);
  free (c.m2);

  if (r != NCG_OK)
    return r;

  return _fit_at (sd, n, nk, ln_os, rnorm);
}

ncg_status_t
ncg_sd_prepare_interp (ncg_sd_t *sd, const double *m2lnp)
{
  const double dbl_limit = 2.0;
  const double thr       = -2.0 * dbl_limit * NCG_LOG_DBL_EPSILON;
  double min_m2lnp = INFINITY, max_m2lnp = -INFINITY;
  ncg_status_t r;
  int n, nk;

  if (sd == NULL || m2lnp == NULL)
    return NCG_ERR_INVALID_ARG;


  for (uint64_t i = 0; i < sd->n; i++)
    if (!isfinite (m2lnp[i]))
    {
      ncg_set_error ("prepare_interp: non-finite m2lnp at %llu", (unsigned long long) i);

      return NCG_ERR_NONFINITE;
    }

  if ((r = ncg_sd_prepare (sd)) != NCG_OK)
    return r;

  /* n_obs rows, n_kernels columns (equal but under a split, where the
   * kernels are the first n_kernels observations); the range is taken over
   * the kernels' entries, the sort over every observation
   * (ncm_stats_dist.c:895-922) */
  n  = (int) sd->n;
  nk = (int) sd->nk;

  for (int i = 0; i < nk; i++)
  {
    min_m2lnp = fmin (min_m2lnp, m2lnp[i]);
    max_m2lnp = fmax (max_m2lnp, m2lnp[i]);
  }

  if (max_m2lnp - min_m2lnp > thr)
  {
    _sv_t *sv = malloc (sizeof (_sv_t) * n);
    int n_cut = 0;

    if (sv == NULL)
      return NCG_ERR_OUT_OF_MEMORY;

    for (int i = 0; i < n; i++)
    {
      sv[i].v   = m2lnp[i];
      sv[i].idx = i;
    }

    qsort (sv, n, sizeof (_sv_t), _sv_cmp);

    for (int i = 0; i < nk; i++)
      if (sv[i].v - min_m2lnp > thr)
      {
        n_cut = i;
        break;
      }

    if (n_cut < (int) (unsigned) (0.5 * n))
    {
      double *w;

      for (int i = 0; i < n_cut; i++)
        if (sv[i].idx >= nk)
        {
          /* the reference would set a weight past its n_kernels-long vector */
          ncg_set_error ("prepare_interp: held-out observation %d is among the %d kept by the range cut",
                         sv[i].idx, n_cut);
          free (sv);

          return NCG_ERR_INVALID_ARG;
        }

      w = malloc (sizeof (double) * nk);

      for (int i = 0; i < nk; i++)
        w[i] = 0.1 / (nk - n_cut);

      for (int i = 0; i < n_cut; i++)
        w[sv[i].idx] = 0.9 / n_cut;

      r = _upload_weights (sd, w);
      sd->interp_branch = 1;
      free (w);
      free (sv);

      return r;
    }

    {
      double *Xc = malloc (sizeof (double) * (size_t) n * sd->d);
      double *mc = malloc (sizeof (double) * n);
      int j      = 0;

      for (int i = 0; i < n; i++)
        if (m2lnp[i] - min_m2lnp <= thr)
        {
          memcpy (Xc + (size_t) j * sd->d, sd->hX + (size_t) i * sd->d, sizeof (double) * sd->d);
          mc[j++] = m2lnp[i];
        }

      if (j != n_cut)
      {
        /* the reference asserts this count (ncm_stats_dist.c:966); under a
         * split the held-out observations can break it */
        ncg_set_error ("prepare_interp: %d observations below the range cut, %d among the kernels", j, n_cut);
        free (Xc);
        free (mc);
        free (sv);

        return NCG_ERR_INVALID_ARG;
      }

      sd->n = 0;
      r     = ncg_sd_add_obs_batch (sd, Xc, (uint64_t) n_cut);

      if (r == NCG_OK)
        r = ncg_sd_prepare_interp (sd, mc);

      if (r == NCG_OK && sd->interp_branch == 0)
        sd->interp_branch = 2;

      free (Xc);
      free (mc);
      free (sv);

      return r;
    }
  }

  /* f_i and the interpolation matrix with rows scaled by 1/f_i */
  {
    double *f = malloc (sizeof (double) * n);
    int32_t bad = 0;
    double rnorm = 0.0;

    if (f == NULL)
      return NCG_ERR_OUT_OF_MEMORY;

    for (int i = 0; i < n; i++)
      f[i] = exp (-0.5 * (m2lnp[i] - min_m2lnp));

    r = ncg_sd_reserve (sd, (void **) &sd->df, &sd->cap.f, sizeof (double) * n);

    if (r == NCG_OK)
    {
      _ws_reset (sd);
      r = _big_reserve (sd, (void **) &sd->nn.IM, &sd->nn.cIM, sizeof (double) * (size_t) n * nk, 1);
    }

    if (r == NCG_OK)
      r = ncg_cuda_status (cudaMemcpyAsync (sd->df, f, sizeof (double) * n, cudaMemcpyHostToDevice, sd->stream), "H2D f");

    free (f);

    if (r != NCG_OK)
      return r;

    if (nk > 20000)
      ncg_set_error ("_ncm_stats_dist_prepare_interp: very large system n = %d!", nk);

    if (sd->cfg.cv_type == NCG_CV_SPLIT)
      r = _split_fit (sd, n, nk, m2lnp, min_m2lnp, &rnorm);
    else
      r = _im_full_nnls (sd, n, nk, &rnorm);

    if (r != NCG_OK)
      return r;

    sd->rnorm = rnorm;

    CK (ncg_launch_normalize_weights (sd->dw, nk, sd->cfg.shrink, sd->nn.info, sd->stream), "normalize");
    CK (cudaMemcpyAsync (&bad, sd->nn.info, sizeof (int32_t), cudaMemcpyDeviceToHost, sd->stream), "D2H");
    CK (ncg_launch_weights_c (sd->dw, sd->dlnnorm, nk, sd->kind, sd->dc, NULL, sd->stream), "weights_c");
    CK (cudaStreamSynchronize (sd->stream), "sync");

    sd->wcum_ready    = 0;
    sd->packmx_ready  = 0;
    sd->gen++;
    sd->interp_branch = 0;

    if (bad)
    {
      ncg_set_error ("prepare_interp: total weight is not positive");

      return NCG_ERR_BAD_WEIGHTS;
    }
  }

  return NCG_OK;
}

/* the interpolation matrix with unit f (n_obs x n_kernels) into sd->nn.IM,
 * asynchronous on the handle's stream */
static ncg_status_t
_raw_IM (ncg_sd_t *sd)
{
  const int n = (int) sd->n, nk = (int) sd->nk;
  ncg_eval_args_t a;
  ncg_status_t r;

  r = ncg_sd_reserve (sd, (void **) &sd->df, &sd->cap.f, sizeof (double) * n);

  if (r == NCG_OK)
  {
    _ws_reset (sd);
    r = _big_reserve (sd, (void **) &sd->nn.IM, &sd->nn.cIM, sizeof (double) * (size_t) n * nk, 1);
  }

  if (r != NCG_OK)
    return r;

  CK (ncg_launch_fill (sd->df, 1.0, n, sd->stream), "fill");

  a.kind        = sd->kind;
  a.kernel      = sd->kernel;
  a.d           = (int32_t) sd->d;
  a.dp          = sd->dp;
  a.n           = nk;
  a.m           = n;
  a.nu          = (sd->kernel == NCG_KERNEL_ST) ? sd->nu : 1.0;
  a.kappa       = -0.5 * (sd->nu + sd->d);
  a.final_shift = 0.0;
  a.d_ln_href   = sd->d * log (sd->href);
  a.inv_href    = 1.0 / sd->href;
  a.c_shift     = 0.0;

  CK (ncg_launch_compute_IM (&a, sd->dX, sd->dpack64, sd->dlnnorm, sd->kernel_lnnorm, sd->df, sd->nn.IM, sd->stream),
      "compute_IM");

  return NCG_OK;
}

ncg_status_t
ncg_sd_compute_IM (ncg_sd_t *sd, double *IM)
{
  ncg_status_t r;

  if (sd == NULL || IM == NULL)
    return NCG_ERR_INVALID_ARG;

  if (!sd->prepared)
    return NCG_ERR_NOT_PREPARED;

  if ((r = _raw_IM (sd)) != NCG_OK)
    return r;

  CK (cudaMemcpyAsync (IM, sd->nn.IM, sizeof (double) * (size_t) sd->n * sd->nk, cudaMemcpyDeviceToHost, sd->stream),
      "D2H IM");
  CK (cudaStreamSynchronize (sd->stream), "sync");

  return NCG_OK;
}

/* row sums of the unit-f interpolation matrix of a square system (n_obs =
 * n_kernels): rowx[i] = sum over j != i of IM[i][j], diag[i] = IM[i][i]
 * (host arrays of n_kernels) */
ncg_status_t
ncg_sd_im_rowsums (ncg_sd_t *sd, double *rowx, double *diag)
{
  const int n = (int) sd->nk;
  ncg_status_t r;

  if (sd->n != sd->nk)
    return NCG_ERR_INVALID_ARG;

  if ((r = _raw_IM (sd)) != NCG_OK)
    return r;

  NRES (mg, cmg, sizeof (double) * 2 * (size_t) n);
  CK (ncg_launch_im_rowsums (sd->nn.IM, n, sd->nn.mg, sd->nn.mg + n, sd->stream), "im_rowsums");
  CK (cudaMemcpyAsync (rowx, sd->nn.mg, sizeof (double) * n, cudaMemcpyDeviceToHost, sd->stream), "D2H rows");
  CK (cudaMemcpyAsync (diag, sd->nn.mg + n, sizeof (double) * n, cudaMemcpyDeviceToHost, sd->stream), "D2H diag");
  CK (cudaStreamSynchronize (sd->stream), "sync");

  return NCG_OK;
}
