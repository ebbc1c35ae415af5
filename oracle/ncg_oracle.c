/*
 * ncg_oracle.c -- CPU oracle for the KDE/VKDE proposal path.
 *
 * TEST INFRASTRUCTURE ONLY (see ncg_oracle.h).  Every function below restates
 * one piece of NumCosmo's FP64 CPU code and cites the file:line it follows;
 * paths are relative to the NumCosmo source tree.  Compile with
 * -ffp-contract=off so that the results are the same on x86_64 and aarch64.
 */
#include "ncg_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_LN2PI 1.8378770664093454835606594728112
#define ORC_LNPI 1.1447298858494001741434273513531
#define ORC_LN2 0.69314718055994530941723212145818
/* GSL_LOG_DBL_EPSILON = log(2^-52) */
#define ORC_LOG_DBL_EPSILON (-3.6043653389117154e+01)

static inline double sq (double x) { return x * x; }

/* ------------------------------------------------------------------------ */
/* Kernels                                                                  */
/* ------------------------------------------------------------------------ */

/* numcosmo/ncm/stats/ncm_stats_dist_kernel_gauss.c:193-199 and
 * numcosmo/ncm/stats/ncm_stats_dist_kernel_st.c:225-238 */
double
orc_kernel_rot_bandwidth (int kernel, double nu, int d, double n)
{
  if (kernel == ORC_GAUSS)
    return pow (4.0 / (n * (d + 2.0)), 1.0 / (d + 4.0));
  else
  {
    const double nuc = (nu >= 3.0) ? nu : 3.0;
    const double dd  = (double) d;

    return pow (
      16.0 * sq (nuc - 2) * (1.0 + dd + nuc) * (3.0 + dd + nuc) /
      ((2.0 + dd) * (dd + nuc) * (2.0 + dd + nuc) * (dd + 2.0 * nuc) * (2.0 + dd + 2.0 * nuc) * n),
      1.0 / (dd + 4.0));
  }
}

/* numcosmo/ncm/algebra/ncm_matrix.c:1158-1186 (frexp range guard) */
double
orc_cholesky_lndet (const double *U, int d)
{
  const double lb = 1.0e-200;
  const double ub = 1.0e+200;
  double detL     = 1.0;
  long exponent   = 0;
  int i;

  for (i = 0; i < d; i++)
  {
    const double Lii   = fabs (U[i * d + i]);
    const double ndetL = detL * Lii;

    if ((ndetL < lb) || (ndetL > ub))
    {
      int exponent_i = 0;

      detL      = frexp (ndetL, &exponent_i);
      exponent += exponent_i;
    }
    else
    {
      detL = ndetL;
    }
  }

  return 2.0 * (log (detL) + exponent * ORC_LN2);
}

/* numcosmo/ncm/stats/ncm_stats_dist_kernel_gauss.c:201-207 and
 * numcosmo/ncm/stats/ncm_stats_dist_kernel_st.c:240-252 */
double
orc_kernel_lnnorm (int kernel, double nu, int d, const double *U)
{
  const double lndet = orc_cholesky_lndet (U, d);

  if (kernel == ORC_GAUSS)
    return 0.5 * (d * ORC_LN2PI + lndet);
  else
  {
    const double lg_lnnorm   = lgamma (nu / 2.0) - lgamma ((nu + d) / 2.0);
    const double chol_lnnorm = 0.5 * lndet;
    const double nc_lnnorm   = (d / 2.0) * (ORC_LNPI + log (nu));

    return lg_lnnorm + nc_lnnorm + chol_lnnorm;
  }
}

/* numcosmo/ncm/stats/ncm_stats_dist_kernel_gauss.c:209-213 and
 * numcosmo/ncm/stats/ncm_stats_dist_kernel_st.c:254-261 */
double
orc_kernel_eval_unnorm (int kernel, double nu, int d, double chi2)
{
  if (kernel == ORC_GAUSS)
    return exp (-0.5 * chi2);
  else
    return pow (1.0 + chi2 / nu, -0.5 * (nu + d));
}

static inline double
_lnt (int kernel, double kappa, double nu, double chi2)
{
  if (kernel == ORC_GAUSS)
    return -0.5 * chi2;
  else
    return kappa * log1p (chi2 / nu);
}

/* Two-pass gamma/lambda of numcosmo/ncm/stats/ncm_stats_dist_kernel_gauss.c:246-290
 * and numcosmo/ncm/stats/ncm_stats_dist_kernel_st.c:295-341 (sum0: per-kernel
 * lnnorms).  The maximum is the first index reaching it; lambda skips it. */
void
orc_kernel_sum0 (int kernel, double nu, int d, int n, const double *chi2,
                 const double *w, const double *lnu, double *lnK,
                 double *gamma, double *lambda)
{
  const double kappa = -0.5 * (nu + d);
  double lnt_max     = -INFINITY;
  int i, i_max       = 0;

  for (i = 0; i < n; i++)
  {
    double lnt_i;

    if (kernel == ORC_GAUSS)
      lnt_i = -0.5 * chi2[i] - lnu[i] + log (w[i]);
    else
      lnt_i = kappa * log1p (chi2[i] / nu) - lnu[i] + log (w[i]);

    if (lnt_i > lnt_max)
    {
      i_max   = i;
      lnt_max = lnt_i;
    }

    lnK[i] = lnt_i;
  }

  lambda[0] = 0.0;

  for (i = 0; i < i_max; i++)
    lambda[0] += exp (lnK[i] - lnt_max);

  for (i = i_max + 1; i < n; i++)
    lambda[0] += exp (lnK[i] - lnt_max);

  gamma[0] = lnt_max;
}

/* numcosmo/ncm/stats/ncm_stats_dist_kernel_gauss.c:292-333 and
 * numcosmo/ncm/stats/ncm_stats_dist_kernel_st.c:343-386 (sum1: shared lnnorm) */
void
orc_kernel_sum1 (int kernel, double nu, int d, int n, const double *chi2,
                 const double *w, double lnnorm, double *lnK,
                 double *gamma, double *lambda)
{
  const double kappa = -0.5 * (nu + d);
  double lnt_max     = -INFINITY;
  int i, i_max       = 0;

  for (i = 0; i < n; i++)
  {
    const double lnt_i = _lnt (kernel, kappa, nu, chi2[i]) + log (w[i]);

    if (lnt_i > lnt_max)
    {
      i_max   = i;
      lnt_max = lnt_i;
    }

    lnK[i] = lnt_i;
  }

  lambda[0] = 0.0;

  for (i = 0; i < i_max; i++)
    lambda[0] += exp (lnK[i] - lnt_max);

  for (i = i_max + 1; i < n; i++)
    lambda[0] += exp (lnK[i] - lnt_max);

  gamma[0] = lnt_max - lnnorm;
}

/* ------------------------------------------------------------------------ */
/* Linear algebra                                                           */
/* ------------------------------------------------------------------------ */

/* Welford mean/covariance with unit weights, restating
 * numcosmo/ncm/stats/ncm_stats_vec.c:511-565 (update) and :2376-2398
 * (get_cov_matrix: diagonal from var, scale by bias_wt = 1/(W - W2/W)).
 * The statistics start from zero (a freshly created NcmStatsVec).
 * rows == NULL means rows 0..nrows-1 in order. */
void
orc_welford_cov (const double *X, const int *rows, int nrows, int d, double *cov)
{
  double *mean  = calloc (d, sizeof (double));
  double *var   = calloc (d, sizeof (double));
  double weight = 0.0, weight2 = 0.0, bias_wt = 0.0;
  const double w = 1.0;
  int t, i, j;

  memset (cov, 0, sizeof (double) * d * d);

  for (t = 0; t < nrows; t++)
  {
    const double *x         = X + (size_t) (rows ? rows[t] : t) * d;
    const double curweight  = weight + w;

    for (i = 0; i < d; i++)
    {
      double mean_i        = mean[i];
      const double x_i     = x[i];
      const double delta_i = x_i - mean_i;
      const double R_i     = delta_i * w / curweight;
      const double dvar    = weight * delta_i * R_i;

      mean_i += R_i;
      mean[i] = mean_i;
      var[i] += dvar;

      for (j = i + 1; j < d; j++)
      {
        const double x_j   = x[j];
        const double mean_j = mean[j];
        const double dC_ij = w * (x_i - mean_i) * (x_j - mean_j);
        const double C_ij  = cov[i * d + j] + dC_ij;

        cov[i * d + j] = C_ij;
        cov[j * d + i] = C_ij;
      }
    }

    weight   = curweight;
    weight2 += w * w;
    bias_wt  = 1.0 / (weight - weight2 / weight);
  }

  for (i = 0; i < d; i++)
    cov[i * d + i] = var[i];

  for (i = 0; i < d * d; i++)
    cov[i] = cov[i] * bias_wt;

  free (mean);
  free (var);
}

/* In-place Cholesky of a row-major SPD matrix into its upper factor,
 * Sigma = U^T U.  Restates ncm_matrix_cholesky_decomp (cm, 'U')
 * (numcosmo/ncm/algebra/ncm_matrix.c:1124-1129) which calls dpotrf with the
 * row/column-major UPLO swap (numcosmo/ncm/algebra/ncm_lapack.c:216-237).
 * Only the upper triangle is read or written.  Returns 0 or j+1 when the
 * leading minor of order j+1 is not positive (LAPACK info). */
int
orc_cholesky_upper (double *A, int d)
{
  int j, i, k;

  for (j = 0; j < d; j++)
  {
    double ajj = A[j * d + j];

    for (k = 0; k < j; k++)
      ajj -= A[k * d + j] * A[k * d + j];

    if (!(ajj > 0.0))
    {
      A[j * d + j] = ajj;

      return j + 1;
    }

    ajj          = sqrt (ajj);
    A[j * d + j] = ajj;

    for (i = j + 1; i < d; i++)
    {
      double aji = A[j * d + i];

      for (k = 0; k < j; k++)
        aji -= A[k * d + j] * A[k * d + i];

      A[j * d + i] = aji / ajj;
    }
  }

  return 0;
}

/* Cyclic Jacobi eigen-decomposition of a symmetric matrix (full storage).
 * eval ascending; evec row i is the unit eigenvector of eval[i].
 * Stands in for LAPACK dsyevr inside nearPD (an eigen-decomposition is
 * unique up to sign/order, which the reconstruction does not see). */
int
orc_sym_eigen (const double *A0, int n, double *eval, double *evec)
{
  double *A = malloc (sizeof (double) * n * n);
  double *V = malloc (sizeof (double) * n * n);
  int *perm = malloc (sizeof (int) * n);
  int p, q, i, sweep;

  memcpy (A, A0, sizeof (double) * n * n);

  for (i = 0; i < n * n; i++)
    V[i] = 0.0;

  for (i = 0; i < n; i++)
    V[i * n + i] = 1.0;

  for (sweep = 0; sweep < 100; sweep++)
  {
    double off = 0.0, diag = 0.0;

    for (p = 0; p < n; p++)
    {
      diag += sq (A[p * n + p]);

      for (q = p + 1; q < n; q++)
        off += sq (A[p * n + q]);
    }

    if (off <= 1.0e-30 * diag || off == 0.0)
      break;

    for (p = 0; p < n - 1; p++)
    {
      for (q = p + 1; q < n; q++)
      {
        const double apq = A[p * n + q];
        double theta, t, c, s;
        int r;

        if (apq == 0.0)
          continue;

        theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
        t     = (theta >= 0.0 ? 1.0 : -1.0) / (fabs (theta) + sqrt (theta * theta + 1.0));
        c     = 1.0 / sqrt (t * t + 1.0);
        s     = t * c;

        for (r = 0; r < n; r++)
        {
          const double arp = A[r * n + p];
          const double arq = A[r * n + q];

          A[r * n + p] = c * arp - s * arq;
          A[r * n + q] = s * arp + c * arq;
        }

        for (r = 0; r < n; r++)
        {
          const double apr = A[p * n + r];
          const double aqr = A[q * n + r];

          A[p * n + r] = c * apr - s * aqr;
          A[q * n + r] = s * apr + c * aqr;
        }

        for (r = 0; r < n; r++)
        {
          const double vrp = V[r * n + p];
          const double vrq = V[r * n + q];

          V[r * n + p] = c * vrp - s * vrq;
          V[r * n + q] = s * vrp + c * vrq;
        }
      }
    }
  }

  for (i = 0; i < n; i++)
    perm[i] = i;

  /* insertion sort by eigenvalue */
  for (p = 1; p < n; p++)
  {
    const int cur = perm[p];

    q = p - 1;

    while (q >= 0 && A[perm[q] * n + perm[q]] > A[cur * n + cur])
    {
      perm[q + 1] = perm[q];
      q--;
    }

    perm[q + 1] = cur;
  }

  for (i = 0; i < n; i++)
  {
    const int c = perm[i];

    eval[i] = A[c * n + c];

    for (p = 0; p < n; p++)
      evec[i * n + p] = V[p * n + c];
  }

  free (A);
  free (V);
  free (perm);

  return 0;
}

/* ------------------------------------------------------------------------ */
/* Robust covariance types (cov-type ROBUST_DIAG, ROBUST)                    */
/* ------------------------------------------------------------------------ */

static int
_dbl_cmp (const void *a, const void *b)
{
  const double x = *(const double *) a, y = *(const double *) b;

  return (x < y) ? -1 : (x > y);
}

/* Qn scale estimator of m values (sorted in place), the statistic GSL's
 * gsl_stats_Qn_from_sorted_data returns (GSL >= 2.8 is not vendored with the
 * reference; this follows the published definition, Rousseeuw & Croux 1993,
 * with the small-sample factors of Croux & Rousseeuw 1992):
 *   Qn = 2.21914 d_m {|x_a - x_b|; a < b}_(k),  k = C(h, 2),  h = floor(m/2) + 1.
 * The k-th smallest difference is found by bisection over the bit patterns
 * of non-negative doubles with a two-pointer count of the pairs at or below
 * the trial value, so the result is exactly one of the differences. */
double
orc_qn (double *v, int m)
{
  static const double dn_small[8] = { 0.399, 0.994, 0.512, 0.844, 0.611, 0.857, 0.669, 0.872 };
  const long long h = m / 2 + 1, kk = h * (h - 1) / 2;
  unsigned long long lo = 0, hi;
  double span, dn;

  if (m < 2)
    return 0.0;

  qsort (v, m, sizeof (double), _dbl_cmp);

  span = v[m - 1] - v[0];

  if (!(span > 0.0))
    span = 0.0;

  memcpy (&hi, &span, sizeof (hi));

  while (lo < hi)
  {
    const unsigned long long mid = lo + ((hi - lo) >> 1);
    double t;
    long long c = 0;
    int a, b = 0;

    memcpy (&t, &mid, sizeof (t));

    /* for each a the largest b with v[b] - v[a] <= t; b never decreases */
    for (a = 0; a < m - 1; a++)
    {
      if (b < a)
        b = a;

      while (b + 1 < m && v[b + 1] - v[a] <= t)
        b++;

      c += b - a;
    }

    if (c >= kk)
      hi = mid;
    else
      lo = mid + 1;
  }

  {
    double q;

    memcpy (&q, &lo, sizeof (q));
    dn = (m <= 9) ? dn_small[m - 2] : ((m & 1) ? m / (m + 1.4) : m / (m + 3.8));

    return 2.21914 * dn * q;
  }
}

/* ncm_stats_vec_compute_cov_robust_diag (ncm_stats_vec.c:1833-1884):
 * cov = diag(Qn(x_i)^2) over the rows (rows == NULL: 0..nrows-1) */
void
orc_cov_robust_diag (const double *X, const int *rows, int nrows, int d, double *cov)
{
  double *v = malloc (sizeof (double) * nrows);
  int i, a;

  memset (cov, 0, sizeof (double) * d * d);

  for (i = 0; i < d; i++)
  {
    double q;

    for (a = 0; a < nrows; a++)
      v[a] = X[(size_t) (rows ? rows[a] : a) * d + i];

    q                = orc_qn (v, nrows);
    cov[i * d + i]   = q * q;
  }

  free (v);
}

/* ncm_stats_vec_compute_cov_robust_ogk (ncm_stats_vec.c:1898-2077), the
 * orthogonalised Gnanadesikan-Kettenring estimate: scales sigma_i = Qn(x_i),
 * y = x * (1/sigma), pairwise C_ij = (Qn(y_i + y_j)^2 - Qn(y_i - y_j)^2) / 4
 * with unit diagonal, eigenvectors E of C (orc_sym_eigen in place of
 * dsyevr), sigma_z_i = Qn(E_i . y), cov = V^T V with V_ij = sigma_z_i E_ij
 * sigma_j.  Full symmetric storage. */
void
orc_cov_robust_ogk (const double *X, const int *rows, int nrows, int d, double *cov)
{
  double *v    = malloc (sizeof (double) * nrows);
  double *y    = malloc (sizeof (double) * (size_t) nrows * d);
  double *C    = calloc ((size_t) d * d, sizeof (double));
  double *E    = malloc (sizeof (double) * d * d);
  double *eval = malloc (sizeof (double) * d);
  double *sx   = malloc (sizeof (double) * d);
  double *sz   = malloc (sizeof (double) * d);
  int i, j, a, r;

  for (i = 0; i < d; i++)
  {
    for (a = 0; a < nrows; a++)
      v[a] = X[(size_t) (rows ? rows[a] : a) * d + i];

    sx[i] = orc_qn (v, nrows);
  }

  for (a = 0; a < nrows; a++)
    for (i = 0; i < d; i++)
      y[(size_t) a * d + i] = X[(size_t) (rows ? rows[a] : a) * d + i] * (1.0 / sx[i]);

  for (i = 0; i < d * d; i++)
    C[i] = 0.0;

  for (i = 0; i < d; i++)
  {
    C[i * d + i] = 1.0;

    for (j = i + 1; j < d; j++)
    {
      double sp, sm;

      for (a = 0; a < nrows; a++)
        v[a] = y[(size_t) a * d + i] + y[(size_t) a * d + j];

      sp = orc_qn (v, nrows);

      for (a = 0; a < nrows; a++)
        v[a] = y[(size_t) a * d + i] - y[(size_t) a * d + j];

      sm = orc_qn (v, nrows);

      C[i * d + j] = 0.25 * (sp * sp - sm * sm);
      C[j * d + i] = C[i * d + j];
    }
  }

  orc_sym_eigen (C, d, eval, E);

  for (i = 0; i < d; i++)
  {
    for (a = 0; a < nrows; a++)
    {
      double z = 0.0;

      for (r = 0; r < d; r++)
        z += E[i * d + r] * y[(size_t) a * d + r];

      v[a] = z;
    }

    sz[i] = orc_qn (v, nrows);
  }

  for (i = 0; i < d; i++)
    for (j = 0; j < d; j++)
      E[i * d + j] = sz[i] * E[i * d + j] * sx[j];

  for (i = 0; i < d; i++)
    for (j = i; j < d; j++)
    {
      double c = 0.0;

      for (r = 0; r < d; r++)
        c += E[r * d + i] * E[r * d + j];

      cov[i * d + j] = c;
      cov[j * d + i] = c;
    }

  free (v);
  free (y);
  free (C);
  free (E);
  free (eval);
  free (sx);
  free (sz);
}

/* Higham (2002) nearest positive-definite matrix with unit-diagonal
 * restoration, restating ncm_matrix_nearPD (numcosmo/ncm/algebra/ncm_matrix.c:1248-1344)
 * with cholesky_decomp = TRUE: on success A holds the upper Cholesky factor
 * of the repaired matrix.  A is symmetric (full storage) on input. */
int
orc_nearPD (double *A, int n, int maxiter)
{
  double *diag = malloc (sizeof (double) * n);
  double *D_S  = calloc (n * n, sizeof (double));
  double *R    = malloc (sizeof (double) * n * n);
  double *eva  = malloc (sizeof (double) * n);
  double *eve  = malloc (sizeof (double) * n * n);
  int iter     = 0;
  int ret      = 0;
  int i, j, k;

  for (i = 0; i < n; i++)
    diag[i] = A[i * n + i];

  while (1)
  {
    double min_pos_ev = INFINITY;

    for (i = 0; i < n * n; i++)
      A[i] -= D_S[i];

    memcpy (R, A, sizeof (double) * n * n);

    orc_sym_eigen (A, n, eva, eve);

    for (i = 0; i < n; i++)
      if (eva[i] > 0.0)
        min_pos_ev = fmin (eva[i], min_pos_ev);

    for (i = 0; i < n; i++)
    {
      if (eva[i] < 0.0)
        eva[i] = min_pos_ev * DBL_EPSILON;

      {
        const double s = sqrt (eva[i]);

        for (k = 0; k < n; k++)
          eve[i * n + k] *= s;
      }
    }

    /* A = eve^T eve (dsyrk, upper), mirrored */
    for (i = 0; i < n; i++)
    {
      for (j = i; j < n; j++)
      {
        double s = 0.0;

        for (k = 0; k < n; k++)
          s += eve[k * n + i] * eve[k * n + j];

        A[i * n + j] = s;
        A[j * n + i] = s;
      }
    }

    for (i = 0; i < n * n; i++)
      D_S[i] = A[i] - R[i];

    for (i = 0; i < n; i++)
      A[i * n + i] = diag[i];

    memcpy (R, A, sizeof (double) * n * n);

    if ((ret = orc_cholesky_upper (R, n)) == 0)
      break;

    if (iter > maxiter)
      break;

    iter++;
  }

  memcpy (A, R, sizeof (double) * n * n);

  free (diag);
  free (D_S);
  free (R);
  free (eva);
  free (eve);

  return ret;
}

/* _cholesky_decomp of numcosmo/ncm/stats/ncm_stats_dist_kde.c:345-367 and
 * numcosmo/ncm/stats/ncm_stats_dist_vkde.c:338-360: Cholesky, else nearPD,
 * else the diagonal.  U gets the upper factor with a zero lower triangle.
 * Returns 0 (plain), 1 (nearPD), 2 (diagonal) or -1 (diagonal not PD). */
int
orc_cholesky_decomp_fallback (const double *cov, double *U, int d, int maxiter)
{
  int ret = 0, i, j;

  memcpy (U, cov, sizeof (double) * d * d);

  if (orc_cholesky_upper (U, d) != 0)
  {
    memcpy (U, cov, sizeof (double) * d * d);
    ret = 1;

    if (orc_nearPD (U, d, maxiter) != 0)
    {
      memset (U, 0, sizeof (double) * d * d);

      for (i = 0; i < d; i++)
        U[i * d + i] = cov[i * d + i];

      ret = 2;

      if (orc_cholesky_upper (U, d) != 0)
        ret = -1;
    }
  }

  for (i = 0; i < d; i++)
    for (j = 0; j < i; j++)
      U[i * d + j] = 0.0;

  return ret;
}

/* Forward solve of U^T y = b for upper U (gsl_blas_dtrsv Upper/Trans/NonUnit),
 * as used by numcosmo/ncm/stats/ncm_stats_dist_vkde.c:703 and
 * numcosmo/ncm/stats/ncm_stats_dist_kde.c:652.  In place on y. */
static void
_trsv_ut (const double *U, int d, double *y)
{
  int r, c;

  for (r = 0; r < d; r++)
  {
    double s = y[r];

    for (c = 0; c < r; c++)
      s -= U[c * d + r] * y[c];

    y[r] = s / U[r * d + r];
  }
}

/* x := U^T x for upper U (gsl_blas_dtrmv Upper/Trans/NonUnit), as used by
 * numcosmo/ncm/stats/ncm_stats_dist_kernel_gauss.c:350-352. */
static void
_trmv_ut (const double *U, int d, double *x)
{
  int r, c;

  for (r = d - 1; r >= 0; r--)
  {
    double s = 0.0;

    for (c = 0; c <= r; c++)
      s += U[c * d + r] * x[c];

    x[r] = s;
  }
}

/* ------------------------------------------------------------------------ */
/* Exact kNN                                                                */
/* ------------------------------------------------------------------------ */

typedef struct { double dist; int idx; } _orc_pair;

static inline int
_pair_less (const _orc_pair *a, const _orc_pair *b)
{
  /* numcosmo/external/misc/rb_knn_list.c:32-40: distance, then index */
  if (a->dist < b->dist)
    return 1;

  if (a->dist > b->dist)
    return 0;

  return a->idx < b->idx;
}

static void
_heap_sift_down (_orc_pair *h, int n, int i)
{
  while (1)
  {
    int l = 2 * i + 1, r = l + 1, m = i;

    if (l < n && _pair_less (&h[m], &h[l]))
      m = l;

    if (r < n && _pair_less (&h[m], &h[r]))
      m = r;

    if (m == i)
      return;

    {
      _orc_pair t = h[i];

      h[i] = h[m];
      h[m] = t;
    }
    i = m;
  }
}

static int
_pair_cmp (const void *a, const void *b)
{
  const _orc_pair *pa = a, *pb = b;

  if (_pair_less (pa, pb))
    return -1;

  if (_pair_less (pb, pa))
    return 1;

  return 0;
}

/* Exact k nearest neighbours (the point itself included) of every row of Y
 * (n x d), in ascending (squared distance, index) order.  The squared
 * distance is summed in coordinate order as in
 * numcosmo/external/misc/kdtree.c:28-38; this replaces kdtree_knn_search
 * (numcosmo/external/misc/kdtree.c:193-320) by exhaustive search. */
void
orc_knn (const double *Y, int n, int d, int k, int *out, int nthreads)
{
  orc_knn_q (Y, n, n, d, k, out, nthreads);
}

/* the k nearest of the n points Y to each of the first nq of them: the
 * kd-tree over all observations queried at the kernels
 * (ncm_stats_dist_vkde.c:378-426) */
void
orc_knn_q (const double *Y, int n, int nq, int d, int k, int *out, int nthreads)
{
  int i;

#ifdef _OPENMP
  #pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (i = 0; i < nq; i++)
  {
    _orc_pair *heap = malloc (sizeof (_orc_pair) * k);
    const double *t = Y + (size_t) i * d;
    int hn          = 0;
    int j, c;

    for (j = 0; j < n; j++)
    {
      const double *p = Y + (size_t) j * d;
      double dist     = 0.0;
      _orc_pair cand;

      for (c = 0; c < d; c++)
        dist += sq (p[c] - t[c]);

      cand.dist = dist;
      cand.idx  = j;

      if (hn < k)
      {
        int h = hn++;

        heap[h] = cand;

        while (h > 0)
        {
          int par = (h - 1) / 2;

          if (_pair_less (&heap[par], &heap[h]))
          {
            _orc_pair tmp = heap[par];

            heap[par] = heap[h];
            heap[h]   = tmp;
            h         = par;
          }
          else
          {
            break;
          }
        }
      }
      else if (_pair_less (&cand, &heap[0]))
      {
        heap[0] = cand;
        _heap_sift_down (heap, hn, 0);
      }
    }

    qsort (heap, hn, sizeof (_orc_pair), _pair_cmp);

    for (j = 0; j < hn; j++)
      out[(size_t) i * k + j] = heap[j].idx;

    free (heap);
  }
}

/* ------------------------------------------------------------------------ */
/* Dense solvers used by NNLS                                               */
/* ------------------------------------------------------------------------ */

/* dposv on the upper triangle (numcosmo/ncm/algebra/ncm_matrix.c:1199-1208):
 * factor M = U^T U, solve U^T U x = b.  Returns the Cholesky info. */
static int
_posv (double *M, int n, double *b)
{
  int ret = orc_cholesky_upper (M, n), r, c;

  if (ret != 0)
    return ret;

  _trsv_ut (M, n, b);

  for (r = n - 1; r >= 0; r--)
  {
    double s = b[r];

    for (c = r + 1; c < n; c++)
      s -= M[r * n + c] * b[c];

    b[r] = s / M[r * n + r];
  }

  return 0;
}

/* Symmetric solve used as the LU fallback (dsysv,
 * numcosmo/ncm/algebra/ncm_nnls.c:573-606): Gaussian elimination with
 * partial pivoting on the full symmetric matrix built from the upper
 * triangle.  Returns >0 when a pivot is exactly zero. */
static int
_sysv (const double *Mu, int n, double *b)
{
  double *A = malloc (sizeof (double) * n * n);
  int r, c, k, ret = 0;

  for (r = 0; r < n; r++)
    for (c = r; c < n; c++)
    {
      A[r * n + c] = Mu[r * n + c];
      A[c * n + r] = Mu[r * n + c];
    }

  for (k = 0; k < n; k++)
  {
    int p       = k;
    double amax = fabs (A[k * n + k]);

    for (r = k + 1; r < n; r++)
      if (fabs (A[r * n + k]) > amax)
      {
        amax = fabs (A[r * n + k]);
        p    = r;
      }

    if (amax == 0.0)
    {
      ret = k + 1;
      break;
    }

    if (p != k)
    {
      for (c = 0; c < n; c++)
      {
        double t = A[k * n + c];

        A[k * n + c] = A[p * n + c];
        A[p * n + c] = t;
      }

      {
        double t = b[k];

        b[k] = b[p];
        b[p] = t;
      }
    }

    for (r = k + 1; r < n; r++)
    {
      const double f = A[r * n + k] / A[k * n + k];

      if (f == 0.0)
        continue;

      for (c = k; c < n; c++)
        A[r * n + c] -= f * A[k * n + c];

      b[r] -= f * b[k];
    }
  }

  if (ret == 0)
  {
    for (r = n - 1; r >= 0; r--)
    {
      double s = b[r];

      for (c = r + 1; c < n; c++)
        s -= A[r * n + c] * b[c];

      b[r] = s / A[r * n + r];
    }
  }

  free (A);

  return ret;
}

/* Least squares min |A_P x - f| by Householder QR, the dgels fallback of
 * numcosmo/ncm/algebra/ncm_nnls.c:608-638.  A is nrows x ncols (row-major),
 * P lists the np columns used; x receives np values. */
static void
_gels (const double *A, int nrows, int ncols, const int *P, int np, const double *f, double *x)
{
  double *Q = malloc (sizeof (double) * (size_t) nrows * np);
  double *y = malloc (sizeof (double) * nrows);
  int r, c, k;

  for (r = 0; r < nrows; r++)
  {
    for (c = 0; c < np; c++)
      Q[(size_t) r * np + c] = A[(size_t) r * ncols + P[c]];

    y[r] = f[r];
  }

  for (k = 0; k < np && k < nrows; k++)
  {
    double nrm = 0.0, alpha, vtv = 0.0;

    for (r = k; r < nrows; r++)
      nrm += sq (Q[(size_t) r * np + k]);

    nrm   = sqrt (nrm);
    alpha = (Q[(size_t) k * np + k] > 0.0) ? -nrm : nrm;

    if (nrm == 0.0)
      continue;

    Q[(size_t) k * np + k] -= alpha;

    for (r = k; r < nrows; r++)
      vtv += sq (Q[(size_t) r * np + k]);

    for (c = k + 1; c < np; c++)
    {
      double s = 0.0;

      for (r = k; r < nrows; r++)
        s += Q[(size_t) r * np + k] * Q[(size_t) r * np + c];

      s = 2.0 * s / vtv;

      for (r = k; r < nrows; r++)
        Q[(size_t) r * np + c] -= s * Q[(size_t) r * np + k];
    }

    {
      double s = 0.0;

      for (r = k; r < nrows; r++)
        s += Q[(size_t) r * np + k] * y[r];

      s = 2.0 * s / vtv;

      for (r = k; r < nrows; r++)
        y[r] -= s * Q[(size_t) r * np + k];
    }

    Q[(size_t) k * np + k] = alpha;
  }

  for (k = np - 1; k >= 0; k--)
  {
    double s = y[k];

    for (c = k + 1; c < np; c++)
      s -= Q[(size_t) k * np + c] * x[c];

    x[k] = (Q[(size_t) k * np + k] != 0.0) ? s / Q[(size_t) k * np + k] : 0.0;
  }

  free (Q);
  free (y);
}

/* ------------------------------------------------------------------------ */
/* NNLS                                                                     */
/* ------------------------------------------------------------------------ */

/* solves of the last orc_nnls_solve that took the LU / the QR fallback */
static int g_nnls_lu, g_nnls_qr;

void
orc_nnls_fallbacks (int *lu, int *qr)
{
  *lu = g_nnls_lu;
  *qr = g_nnls_qr;
}

typedef struct
{
  const double *A;
  int nrows, ncols, nthreads;
  const double *f;
  double *M;      /* ncols x ncols, upper triangle = A^T A */
  double *b;      /* A^T f */
  double *Msub;   /* work */
  double *xsub;   /* work */
  int *Psub;      /* work */
} _orc_nnls;

/* solve the normal equations restricted to the set P (sorted index list in
 * mask form), NORMAL umethod with the LU and QR fallbacks:
 * numcosmo/ncm/algebra/ncm_nnls.c:544-571,640-690 */
static void
_nnls_solve_unconstrained (_orc_nnls *s, const char *inP, double *x)
{
  int np = 0, i, j, ret;

  for (i = 0; i < s->ncols; i++)
    if (inP[i])
      s->Psub[np++] = i;

  for (i = 0; i < np; i++)
  {
    for (j = i; j < np; j++)
      s->Msub[i * np + j] = s->M[(size_t) s->Psub[i] * s->ncols + s->Psub[j]];

    s->xsub[i] = s->b[s->Psub[i]];
  }

  for (i = 0; i < s->ncols; i++)
    x[i] = 0.0;

  if (np == 0)
    return;

  ret = _posv (s->Msub, np, s->xsub);

  if (ret > 0)
  {
    g_nnls_lu++;
    for (i = 0; i < np; i++)
    {
      for (j = i; j < np; j++)
        s->Msub[i * np + j] = s->M[(size_t) s->Psub[i] * s->ncols + s->Psub[j]];

      s->xsub[i] = s->b[s->Psub[i]];
    }

    ret = _sysv (s->Msub, np, s->xsub);

    if (ret > 0)
    {
      g_nnls_qr++;
      _gels (s->A, s->nrows, s->ncols, s->Psub, np, s->f, s->xsub);
    }
  }

  for (i = 0; i < np; i++)
    x[s->Psub[i]] = s->xsub[i];
}

typedef struct { double v; int pos; } _orc_vi;

static int
_vi_cmp_asc (const void *a, const void *b)
{
  const _orc_vi *pa = a, *pb = b;

  if (pa->v < pb->v) return -1;
  if (pa->v > pb->v) return 1;
  return (pa->pos < pb->pos) ? -1 : (pa->pos > pb->pos);
}

static int
_vi_cmp_desc (const void *a, const void *b)
{
  const _orc_vi *pa = a, *pb = b;

  if (pa->v > pb->v) return -1;
  if (pa->v < pb->v) return 1;
  return (pa->pos < pb->pos) ? -1 : (pa->pos > pb->pos);
}

/* _ncm_nnls_solve_feasible, numcosmo/ncm/algebra/ncm_nnls.c:728-751, with
 * ncm_iset_get_subset_vec_lt (numcosmo/ncm/core/ncm_iset.c:853-875) and
 * ncm_iset_remove_smallest_subset (numcosmo/ncm/core/ncm_iset.c:920-975).
 * Ties in the smallest-value selection go to the lower index. */
static void
_nnls_solve_feasible (_orc_nnls *s, char *inP, double *x, int max_remove)
{
  _orc_vi *inv = malloc (sizeof (_orc_vi) * s->ncols);

  _nnls_solve_unconstrained (s, inP, x);

  while (1)
  {
    int ninv = 0, i;

    for (i = 0; i < s->ncols; i++)
      if (inP[i] && x[i] < 1.0e-300)
      {
        inv[ninv].v   = x[i];
        inv[ninv].pos = i;
        ninv++;
      }

    if (ninv == 0)
      break;

    if (max_remove >= ninv)
    {
      for (i = 0; i < ninv; i++)
        inP[inv[i].pos] = 0;
    }
    else
    {
      qsort (inv, ninv, sizeof (_orc_vi), _vi_cmp_asc);

      for (i = 0; i < max_remove; i++)
        inP[inv[i].pos] = 0;
    }

    _nnls_solve_unconstrained (s, inP, x);
  }

  free (inv);
}

/* |f - A x| and the residual vector (ncm_nnls.c:700-711) */
static double
_nnls_residuals (_orc_nnls *s, const double *x, double *res)
{
  double rn = 0.0;
  int r;

#ifdef _OPENMP
  #pragma omp parallel for num_threads(s->nthreads > 0 ? s->nthreads : 1)
#endif
  for (r = 0; r < s->nrows; r++)
  {
    const double *a = s->A + (size_t) r * s->ncols;
    double acc      = 0.0;
    int c;

    for (c = 0; c < s->ncols; c++)
      acc += a[c] * x[c];

    res[r] = s->f[r] - acc;
  }

  for (r = 0; r < s->nrows; r++)
    rn += res[r] * res[r];

  return sqrt (rn);
}

/* mgrad = A^T res (ncm_nnls.c:713-717) */
static void
_nnls_mgrad (_orc_nnls *s, const double *res, double *mgrad)
{
  int c, r;

  for (c = 0; c < s->ncols; c++)
    mgrad[c] = 0.0;

  for (r = 0; r < s->nrows; r++)
  {
    const double *a = s->A + (size_t) r * s->ncols;
    const double rr = res[r];

    for (c = 0; c < s->ncols; c++)
      mgrad[c] += a[c] * rr;
  }
}

/* ncm_iset_add_largest_subset (numcosmo/ncm/core/ncm_iset.c:994-1078):
 * among indices not in P with v > min, add the min(k, max(k*add_frac, 1))
 * largest.  Ties go to the lower index. */
static int
_iset_add_largest (char *inP, int n, const double *v, double vmin, double add_frac)
{
  _orc_vi *cand = malloc (sizeof (_orc_vi) * n);
  int k = 0, adds, i, csize = 0;

  for (i = 0; i < n; i++)
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
    qsort (cand, k, sizeof (_orc_vi), _vi_cmp_desc);

    for (i = 0; i < adds; i++)
      inP[cand[i].pos] = 1;
  }

  free (cand);

  return adds;
}

/* ncm_nnls_solve with NCM_NNLS_UMETHOD_NORMAL and reltol = DBL_EPSILON
 * (numcosmo/ncm/algebra/ncm_nnls.c:767-871; reltol default :271-274).
 * A is nrows x ncols row-major; returns the residual norm. */
double
orc_nnls_solve (const double *A, int nrows, int ncols, const double *f, double *x, int nthreads)
{
  const double reltol = DBL_EPSILON;
  _orc_nnls s;
  char *P     = malloc (ncols);

  g_nnls_lu = g_nnls_qr = 0;

  char *Ptry  = malloc (ncols);
  double *res = malloc (sizeof (double) * nrows);
  double *rtr = malloc (sizeof (double) * nrows);
  double *xtr = malloc (sizeof (double) * ncols);
  double *mg  = malloc (sizeof (double) * ncols);
  double rnorm;
  int i;

  s.A        = A;
  s.nrows    = nrows;
  s.ncols    = ncols;
  s.f        = f;
  s.nthreads = nthreads;
  s.M        = calloc ((size_t) ncols * ncols, sizeof (double));
  s.b        = malloc (sizeof (double) * ncols);
  s.Msub     = malloc (sizeof (double) * (size_t) ncols * ncols);
  s.xsub     = malloc (sizeof (double) * ncols);
  s.Psub     = malloc (sizeof (int) * ncols);

  /* M = A^T A, upper triangle (ncm_matrix_square_to_sym, ncm_matrix.c:1548-1572) */
#ifdef _OPENMP
  #pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (i = 0; i < ncols; i++)
  {
    double *Mi = s.M + (size_t) i * ncols;
    int r, c;

    for (r = 0; r < nrows; r++)
    {
      const double *a = A + (size_t) r * ncols;
      const double ai = a[i];

      for (c = i; c < ncols; c++)
        Mi[c] += ai * a[c];
    }
  }

  /* b = A^T f */
  for (i = 0; i < ncols; i++)
    s.b[i] = 0.0;

  for (i = 0; i < nrows; i++)
  {
    const double *a = A + (size_t) i * ncols;
    int c;

    for (c = 0; c < ncols; c++)
      s.b[c] += a[c] * f[i];
  }

  for (i = 0; i < ncols; i++)
    P[i] = 1;

  _nnls_solve_feasible (&s, P, x, ncols);
  rnorm = _nnls_residuals (&s, x, res);
  _nnls_mgrad (&s, res, mg);

  while (1)
  {
    double add_frac = 1.0;
    int finish      = 0;

    while (1)
    {
      double lrnorm;
      int added;

      memcpy (Ptry, P, ncols);
      added     = _iset_add_largest (Ptry, ncols, mg, rnorm * reltol, add_frac);
      add_frac *= 0.5;

      if (added == 0)
      {
        finish = 1;
        break;
      }

      _nnls_solve_feasible (&s, Ptry, xtr, added);
      lrnorm = _nnls_residuals (&s, xtr, rtr);

      if (rnorm - lrnorm > rnorm * reltol)
      {
        memcpy (P, Ptry, ncols);
        memcpy (x, xtr, sizeof (double) * ncols);
        memcpy (res, rtr, sizeof (double) * nrows);
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

    _nnls_mgrad (&s, res, mg);
  }

  free (P);
  free (Ptry);
  free (res);
  free (rtr);
  free (xtr);
  free (mg);
  free (s.M);
  free (s.b);
  free (s.Msub);
  free (s.xsub);
  free (s.Psub);

  return rnorm;
}

/* ------------------------------------------------------------------------ */
/* StatsDist object                                                         */
/* ------------------------------------------------------------------------ */

struct orc_sd
{
  int kind, kernel, d;
  double nu;
  double over_smooth, shrink, local_frac;
  int use_rot_href, nearPD_maxiter, nthreads, cov_type;
  double *cov_fixed;      /* cov-type FIXED: the global covariance, d x d (NULL: unset) */

  int n;                  /* observations (n_obs)                       */
  double *X;
  int cv_type, nk;         /* CV type; kernels (n_kernels) of the prepare */
  double split_frac;

  int prepared, k, wcum_ready, interp_branch, chol_fallbacks;
  double href, kernel_lnnorm, rnorm;
  double *weights, *wcum;
  double *cov, *U;
  double *Y;
  double *Ui;
  double *lnnorms;
  int *knn;
  double *loo_draws;      /* LOO Monte Carlo: per pair u, z1[d], (c1), z2[d], (c2) */
  long loo_npairs;
  int loo_short;          /* a LOO objective ran out of draws                */
  double *split_draws;    /* CV_SPLIT: unit gaussians of the restarts, in order */
  int no_fit;             /* checker's knob: skip the CV bandwidth fits          */
  long split_ndraws, split_pos;
};

orc_sd *
orc_sd_new (int kind, int kernel, double nu, int d)
{
  orc_sd *sd = calloc (1, sizeof (orc_sd));

  sd->kind           = kind;
  sd->kernel         = kernel;
  sd->nu             = nu;
  sd->d              = d;
  sd->over_smooth    = 1.0;
  sd->shrink         = 0.01;
  sd->local_frac     = 0.05;
  sd->use_rot_href   = 0;
  sd->nearPD_maxiter = 200;
  sd->nthreads       = 1;
  sd->split_frac     = 0.5;   /* "split-frac" construct-time default, ncm_stats_dist.c:428-434 */
  sd->cov            = calloc (d * d, sizeof (double));
  sd->U              = calloc (d * d, sizeof (double));

  return sd;
}

static void
_orc_sd_free_prepared (orc_sd *sd)
{
  free (sd->weights);
  free (sd->wcum);
  free (sd->Y);
  free (sd->Ui);
  free (sd->lnnorms);
  free (sd->knn);
  sd->weights = sd->wcum = sd->Y = sd->Ui = sd->lnnorms = NULL;
  sd->knn      = NULL;
  sd->prepared = 0;
}

void
orc_sd_free (orc_sd *sd)
{
  if (sd == NULL)
    return;

  free (sd->split_draws);
  free (sd->loo_draws);
  free (sd->cov_fixed);
  _orc_sd_free_prepared (sd);
  free (sd->X);
  free (sd->cov);
  free (sd->U);
  free (sd);
}

void
orc_sd_set_params (orc_sd *sd, double over_smooth, double shrink, double local_frac,
                   int use_rot_href, int nearPD_maxiter)
{
  sd->over_smooth    = over_smooth;
  sd->shrink         = shrink;
  sd->local_frac     = local_frac;
  sd->use_rot_href   = use_rot_href;
  sd->nearPD_maxiter = nearPD_maxiter;
}

void
orc_sd_set_threads (orc_sd *sd, int nthreads)
{
  sd->nthreads = nthreads > 0 ? nthreads : 1;
}

/* ncm_stats_dist_reset + add_obs for every row (ncm_stats_dist.c:1680-1686,1790-1796) */
void
orc_sd_set_sample (orc_sd *sd, const double *X, int n)
{
  _orc_sd_free_prepared (sd);
  free (sd->X);
  sd->n = n;
  sd->X = malloc (sizeof (double) * (size_t) n * sd->d);
  memcpy (sd->X, X, sizeof (double) * (size_t) n * sd->d);
}

/* NcmStatsDistCV and the split fraction (ncm_stats_dist_set_split_frac,
 * ncm_stats_dist.c:1303-1311) */
void
orc_sd_set_cv (orc_sd *sd, int cv_type, double split_frac)
{
  sd->cv_type    = cv_type;
  sd->split_frac = split_frac;
}

/* get_href: ncm_stats_dist.c:476-482 (KDE, with n_kernels) and ncm_stats_dist_vkde.c:317-335 (VKDE) */
static double
_orc_get_href (orc_sd *sd)
{
  const double base = sd->over_smooth * orc_kernel_rot_bandwidth (sd->kernel, sd->nu, sd->d, (double) sd->nk);

  if (sd->kind == ORC_KDE)
    return base;

  if (sd->use_rot_href)
    return base / sd->local_frac;

  return sd->over_smooth;
}

/* _ncm_stats_dist_prepare (ncm_stats_dist.c:703-789, CV_NONE) with
 * _ncm_stats_dist_kde_prepare_kernel (ncm_stats_dist_kde.c:379-490, cov SAMPLE)
 * and _ncm_stats_dist_vkde_prepare_kernel / build_cov_array_kdtree
 * (ncm_stats_dist_vkde.c:363-516). */
/* the covariance of cov-type (ncm_stats_dist_kde.c:404-444; VKDE local
 * neighbourhoods ncm_stats_dist_vkde.c:462-476, where FIXED means SAMPLE) */
static void
_orc_cov (orc_sd *sd, const int *rows, int nrows, double *cov)
{
  switch (sd->cov_type)
  {
    case ORC_COV_ROBUST_DIAG:
      orc_cov_robust_diag (sd->X, rows, nrows, sd->d, cov);
      break;
    case ORC_COV_ROBUST:
      orc_cov_robust_ogk (sd->X, rows, nrows, sd->d, cov);
      break;
    default:
      orc_welford_cov (sd->X, rows, nrows, sd->d, cov);
      break;
  }
}

void
orc_sd_set_cov_type (orc_sd *sd, int cov_type)
{
  sd->cov_type = cov_type;
}

/* ncm_stats_dist_kde_set_cov_fixed (ncm_stats_dist_kde.c:825-845): a copy of
 * the matrix, the global covariance of cov-type FIXED */
void
orc_sd_set_cov_fixed (orc_sd *sd, const double *cov)
{
  const size_t bytes = sizeof (double) * (size_t) sd->d * sd->d;

  if (sd->cov_fixed == NULL)
    sd->cov_fixed = malloc (bytes);

  memcpy (sd->cov_fixed, cov, bytes);
}

static int _orc_split_nofit (orc_sd *sd);
static int _orc_loo_fit (orc_sd *sd);

/* _ncm_stats_dist_prepare (ncm_stats_dist.c:703-789): n_obs = n; n_kernels =
 * n, or ceil(n split_frac) for the split CV types (the first n_kernels
 * observations are the kernels, the rest only enter the VKDE neighbourhoods
 * and the cross-validation) */
int
orc_sd_prepare (orc_sd *sd)
{
  const int d = sd->d, n = sd->n;
  int i, fb;

  _orc_sd_free_prepared (sd);
  sd->chol_fallbacks = 0;

  if (n <= d)
    return ORC_ERR_SAMPLE_TOO_SMALL;

  if (sd->cv_type == ORC_CV_SPLIT_NOFIT || sd->cv_type == ORC_CV_SPLIT)
  {
    if (!(sd->split_frac >= 0.01 && sd->split_frac <= 1.0))
      return ORC_ERR_INVALID;

    sd->nk = (int) ceil (n * sd->split_frac);

    if (sd->nk <= d)
      return ORC_ERR_SAMPLE_TOO_SMALL;
  }
  else if (sd->cv_type == ORC_CV_NONE || sd->cv_type == ORC_CV_LOO)
    sd->nk = n;
  else
    return ORC_ERR_INVALID;

  const int nk = sd->nk;

  if (sd->kind == ORC_VKDE && sd->local_frac * n < 2)
    return ORC_ERR_TOO_FEW_LOCAL;

  /* the robust estimates' minimum (ncm_stats_vec.c:1841-1843, 1911-1913) */
  if ((sd->cov_type == ORC_COV_ROBUST_DIAG || sd->cov_type == ORC_COV_ROBUST) &&
      (n < 4 || (sd->kind == ORC_VKDE && (int) (size_t) ((sd->local_frac * n > 2) ? sd->local_frac * n : 2) < 4)))
    return ORC_ERR_SAMPLE_TOO_SMALL;

  /* global covariance over the kernels, Cholesky, lnnorm, whitened sample */
  if (sd->cov_type == ORC_COV_FIXED)
  {
    /* ncm_stats_dist_kde.c:414-421: the fixed matrix and its factor from
     * set_cov_fixed / set_cov_type (:791-797, 838-845), a plain Cholesky
     * decomposition with no nearPD repair (not positive definite: error) */
    if (sd->cov_fixed == NULL)
      return ORC_ERR_INVALID;

    memcpy (sd->cov, sd->cov_fixed, sizeof (double) * d * d);
    memcpy (sd->U, sd->cov_fixed, sizeof (double) * d * d);

    if (orc_cholesky_upper (sd->U, d) != 0)
      return ORC_ERR_NOT_PD;

    for (i = 0; i < d; i++)
    {
      int j;

      for (j = 0; j < i; j++)
        sd->U[i * d + j] = 0.0;
    }
  }
  else
  {
    _orc_cov (sd, NULL, nk, sd->cov);
    fb = orc_cholesky_decomp_fallback (sd->cov, sd->U, d, sd->nearPD_maxiter);

    if (fb < 0)
      return ORC_ERR_NOT_PD;

    sd->chol_fallbacks += (fb > 0);
  }
  sd->kernel_lnnorm   = orc_kernel_lnnorm (sd->kernel, sd->nu, d, sd->U);

  sd->Y = malloc (sizeof (double) * (size_t) n * d);

  /* invUsample = sample * U^{-1} (gsl_blas_dtrsm Right/Upper/NoTrans, kde.c:477-480) */
  for (i = 0; i < n; i++)
  {
    const double *x = sd->X + (size_t) i * d;
    double *y       = sd->Y + (size_t) i * d;
    int j, kk;

    for (j = 0; j < d; j++)
    {
      double s = x[j];

      for (kk = 0; kk < j; kk++)
        s -= y[kk] * sd->U[kk * d + j];

      y[j] = s / sd->U[j * d + j];
    }
  }

  if (sd->kind == ORC_VKDE)
  {
    const double kd = (sd->local_frac * n > 2) ? sd->local_frac * n : 2;
    const int k     = (int) (size_t) kd;
    int bad         = 0;

    sd->k       = k;
    sd->knn     = malloc (sizeof (int) * (size_t) nk * k);
    sd->Ui      = malloc (sizeof (double) * (size_t) nk * d * d);
    sd->lnnorms = malloc (sizeof (double) * nk);

    orc_knn_q (sd->Y, n, nk, d, k, sd->knn, sd->nthreads);

#ifdef _OPENMP
    #pragma omp parallel for schedule(dynamic, 8) num_threads(sd->nthreads) reduction(+:bad)
#endif
    for (i = 0; i < nk; i++)
    {
      double *cov_i = malloc (sizeof (double) * d * d);
      double *U_i   = sd->Ui + (size_t) i * d * d;
      int r;

      _orc_cov (sd, sd->knn + (size_t) i * k, k, cov_i);
      r = orc_cholesky_decomp_fallback (cov_i, U_i, d, sd->nearPD_maxiter);

      if (r < 0)
        bad++;
      else
        sd->lnnorms[i] = orc_kernel_lnnorm (sd->kernel, sd->nu, d, U_i);

      if (r > 0)
      {
#ifdef _OPENMP
        #pragma omp atomic
#endif
        sd->chol_fallbacks++;
      }

      free (cov_i);
    }

    if (bad)
      return ORC_ERR_NOT_PD;
  }

  sd->weights = malloc (sizeof (double) * nk);
  sd->wcum    = malloc (sizeof (double) * (nk + 1));

  sd->href = _orc_get_href (sd);

  for (i = 0; i < nk; i++)
    sd->weights[i] = 1.0 / (1.0 * nk);

  sd->wcum_ready    = 0;
  sd->prepared      = 1;
  sd->interp_branch = 0;
  sd->rnorm         = 0.0;

  if (sd->no_fit)
    return ORC_OK;

  if (sd->cv_type == ORC_CV_SPLIT_NOFIT)
    return _orc_split_nofit (sd);

  if (sd->cv_type == ORC_CV_LOO)
    return _orc_loo_fit (sd);

  return ORC_OK;
}

/* IM[j][i], n_obs x n_kernels row-major: compute_IM of
 * ncm_stats_dist_kde.c:493-557 (KDE: the symmetric kernel block, then the
 * held-out rows against every kernel) and ncm_stats_dist_vkde.c:518-606
 * (VKDE: kernel by kernel over every observation). */
int
orc_sd_compute_IM (orc_sd *sd, double *IM)
{
  const int d = sd->d, n = sd->n, nk = sd->nk;
  const double href2 = sd->href * sd->href;
  int i;

  if (!sd->prepared)
    return ORC_ERR_NOT_PREPARED;

  if (sd->kind == ORC_KDE)
  {
    const double scale = exp (-(sd->kernel_lnnorm + d * log (sd->href)));

#ifdef _OPENMP
    #pragma omp parallel for schedule(dynamic, 8) num_threads(sd->nthreads)
#endif
    for (i = 0; i < nk; i++)
    {
      const double *yi = sd->Y + (size_t) i * d;
      int j, kk;

      IM[(size_t) i * nk + i] = 0.0;

      for (j = i + 1; j < nk; j++)
      {
        const double *yj = sd->Y + (size_t) j * d;
        double chi2      = 0.0;

        for (kk = 0; kk < d; kk++)
          chi2 += sq (yi[kk] - yj[kk]);

        chi2 = chi2 / href2;

        IM[(size_t) i * nk + j] = chi2;
        IM[(size_t) j * nk + i] = chi2;
      }
    }

#ifdef _OPENMP
    #pragma omp parallel for schedule(dynamic, 8) num_threads(sd->nthreads)
#endif
    for (i = nk; i < n; i++)
    {
      const double *yi = sd->Y + (size_t) i * d;
      int j, kk;

      for (j = 0; j < nk; j++)
      {
        const double *yj = sd->Y + (size_t) j * d;
        double chi2      = 0.0;

        for (kk = 0; kk < d; kk++)
          chi2 += sq (yi[kk] - yj[kk]);

        IM[(size_t) i * nk + j] = chi2 / href2;
      }
    }

#ifdef _OPENMP
    #pragma omp parallel for num_threads(sd->nthreads)
#endif
    for (i = 0; i < n; i++)
    {
      int j;

      for (j = 0; j < nk; j++)
        IM[(size_t) i * nk + j] = orc_kernel_eval_unnorm (sd->kernel, sd->nu, d, IM[(size_t) i * nk + j]) * scale;
    }
  }
  else
  {
    const double one_href2   = 1.0 / href2;
    const double lnnorm_href = d * log (sd->href);

#ifdef _OPENMP
    #pragma omp parallel for schedule(dynamic, 8) num_threads(sd->nthreads)
#endif
    for (i = 0; i < nk; i++)
    {
      const double *U_i   = sd->Ui + (size_t) i * d * d;
      const double *th_i  = sd->X + (size_t) i * d;
      const double norm_i = exp (sd->lnnorms[i] + lnnorm_href);
      const double inv_n  = 1.0 / norm_i;
      double *y           = malloc (sizeof (double) * d);
      int j, kk;

      for (j = 0; j < n; j++)
      {
        const double *xj = sd->X + (size_t) j * d;
        double chi2      = 0.0;

        for (kk = 0; kk < d; kk++)
          y[kk] = xj[kk] - th_i[kk];

        _trsv_ut (U_i, d, y);

        for (kk = 0; kk < d; kk++)
          chi2 += y[kk] * y[kk];

        chi2                    = chi2 * one_href2;
        IM[(size_t) j * nk + i] = orc_kernel_eval_unnorm (sd->kernel, sd->nu, d, chi2) * inv_n;
      }

      free (y);
    }
  }

  return ORC_OK;
}

/* prepare_interp, CV_NONE branch: ncm_stats_dist.c:878-1094 */
typedef struct { double v; int idx; } _orc_sortv;

static int
_sortv_cmp (const void *a, const void *b)
{
  const _orc_sortv *pa = a, *pb = b;

  if (pa->v < pb->v) return -1;
  if (pa->v > pb->v) return 1;
  return (pa->idx < pb->idx) ? -1 : (pa->idx > pb->idx);
}

/* _ncm_stats_dist_compute_IM_full (ncm_stats_dist.c:791-804: row i times
 * 1/f_i) at the current href, then the NNLS fit into the weights; returns rnorm */
static double
_orc_im_full_nnls (orc_sd *sd, double *IM, const double *f, const double *f1)
{
  const int n = sd->n, nk = sd->nk;
  int i;

  orc_sd_compute_IM (sd, IM);

#ifdef _OPENMP
  #pragma omp parallel for num_threads(sd->nthreads)
#endif
  for (i = 0; i < n; i++)
  {
    const double s = 1.0 / f[i];
    int j;

    for (j = 0; j < nk; j++)
      IM[(size_t) i * nk + j] *= s;
  }

  return orc_nnls_solve (IM, n, nk, f1, sd->weights, sd->nthreads);
}

/* |y|^2 in levmar's accumulation order (LEVMAR_L2NRMXMY): blocks of eight
 * downwards into four partial sums, the remainder upwards, then the sum */
static double
_orc_l2_lm (const double *y, int n)
{
  const int blockn = (n >> 3) << 3;
  double s[4] = { 0.0, 0.0, 0.0, 0.0 };
  int i, j, t;

  for (i = blockn - 1; i > 0; i -= 8)
    for (j = 0; j < 8; j++)
      s[j & 3] += y[i - j] * y[i - j];

  for (i = blockn, t = 7 - (n - blockn); i < n; i++, t++)
    s[t & 3] += y[i] * y[i];

  return ((s[0] + s[1]) + s[2]) + s[3];
}

/* dlevmar_dif (numcosmo/external/levmar/lm_core.c:439-830) restated for one
 * parameter and a zero measurement vector: Levenberg-Marquardt with
 * Nielsen's damping rule (mu *= max(1/3, 1 - (2 dF/dL - 1)^3) on success,
 * mu *= nu, nu *= 2 on failure), a forward-difference Jacobian with step
 * max(1e-4 |p|, delta), refreshed every K = 10 Broyden rank-one updates or
 * after a run of failures; stops on |e|^2 <= eps3, |J^T e| <= eps1,
 * Dp^2 <= eps2^2 p^2, Dp^2 >= (p^2 + eps2) / 1e-24, a non-finite |e|^2 or
 * itmax.  opts = (tau, eps1, eps2, eps3, delta).  f fills hx (n values) at
 * p; returns the number of iterations. */
int
orc_lm1_dif (orc_lm_fn func, double *p, int n, int itmax, const double *opts, void *ctx)
{
  const double tau = opts[0], eps1 = opts[1], eps2 = opts[2], eps2_sq = opts[2] * opts[2], eps3 = opts[3];
  const double delta = opts[4];
  const double one_third = 0.3333333334, lm_eps = 1.0e-12;
  double *hx   = malloc (sizeof (double) * n), *wrk = malloc (sizeof (double) * n);
  double *jac  = malloc (sizeof (double) * n), *e = malloc (sizeof (double) * n);
  double p_eL2, mu = 0.0, jacTe = 0.0, jacTjac = 0.0, jacTe_inf = 0.0, p_L2 = 0.0;
  int nu = 20, updjac = 0, updp = 1, newjac = 0, k = 0, i;
  const int K = 10;

  func (*p, hx, n, ctx);

  for (i = 0; i < n; i++)
    e[i] = -hx[i];

  p_eL2 = _orc_l2_lm (e, n);

  if (isfinite (p_eL2))
    for (k = 0; k < itmax; k++)
    {
      if (p_eL2 <= eps3)
        break;

      if ((updp && nu > 16) || updjac == K)
      {
        double d = fabs (1.0e-4 * *p);

        if (d < delta)
          d = delta;

        func (*p + d, wrk, n, ctx);
        d = 1.0 / d;

        for (i = 0; i < n; i++)
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
          for (i = n - 1; i >= 0; i--)
          {
            jacTjac += jac[i] * jac[i];
            jacTe   += jac[i] * e[i];
          }
        else
          for (i = 0; i < n; i++)
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
          const double Dp    = jacTe / A;
          const double pDp   = *p + Dp;
          const double Dp_L2 = Dp * Dp;
          double pDp_eL2, dF, dL;

          if (Dp_L2 <= eps2_sq * p_L2)
            break;

          if (Dp_L2 >= (p_L2 + eps2) / (lm_eps * lm_eps))
            break;

          func (pDp, wrk, n, ctx);
          pDp_eL2 = _orc_l2_lm (wrk, n);

          if (!isfinite (pDp_eL2))
            break;

          dF = p_eL2 - pDp_eL2;

          if (updp || dF > 0.0)
          {
            for (i = 0; i < n; i++)
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

            t  = 1.0 - t * t * t;
            mu = mu * ((t >= one_third) ? t : one_third);
            nu = 2;
            *p = pDp;

            for (i = 0; i < n; i++)
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

  free (hx);
  free (wrk);
  free (jac);
  free (e);

  return k;
}

typedef struct
{
  orc_sd *sd;
  const double *m2lnp, *f, *f1;
  double min_m2lnp, *IM, *m2;
} _orc_split_ctx;

/* _ncm_stats_dist_prepare_interp_fit_nnls_f (ncm_stats_dist.c:815-846) */
static void
_orc_split_f (double p, double *hx, int n, void *vctx)
{
  _orc_split_ctx *c = vctx;
  orc_sd *sd        = c->sd;
  int i;

  sd->over_smooth = exp (p);
  sd->href        = _orc_get_href (sd);
  _orc_im_full_nnls (sd, c->IM, c->f, c->f1);
  orc_sd_eval_m2lnp_batch (sd, sd->X, n, c->m2);

  for (i = 0; i < n; i++)
    hx[i] = expm1 (-0.5 * (c->m2[i] - (c->m2lnp[i] - c->min_m2lnp)));
}

/* CV_SPLIT (ncm_stats_dist.c:1018-1066) */
static int
_orc_split_fit (orc_sd *sd, const double *m2lnp, double min_m2lnp, double *IM, const double *f, const double *f1)
{
  static const double opts[5] = { 1.0e-3, 1.0e-7, 1.0e-7, 1.0e-10, 1.0e-6 };
  double ln_os = log (sd->over_smooth), rnorm0;
  _orc_split_ctx c;
  int i;

  rnorm0 = _orc_im_full_nnls (sd, IM, f, f1);

  for (i = 0; i < 10; i++)
  {
    double ln_os_try, rnorm_try;

    if (sd->split_pos >= sd->split_ndraws)
      return ORC_ERR_INVALID;

    ln_os_try = sd->split_draws[sd->split_pos++] * 0.5 + ln_os;

    sd->over_smooth = exp (ln_os_try);
    sd->href        = _orc_get_href (sd);
    rnorm_try       = _orc_im_full_nnls (sd, IM, f, f1);

    if (rnorm_try < rnorm0)
    {
      ln_os  = ln_os_try;
      rnorm0 = rnorm_try;
    }
  }

  c.sd        = sd;
  c.m2lnp     = m2lnp;
  c.f         = f;
  c.f1        = f1;
  c.min_m2lnp = min_m2lnp;
  c.IM        = IM;
  c.m2        = malloc (sizeof (double) * sd->n);
  orc_lm1_dif (_orc_split_f, &ln_os, sd->n, 10000, opts, &c);
  free (c.m2);

  sd->over_smooth = exp (ln_os);
  sd->href        = _orc_get_href (sd);
  sd->rnorm       = _orc_im_full_nnls (sd, IM, f, f1);

  return ORC_OK;
}

void
orc_sd_set_split_draws (orc_sd *sd, long n, const double *g)
{
  free (sd->split_draws);
  sd->split_draws  = malloc (sizeof (double) * (size_t) (n > 0 ? n : 1));
  sd->split_ndraws = n;
  sd->split_pos    = 0;
  memcpy (sd->split_draws, g, sizeof (double) * (size_t) n);
}

/* m2lnp has n_obs entries.  Under a split the range is taken over the
 * kernels' entries, the sort over all observations (ncm_stats_dist.c:895-922);
 * where the reference would index a weight past n_kernels (a held-out
 * observation among the n_cut lowest) or find a different count of
 * observations below the cut than n_cut (its g_assert at :966), this returns
 * ORC_ERR_INVALID. */
int
orc_sd_prepare_interp (orc_sd *sd, const double *m2lnp)
{
  const double dbl_limit = 2.0;
  const double thr       = -2.0 * dbl_limit * ORC_LOG_DBL_EPSILON;
  double min_m2lnp = INFINITY, max_m2lnp = -INFINITY;
  int ret, i, n, nk;


  ret = orc_sd_prepare (sd);

  if (ret != ORC_OK)
    return ret;

  n  = sd->n;
  nk = sd->nk;

  for (i = 0; i < nk; i++)
  {
    min_m2lnp = fmin (min_m2lnp, m2lnp[i]);
    max_m2lnp = fmax (max_m2lnp, m2lnp[i]);
  }

  if (max_m2lnp - min_m2lnp > thr)
  {
    _orc_sortv *s = malloc (sizeof (_orc_sortv) * n);
    int n_cut     = 0;

    for (i = 0; i < n; i++)
    {
      s[i].v   = m2lnp[i];
      s[i].idx = i;
    }

    qsort (s, n, sizeof (_orc_sortv), _sortv_cmp);

    for (i = 0; i < nk; i++)
      if (s[i].v - min_m2lnp > thr)
      {
        n_cut = i;
        break;
      }

    if (n_cut < (int) (unsigned) (0.5 * n))
    {
      for (i = 0; i < n_cut; i++)
        if (s[i].idx >= nk)
        {
          free (s);

          return ORC_ERR_INVALID;
        }

      for (i = 0; i < nk; i++)
        sd->weights[i] = 0.1 / (nk - n_cut);

      for (i = 0; i < n_cut; i++)
        sd->weights[s[i].idx] = 0.9 / n_cut;

      sd->interp_branch = 1;
      sd->wcum_ready    = 0;
      free (s);

      return ORC_OK;
    }

    {
      double *Xc = malloc (sizeof (double) * (size_t) n * sd->d);
      double *mc = malloc (sizeof (double) * n);
      int j      = 0;

      for (i = 0; i < n; i++)
        if (m2lnp[i] - min_m2lnp <= thr)
        {
          memcpy (Xc + (size_t) j * sd->d, sd->X + (size_t) i * sd->d, sizeof (double) * sd->d);
          mc[j++] = m2lnp[i];
        }

      if (j != n_cut)
        ret = ORC_ERR_INVALID;
      else
      {
        orc_sd_set_sample (sd, Xc, n_cut);
        ret = orc_sd_prepare_interp (sd, mc);
      }

      if (ret == ORC_OK && sd->interp_branch == 0)
        sd->interp_branch = 2;

      free (Xc);
      free (mc);
      free (s);

      return ret;
    }
  }

  {
    double *IM = malloc (sizeof (double) * (size_t) n * nk);
    double *f  = malloc (sizeof (double) * n);
    double *f1 = malloc (sizeof (double) * n);
    double total_weight = 0.0;

    for (i = 0; i < nk; i++)
      sd->weights[i] = 0.0;

    for (i = 0; i < n; i++)
    {
      f[i]  = exp (-0.5 * (m2lnp[i] - min_m2lnp));
      f1[i] = 1.0;
    }

    if (sd->cv_type == ORC_CV_SPLIT)
    {
      ret = _orc_split_fit (sd, m2lnp, min_m2lnp, IM, f, f1);

      if (ret != ORC_OK)
      {
        free (IM);
        free (f);
        free (f1);

        return ret;
      }
    }
    else
      sd->rnorm = _orc_im_full_nnls (sd, IM, f, f1);

    for (i = 0; i < nk; i++)
      total_weight += sd->weights[i];

    if (!(total_weight > 0.0))
    {
      free (IM);
      free (f);
      free (f1);

      return ORC_ERR_BAD_INPUT;
    }

    {
      const double sc = (1.0 - sd->shrink) / total_weight;
      const double ad = sd->shrink / nk;

      for (i = 0; i < nk; i++)
        sd->weights[i] = sd->weights[i] * sc + ad;
    }

    sd->interp_branch = 0;
    sd->wcum_ready    = 0;

    free (IM);
    free (f);
    free (f1);
  }

  return ORC_OK;
}

/* _ncm_stats_dist_vkde_eval_weights_m2lnp (ncm_stats_dist_vkde.c:682-723) and
 * _ncm_stats_dist_kde_eval_weights_m2lnp (ncm_stats_dist_kde.c:640-681) */
static double
_orc_eval_m2lnp_ws (orc_sd *sd, const double *x, double *chi2, double *lnK, double *y)
{
  const int d = sd->d, n = sd->nk;
  const double href2 = sd->href * sd->href;
  double gamma, lambda;
  int i, kk;

  if (sd->kind == ORC_VKDE)
  {
    const double one_href2 = 1.0 / href2;

    for (i = 0; i < n; i++)
    {
      const double *th = sd->X + (size_t) i * d;
      double c2        = 0.0;

      for (kk = 0; kk < d; kk++)
        y[kk] = x[kk] - th[kk];

      _trsv_ut (sd->Ui + (size_t) i * d * d, d, y);

      for (kk = 0; kk < d; kk++)
        c2 += y[kk] * y[kk];

      chi2[i] = c2 * one_href2;
    }

    orc_kernel_sum0 (sd->kernel, sd->nu, d, n, chi2, sd->weights, sd->lnnorms, lnK, &gamma, &lambda);
  }
  else
  {
    for (kk = 0; kk < d; kk++)
      y[kk] = x[kk];

    _trsv_ut (sd->U, d, y);

    for (i = 0; i < n; i++)
    {
      const double *row = sd->Y + (size_t) i * d;
      double c2         = 0.0;

      for (kk = 0; kk < d; kk++)
        c2 += sq (row[kk] - y[kk]);

      chi2[i] = c2 / href2;
    }

    orc_kernel_sum1 (sd->kernel, sd->nu, d, n, chi2, sd->weights, sd->kernel_lnnorm, lnK, &gamma, &lambda);
  }

  return -2.0 * (gamma + log1p (lambda) - d * log (sd->href));
}

double
orc_sd_eval_m2lnp (orc_sd *sd, const double *x)
{
  double *chi2 = malloc (sizeof (double) * sd->nk);
  double *lnK  = malloc (sizeof (double) * sd->nk);
  double *y    = malloc (sizeof (double) * sd->d);
  double r     = _orc_eval_m2lnp_ws (sd, x, chi2, lnK, y);

  free (chi2);
  free (lnK);
  free (y);

  return r;
}

void
orc_sd_eval_m2lnp_batch (orc_sd *sd, const double *X, int m, double *out)
{
#ifdef _OPENMP
  #pragma omp parallel num_threads(sd->nthreads)
#endif
  {
    double *chi2 = malloc (sizeof (double) * sd->nk);
    double *lnK  = malloc (sizeof (double) * sd->nk);
    double *y    = malloc (sizeof (double) * sd->d);
    int j;

#ifdef _OPENMP
    #pragma omp for schedule(dynamic, 4)
#endif
    for (j = 0; j < m; j++)
      out[j] = _orc_eval_m2lnp_ws (sd, X + (size_t) j * sd->d, chi2, lnK, y);

    free (chi2);
    free (lnK);
    free (y);
  }
}

/* linear-space density: ncm_stats_dist_kde.c:597-637, ncm_stats_dist_vkde.c:632-679 */
double
orc_sd_eval (orc_sd *sd, const double *x)
{
  const int d = sd->d, n = sd->nk;
  const double href2 = sd->href * sd->href;
  double *y = malloc (sizeof (double) * d);
  double s  = 0.0, res;
  int i, kk;

  if (sd->kind == ORC_VKDE)
  {
    const double one_href2 = 1.0 / href2;

    for (i = 0; i < n; i++)
    {
      const double *th = sd->X + (size_t) i * d;
      double c2        = 0.0;

      for (kk = 0; kk < d; kk++)
        y[kk] = x[kk] - th[kk];

      _trsv_ut (sd->Ui + (size_t) i * d * d, d, y);

      for (kk = 0; kk < d; kk++)
        c2 += y[kk] * y[kk];

      c2 = c2 * one_href2;
      s += sd->weights[i] * (orc_kernel_eval_unnorm (sd->kernel, sd->nu, d, c2) / exp (sd->lnnorms[i]));
    }

    res = s / pow (sd->href, d);
  }
  else
  {
    for (kk = 0; kk < d; kk++)
      y[kk] = x[kk];

    _trsv_ut (sd->U, d, y);

    for (i = 0; i < n; i++)
    {
      const double *row = sd->Y + (size_t) i * d;
      double c2         = 0.0;

      for (kk = 0; kk < d; kk++)
        c2 += sq (row[kk] - y[kk]);

      c2 = c2 / href2;
      s += orc_kernel_eval_unnorm (sd->kernel, sd->nu, d, c2) * sd->weights[i];
    }

    res = s * exp (-(sd->kernel_lnnorm + d * log (sd->href)));
  }

  free (y);

  return res;
}

void
orc_sd_eval_batch (orc_sd *sd, const double *X, int m, double *out)
{
  int j;

#ifdef _OPENMP
  #pragma omp parallel for schedule(dynamic, 4) num_threads(sd->nthreads)
#endif
  for (j = 0; j < m; j++)
    out[j] = orc_sd_eval (sd, X + (size_t) j * sd->d);
}

/* ncm_stats_dist_kernel_choose (ncm_stats_dist.c:1565-1606) with p = u */
int
orc_sd_kernel_choose (orc_sd *sd, double p)
{
  const int n = sd->nk;
  int ilo = 0, ihi = n;

  if (!sd->wcum_ready)
  {
    double cum = 0.0;
    int i;

    sd->wcum[0] = cum;

    for (i = 0; i < n; i++)
    {
      cum            += sd->weights[i];
      sd->wcum[i + 1] = cum;
    }

    {
      const double s = 1.0 / cum;

      for (i = 0; i <= n; i++)
        sd->wcum[i] = sd->wcum[i] * s;
    }

    sd->wcum_ready = 1;
  }

  while (ihi > ilo + 1)
  {
    int mi = (ihi + ilo) / 2;

    if (sd->wcum[mi] > p)
      ihi = mi;
    else
      ilo = mi;
  }

  return ilo;
}

/* ncm_stats_dist_sample (ncm_stats_dist.c:1618-1627) with the kernel draws of
 * ncm_stats_dist_kernel_gauss.c:335-355 and ncm_stats_dist_kernel_st.c:388-414:
 * x = theta_i + s * U_i^T (h z), s = 1 (Gauss) or sqrt(nu/chisq) (ST). */
static void _orc_sample_at (orc_sd *sd, int i, const double *z, double chisq, double *x);

int
orc_sd_sample (orc_sd *sd, double u, const double *z, double chisq, double *x)
{
  const int i = orc_sd_kernel_choose (sd, u);

  _orc_sample_at (sd, i, z, chisq, x);

  return i;
}

/* the draw of ncm_stats_dist_kernel_{gauss,st}_sample from kernel i */
static void
_orc_sample_at (orc_sd *sd, int i, const double *z, double chisq, double *x)
{
  const int d = sd->d;
  const double *U   = (sd->kind == ORC_VKDE) ? sd->Ui + (size_t) i * d * d : sd->U;
  const double *mu  = sd->X + (size_t) i * d;
  int kk;

  for (kk = 0; kk < d; kk++)
    x[kk] = z[kk] * sd->href;

  _trmv_ut (U, d, x);

  if (sd->kernel == ORC_ST)
  {
    const double chi_scale = sqrt (sd->nu / chisq);

    for (kk = 0; kk < d; kk++)
      x[kk] = x[kk] * chi_scale;
  }

  for (kk = 0; kk < d; kk++)
    x[kk] = x[kk] + mu[kk];
}

void
orc_sd_sample_batch (orc_sd *sd, int n, const double *u, const double *z,
                     const double *chisq, double *x, int *idx)
{
  int j;

  for (j = 0; j < n; j++)
    idx[j] = orc_sd_sample (sd, u[j], z + (size_t) j * sd->d,
                            chisq ? chisq[j] : 1.0, x + (size_t) j * sd->d);
}

int orc_sd_get_n (orc_sd *sd) { return sd->n; }
int orc_sd_get_k (orc_sd *sd) { return sd->k; }
double orc_sd_get_href (orc_sd *sd) { return sd->href; }
double orc_sd_get_rnorm (orc_sd *sd) { return sd->rnorm; }
double orc_sd_get_kernel_lnnorm (orc_sd *sd) { return sd->kernel_lnnorm; }
int orc_sd_get_interp_branch (orc_sd *sd) { return sd->interp_branch; }
int orc_sd_get_chol_fallbacks (orc_sd *sd) { return sd->chol_fallbacks; }

void orc_sd_get_weights (orc_sd *sd, double *w) { memcpy (w, sd->weights, sizeof (double) * sd->nk); }
int orc_sd_get_nk (orc_sd *sd) { return sd->nk; }
double orc_sd_get_over_smooth (orc_sd *sd) { return sd->over_smooth; }
void orc_sd_get_sample (orc_sd *sd, double *X) { memcpy (X, sd->X, sizeof (double) * (size_t) sd->n * sd->d); }
void orc_sd_get_cov (orc_sd *sd, double *cov) { memcpy (cov, sd->cov, sizeof (double) * sd->d * sd->d); }
void orc_sd_get_U (orc_sd *sd, double *U) { memcpy (U, sd->U, sizeof (double) * sd->d * sd->d); }
void orc_sd_get_invUsample (orc_sd *sd, double *Y) { memcpy (Y, sd->Y, sizeof (double) * (size_t) sd->n * sd->d); }

void
orc_sd_get_Ui (orc_sd *sd, int i, double *U)
{
  if (sd->kind == ORC_VKDE)
    memcpy (U, sd->Ui + (size_t) i * sd->d * sd->d, sizeof (double) * sd->d * sd->d);
  else
    memcpy (U, sd->U, sizeof (double) * sd->d * sd->d);
}

void
orc_sd_get_lnnorms (orc_sd *sd, double *lnnorms)
{
  int i;

  for (i = 0; i < sd->nk; i++)
    lnnorms[i] = (sd->kind == ORC_VKDE) ? sd->lnnorms[i] : sd->kernel_lnnorm;
}

void
orc_sd_get_knn (orc_sd *sd, int *knn)
{
  if (sd->knn)
    memcpy (knn, sd->knn, sizeof (int) * (size_t) sd->nk * sd->k);
}

/* ------------------------------------------------------------------------ */
/* CV_SPLIT_NOFIT: the bandwidth fit of _ncm_stats_dist_prepare              */
/* (ncm_stats_dist.c:768-770, objective _ncm_stats_dist_m2lnp :484-511,      */
/* minimiser _ncm_stats_dist_minimize_obj :660-701).                         */
/* ------------------------------------------------------------------------ */

/* over_smooth = exp(lnos), then the sum, in observation order, of -2 ln p of
 * the held-out observations n_kernels .. n_obs - 1 under the kernels */
static double
_orc_split_obj (orc_sd *sd, double lnos, double *buf)
{
  const int nh = sd->n - sd->nk;
  double s     = 0.0;
  int i;

  sd->over_smooth = exp (lnos);
  sd->href        = _orc_get_href (sd);

  orc_sd_eval_m2lnp_batch (sd, sd->X + (size_t) sd->nk * sd->d, nh, buf);

  for (i = 0; i < nh; i++)
    s += buf[i];

  return s;
}

/* One-dimensional Nelder-Mead in the form of GSL's nmsimplex2 (the
 * minimiser the reference allocates, ncm_stats_dist.c:175), restated from the
 * method's published description: a simplex of the start and the start plus
 * the step 0.1; each iteration reflects the worst vertex through the others'
 * centroid, tries the doubled step when the reflection is the new best,
 * otherwise contracts halfway towards the worst vertex and, failing that,
 * shrinks towards the best; the size is the vertices' RMS distance from
 * their centroid and the fit stops below 1e-3 or after 1000 iterations.
 * As in the reference, the bandwidth left set is the one of the objective's
 * last evaluation, not necessarily the best vertex. */
typedef double (*_orc_obj_fn) (orc_sd *sd, double lnos, void *ctx);

static double
_orc_split_obj_cb (orc_sd *sd, double lnos, void *ctx)
{
  return _orc_split_obj (sd, lnos, (double *) ctx);
}

static int
_orc_nm (orc_sd *sd, _orc_obj_fn obj, void *ctx)
{
  double x[2], f[2];
  int iter;

  x[0] = log (sd->over_smooth);
  x[1] = x[0] + 0.1;
  f[0] = obj (sd, x[0], ctx);
  f[1] = obj (sd, x[1], ctx);

  for (iter = 1; iter <= 1000; iter++)
  {
    const int hi    = (f[1] > f[0]) ? 1 : 0;
    const int lo    = 1 - hi;
    const double c  = x[lo];                 /* centroid of the vertices but the worst */
    const double xr = 2.0 * c - x[hi];
    const double fr = obj (sd, xr, ctx);

    if (isfinite (fr) && fr < f[lo])
    {
      const double xe = 3.0 * c - 2.0 * x[hi];
      const double fe = obj (sd, xe, ctx);

      if (isfinite (fe) && fe < f[lo])
      {
        x[hi] = xe;
        f[hi] = fe;
      }
      else
      {
        x[hi] = xr;
        f[hi] = fr;
      }
    }
    else if (!isfinite (fr) || fr > f[lo])
    {
      if (isfinite (fr) && fr <= f[hi])
      {
        x[hi] = xr;
        f[hi] = fr;
      }

      {
        const double xc = 0.5 * c + 0.5 * x[hi];
        const double fc = obj (sd, xc, ctx);

        if (isfinite (fc) && fc <= f[hi])
        {
          x[hi] = xc;
          f[hi] = fc;
        }
        else
        {
          x[hi] = 0.5 * (x[hi] + x[lo]);
          f[hi] = obj (sd, x[hi], ctx);
        }
      }
    }
    else
    {
      x[hi] = xr;
      f[hi] = fr;
    }

    if (0.5 * fabs (x[0] - x[1]) < 1.0e-3)
      break;
  }

  return ORC_OK;
}

int
orc_nm_split_fit (orc_sd *sd)
{
  double *buf = malloc (sizeof (double) * (size_t) (sd->n - sd->nk + 1));
  const int r = _orc_nm (sd, _orc_split_obj_cb, buf);

  free (buf);

  return r;
}

static int
_orc_split_nofit (orc_sd *sd)
{
  return orc_nm_split_fit (sd);
}

/* ------------------------------------------------------------------------ */
/* CV_LOO: the bandwidth fit of _ncm_stats_dist_prepare (ncm_stats_dist.c:   */
/* 760-765): Nelder-Mead (as above) on the AMISE, in closed form for a       */
/* Gaussian KDE (_ncm_stats_dist_amise_kde_gauss, :513-557) and with a       */
/* Monte Carlo integral otherwise (_ncm_stats_dist_amise, :561-658).         */
/* ------------------------------------------------------------------------ */

void
orc_sd_set_loo_draws (orc_sd *sd, long npairs, const double *u, const double *z1, const double *c1,
                      const double *z2, const double *c2)
{
  const int d = sd->d, st = (sd->kernel == ORC_ST);
  const int stride = 1 + 2 * d + 2 * st;
  long k;

  free (sd->loo_draws);
  sd->loo_draws  = malloc (sizeof (double) * (size_t) npairs * stride);
  sd->loo_npairs = npairs;

  for (k = 0; k < npairs; k++)
  {
    double *p = sd->loo_draws + (size_t) k * stride;
    int c;

    *p++ = u[k];

    for (c = 0; c < d; c++)
      *p++ = z1[(size_t) k * d + c];

    if (st)
      *p++ = c1[k];

    for (c = 0; c < d; c++)
      *p++ = z2[(size_t) k * d + c];

    if (st)
      *p++ = c2[k];
  }
}

int orc_sd_get_loo_short (orc_sd *sd) { return sd->loo_short; }

/* sum_ij IM_ij / n^2 at href = sqrt(2) h, minus the off-diagonal
 * 2 IM_ij / (n (n - 1)) at h, in the reference's order */
static double
_orc_amise_kde_gauss (orc_sd *sd, double lnos, void *ctx)
{
  double *IM   = ctx;
  const int n  = sd->nk;
  const double n2 = (double) n * (double) n;
  const double nn1 = (double) ((unsigned) n * (unsigned) (n - 1));
  double amise = 0.0;
  int i, j;

  sd->over_smooth = exp (lnos);
  sd->href        = sqrt (2.0) * _orc_get_href (sd);
  orc_sd_compute_IM (sd, IM);

  for (i = 0; i < n; i++)
    for (j = 0; j < n; j++)
      amise += IM[(size_t) i * n + j] / n2;

  sd->over_smooth = exp (lnos);
  sd->href        = _orc_get_href (sd);
  orc_sd_compute_IM (sd, IM);

  for (i = 0; i < n; i++)
  {
    for (j = 0; j < i; j++)
      amise -= 2.0 * IM[(size_t) i * n + j] / nn1;

    for (j = i + 1; j < n; j++)
      amise -= 2.0 * IM[(size_t) i * n + j] / nn1;
  }

  return amise;
}

typedef struct { double v; size_t idx; } _orc_sidx;

static int
_sidx_cmp (const void *a, const void *b)
{
  const _orc_sidx *pa = a, *pb = b;

  if (pa->v < pb->v) return -1;
  if (pa->v > pb->v) return 1;
  return (pa->idx < pb->idx) ? -1 : (pa->idx > pb->idx);
}

/* ncm_stats_vec_update with weight 1 on (p1, p2) (ncm_stats_vec.c:511-565) */
typedef struct { double w, w2, bias, m[2], v[2], c01; } _orc_sv2;

static void
_orc_sv2_update (_orc_sv2 *s, const double *x)
{
  const double curweight = s->w + 1.0;
  int i;

  for (i = 0; i < 2; i++)
  {
    const double delta = x[i] - s->m[i];
    const double R     = delta * 1.0 / curweight;
    const double dvar  = s->w * delta * R;

    s->m[i] += R;
    s->v[i] += dvar;

    if (i == 0)
      s->c01 += 1.0 * (x[0] - s->m[0]) * (x[1] - s->m[1]);
  }

  s->w     = curweight;
  s->w2   += 1.0;
  s->bias  = 1.0 / (s->w - s->w2 / s->w);
}

/* ncm_stats_dist_sample2 (ncm_stats_dist.c:1633-1651) from draw pair k, then
 * ncm_stats_dist_eval at both points */
static void
_orc_mc_pair (orc_sd *sd, const size_t *sorted, long k, double *x1, double *x2, double *p)
{
  const int d = sd->d, st = (sd->kernel == ORC_ST), n = sd->n;
  const double *q = sd->loo_draws + (size_t) k * (1 + 2 * d + 2 * st);
  const int i = orc_sd_kernel_choose (sd, q[0]);

  _orc_sample_at (sd, (int) sorted[i], q + 1, st ? q[1 + d] : 1.0, x1);
  _orc_sample_at (sd, (int) sorted[n - 1 - i], q + 1 + d + st, st ? q[1 + 2 * d + 1] : 1.0, x2);
  p[0] = orc_sd_eval (sd, x1);
  p[1] = orc_sd_eval (sd, x2);
}

static double
_orc_amise (orc_sd *sd, double lnos, void *ctx)
{
  double *IM   = ctx;
  const int n  = sd->nk;
  const double nn1 = (double) ((unsigned) n * (unsigned) (n - 1));
  double amise = 0.0, mean = 0.0;
  _orc_sidx *srt = malloc (sizeof (_orc_sidx) * n);
  size_t *sorted = malloc (sizeof (size_t) * n);
  double *x1 = malloc (sizeof (double) * sd->d), *x2 = malloc (sizeof (double) * sd->d);
  _orc_sv2 sv;
  long k = 0, i;
  int a, j;

  sd->over_smooth = exp (lnos);
  sd->href        = _orc_get_href (sd);
  orc_sd_compute_IM (sd, IM);

  for (a = 0; a < n; a++)
  {
    double row_sum = 0.0;

    for (j = 0; j < a; j++)
      row_sum += IM[(size_t) a * n + j];

    for (j = a + 1; j < n; j++)
      row_sum += IM[(size_t) a * n + j];

    amise -= 2.0 * row_sum / nn1;

    srt[a].v   = (row_sum + IM[(size_t) a * n + a]) / n;
    srt[a].idx = (size_t) a;
  }

  /* gsl_sort_index: ascending (ties, absent for distinct sums, by index) */
  qsort (srt, n, sizeof (_orc_sidx), _sidx_cmp);

  for (a = 0; a < n; a++)
    sorted[a] = srt[a].idx;

  memset (&sv, 0, sizeof (sv));

  for (i = 0; i < 100 + 100000000L; i++)
  {
    double p[2];

    if (k >= sd->loo_npairs)
    {
      sd->loo_short = 1;
      amise = NAN;
      break;
    }

    _orc_mc_pair (sd, sorted, k++, x1, x2, p);
    _orc_sv2_update (&sv, p);

    if (i >= 100)
    {
      const long it = i - 100;
      const double var = 0.25 * (sv.v[0] * sv.bias + sv.v[1] * sv.bias + 2.0 * (sv.c01 * sv.bias));
      const double msd = sqrt (var / (it + 101.0)) / (mean = 0.5 * (sv.m[0] + sv.m[1]));

      if (msd < 1.0e-2)
        break;
    }
  }

  amise += mean;

  free (srt);
  free (sorted);
  free (x1);
  free (x2);

  return amise;
}

static int
_orc_loo_fit (orc_sd *sd)
{
  double *IM = malloc (sizeof (double) * (size_t) sd->nk * sd->nk);
  int r;

  sd->loo_short = 0;

  if (sd->kind == ORC_KDE && sd->kernel == ORC_GAUSS)
    r = _orc_nm (sd, _orc_amise_kde_gauss, IM);
  else if (sd->loo_draws == NULL)
    r = ORC_ERR_INVALID;
  else
    r = _orc_nm (sd, _orc_amise, IM);

  free (IM);

  if (r == ORC_OK && sd->loo_short)
    r = ORC_ERR_INVALID;

  return r;
}

/* the kernel layout of the CV type without its bandwidth fit: the weight fit
 * at a given over-smoothing (a checker's knob; the reference has none) */
void orc_sd_set_no_fit (orc_sd *sd, int no_fit) { sd->no_fit = no_fit; }
