/*
 * Flat driver over NumCosmo's vendored levmar (numcosmo/external/levmar),
 * linked only into oracle/_ref/liblevmar_ref.so (test infrastructure): it
 * runs dlevmar_dif, as _ncm_stats_dist_prepare_interp calls it for CV_SPLIT
 * (numcosmo/ncm/stats/ncm_stats_dist.c:1018-1066: one parameter, a NULL
 * measurement vector, 10000 iterations), on a caller's scalar function, so
 * the oracle's restatement of the method can be pinned to it.
 */
#include <stdlib.h>
#include "levmar.h"

typedef void (*ref_lm_fn) (double p, double *hx, int n, void *ctx);

typedef struct { ref_lm_fn f; void *ctx; } tramp_t;

static void
_tramp (double *p, double *hx, int m, int n, void *adata)
{
  tramp_t *t = adata;

  (void) m;
  t->f (p[0], hx, n, t->ctx);
}

int
ref_levmar_dif1 (ref_lm_fn f, double *p, int n, int itmax, double *opts, void *ctx, double *info)
{
  tramp_t t = { f, ctx };
  double cov;
  double *work = malloc (sizeof (double) * LM_DIF_WORKSZ (1, n));
  int r = dlevmar_dif (_tramp, p, NULL, 1, n, itmax, opts, info, work, &cov, &t);

  free (work);

  return r;
}
