/*
 * capi_driver.c -- drives libncg.so from plain C, the way the GObject shim
 * NcmStatsDistVKDEGPU would: create a handle, add the observations, prepare,
 * evaluate -2 ln p, draw samples, fit the weights, read the kernels back.
 * Built with gcc against include/ncg.h alone (no Python, no CUDA headers).
 *
 *   capi_driver --version
 *   capi_driver DIR kind kernel dim nu n m ns
 *
 * DIR holds raw little-endian doubles written by the caller: centres.f64
 * (n x dim), points.f64 (m x dim), u.f64 (ns), z.f64 (ns x dim), chisq.f64
 * (ns, Student-t only), target.f64 (n: -2 ln L at the centres).  The driver
 * writes m2lnp.f64 (m), x.f64 (ns x dim), idx.i32 (ns), weights.f64 (n),
 * m2lnp_fit.f64 (m, after prepare_interp), Ki.f64 (dim + dim^2 + 2, kernel 0).
 * Exit status 0 on success, otherwise the failing call is printed.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ncg.h"

#define CHECK(call)                                                                            \
  do {                                                                                         \
    ncg_status_t st_ = (call);                                                                 \
    if (st_ != NCG_OK)                                                                         \
    {                                                                                          \
      fprintf (stderr, "%s failed: %s (%s)\n", #call, ncg_status_string (st_), ncg_last_error ()); \
      return 1;                                                                                \
    }                                                                                          \
  } while (0)

static void *
_read (const char *dir, const char *name, size_t bytes)
{
  char path[4096];
  FILE *f;
  void *p = malloc (bytes ? bytes : 1);

  snprintf (path, sizeof path, "%s/%s", dir, name);
  f = fopen (path, "rb");

  if (f == NULL || p == NULL || fread (p, 1, bytes, f) != bytes)
  {
    fprintf (stderr, "cannot read %zu bytes from %s\n", bytes, path);
    exit (2);
  }

  fclose (f);

  return p;
}

static int
_write (const char *dir, const char *name, const void *p, size_t bytes)
{
  char path[4096];
  FILE *f;

  snprintf (path, sizeof path, "%s/%s", dir, name);
  f = fopen (path, "wb");

  if (f == NULL || fwrite (p, 1, bytes, f) != bytes)
  {
    fprintf (stderr, "cannot write %s\n", path);
    return 1;
  }

  fclose (f);

  return 0;
}

int
main (int argc, char **argv)
{
  if (argc == 2 && strcmp (argv[1], "--version") == 0)
  {
    printf ("%s\n%s\n", ncg_version (), ncg_status_string (NCG_ERR_SAMPLE_TOO_SMALL));

    return 0;
  }

  if (argc != 9)
  {
    fprintf (stderr, "usage: %s DIR kind kernel dim nu n m ns | --version\n", argv[0]);

    return 2;
  }

  const char *dir   = argv[1];
  const int kind    = atoi (argv[2]), kernel = atoi (argv[3]);
  const unsigned d  = (unsigned) atoi (argv[4]);
  const double nu   = atof (argv[5]);
  const uint64_t n  = strtoull (argv[6], NULL, 10), m = strtoull (argv[7], NULL, 10), ns = strtoull (argv[8], NULL, 10);
  double *X         = _read (dir, "centres.f64", n * d * sizeof (double));
  double *P         = _read (dir, "points.f64", m * d * sizeof (double));
  double *u         = _read (dir, "u.f64", ns * sizeof (double));
  double *z         = _read (dir, "z.f64", ns * d * sizeof (double));
  double *cs        = kernel == NCG_KERNEL_ST ? _read (dir, "chisq.f64", ns * sizeof (double)) : NULL;
  double *target    = _read (dir, "target.f64", n * sizeof (double));
  double *m2lnp     = malloc (m * sizeof (double));
  double *xs        = malloc (ns * d * sizeof (double));
  int32_t *idx      = malloc (ns * sizeof (int32_t));
  double *w         = malloc (n * sizeof (double));
  double *Ki        = malloc ((d + d * d + 2) * sizeof (double));
  ncg_sd_config_t cfg;
  ncg_sd_t *sd = NULL;
  uint64_t nk;

  ncg_sd_config_init (&cfg);
  CHECK (ncg_sd_new ((ncg_kind_t) kind, (ncg_kernel_t) kernel, d, nu, &cfg, &sd));

  /* ncm_stats_dist_reset + add_obs per point, as the walker fills the sample */
  CHECK (ncg_sd_reset (sd));
  for (uint64_t i = 0; i < n; i++)
    CHECK (ncg_sd_add_obs (sd, X + i * d));

  CHECK (ncg_sd_prepare (sd));
  CHECK (ncg_sd_eval_m2lnp_batch (sd, P, m, m2lnp));
  CHECK (ncg_sd_sample_batch (sd, u, z, cs, ns, xs, idx));

  if (_write (dir, "m2lnp.f64", m2lnp, m * sizeof (double)) || _write (dir, "x.f64", xs, ns * d * sizeof (double)) ||
      _write (dir, "idx.i32", idx, ns * sizeof (int32_t)))
    return 1;

  /* the weight fit and the per-point eval the walker uses afterwards */
  CHECK (ncg_sd_prepare_interp (sd, target));
  CHECK (ncg_sd_get_n_kernels (sd, &nk));
  CHECK (ncg_sd_get_weights (sd, w));
  for (uint64_t j = 0; j < m; j++)
    CHECK (ncg_sd_eval_m2lnp (sd, P + j * d, m2lnp + j));
  CHECK (ncg_sd_get_Ki (sd, 0, Ki, Ki + d, Ki + d + d * d, Ki + d + d * d + 1));

  if (_write (dir, "weights.f64", w, nk * sizeof (double)) || _write (dir, "m2lnp_fit.f64", m2lnp, m * sizeof (double)) ||
      _write (dir, "Ki.f64", Ki, (d + d * d + 2) * sizeof (double)))
    return 1;

  CHECK (ncg_sd_free (sd));
  printf ("ok n_kernels=%llu\n", (unsigned long long) nk);

  free (X); free (P); free (u); free (z); free (cs); free (target);
  free (m2lnp); free (xs); free (idx); free (w); free (Ki);

  return 0;
}
