/*
 * ncg_server.c -- the serving loop (ncg_server_*): concurrent APES chains,
 * one request = one APES step of one chain.
 *
 * Threads: `slots` workers share one mutex-protected scheduler state.  A
 * worker takes the oldest pending request whose chain is idle and either
 * resident or admissible within the device-memory budget (evicting idle
 * chains, least recently used first, when that makes room), runs the step
 * on the chain's own stream and records the result.  Requests of one chain
 * run in submission order; requests of different chains run concurrently,
 * so their kernels overlap on the device.
 *
 * Memory: a resident chain holds its StatsDist state and the step buffers
 * (estimated by _chain_bytes); each worker holds one arena for the O(n^2)
 * prepare_interp matrices (ncg_sd_set_workspace), sized for the largest
 * chain added, allocated at the worker's first step.  Both count against
 * hbm_budget.  An evicted chain keeps its
 * walkers, -2 ln L and RNG on the host and is rebuilt on its next step.
 *
 * A step is one APES half-move (numcosmo/ncm/fit/ncm_fit_esmcmc_walker_apes.c:
 * 739-919, see _run_step): the half that moves draws its proposals from the
 * fit of the other half.  The RNG draws come from the chain's own MT19937
 * stream in a fixed order, so a chain's trajectory is the same whatever else
 * the server runs.
 */
#define _POSIX_C_SOURCE 200809L

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <cuda_runtime_api.h>

#include "ncg_internal.h"
#include "ncg_host.h"

enum { CH_WAITING = 0, CH_LOADING, CH_RESIDENT, CH_EVICTING };
enum { RQ_PENDING = 0, RQ_RUNNING, RQ_DONE };

typedef struct
{
  ncg_chain_desc_t desc;
  double *X, *m2, *L;                 /* host state (pinned), target factor */
  double *hu, *hz, *hch, *hacc;       /* host draws (pinned) */
  double *lb, *ub, *hprop;            /* bounds (+-inf when none), proposals of a bounded step (pinned) */
  int32_t *hmap;                      /* moving walker of each compacted draw */
  int bounded;                        /* some bound is finite */
  uint32_t explore_left;              /* half-moves still in the exploration phase */
  ncg_rng_t *rng;
  int state, running;
  int64_t npending;
  uint64_t steps, last_used, bytes;
  ncg_sd_t *sd;
  cudaStream_t stream;                /* the handle's stream while resident */
  void *dbuf;                         /* step buffers, one allocation */
} chain_t;

typedef struct
{
  int32_t chain;
  int state;
  ncg_step_result_t res;
} req_t;

typedef struct
{
  ncg_server_t *s;
  int idx;
  pthread_t th;
  void *ws;
  size_t ws_bytes;
} worker_t;

struct ncg_server
{
  ncg_server_config_t cfg;
  pthread_mutex_t mu;
  pthread_cond_t cv_work, cv_done;
  int stop, started;
  chain_t *ch;
  int nch, capch;
  req_t *rq;
  int64_t nrq, caprq, first_pending;
  uint64_t reserved, peak;
  uint64_t admitted, evicted, failed, completed;
  int running;
  uint64_t tick, scan;
  uint64_t *stamp;
  size_t ws_size;
  uint64_t n_max;                     /* largest chain added */
  cudaMemPool_t pool;                 /* chain buffers, stream-ordered; keeps up to the budget cached */
  worker_t *w;
  struct timespec t0;
};

static double
_now (const ncg_server_t *s)
{
  struct timespec t;

  clock_gettime (CLOCK_MONOTONIC, &t);

  return (double) (t.tv_sec - s->t0.tv_sec) + 1e-9 * (double) (t.tv_nsec - s->t0.tv_nsec);
}

double
ncg_server_clock (ncg_server_t *s)
{
  return s ? _now (s) : 0.0;
}

ncg_status_t
ncg_server_config_init (ncg_server_config_t *cfg)
{
  if (cfg == NULL)
    return NCG_ERR_INVALID_ARG;

  memset (cfg, 0, sizeof (*cfg));
  cfg->device     = 0;
  cfg->slots      = 4;
  cfg->precision  = NCG_PREC_MIXED;
  cfg->hbm_budget = (uint64_t) 40 << 30;

  return NCG_OK;
}

/* ------------------------------------------------------------ accounting */

/* step buffers of a chain (one half of N = n/2 walkers moves per step):
 * proposals, the 2N eval points, fit and target values, the moving half's
 * walkers and -2 ln L, the draws, the accept counter */
static size_t
_dbuf_doubles (const ncg_chain_desc_t *c)
{
  const size_t n = c->n / 2, d = c->dim;

  return n * d /* prop */ + 2 * n * d /* pts */ + 2 * n /* q */ + n /* tl */ + d * d /* L */ + n * d /* X */ +
         n /* m2 */ + n /* u */ + n * d /* z */ + n /* chisq */ + n /* acc u */ + 8 /* counter */ +
         3 * d /* random-walk std, bounds */;
}

/* device bytes a resident chain holds (its handle's state and scratch, and
 * the step buffers): an estimate from the layouts of the handle's buffers,
 * with 10 % and 4 MiB of slack */
static uint64_t
_chain_bytes (const ncg_chain_desc_t *c, int mixed)
{
  const double n = (double) (c->n / 2), d = c->dim;   /* the fit's kernels */
  const int dp   = ncg_pad_dim ((int) c->dim);
  double b       = 0.0;

  b += 8.0 * n * d * 3.0;                                   /* X, Y, staging  */
  b += 8.0 * n * ncg_pack64_stride (c->kind, dp);           /* pack64         */
  b += 8.0 * n * 8.0;                                       /* per-kernel vectors */
  b += 8.0 * 24.0 * n + 8.0 * n * ceil (n / 256.0);         /* NNLS vectors, gemv scratch */
  b += (double) ncg_pcg_trinv_bytes ((int) n) + (double) ncg_syrk_tc_pack_bytes ((int) n, 64);  /* preconditioner */
  b += 16.0 * 2.0 * n * 16.0;                               /* eval partials (<= 16 slices of 2n) */

  if (c->kind == NCG_VKDE)
  {
    const double lf = (c->local_frac > 0.0) ? c->local_frac : 0.05;
    const double k  = fmax (lf * n, 2.0);

    b += 8.0 * n * d * d;                                   /* U_i            */
    b += 4.0 * n * k;                                       /* kNN            */
    b += (double) ncg_knn_scratch_bytes ((int) (c->n / 2), (int) c->dim, (int) k);
  }

  if (mixed)
  {
    b += (double) ncg_packmx_bytes (c->kind, (int) (c->n / 2), dp);

    if (ncg_tc_supported (c->kind, dp))
      b += (double) ncg_tc_B_bytes ((int) (c->n / 2), dp) + (double) ncg_tc_scratch_bytes ((int64_t) c->n, (int) (c->n / 2), dp);
  }

  b += 8.0 * (double) _dbuf_doubles (c) + 8.0 * 2.0 * n * d;   /* + the walkers' host-side copy staging */

  return (uint64_t) (1.1 * b) + ((uint64_t) 4 << 20);
}

/* every worker's arena fits the largest chain added so far, so a chain can
 * run on any worker and the arenas never need to shrink */
static size_t
_ws_need (const ncg_server_t *s)
{
  return s->ws_size;
}

/* ------------------------------------------------------------- lifecycle */

static void *_worker_main (void *arg);

ncg_status_t
ncg_server_new (const ncg_server_config_t *cfg, ncg_server_t **out)
{
  ncg_server_t *s;

  if (cfg == NULL || out == NULL || cfg->slots < 1 || cfg->slots > 64 ||
      (cfg->precision != NCG_PREC_FP64 && cfg->precision != NCG_PREC_MIXED && cfg->precision != NCG_PREC_MIXED_SIMT))
    return NCG_ERR_INVALID_ARG;

  *out = NULL;

  if (cudaSetDevice (cfg->device) != cudaSuccess)
    return ncg_cuda_status (cudaGetLastError (), "cudaSetDevice");

  s = calloc (1, sizeof (*s));

  if (s == NULL)
    return NCG_ERR_OUT_OF_MEMORY;

  s->cfg = *cfg;
  pthread_mutex_init (&s->mu, NULL);
  pthread_cond_init (&s->cv_work, NULL);
  pthread_cond_init (&s->cv_done, NULL);
  clock_gettime (CLOCK_MONOTONIC, &s->t0);

  s->w = calloc ((size_t) cfg->slots, sizeof (worker_t));

  if (s->w == NULL)
  {
    free (s);

    return NCG_ERR_OUT_OF_MEMORY;
  }

  /* Chain handles and step buffers come from a pool of the server's own, on
   * each chain's stream: loading and evicting a chain then synchronises
   * neither the device nor the other chains' streams (cudaMalloc/cudaFree
   * would).  Freed blocks stay cached up to the budget. */
  {
    struct cudaMemPoolProps pp;
    uint64_t thr = cfg->hbm_budget;

    memset (&pp, 0, sizeof (pp));
    pp.allocType     = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id   = cfg->device;

    if (cudaMemPoolCreate (&s->pool, &pp) != cudaSuccess ||
        cudaMemPoolSetAttribute (s->pool, cudaMemPoolAttrReleaseThreshold, &thr) != cudaSuccess)
    {
      const ncg_status_t r = ncg_cuda_status (cudaGetLastError (), "cudaMemPoolCreate");

      if (s->pool)
        cudaMemPoolDestroy (s->pool);

      free (s->w);
      free (s);

      return r;
    }
  }

  for (int i = 0; i < cfg->slots; i++)
  {
    s->w[i].s   = s;
    s->w[i].idx = i;

    if (pthread_create (&s->w[i].th, NULL, _worker_main, &s->w[i]) != 0)
    {
      pthread_mutex_lock (&s->mu);
      s->stop = 1;
      pthread_cond_broadcast (&s->cv_work);
      pthread_mutex_unlock (&s->mu);

      for (int j = 0; j < i; j++)
        pthread_join (s->w[j].th, NULL);

      cudaMemPoolDestroy (s->pool);
      free (s->w);
      free (s);

      return NCG_ERR_OUT_OF_MEMORY;
    }
  }

  s->started = cfg->slots;
  *out       = s;

  return NCG_OK;
}

/* the host side of a chain (NULL-safe) */
static void
_chain_free_host (chain_t *c)
{
  ncg_rng_free (c->rng);
  cudaFreeHost (c->X);
  cudaFreeHost (c->m2);
  cudaFreeHost (c->hu);
  cudaFreeHost (c->hz);
  cudaFreeHost (c->hch);
  cudaFreeHost (c->hacc);
  cudaFreeHost (c->hprop);
  free (c->L);
  free (c->lb);
  free (c->ub);
  free (c->hmap);
  c->rng  = NULL;
  c->X    = c->m2 = c->hu = c->hz = c->hch = c->hacc = c->hprop = c->L = c->lb = c->ub = NULL;
  c->hmap = NULL;
}

static void
_chain_unload (chain_t *c)
{
  if (c->dbuf)
    cudaFreeAsync (c->dbuf, c->stream);

  if (c->sd)
    ncg_sd_free (c->sd);  /* frees on c->stream and synchronises it */

  if (c->stream)
    cudaStreamDestroy (c->stream);

  c->sd     = NULL;
  c->stream = NULL;
  c->dbuf   = NULL;
}

void
ncg_server_free (ncg_server_t *s)
{
  if (s == NULL)
    return;

  pthread_mutex_lock (&s->mu);
  s->stop = 1;
  pthread_cond_broadcast (&s->cv_work);
  pthread_mutex_unlock (&s->mu);

  for (int i = 0; i < s->started; i++)
    pthread_join (s->w[i].th, NULL);

  cudaSetDevice (s->cfg.device);

  for (int i = 0; i < s->cfg.slots; i++)
    if (s->w[i].ws)
      cudaFree (s->w[i].ws);

  for (int i = 0; i < s->nch; i++)
  {
    chain_t *c = &s->ch[i];

    _chain_unload (c);
    _chain_free_host (c);
  }

  if (s->pool)
    cudaMemPoolDestroy (s->pool);

  pthread_mutex_destroy (&s->mu);
  pthread_cond_destroy (&s->cv_work);
  pthread_cond_destroy (&s->cv_done);
  free (s->ch);
  free (s->rq);
  free (s->stamp);
  free (s->w);
  free (s);
}

/* -2 ln L of the Gaussian target (host, for the initial walkers) */
static double
_target_host (const double *L, const double *x, int d)
{
  double y[NCG_DMAX], s = 0.0;

  for (int r = 0; r < d; r++)
  {
    double v = x[r];

    for (int c = 0; c < r; c++)
      v = fma (-L[r * d + c], y[c], v);

    y[r] = v / L[r * d + r];
    s    = fma (y[r], y[r], s);
  }

  return s;
}

/* a chain from its description; with m2 the walkers' -2 ln L, with rng_state
 * the generator's state and with steps the steps already taken (a restored
 * chain), else computed, seeded and zero */
static ncg_status_t
_add_chain (ncg_server_t *s, const ncg_chain_desc_t *c, const double *m2, const void *rng_state, uint64_t steps,
            int32_t *chain_id)
{
  chain_t ch;
  const size_t n = c ? c->n : 0, d = c ? c->dim : 0;

  if (s == NULL || c == NULL || c->X0 == NULL || c->target_L == NULL || d < 1 || d > NCG_DMAX || n < 4 ||
      (n & 1) || n > (1u << 24) || (c->kind != NCG_KDE && c->kind != NCG_VKDE) ||
      (c->kernel != NCG_KERNEL_GAUSS && c->kernel != NCG_KERNEL_ST) ||
      !(c->random_walk_prob >= 0.0 && c->random_walk_prob < 1.0))
    return NCG_ERR_INVALID_ARG;

  for (size_t r = 0; r < d; r++)
  {
    const double lo = c->lb ? c->lb[r] : -INFINITY, hi = c->ub ? c->ub[r] : INFINITY;

    if (!(lo < hi))
    {
      ncg_set_error ("ncg_server_add_chain: bounds of parameter %zu are empty", r);

      return NCG_ERR_INVALID_ARG;
    }

    for (size_t j = 0; j < n; j++)
      if (c->X0[j * d + r] < lo || c->X0[j * d + r] > hi)
      {
        ncg_set_error ("ncg_server_add_chain: walker %zu is outside the bounds", j);

        return NCG_ERR_INVALID_ARG;
      }
  }

  for (size_t r = 0; r < d; r++)
    if (!(c->target_L[r * d + r] > 0.0))
    {
      ncg_set_error ("ncg_server_add_chain: target factor has a non-positive diagonal");

      return NCG_ERR_INVALID_ARG;
    }

  memset (&ch, 0, sizeof (ch));
  ch.desc = *c;

  if (cudaSetDevice (s->cfg.device) != cudaSuccess ||
      cudaHostAlloc ((void **) &ch.X, sizeof (double) * n * d, cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc ((void **) &ch.m2, sizeof (double) * n, cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc ((void **) &ch.hu, sizeof (double) * n, cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc ((void **) &ch.hz, sizeof (double) * n * d, cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc ((void **) &ch.hch, sizeof (double) * n, cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc ((void **) &ch.hacc, sizeof (double) * n, cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc ((void **) &ch.hprop, sizeof (double) * (n / 2) * d, cudaHostAllocDefault) != cudaSuccess)
  {
    _chain_free_host (&ch);

    return ncg_cuda_status (cudaGetLastError (), "cudaHostAlloc");
  }

  ch.L    = malloc (sizeof (double) * d * d);
  ch.lb   = malloc (sizeof (double) * d);
  ch.ub   = malloc (sizeof (double) * d);
  ch.hmap = malloc (sizeof (int32_t) * n);   /* pending walkers | compacted draws */

  if (ch.L == NULL || ch.lb == NULL || ch.ub == NULL || ch.hmap == NULL || ncg_rng_new (c->seed, &ch.rng) != NCG_OK ||
      (rng_state != NULL && ncg_rng_set_state (ch.rng, rng_state) != NCG_OK))
  {
    _chain_free_host (&ch);

    return NCG_ERR_OUT_OF_MEMORY;
  }

  memcpy (ch.X, c->X0, sizeof (double) * n * d);
  memcpy (ch.L, c->target_L, sizeof (double) * d * d);

  for (size_t r = 0; r < d; r++)
  {
    ch.lb[r]    = c->lb ? c->lb[r] : -INFINITY;
    ch.ub[r]    = c->ub ? c->ub[r] : INFINITY;
    ch.bounded |= isfinite (ch.lb[r]) || isfinite (ch.ub[r]);
  }

  ch.explore_left = c->exploration;

  for (size_t j = 0; j < n; j++)
    ch.m2[j] = m2 ? m2[j] : _target_host (ch.L, ch.X + j * d, (int) d);

  ch.steps = steps;

  ch.desc.X0       = NULL;
  ch.desc.target_L = NULL;
  ch.desc.lb       = NULL;
  ch.desc.ub       = NULL;
  ch.bytes         = _chain_bytes (&ch.desc, s->cfg.precision != NCG_PREC_FP64);

  pthread_mutex_lock (&s->mu);

  if (s->nch == s->capch)
  {
    const int nc    = s->capch ? 2 * s->capch : 64;
    chain_t *nchs   = realloc (s->ch, sizeof (chain_t) * nc);
    uint64_t *nstmp = realloc (s->stamp, sizeof (uint64_t) * nc);

    if (nchs)
      s->ch = nchs;

    if (nstmp)
      s->stamp = nstmp;

    if (nchs == NULL || nstmp == NULL)
    {
      pthread_mutex_unlock (&s->mu);
      _chain_free_host (&ch);

      return NCG_ERR_OUT_OF_MEMORY;
    }

    s->capch = nc;
  }

  s->ch[s->nch]    = ch;
  s->stamp[s->nch] = 0;

  {
    const size_t ws = ncg_sd_workspace_bytes_for (ch.desc.n / 2, s->cfg.precision != NCG_PREC_FP64);

    if (ws > s->ws_size)
      s->ws_size = ws;

    if (ch.desc.n > s->n_max)
      s->n_max = ch.desc.n;
  }

  if (chain_id)
    *chain_id = s->nch;

  s->nch++;
  pthread_mutex_unlock (&s->mu);

  return NCG_OK;
}

ncg_status_t
ncg_server_add_chain (ncg_server_t *s, const ncg_chain_desc_t *c, int32_t *chain_id)
{
  return _add_chain (s, c, NULL, NULL, 0, chain_id);
}

/* ------------------------------------------------------------ checkpoints */

#define CKPT_MAGIC "NCGCKPT1"
#define CKPT_VERSION 2u

typedef struct
{
  FILE *f;
  uint64_t h;   /* FNV-1a of the bytes so far */
  int ok;
} ckio_t;

static void
_fnv (ckio_t *io, const void *p, size_t n)
{
  const unsigned char *b = p;

  for (size_t i = 0; i < n; i++)
  {
    io->h ^= b[i];
    io->h *= 1099511628211ull;
  }
}

static void
_put (ckio_t *io, const void *p, size_t n)
{
  if (io->ok && fwrite (p, 1, n, io->f) != n)
    io->ok = 0;

  _fnv (io, p, n);
}

static void
_get (ckio_t *io, void *p, size_t n)
{
  if (io->ok && fread (p, 1, n, io->f) != n)
    io->ok = 0;

  if (io->ok)
    _fnv (io, p, n);
}

/* the scalar part of a chain description, field by field (the struct's
 * pointers and padding are not written) */
static void
_io_desc (ckio_t *io, ncg_chain_desc_t *c, int writing)
{
#define IOF(f) do { if (writing) _put (io, &c->f, sizeof (c->f)); else _get (io, &c->f, sizeof (c->f)); } while (0)
  IOF (kind);
  IOF (kernel);
  IOF (dim);
  IOF (n);
  IOF (nu);
  IOF (over_smooth);
  IOF (local_frac);
  IOF (seed);
  IOF (random_walk_prob);
  IOF (exploration);
#undef IOF
}

ncg_status_t
ncg_server_checkpoint (ncg_server_t *s, const char *path)
{
  const size_t rs = ncg_rng_state_bytes ();
  char *tmp;
  ckio_t io = { NULL, 14695981039346656037ull, 1 };
  ncg_status_t r = NCG_OK;

  if (s == NULL || path == NULL)
    return NCG_ERR_INVALID_ARG;

  tmp = malloc (strlen (path) + 8);

  if (tmp == NULL)
    return NCG_ERR_OUT_OF_MEMORY;

  sprintf (tmp, "%s.tmp", path);
  pthread_mutex_lock (&s->mu);

  if (s->running > 0)
    r = NCG_ERR_BUSY;

  for (int64_t q = s->first_pending; q < s->nrq; q++)
    if (s->rq[q].state != RQ_DONE)
      r = NCG_ERR_BUSY;

  if (r == NCG_OK && (io.f = fopen (tmp, "wb")) == NULL)
  {
    ncg_set_error ("ncg_server_checkpoint: cannot open %s", tmp);
    r = NCG_ERR_INVALID_ARG;
  }

  if (r == NCG_OK)
  {
    const uint32_t ver = CKPT_VERSION, nch = (uint32_t) s->nch, rsz = (uint32_t) rs;
    unsigned char *st = malloc (rs);

    _put (&io, CKPT_MAGIC, 8);
    _put (&io, &ver, sizeof (ver));
    _put (&io, &nch, sizeof (nch));
    _put (&io, &rsz, sizeof (rsz));

    for (int i = 0; i < s->nch && st != NULL; i++)
    {
      chain_t *c     = &s->ch[i];
      const size_t n = c->desc.n, d = c->desc.dim;

      ncg_chain_desc_t dsc = c->desc;

      dsc.exploration = c->explore_left;
      _io_desc (&io, &dsc, 1);
      _put (&io, &c->steps, sizeof (c->steps));
      _put (&io, c->lb, sizeof (double) * d);
      _put (&io, c->ub, sizeof (double) * d);
      _put (&io, c->X, sizeof (double) * n * d);
      _put (&io, c->m2, sizeof (double) * n);
      _put (&io, c->L, sizeof (double) * d * d);
      ncg_rng_get_state (c->rng, st);
      _put (&io, st, rs);
    }

    {
      const uint64_t h = io.h;

      _put (&io, &h, sizeof (h));
    }

    if (st == NULL)
      io.ok = 0;

    free (st);

    if (fclose (io.f) != 0)
      io.ok = 0;

    if (!io.ok || rename (tmp, path) != 0)
    {
      ncg_set_error ("ncg_server_checkpoint: writing %s failed", path);
      remove (tmp);
      r = NCG_ERR_INVALID_ARG;
    }
  }

  pthread_mutex_unlock (&s->mu);
  free (tmp);

  return r;
}

ncg_status_t
ncg_server_restore (ncg_server_t *s, const char *path, int32_t *first_id, int32_t *count)
{
  const size_t rs = ncg_rng_state_bytes ();
  ckio_t io = { NULL, 14695981039346656037ull, 1 };
  char magic[8];
  uint32_t ver = 0, nch = 0, rsz = 0;
  ncg_chain_desc_t *descs = NULL;
  double **X = NULL, **m2 = NULL, **L = NULL, **lb = NULL, **ub = NULL;
  unsigned char *st = NULL;
  uint64_t *steps = NULL;
  ncg_status_t r = NCG_OK;
  uint32_t got = 0;

  if (s == NULL || path == NULL)
    return NCG_ERR_INVALID_ARG;

  if ((io.f = fopen (path, "rb")) == NULL)
  {
    ncg_set_error ("ncg_server_restore: cannot open %s", path);

    return NCG_ERR_INVALID_ARG;
  }

  _get (&io, magic, 8);
  _get (&io, &ver, sizeof (ver));
  _get (&io, &nch, sizeof (nch));
  _get (&io, &rsz, sizeof (rsz));

  if (!io.ok || memcmp (magic, CKPT_MAGIC, 8) != 0 || ver != CKPT_VERSION || rsz != rs || nch > (1u << 20))
  {
    ncg_set_error ("ncg_server_restore: %s is not a version-%u checkpoint", path, CKPT_VERSION);
    fclose (io.f);

    return NCG_ERR_INVALID_ARG;
  }

  descs = calloc (nch ? nch : 1, sizeof (*descs));
  X     = calloc (nch ? nch : 1, sizeof (*X));
  m2    = calloc (nch ? nch : 1, sizeof (*m2));
  L     = calloc (nch ? nch : 1, sizeof (*L));
  steps = calloc (nch ? nch : 1, sizeof (*steps));
  lb    = calloc (nch ? nch : 1, sizeof (*lb));
  ub    = calloc (nch ? nch : 1, sizeof (*ub));
  st    = malloc (rs * (nch ? nch : 1));

  if (!descs || !X || !m2 || !L || !steps || !st || !lb || !ub)
    r = NCG_ERR_OUT_OF_MEMORY;

  for (; r == NCG_OK && got < nch; got++)
  {
    ncg_chain_desc_t *c = &descs[got];
    size_t n, d;

    _io_desc (&io, c, 0);
    n = c->n;
    d = c->dim;

    if (!io.ok || d < 1 || d > NCG_DMAX || n < 4 || (n & 1) || n > (1u << 24))
    {
      r = NCG_ERR_INVALID_ARG;
      break;
    }

    X[got]  = malloc (sizeof (double) * n * d);
    m2[got] = malloc (sizeof (double) * n);
    L[got]  = malloc (sizeof (double) * d * d);
    lb[got] = malloc (sizeof (double) * d);
    ub[got] = malloc (sizeof (double) * d);

    if (!X[got] || !m2[got] || !L[got] || !lb[got] || !ub[got])
    {
      r = NCG_ERR_OUT_OF_MEMORY;
      got++;
      break;
    }

    _get (&io, &steps[got], sizeof (uint64_t));
    _get (&io, lb[got], sizeof (double) * d);
    _get (&io, ub[got], sizeof (double) * d);
    _get (&io, X[got], sizeof (double) * n * d);
    _get (&io, m2[got], sizeof (double) * n);
    _get (&io, L[got], sizeof (double) * d * d);
    _get (&io, st + rs * got, rs);
  }

  if (r == NCG_OK)
  {
    const uint64_t h = io.h;
    uint64_t want = 0;

    _get (&io, &want, sizeof (want));

    if (!io.ok || want != h)
      r = NCG_ERR_INVALID_ARG;
  }

  fclose (io.f);

  if (r == NCG_ERR_INVALID_ARG)
    ncg_set_error ("ncg_server_restore: %s is truncated or corrupt", path);

  if (r == NCG_OK)
  {
    int32_t id = -1;

    for (uint32_t i = 0; i < nch && r == NCG_OK; i++)
    {
      descs[i].X0       = X[i];
      descs[i].target_L = L[i];
      descs[i].lb       = lb[i];
      descs[i].ub       = ub[i];
      r = _add_chain (s, &descs[i], m2[i], st + rs * i, steps[i], &id);

      if (r == NCG_OK && i == 0 && first_id)
        *first_id = id;
    }

    if (count)
      *count = (r == NCG_OK) ? (int32_t) nch : 0;
  }

  for (uint32_t i = 0; i < got && X && lb && ub; i++)
  {
    free (X[i]);
    free (m2[i]);
    free (L[i]);
    free (lb[i]);
    free (ub[i]);
  }

  free (descs);
  free (X);
  free (m2);
  free (L);
  free (steps);
  free (st);
  free (lb);
  free (ub);

  return r;
}

ncg_status_t
ncg_server_submit (ncg_server_t *s, int32_t chain_id, int64_t *request_id)
{
  if (s == NULL)
    return NCG_ERR_INVALID_ARG;

  pthread_mutex_lock (&s->mu);

  if (chain_id < 0 || chain_id >= s->nch || s->stop)
  {
    pthread_mutex_unlock (&s->mu);

    return NCG_ERR_INVALID_ARG;
  }

  if (s->nrq == s->caprq)
  {
    const int64_t nc = s->caprq ? 2 * s->caprq : 1024;
    req_t *nr        = realloc (s->rq, sizeof (req_t) * (size_t) nc);

    if (nr == NULL)
    {
      pthread_mutex_unlock (&s->mu);

      return NCG_ERR_OUT_OF_MEMORY;
    }

    s->rq    = nr;
    s->caprq = nc;
  }

  {
    req_t *r = &s->rq[s->nrq];

    memset (r, 0, sizeof (*r));
    r->chain        = chain_id;
    r->state        = RQ_PENDING;
    r->res.request  = s->nrq;
    r->res.chain    = chain_id;
    r->res.t_arrive = _now (s);
  }

  if (request_id)
    *request_id = s->nrq;

  s->nrq++;
  s->ch[chain_id].npending++;
  pthread_cond_broadcast (&s->cv_work);
  pthread_mutex_unlock (&s->mu);

  return NCG_OK;
}

ncg_status_t
ncg_server_wait (ncg_server_t *s, int64_t request_id, ncg_step_result_t *res)
{
  if (s == NULL)
    return NCG_ERR_INVALID_ARG;

  pthread_mutex_lock (&s->mu);

  if (request_id < 0 || request_id >= s->nrq)
  {
    pthread_mutex_unlock (&s->mu);

    return NCG_ERR_INVALID_ARG;
  }

  while (s->rq[request_id].state != RQ_DONE && !s->stop)
    pthread_cond_wait (&s->cv_done, &s->mu);

  if (s->rq[request_id].state != RQ_DONE)
  {
    pthread_mutex_unlock (&s->mu);

    return NCG_ERR_BUSY;
  }

  if (res)
    *res = s->rq[request_id].res;

  {
    const ncg_status_t st = (ncg_status_t) s->rq[request_id].res.status;

    pthread_mutex_unlock (&s->mu);

    return st;
  }
}

ncg_status_t
ncg_server_drain (ncg_server_t *s)
{
  if (s == NULL)
    return NCG_ERR_INVALID_ARG;

  pthread_mutex_lock (&s->mu);

  while (s->completed + s->failed < (uint64_t) s->nrq && !s->stop)
    pthread_cond_wait (&s->cv_done, &s->mu);

  pthread_mutex_unlock (&s->mu);

  return NCG_OK;
}

static int
_dcmp (const void *a, const void *b)
{
  const double x = *(const double *) a, y = *(const double *) b;

  return (x < y) ? -1 : (x > y);
}

ncg_status_t
ncg_server_get_stats (ncg_server_t *s, ncg_server_stats_t *st)
{
  if (s == NULL || st == NULL)
    return NCG_ERR_INVALID_ARG;

  memset (st, 0, sizeof (*st));
  pthread_mutex_lock (&s->mu);

  st->submitted           = (uint64_t) s->nrq;
  st->completed           = s->completed;
  st->failed              = s->failed;
  st->admitted            = s->admitted;
  st->evicted             = s->evicted;
  st->reserved_bytes      = s->reserved;
  st->peak_reserved_bytes = s->peak;

  {
    double *lat   = malloc (sizeof (double) * (size_t) (s->nrq > 0 ? s->nrq : 1));
    int64_t k     = 0;
    double first  = INFINITY, last = 0.0, sum = 0.0;

    if (lat == NULL)
    {
      pthread_mutex_unlock (&s->mu);

      return NCG_ERR_OUT_OF_MEMORY;
    }

    for (int64_t i = 0; i < s->nrq; i++)
    {
      const ncg_step_result_t *r = &s->rq[i].res;

      if (s->rq[i].state != RQ_DONE || r->status != NCG_OK)
        continue;

      lat[k] = 1e3 * (r->t_done - r->t_arrive);
      sum   += lat[k];
      first  = fmin (first, r->t_arrive);
      last   = fmax (last, r->t_done);
      st->pairs += (double) r->pairs;
      k++;
    }

    if (k > 0)
    {
      qsort (lat, (size_t) k, sizeof (double), _dcmp);
      st->p50_ms  = lat[(int64_t) ceil (0.50 * k) - 1];
      st->p99_ms  = lat[(int64_t) ceil (0.99 * k) - 1];
      st->mean_ms = sum / k;
      st->max_ms  = lat[k - 1];
      st->span_s  = last - first;
    }

    free (lat);
  }

  pthread_mutex_unlock (&s->mu);

  return NCG_OK;
}

ncg_status_t
ncg_server_get_chain (ncg_server_t *s, int32_t chain_id, double *X, double *m2lnL)
{
  if (s == NULL)
    return NCG_ERR_INVALID_ARG;

  pthread_mutex_lock (&s->mu);

  if (chain_id < 0 || chain_id >= s->nch || s->ch[chain_id].running)
  {
    pthread_mutex_unlock (&s->mu);

    return (chain_id < 0 || chain_id >= s->nch) ? NCG_ERR_INVALID_ARG : NCG_ERR_BUSY;
  }

  {
    const chain_t *c = &s->ch[chain_id];

    if (X)
      memcpy (X, c->X, sizeof (double) * c->desc.n * c->desc.dim);

    if (m2lnL)
      memcpy (m2lnL, c->m2, sizeof (double) * c->desc.n);
  }

  pthread_mutex_unlock (&s->mu);

  return NCG_OK;
}

ncg_status_t
ncg_server_get_chain_info (ncg_server_t *s, int32_t chain_id, ncg_chain_desc_t *desc, uint64_t *steps)
{
  if (s == NULL)
    return NCG_ERR_INVALID_ARG;

  pthread_mutex_lock (&s->mu);

  if (chain_id < 0 || chain_id >= s->nch)
  {
    pthread_mutex_unlock (&s->mu);

    return NCG_ERR_INVALID_ARG;
  }

  if (desc)
    *desc = s->ch[chain_id].desc;

  if (steps)
    *steps = s->ch[chain_id].steps;

  pthread_mutex_unlock (&s->mu);

  return NCG_OK;
}

/* -------------------------------------------------------------- the step */

#define SK(call)                          \
  do {                                    \
    ncg_status_t _s = (call);             \
    if (_s != NCG_OK)                     \
      return _s;                          \
  } while (0)

#define SC(call, where) SK (ncg_cuda_status ((call), (where)))

static ncg_status_t
_chain_load (ncg_server_t *s, chain_t *c)
{
  const ncg_chain_desc_t *dsc = &c->desc;
  ncg_sd_config_t cfg;

  ncg_sd_config_init (&cfg);
  cfg.device    = s->cfg.device;
  cfg.precision = (ncg_precision_t) s->cfg.precision;

  if (dsc->over_smooth > 0.0)
    cfg.over_smooth = dsc->over_smooth;

  if (dsc->local_frac > 0.0)
    cfg.local_frac = dsc->local_frac;

  cfg.async_alloc = 1;
  SK (ncg_sd_new ((ncg_kind_t) dsc->kind, (ncg_kernel_t) dsc->kernel, dsc->dim, dsc->nu, &cfg, &c->sd));
  c->sd->pool = s->pool;

  /* Stream priority by step size: the chains of more than half the largest
   * size (the tail of the latency distribution) run on high-priority streams,
   * so the block scheduler starts their pending CTAs before those of small
   * chains.  It reorders nothing inside a step, so results do not depend on
   * it. */
  {
    int lo = 0, hi = 0;

    SC (cudaDeviceGetStreamPriorityRange (&lo, &hi), "stream priorities");
    SC (cudaStreamCreateWithPriority (&c->stream, cudaStreamNonBlocking,
                                      (dsc->n * 2 > s->n_max) ? hi : lo), "stream");
    SK (ncg_sd_set_stream (c->sd, c->stream));
  }
  SC (cudaMallocFromPoolAsync (&c->dbuf, sizeof (double) * _dbuf_doubles (dsc), s->pool, c->stream),
      "cudaMallocFromPoolAsync");
  SC (cudaMemcpyAsync ((double *) c->dbuf + 3 * (dsc->n / 2) * dsc->dim + 3 * (dsc->n / 2), c->L,
                       sizeof (double) * dsc->dim * dsc->dim, cudaMemcpyHostToDevice, c->sd->stream), "H2D L");

  return NCG_OK;
}

/* Proposals of a step with bounds or the random-walk mixture, into c->hprop
 * (_ncm_fit_esmcmc_walker_apes_sample, ncm_fit_esmcmc_walker_apes.c:717-737):
 * walker by walker, in order, each attempt draws the mixture component (a
 * uniform, when the random walk is on), then either a random-walk proposal
 * coordinate by coordinate from the truncated Gaussian (:695-715, on the host)
 * or a draw of the fit (sampled on the device); a fit draw outside the bounds
 * is attempted again before the next walker draws, so the chain consumes its
 * stream in the reference's order.  The device samples a window of walkers'
 * first attempts at once; at the first walker whose fit draw falls outside,
 * the generator is rewound to the window's start and the window's draws are
 * replayed up to that attempt, and the next window starts with that walker's
 * next attempt.  A step without rejections takes one window.  With std the
 * random walk's scales, 0.25 sqrt(cov_ii) of the fit (:646-693). */
#define NCG_PROPOSAL_ROUNDS 200000
#define NCG_PROPOSAL_WINDOW_MIN 64

/* one attempt of walker j: a random-walk proposal into hprop (returns 1), or
 * the fit draw's stream into (u, z, ch) (returns 0) */
static ncg_status_t
_attempt (chain_t *c, uint64_t d, const double *Xh, const double *std, int32_t j, double *u, double *z, double *ch,
          int *rw)
{
  const ncg_chain_desc_t *dsc = &c->desc;

  *rw = 0;

  if (dsc->random_walk_prob > 0.0 && ncg_rng_uniform_pos (c->rng) < dsc->random_walk_prob)
  {
    for (uint64_t i = 0; i < d; i++)
    {
      double x;
      int tries = 0;

      do {
        if (++tries > (1 << 20))
        {
          ncg_set_error ("random walk: no draw inside the bounds of parameter %llu", (unsigned long long) i);

          return NCG_ERR_TIMEOUT;
        }

        x = ncg_rng_ugaussian (c->rng) * std[i] + Xh[(uint64_t) j * d + i];
      } while (x < c->lb[i] || x > c->ub[i]);

      c->hprop[(uint64_t) j * d + i] = x;
    }

    *rw = 1;

    return NCG_OK;
  }

  return ncg_rng_sample_stream (c->rng, (ncg_kernel_t) dsc->kernel, (uint32_t) d, dsc->nu, 1, u, z, ch);
}

static ncg_status_t
_proposals (chain_t *c, ncg_sd_t *sd, cudaStream_t st, uint64_t n, uint64_t d, const double *Xh, double *du,
            double *dz, double *dch, double *dtmp, double *std)
{
  const ncg_chain_desc_t *dsc = &c->desc;
  const double p   = dsc->random_walk_prob;
  const int stk    = dsc->kernel == NCG_KERNEL_ST;
  int32_t *map     = c->hmap + n;
  uint64_t w0 = 0, win = n;
  unsigned char state[4096];
  double scratch[NCG_DMAX + 2];
  ncg_status_t r;

  if (ncg_rng_state_bytes () > sizeof (state))
    return NCG_ERR_INVALID_ARG;

  if (p > 0.0)
  {
    double cov[NCG_DMAX * NCG_DMAX];

    SK (ncg_sd_get_full_cov (sd, cov));

    for (uint64_t i = 0; i < d; i++)
    {
      if (!(cov[i * d + i] > 0.0))
      {
        ncg_set_error ("random walk: diagonal element %llu of the fit's covariance is not positive",
                       (unsigned long long) i);

        return NCG_ERR_NOT_PD;
      }

      std[i] = sqrt (cov[i * d + i]) * 0.25;
    }
  }

  for (int round = 0; w0 < n; round++)
  {
    const uint64_t w1 = (w0 + win < n) ? w0 + win : n;
    uint64_t kc = 0;
    int rw;

    if (round == NCG_PROPOSAL_ROUNDS)
    {
      ncg_set_error ("no proposal inside the bounds after %d rounds", NCG_PROPOSAL_ROUNDS);

      return NCG_ERR_TIMEOUT;
    }

    SK (ncg_rng_get_state (c->rng, state));

    for (uint64_t j = w0; j < w1; j++)
    {
      if ((r = _attempt (c, d, Xh, std, (int32_t) j, c->hu + kc, c->hz + kc * d, stk ? c->hch + kc : NULL, &rw)) !=
          NCG_OK)
        return r;

      if (!rw)
        map[kc++] = (int32_t) j;
    }

    if (kc == 0)
    {
      w0  = w1;
      win = 2 * win;
      continue;
    }

    SC (cudaMemcpyAsync (du, c->hu, sizeof (double) * kc, cudaMemcpyHostToDevice, st), "H2D u");
    SC (cudaMemcpyAsync (dz, c->hz, sizeof (double) * kc * d, cudaMemcpyHostToDevice, st), "H2D z");

    if (stk)
      SC (cudaMemcpyAsync (dch, c->hch, sizeof (double) * kc, cudaMemcpyHostToDevice, st), "H2D chisq");

    SK (ncg_sd_sample_batch_device (sd, du, dz, stk ? dch : NULL, kc, dtmp, NULL));
    SC (cudaMemcpyAsync (c->hz, dtmp, sizeof (double) * kc * d, cudaMemcpyDeviceToHost, st), "D2H draws");
    SC (cudaStreamSynchronize (st), "sync");

    {
      uint64_t a;

      for (a = 0; a < kc; a++)
      {
        const double *x = c->hz + a * d;
        int in          = 1;

        for (uint64_t i = 0; i < d; i++)
          in &= (x[i] >= c->lb[i]) & (x[i] <= c->ub[i]);

        if (!in)
          break;

        memcpy (c->hprop + (uint64_t) map[a] * d, x, sizeof (double) * d);
      }

      if (a == kc)
      {
        /* every attempt of the window landed: the next window doubles */
        w0  = w1;
        win = 2 * win;
        continue;
      }

      /* walker f's fit draw fell outside: rewind to the window's start and
       * replay the draws up to and including f's attempt (the walkers before
       * f keep the proposals they have); f attempts again next */
      {
        const int32_t f = map[a];

        SK (ncg_rng_set_state (c->rng, state));

        for (uint64_t j = w0; j <= (uint64_t) f; j++)
          if ((r = _attempt (c, d, Xh, std, (int32_t) j, scratch, scratch + 1, stk ? scratch + 1 + d : NULL, &rw)) !=
              NCG_OK)
            return r;

        win = 4 * ((uint64_t) f - w0 + 1);
        win = (win < NCG_PROPOSAL_WINDOW_MIN) ? NCG_PROPOSAL_WINDOW_MIN : win;
        w0  = (uint64_t) f;
      }
    }
  }

  return NCG_OK;
}

/* One APES half-move (ncm_fit_esmcmc_walker_apes.c:739-919): the walkers are
 * two halves of N = n/2; step k moves half h = k mod 2 with proposals from the
 * fit of the other half o (prepare_interp on its walkers and their -2 ln L),
 * the fit evaluated at the proposals and at half h's walkers (m2lnp_star,
 * m2lnp_cur, apes.c:872-873), the target at the proposals, and the test
 * exp(-((m2lnL* - m2lnp*) - (m2lnL - m2lnp))/2) (apes.c:897-902), with the
 * random-walk mixture, bounds and exploration phase when the chain has them. */
static ncg_status_t
_run_step (ncg_server_t *s, worker_t *w, chain_t *c, ncg_step_result_t *res)
{
  const ncg_chain_desc_t *dsc = &c->desc;
  const uint64_t nw = dsc->n, n = nw / 2, d = dsc->dim;
  const uint64_t h = c->steps & 1, o = 1 - h;
  double *Xh       = c->X + h * n * d, *m2h = c->m2 + h * n;
  ncg_sd_t *sd     = c->sd;
  cudaStream_t st  = sd->stream;
  double *b        = (double *) c->dbuf;
  double *dprop    = b;
  double *dpts     = dprop + n * d;
  double *dq       = dpts + 2 * n * d;
  double *dtl      = dq + 2 * n;
  double *dL       = dtl + n;
  double *dX       = dL + d * d;
  double *dm2      = dX + n * d;
  double *du       = dm2 + n;
  double *dz       = du + n;
  double *dch      = dz + n * d;
  double *dacc     = dch + n;
  unsigned long long *dcount = (unsigned long long *) (dacc + n);
  double *drw      = dacc + n + 8;   /* std | lb | ub */
  unsigned long long hcount  = 0;
  const int mix     = dsc->random_walk_prob > 0.0;
  const int explore = c->explore_left > 0;
  double std[NCG_DMAX];

  (void) s;

  SK (ncg_sd_set_workspace (sd, w->ws, w->ws_bytes));

  /* fit the other half */
  SK (ncg_sd_reset (sd));
  SK (ncg_sd_add_obs_batch (sd, c->X + o * n * d, n));
  SK (ncg_sd_prepare_interp (sd, c->m2 + o * n));

  if (!mix && !c->bounded)
  {
    /* the chain's draws, in a fixed order: the sample stream, then one
     * uniform per moving walker for the accept test */
    SK (ncg_rng_sample_stream (c->rng, (ncg_kernel_t) dsc->kernel, (uint32_t) d, dsc->nu, n, c->hu, c->hz,
                               dsc->kernel == NCG_KERNEL_ST ? c->hch : NULL));

    for (uint64_t j = 0; j < n; j++)
      c->hacc[j] = ncg_rng_uniform_pos (c->rng);

    SC (cudaMemcpyAsync (du, c->hu, sizeof (double) * n, cudaMemcpyHostToDevice, st), "H2D u");
    SC (cudaMemcpyAsync (dz, c->hz, sizeof (double) * n * d, cudaMemcpyHostToDevice, st), "H2D z");

    if (dsc->kernel == NCG_KERNEL_ST)
      SC (cudaMemcpyAsync (dch, c->hch, sizeof (double) * n, cudaMemcpyHostToDevice, st), "H2D chisq");

    SC (cudaMemcpyAsync (dacc, c->hacc, sizeof (double) * n, cudaMemcpyHostToDevice, st), "H2D u accept");
    SC (cudaMemcpyAsync (dX, Xh, sizeof (double) * n * d, cudaMemcpyHostToDevice, st), "H2D walkers");
    SC (cudaMemcpyAsync (dm2, m2h, sizeof (double) * n, cudaMemcpyHostToDevice, st), "H2D m2lnL");

    /* proposals from the fit */
    SK (ncg_sd_sample_batch_device (sd, du, dz, dsc->kernel == NCG_KERNEL_ST ? dch : NULL, n, dprop, NULL));
  }
  else
  {
    /* proposals in rounds (the pair-point buffer is their scratch), then the
     * accept uniforms */
    SK (_proposals (c, sd, st, n, d, Xh, du, dz, dch, dpts, std));

    for (uint64_t j = 0; j < n; j++)
      c->hacc[j] = ncg_rng_uniform_pos (c->rng);

    SC (cudaMemcpyAsync (dacc, c->hacc, sizeof (double) * n, cudaMemcpyHostToDevice, st), "H2D u accept");
    SC (cudaMemcpyAsync (dX, Xh, sizeof (double) * n * d, cudaMemcpyHostToDevice, st), "H2D walkers");
    SC (cudaMemcpyAsync (dm2, m2h, sizeof (double) * n, cudaMemcpyHostToDevice, st), "H2D m2lnL");
    SC (cudaMemcpyAsync (dprop, c->hprop, sizeof (double) * n * d, cudaMemcpyHostToDevice, st), "H2D proposals");

    if (mix)
    {
      SC (cudaMemcpyAsync (drw, std, sizeof (double) * d, cudaMemcpyHostToDevice, st), "H2D std");
      SC (cudaMemcpyAsync (drw + d, c->lb, sizeof (double) * d, cudaMemcpyHostToDevice, st), "H2D lb");
      SC (cudaMemcpyAsync (drw + 2 * d, c->ub, sizeof (double) * d, cudaMemcpyHostToDevice, st), "H2D ub");
    }
  }

  SC (cudaMemcpyAsync (dpts, dprop, sizeof (double) * n * d, cudaMemcpyDeviceToDevice, st), "D2D proposals");
  SC (cudaMemcpyAsync (dpts + n * d, dX, sizeof (double) * n * d, cudaMemcpyDeviceToDevice, st), "D2D walkers");
  SK (ncg_sd_eval_m2lnp_device (sd, dpts, 2 * n, dq));
  SC (ncg_launch_serve_target (dprop, (int64_t) n, (int) d, dL, dtl, st), "target");

  if (mix)
    SC (ncg_launch_serve_mix (dq, dX, dprop, drw, (int64_t) n, (int) d, dsc->random_walk_prob, st), "mixture");

  SC (ncg_launch_serve_accept (dX, dm2, dprop, dtl, dq, dacc, (int64_t) n, (int) d, explore, dcount, st), "accept");

  SC (cudaMemcpyAsync (Xh, dX, sizeof (double) * n * d, cudaMemcpyDeviceToHost, st), "D2H walkers");
  SC (cudaMemcpyAsync (m2h, dm2, sizeof (double) * n, cudaMemcpyDeviceToHost, st), "D2H m2lnL");
  SC (cudaMemcpyAsync (&hcount, dcount, sizeof (hcount), cudaMemcpyDeviceToHost, st), "D2H count");
  SC (cudaStreamSynchronize (st), "sync");

  {
    double m = 0.0, x = 0.0;

    for (uint64_t j = 0; j < nw; j++)
      m += c->m2[j];

    for (uint64_t j = 0; j < nw * d; j++)
      x += c->X[j];

    res->accepted   = hcount;
    res->mean_m2lnL = m / (double) nw;
    res->state_sum  = x;
    res->pairs      = 3 * n * n;
  }

  return NCG_OK;
}

/* ------------------------------------------------------------- scheduler */

typedef struct
{
  int64_t req;
  int victims[64];
  int nvictims;
  size_t ws_grow;
  int load;
} pick_t;

/* under the lock: the next request this worker can run, with the chains to
 * evict and the workspace growth it needs; or a request that can never fit
 * (failed here) */
static int
_pick (ncg_server_t *s, worker_t *w, pick_t *pk)
{
  const uint64_t budget = s->cfg.hbm_budget;

  s->scan++;
  memset (pk, 0, sizeof (*pk));
  pk->req = -1;

  while (s->first_pending < s->nrq && s->rq[s->first_pending].state != RQ_PENDING)
    s->first_pending++;

  for (int64_t r = s->first_pending; r < s->nrq; r++)
  {
    if (s->rq[r].state != RQ_PENDING)
      continue;

    const int ci = s->rq[r].chain;
    chain_t *c   = &s->ch[ci];

    if (s->stamp[ci] == s->scan)
      continue;   /* not the chain's oldest request */

    s->stamp[ci] = s->scan;

    if (c->running || c->state == CH_LOADING || c->state == CH_EVICTING)
      continue;

    {
      const size_t need_ws = _ws_need (s);
      const size_t grow    = (need_ws > w->ws_bytes) ? need_ws - w->ws_bytes : 0;
      const uint64_t need  = grow + ((c->state == CH_RESIDENT) ? 0 : c->bytes);

      if (s->reserved + need <= budget)
      {
        pk->req     = r;
        pk->ws_grow = grow;
        pk->load    = (c->state != CH_RESIDENT);

        return 1;
      }

      /* evict idle resident chains, least recently used first */
      {
        uint64_t freed = 0, evictable = 0;
        int nv = 0;

        for (int i = 0; i < s->nch; i++)
        {
          const chain_t *v = &s->ch[i];

          if (v->state == CH_RESIDENT && !v->running && v->npending == 0)
            evictable += v->bytes;
        }

        if (s->reserved - evictable + need <= budget)
        {
          while (s->reserved - freed + need > budget && nv < 64)
          {
            int best = -1;

            for (int i = 0; i < s->nch; i++)
            {
              const chain_t *v = &s->ch[i];
              int taken        = 0;

              for (int k = 0; k < nv; k++)
                taken |= (pk->victims[k] == i);

              if (!taken && v->state == CH_RESIDENT && !v->running && v->npending == 0 &&
                  (best < 0 || v->last_used < s->ch[best].last_used))
                best = i;
            }

            if (best < 0)
              break;

            pk->victims[nv++] = best;
            freed            += s->ch[best].bytes;
          }

          if (s->reserved - freed + need <= budget)
          {
            pk->req      = r;
            pk->ws_grow  = grow;
            pk->load     = (c->state != CH_RESIDENT);
            pk->nvictims = nv;

            return 1;
          }
        }
        else if (s->running == 0)
        {
          /* nothing runs and evicting every idle chain does not make room:
           * the request can never run */
          s->rq[r].state      = RQ_DONE;
          s->rq[r].res.status = NCG_ERR_OUT_OF_MEMORY;
          s->rq[r].res.t_done = _now (s);
          snprintf (s->rq[r].res.detail, sizeof (s->rq[r].res.detail),
                    "chain needs %llu bytes + a %zu-byte workspace, budget %llu, %llu reserved",
                    (unsigned long long) c->bytes, need_ws, (unsigned long long) budget,
                    (unsigned long long) s->reserved);
          c->npending--;
          s->failed++;
          pthread_cond_broadcast (&s->cv_done);

          return 2;
        }
      }
    }
  }

  return 0;
}

static void *
_worker_main (void *arg)
{
  worker_t *w     = arg;
  ncg_server_t *s = w->s;

  cudaSetDevice (s->cfg.device);
  pthread_mutex_lock (&s->mu);

  for (;;)
  {
    pick_t pk;
    int got;

    if (s->stop)
      break;

    got = _pick (s, w, &pk);

    if (got == 2)
      continue;

    if (got == 0)
    {
      pthread_cond_wait (&s->cv_work, &s->mu);
      continue;
    }

    /* claim under the lock */
    req_t *rq     = &s->rq[pk.req];
    const int ci  = rq->chain;
    chain_t *c    = &s->ch[ci];

    rq->state        = RQ_RUNNING;
    rq->res.t_start  = _now (s);
    rq->res.step     = c->steps;
    c->running       = 1;
    c->npending--;
    s->running++;

    for (int k = 0; k < pk.nvictims; k++)
    {
      s->ch[pk.victims[k]].state = CH_EVICTING;
      s->reserved               -= s->ch[pk.victims[k]].bytes;
    }

    if (pk.load)
    {
      c->state     = CH_LOADING;
      s->reserved += c->bytes;
      s->admitted++;
    }

    s->reserved += pk.ws_grow;

    if (s->reserved > s->peak)
      s->peak = s->reserved;

    pthread_mutex_unlock (&s->mu);

    /* device work outside the lock */
    ncg_status_t st = NCG_OK;

    for (int k = 0; k < pk.nvictims; k++)
      _chain_unload (&s->ch[pk.victims[k]]);

    size_t ws_lost = 0;   /* arena bytes reserved but not held after a failed allocation */

    if (pk.ws_grow > 0)
    {
      const size_t nb = w->ws_bytes + pk.ws_grow;

      if (w->ws)
        cudaFree (w->ws);

      w->ws       = NULL;
      w->ws_bytes = 0;

      if (cudaMalloc (&w->ws, nb) == cudaSuccess)
      {
        w->ws_bytes = nb;
      }
      else
      {
        cudaGetLastError ();
        w->ws   = NULL;
        ws_lost = nb;
        st      = NCG_ERR_OUT_OF_MEMORY;
        ncg_set_error ("serving: workspace of %zu bytes could not be allocated", nb);
      }
    }

    if (st == NCG_OK && pk.load && (st = _chain_load (s, c)) != NCG_OK)
      _chain_unload (c);

    if (st == NCG_OK)
      st = _run_step (s, w, c, &rq->res);

    pthread_mutex_lock (&s->mu);
    rq = &s->rq[pk.req];   /* the request array may have moved */

    for (int k = 0; k < pk.nvictims; k++)
    {
      s->ch[pk.victims[k]].state = CH_WAITING;
      s->evicted++;
    }

    s->reserved -= ws_lost;

    if (pk.load)
      c->state = (c->sd != NULL && c->dbuf != NULL) ? CH_RESIDENT : CH_WAITING;

    if (pk.load && c->state == CH_WAITING)
      s->reserved -= c->bytes;

    rq->res.status = st;
    rq->res.t_done = _now (s);

    if (st != NCG_OK)
    {
      strncpy (rq->res.detail, ncg_last_error (), sizeof (rq->res.detail) - 1);
      rq->res.detail[sizeof (rq->res.detail) - 1] = '\0';
    }
    rq->state      = RQ_DONE;
    c->running     = 0;
    c->last_used   = ++s->tick;
    s->running--;

    if (st == NCG_OK)
    {
      c->steps++;
      s->completed++;

      if (c->explore_left > 0)
        c->explore_left--;
    }
    else
    {
      s->failed++;
    }

    pthread_cond_broadcast (&s->cv_done);
    pthread_cond_broadcast (&s->cv_work);
  }

  pthread_mutex_unlock (&s->mu);

  return NULL;
}
