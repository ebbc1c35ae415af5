/*
 * ncg_batch.c -- host side of the multi-problem eval (ncg_batch_*): the plan
 * (per-problem slicing, work list, partial-sum layout), its capture into a
 * CUDA graph, and the autotuner that picks the plan's parameters by timing
 * them on the device.
 *
 * The reference has no such object: APES evaluates one NcmStatsDist at a
 * time (numcosmo/ncm/fit/ncm_fit_esmcmc_walker_apes.c:828-873).  A batch
 * holds borrowed, prepared ncg_sd_t handles and the point count each is
 * evaluated at; every launch reads the handles' current device state.
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <cuda_runtime_api.h>

#include "ncg_internal.h"
#include "ncg_host.h"

#define CK(call, where)                                   \
  do {                                                    \
    ncg_status_t _s = ncg_cuda_status ((call), (where));  \
    if (_s != NCG_OK)                                     \
      return _s;                                          \
  } while (0)

enum { BP_FP64 = 0, BP_MIXED = 1 };

/* Longest kernel slice of a mixed tile: a slice's lambda is an FP32 sum, so
 * its rounding grows with the slice length; the slices are combined in FP64.
 * 1024 keeps the sum's relative rounding near 1e-6 worst case. */
#define NCG_BATCH_MIXED_KMAX 1024

typedef struct ncg_bplan
{
  int valid;                   /* built for the current problem list and generations */
  ncg_batch_params_t prm;
  int tuned;
  int nlaunch;                 /* 1, or 2 for the split schedule */
  int set[2], grid[2], nitems[2];
  ncg_bprob_t *hp;
  ncg_bprob_t *dp;
  size_t cap_dp;
  int32_t *hitems, *ditems;    /* both launches' items, launch 1 after launch 0 */
  size_t cap_items;
  void *dpart;
  size_t cap_part;
  int32_t *dcnt;
  size_t cap_cnt;
  int32_t *dcounter;           /* one per launch */
  cudaGraphExec_t ge;
  const double *gX;
  double *gout;
  int n_fp64_tiles;            /* problems served by FP64 tiles in this plan */
  int32_t *tcp;                /* problems on the tensor-core kernel */
  int ntcp, cap_tcp;
  int32_t *brp;                /* branch schedule (tc = 2): every problem, largest first */
  int8_t *brk;                 /* its launch: 0 FP64 tiles, 1 FP32 SIMT tiles, 2 tensor cores */
  int nbrp, cap_brp;
  int64_t pairs;
  int64_t captures, launches;
} ncg_bplan_t;

/* streams the tensor-core launches of a plan are spread over */
#define NCG_BATCH_TC_STREAMS 4
/* streams the branch schedule's launches are spread over */
#define NCG_BATCH_BR_STREAMS 16

struct ncg_batch
{
  int device, nsm;
  cudaStream_t s1, s2, stc[NCG_BATCH_TC_STREAMS], sbr[NCG_BATCH_BR_STREAMS];
  cudaEvent_t ev_in, ev_fork, ev_join, ev_out, t0, t1, ev_tc[NCG_BATCH_TC_STREAMS], ev_br[NCG_BATCH_BR_STREAMS];
  int n, cap;
  ncg_sd_t **sd;
  uint64_t *m, *gen;
  int64_t *x_off, *out_off;
  int64_t x_total, out_total;
  ncg_bplan_t plan[2];
  double *dX, *dout;
  size_t cap_dX, cap_dout;
};

static void
_plan_release (ncg_bplan_t *p)
{
  if (p->ge)
    cudaGraphExecDestroy (p->ge);

  p->ge   = NULL;
  p->gX   = NULL;
  p->gout = NULL;
}

static void
_plan_free (ncg_bplan_t *p)
{
  _plan_release (p);
  free (p->hp);
  free (p->hitems);
  free (p->tcp);
  free (p->brp);
  free (p->brk);

  if (p->dp)
    cudaFree (p->dp);

  if (p->ditems)
    cudaFree (p->ditems);

  if (p->dpart)
    cudaFree (p->dpart);

  if (p->dcnt)
    cudaFree (p->dcnt);

  if (p->dcounter)
    cudaFree (p->dcounter);

  memset (p, 0, sizeof (*p));
}

ncg_status_t
ncg_batch_params_init (ncg_batch_params_t *p)
{
  if (p == NULL)
    return NCG_ERR_INVALID_ARG;

  p->items_per_cta = 8.0;
  p->ctas_per_sm   = 0;
  p->order         = 1;
  p->split         = 0;
  p->tc            = 1;

  return NCG_OK;
}

ncg_status_t
ncg_batch_new (int device, ncg_batch_t **out)
{
  ncg_batch_t *b;

  if (out == NULL)
    return NCG_ERR_INVALID_ARG;

  *out = NULL;
  CK (cudaSetDevice (device), "cudaSetDevice");

  b = calloc (1, sizeof (*b));

  if (b == NULL)
    return NCG_ERR_OUT_OF_MEMORY;

  b->device = device;
  CK (cudaDeviceGetAttribute (&b->nsm, cudaDevAttrMultiProcessorCount, device), "SM count");
  CK (cudaStreamCreateWithFlags (&b->s1, cudaStreamNonBlocking), "stream");
  CK (cudaStreamCreateWithFlags (&b->s2, cudaStreamNonBlocking), "stream");
  CK (cudaEventCreateWithFlags (&b->ev_in, cudaEventDisableTiming), "event");
  CK (cudaEventCreateWithFlags (&b->ev_fork, cudaEventDisableTiming), "event");
  CK (cudaEventCreateWithFlags (&b->ev_join, cudaEventDisableTiming), "event");
  CK (cudaEventCreateWithFlags (&b->ev_out, cudaEventDisableTiming), "event");
  CK (cudaEventCreate (&b->t0), "event");
  CK (cudaEventCreate (&b->t1), "event");

  for (int k = 0; k < NCG_BATCH_TC_STREAMS; k++)
  {
    CK (cudaStreamCreateWithFlags (&b->stc[k], cudaStreamNonBlocking), "stream");
    CK (cudaEventCreateWithFlags (&b->ev_tc[k], cudaEventDisableTiming), "event");
  }

  for (int k = 0; k < NCG_BATCH_BR_STREAMS; k++)
  {
    CK (cudaStreamCreateWithFlags (&b->sbr[k], cudaStreamNonBlocking), "stream");
    CK (cudaEventCreateWithFlags (&b->ev_br[k], cudaEventDisableTiming), "event");
  }

  for (int k = 0; k < 2; k++)
    ncg_batch_params_init (&b->plan[k].prm);

  *out = b;

  return NCG_OK;
}

void
ncg_batch_free (ncg_batch_t *b)
{
  if (b == NULL)
    return;

  cudaSetDevice (b->device);
  cudaStreamSynchronize (b->s1);
  cudaStreamSynchronize (b->s2);

  for (int k = 0; k < 2; k++)
    _plan_free (&b->plan[k]);

  if (b->dX)
    cudaFree (b->dX);

  if (b->dout)
    cudaFree (b->dout);

  cudaEventDestroy (b->ev_in);
  cudaEventDestroy (b->ev_fork);
  cudaEventDestroy (b->ev_join);
  cudaEventDestroy (b->ev_out);
  cudaEventDestroy (b->t0);
  cudaEventDestroy (b->t1);
  for (int k = 0; k < NCG_BATCH_TC_STREAMS; k++)
  {
    cudaStreamSynchronize (b->stc[k]);
    cudaEventDestroy (b->ev_tc[k]);
    cudaStreamDestroy (b->stc[k]);
  }

  for (int k = 0; k < NCG_BATCH_BR_STREAMS; k++)
  {
    if (b->sbr[k])
    {
      cudaStreamSynchronize (b->sbr[k]);
      cudaStreamDestroy (b->sbr[k]);
    }

    if (b->ev_br[k])
      cudaEventDestroy (b->ev_br[k]);
  }

  cudaStreamDestroy (b->s1);
  cudaStreamDestroy (b->s2);
  free (b->sd);
  free (b->m);
  free (b->gen);
  free (b->x_off);
  free (b->out_off);
  free (b);
}

static void
_invalidate (ncg_batch_t *b)
{
  for (int k = 0; k < 2; k++)
  {
    b->plan[k].valid = 0;
    _plan_release (&b->plan[k]);
  }
}

ncg_status_t
ncg_batch_add (ncg_batch_t *b, ncg_sd_t *sd, uint64_t m, int32_t *slot)
{
  if (b == NULL || sd == NULL || m == 0 || m > (uint64_t) INT32_MAX * 64)
    return NCG_ERR_INVALID_ARG;

  if (sd->cfg.device != b->device)
  {
    ncg_set_error ("ncg_batch_add: handle on device %d, batch on device %d", sd->cfg.device, b->device);

    return NCG_ERR_INVALID_ARG;
  }

  if (b->n == b->cap)
  {
    const int nc = b->cap ? 2 * b->cap : 64;
    void *p[5] = {
      realloc (b->sd, sizeof (*b->sd) * nc), realloc (b->m, sizeof (*b->m) * nc), realloc (b->gen, sizeof (*b->gen) * nc),
      realloc (b->x_off, sizeof (*b->x_off) * nc), realloc (b->out_off, sizeof (*b->out_off) * nc),
    };

    if (p[0]) b->sd = p[0];
    if (p[1]) b->m = p[1];
    if (p[2]) b->gen = p[2];
    if (p[3]) b->x_off = p[3];
    if (p[4]) b->out_off = p[4];

    if (!p[0] || !p[1] || !p[2] || !p[3] || !p[4])
      return NCG_ERR_OUT_OF_MEMORY;

    b->cap = nc;
  }

  b->sd[b->n]      = sd;
  b->m[b->n]       = m;
  b->gen[b->n]     = 0;
  b->x_off[b->n]   = b->x_total;
  b->out_off[b->n] = b->out_total;
  b->x_total      += (int64_t) m * sd->d;
  b->out_total    += (int64_t) m;

  if (slot)
    *slot = b->n;

  b->n++;
  _invalidate (b);

  return NCG_OK;
}

ncg_status_t
ncg_batch_clear (ncg_batch_t *b)
{
  if (b == NULL)
    return NCG_ERR_INVALID_ARG;

  cudaSetDevice (b->device);
  cudaStreamSynchronize (b->s1);
  b->n         = 0;
  b->x_total   = 0;
  b->out_total = 0;
  _invalidate (b);

  return NCG_OK;
}

ncg_status_t
ncg_batch_layout (ncg_batch_t *b, int64_t *x_off, int64_t *out_off, int64_t totals[2])
{
  if (b == NULL)
    return NCG_ERR_INVALID_ARG;

  if (x_off)
    memcpy (x_off, b->x_off, sizeof (int64_t) * b->n);

  if (out_off)
    memcpy (out_off, b->out_off, sizeof (int64_t) * b->n);

  if (totals)
  {
    totals[0] = b->x_total;
    totals[1] = b->out_total;
  }

  return NCG_OK;
}

/* ------------------------------------------------------------------ plan */

/* work of one (point, kernel) pair of a problem, in the units of the tile
 * arithmetic: VKDE d(d+1)/2 + 2d, KDE 2d (whitening of the point is per
 * point, not per pair) */
static double
_pair_cost (const ncg_sd_t *sd)
{
  const double dp = sd->dp;

  return (sd->kind == NCG_VKDE) ? dp * (dp + 1.0) / 2.0 + 2.0 * dp : 2.0 * dp;
}

typedef struct { double cost; int32_t p, local; } _bitem_t;

static int
_item_cmp_lpt (const void *x, const void *y)
{
  const _bitem_t *a = x, *b = y;

  if (a->cost > b->cost) return -1;
  if (a->cost < b->cost) return 1;
  if (a->p != b->p) return (a->p < b->p) ? -1 : 1;
  return (a->local < b->local) ? -1 : (a->local > b->local);
}

static ncg_status_t
_reserve (void **ptr, size_t *cap, size_t bytes)
{
  return ncg_dev_reserve (ptr, cap, bytes);
}

static int
_is_tc (const ncg_bplan_t *P, int i)
{
  for (int k = 0; k < P->ntcp; k++)
    if (P->tcp[k] == i)
      return 1;

  return 0;
}

static ncg_status_t
_build_plan (ncg_batch_t *b, int mixed)
{
  ncg_bplan_t *P = &b->plan[mixed];
  const ncg_batch_params_t *prm = &P->prm;
  double total = 0.0;
  int64_t nitems = 0;
  size_t part_bytes = 0, cnt = 0;
  ncg_status_t r;

  _plan_release (P);
  P->valid        = 0;
  P->n_fp64_tiles = 0;
  P->pairs        = 0;

  if (b->n == 0)
    return NCG_OK;

  {
    ncg_bprob_t *hp = realloc (P->hp, sizeof (ncg_bprob_t) * b->n);

    if (hp == NULL)
      return NCG_ERR_OUT_OF_MEMORY;

    P->hp = hp;
  }

  if (P->cap_tcp < b->n)
  {
    int32_t *t = realloc (P->tcp, sizeof (int32_t) * b->n);

    if (t == NULL)
      return NCG_ERR_OUT_OF_MEMORY;

    P->tcp     = t;
    P->cap_tcp = b->n;
  }

  P->ntcp = 0;
  P->nbrp = 0;

  if (prm->tc == 2 && P->cap_brp < b->n)
  {
    int32_t *t = realloc (P->brp, sizeof (int32_t) * b->n);
    int8_t *k8 = t ? realloc (P->brk, sizeof (int8_t) * b->n) : NULL;

    if (t)
      P->brp = t;

    if (k8 == NULL)
      return NCG_ERR_OUT_OF_MEMORY;

    P->brk     = k8;
    P->cap_brp = b->n;
  }

  /* per-problem arithmetic and state */
  for (int i = 0; i < b->n; i++)
  {
    ncg_sd_t *sd    = b->sd[i];
    ncg_bprob_t *q  = &P->hp[i];
    int tmix        = 0;

    if (!sd->prepared)
    {
      ncg_set_error ("ncg_batch: problem %d is not prepared", i);

      return NCG_ERR_NOT_PREPARED;
    }

    if (mixed)
    {
      if ((r = ncg_sd_ensure_packmx (sd)) != NCG_OK)
        return r;

      tmix = (sd->mixed_kappa <= NCG_MIXED_KAPPA_MAX);

      /* a tensor-core problem: its operand passes its check; its scratch is
       * reserved now, since nothing may allocate inside the captured graph */
      if (tmix && prm->tc && ncg_tc_supported (sd->kind, sd->dp))
      {
        if ((r = ncg_sd_ensure_tc (sd)) != NCG_OK)
          return r;

        if (sd->tc_ok)
        {
          if ((r = ncg_sd_reserve (sd, (void **) &sd->dscratch, &sd->cap.scratch,
                                   ncg_tc_scratch_bytes ((int64_t) b->m[i], (int) sd->nk, sd->dp))) != NCG_OK)
            return r;

          CK (cudaStreamSynchronize (sd->stream), "sync");

          P->tcp[P->ntcp++] = i;
        }
      }
    }

    if (mixed && !tmix)
      P->n_fp64_tiles++;

    /* the branch schedule: a problem off the tensor cores runs its own
     * specialised tile kernel (FP32 SIMT, or FP64), whose scratch is
     * reserved now */
    if (prm->tc == 2)
    {
      const int on_tc = (P->ntcp > 0 && P->tcp[P->ntcp - 1] == i);

      P->brk[P->nbrp]   = on_tc ? 2 : ((mixed && tmix) ? 1 : 0);
      P->brp[P->nbrp++] = i;

      if (!on_tc)
      {
        ncg_eval_args_t a;

        ncg_sd_fill_args (sd, b->m[i], &a);

        if ((r = ncg_sd_reserve (sd, (void **) &sd->dscratch, &sd->cap.scratch,
                                 ncg_eval_scratch_bytes (&a, (mixed && tmix) ? NCG_PREC_MIXED_SIMT : NCG_PREC_FP64)))
            != NCG_OK)
          return r;

        CK (cudaStreamSynchronize (sd->stream), "sync");
      }
    }

    memset (q, 0, sizeof (*q));
    ncg_sd_fill_args (sd, b->m[i], &q->a);
    q->pack64  = sd->dpack64;
    q->c       = sd->dc;
    q->Vg      = sd->dVg;
    q->mu      = (tmix && sd->kind == NCG_VKDE) ? sd->dmu : NULL;
    q->packmx  = tmix ? sd->dpackmx : NULL;
    q->dshift  = tmix ? ncg_packmx_cshift (sd->dpackmx, sd->kind, (int) sd->nk, sd->dp) : NULL;
    q->x_off   = b->x_off[i];
    q->out_off = b->out_off[i];
    q->cls     = NCG_BCLS (tmix, sd->dp, sd->kind, sd->kernel);
    q->bx      = (int32_t) ((b->m[i] + 127) / 128);
    total     += (double) b->m[i] * (double) sd->nk * _pair_cost (sd);
    P->pairs  += (int64_t) b->m[i] * (int64_t) sd->nk;
    b->gen[i]  = sd->gen;
  }

  /* launches and grids */
  P->nlaunch = prm->split ? 2 : 1;
  P->set[0]  = prm->split ? NCG_BSET_SMALL : NCG_BSET_ALL;
  P->set[1]  = NCG_BSET_LARGE;

  for (int l = 0; l < P->nlaunch; l++)
  {
    const int occ = ncg_batch_ctas_per_sm (mixed, P->set[l]);
    const int cps = (prm->ctas_per_sm > 0 && prm->ctas_per_sm < occ) ? prm->ctas_per_sm : occ;

    P->grid[l] = b->nsm * cps;
  }

  /* slicing: items of about equal work, items_per_cta per resident CTA */
  {
    const double per_item = total / ((double) P->grid[0] * (prm->items_per_cta > 1.0 ? prm->items_per_cta : 1.0));

    for (int i = 0; i < b->n; i++)
    {
      ncg_sd_t *sd   = b->sd[i];
      ncg_bprob_t *q = &P->hp[i];
      const int kc   = ncg_batch_chunk (q->cls);
      const int n    = (int) sd->nk;
      double want    = per_item / (128.0 * _pair_cost (sd));
      int kper;

      if (q->cls >= NCG_BCLS (1, 4, 0, 0) && want > NCG_BATCH_MIXED_KMAX)
        want = NCG_BATCH_MIXED_KMAX;

      if (want < kc)
        want = kc;

      if (want > n)
        want = n;

      kper    = (int) ceil (want);
      kper    = ((kper + kc - 1) / kc) * kc;
      q->kper = kper;
      q->ns   = (n + kper - 1) / kper;
      nitems += (int64_t) q->bx * q->ns;

      part_bytes  = (part_bytes + 255) & ~(size_t) 255;
      q->part     = (void *) part_bytes;   /* offset, relocated below */
      part_bytes += (size_t) q->ns * b->m[i] * ((q->cls >= NCG_BCLS (1, 4, 0, 0)) ? 8 : 16);
      q->tile_cnt = (int32_t *) (uintptr_t) cnt;
      cnt        += (size_t) q->bx;
    }
  }

  if (nitems > INT32_MAX)
  {
    ncg_set_error ("ncg_batch: %lld work items exceed the work list", (long long) nitems);

    return NCG_ERR_INVALID_ARG;
  }

  if ((r = _reserve (&P->dpart, &P->cap_part, part_bytes)) != NCG_OK)
    return r;

  {
    const size_t old = P->cap_cnt;

    if ((r = _reserve ((void **) &P->dcnt, &P->cap_cnt, sizeof (int32_t) * cnt)) != NCG_OK)
      return r;

    (void) old;
  }

  CK (cudaMemsetAsync (P->dcnt, 0, sizeof (int32_t) * cnt, b->s1), "memset tile counts");

  if (P->dcounter == NULL)
    CK (cudaMalloc ((void **) &P->dcounter, 2 * sizeof (int32_t)), "cudaMalloc");

  for (int i = 0; i < b->n; i++)
  {
    P->hp[i].part     = (char *) P->dpart + (size_t) P->hp[i].part;
    P->hp[i].tile_cnt = P->dcnt + (size_t) (uintptr_t) P->hp[i].tile_cnt;
  }

  /* work list, grouped by launch, in the requested order */
  {
    _bitem_t *it = malloc (sizeof (_bitem_t) * (size_t) (nitems > 0 ? nitems : 1));
    int32_t *hi  = realloc (P->hitems, sizeof (int32_t) * 2 * (size_t) (nitems > 0 ? nitems : 1));
    int64_t k    = 0;

    if (it == NULL || hi == NULL)
    {
      free (it);

      if (hi)
        P->hitems = hi;

      return NCG_ERR_OUT_OF_MEMORY;
    }

    P->hitems = hi;

    for (int l = 0; l < P->nlaunch; l++)
    {
      const int64_t k0 = k;

      for (int i = 0; i < b->n; i++)
      {
        const ncg_bprob_t *q = &P->hp[i];
        const int dp         = b->sd[i]->dp;
        const int in_set     = (P->set[l] == NCG_BSET_ALL) ||
                               (P->set[l] == NCG_BSET_SMALL && dp <= NCG_BSET_SPLIT_DP) ||
                               (P->set[l] == NCG_BSET_LARGE && dp > NCG_BSET_SPLIT_DP);

        if (!in_set || _is_tc (P, i) || prm->tc == 2)
          continue;

        for (int sy = 0; sy < q->ns; sy++)
        {
          const int kk      = (sy == q->ns - 1) ? (int) b->sd[i]->n - sy * q->kper : q->kper;
          const double cost = (double) kk * _pair_cost (b->sd[i]);

          for (int x = 0; x < q->bx; x++)
          {
            it[k].cost  = cost * (double) ((x == q->bx - 1) ? (int64_t) b->m[i] - (int64_t) x * 128 : 128);
            it[k].p     = i;
            it[k].local = sy * q->bx + x;
            k++;
          }
        }
      }

      if (prm->order == 1)
        qsort (it + k0, (size_t) (k - k0), sizeof (_bitem_t), _item_cmp_lpt);

      P->nitems[l] = (int) (k - k0);
    }

    for (int64_t e = 0; e < k; e++)
    {
      hi[2 * e]     = it[e].p;
      hi[2 * e + 1] = it[e].local;
    }

    free (it);
  }

  if ((r = _reserve ((void **) &P->dp, &P->cap_dp, sizeof (ncg_bprob_t) * b->n)) != NCG_OK)
    return r;

  if ((r = _reserve ((void **) &P->ditems, &P->cap_items, sizeof (int32_t) * 2 * (size_t) (nitems > 0 ? nitems : 1))) != NCG_OK)
    return r;

  CK (cudaMemcpyAsync (P->dp, P->hp, sizeof (ncg_bprob_t) * b->n, cudaMemcpyHostToDevice, b->s1), "H2D problems");
  CK (cudaMemcpyAsync (P->ditems, P->hitems, sizeof (int32_t) * 2 * (size_t) nitems, cudaMemcpyHostToDevice, b->s1),
      "H2D items");
  CK (cudaStreamSynchronize (b->s1), "sync");
  P->valid = 1;

  return NCG_OK;
}

/* the tensor-core problems of a plan, spread over the TC streams forked from
 * s1 and joined back into it */
static ncg_status_t
_enqueue_tc (ncg_batch_t *b, ncg_bplan_t *P, const double *dX, double *dout)
{
  const int ns = (P->ntcp < NCG_BATCH_TC_STREAMS) ? P->ntcp : NCG_BATCH_TC_STREAMS;

  if (ns == 0)
    return NCG_OK;

  CK (cudaEventRecord (b->ev_fork, b->s1), "record");

  for (int k = 0; k < ns; k++)
    CK (cudaStreamWaitEvent (b->stc[k], b->ev_fork, 0), "wait");

  for (int k = 0; k < P->ntcp; k++)
  {
    const int i = P->tcp[k];
    ncg_sd_t *sd = b->sd[i];
    ncg_eval_args_t a;

    ncg_sd_fill_args (sd, b->m[i], &a);
    CK (ncg_launch_eval_tc (&a, dX + b->x_off[i], sd->dtcB, sd->dmu, sd->dVg,
                            ncg_packmx_cshift (sd->dpackmx, sd->kind, (int) sd->nk, sd->dp), sd->dscratch,
                            dout + b->out_off[i], sd->d_flag_alias, NULL, b->stc[k % ns]), "batch eval_tc");
  }

  for (int k = 0; k < ns; k++)
  {
    CK (cudaEventRecord (b->ev_tc[k], b->stc[k]), "record");
    CK (cudaStreamWaitEvent (b->s1, b->ev_tc[k], 0), "wait");
  }

  return NCG_OK;
}

typedef struct { double cost; int32_t k; } _brc_t;

static int
_brc_desc (const void *x, const void *y)
{
  const _brc_t *a = x, *c = y;

  if (a->cost > c->cost) return -1;
  if (a->cost < c->cost) return 1;
  return (a->k < c->k) ? -1 : (a->k > c->k);
}

/* The branch schedule (tc = 2): every problem is one launch of the kernel its
 * own eval would use (tensor cores, FP32 SIMT tiles or FP64 tiles), the
 * problems spread over NCG_BATCH_BR_STREAMS streams forked from s1, largest
 * first, each to the stream with the least work so far (longest processing
 * time first); captured, the streams are parallel branches of the graph. */
static ncg_status_t
_enqueue_branches (ncg_batch_t *b, ncg_bplan_t *P, const double *dX, double *dout)
{
  const int ns = (P->nbrp < NCG_BATCH_BR_STREAMS) ? P->nbrp : NCG_BATCH_BR_STREAMS;
  double load[NCG_BATCH_BR_STREAMS];
  _brc_t *ord;

  if (ns == 0)
    return NCG_OK;

  if ((ord = malloc (sizeof (_brc_t) * P->nbrp)) == NULL)
    return NCG_ERR_OUT_OF_MEMORY;

  for (int k = 0; k < P->nbrp; k++)
  {
    const int i = P->brp[k];

    /* tensor-core pairs at about a quarter of the FP32 SIMT pair time */
    ord[k].cost = (double) b->m[i] * (double) b->sd[i]->nk * _pair_cost (b->sd[i]) * ((P->brk[k] == 2) ? 0.25 : 1.0);
    ord[k].k    = k;
  }

  qsort (ord, P->nbrp, sizeof (_brc_t), _brc_desc);

  {
    ncg_status_t r = ncg_cuda_status (cudaEventRecord (b->ev_fork, b->s1), "record");

    for (int k = 0; k < ns && r == NCG_OK; k++)
    {
      load[k] = 0.0;
      r       = ncg_cuda_status (cudaStreamWaitEvent (b->sbr[k], b->ev_fork, 0), "wait");
    }

    for (int q = 0; q < P->nbrp && r == NCG_OK; q++)
    {
      const int k   = ord[q].k, i = P->brp[k];
      ncg_sd_t *sd  = b->sd[i];
      int best      = 0;
      ncg_eval_args_t a;

      for (int t = 1; t < ns; t++)
        if (load[t] < load[best])
          best = t;

      load[best] += ord[q].cost;
      ncg_sd_fill_args (sd, b->m[i], &a);

      if (P->brk[k] == 2)
        r = ncg_cuda_status (ncg_launch_eval_tc (&a, dX + b->x_off[i], sd->dtcB, sd->dmu, sd->dVg,
                                                 ncg_packmx_cshift (sd->dpackmx, sd->kind, (int) sd->nk, sd->dp),
                                                 sd->dscratch, dout + b->out_off[i], sd->d_flag_alias, NULL,
                                                 b->sbr[best]), "batch eval_tc");
      else if (P->brk[k] == 1)
        r = ncg_cuda_status (ncg_launch_eval_m2lnp_mixed (&a, dX + b->x_off[i], sd->dpackmx, sd->dmu, sd->dVg,
                                                          dout + b->out_off[i], sd->dscratch, b->sbr[best]),
                             "batch eval_mixed");
      else
        r = ncg_cuda_status (ncg_launch_eval_m2lnp_fp64 (&a, dX + b->x_off[i], sd->dpack64, sd->dc, sd->dVg,
                                                         dout + b->out_off[i], sd->dscratch, 0, b->sbr[best]),
                             "batch eval_fp64");
    }

    for (int k = 0; k < ns && r == NCG_OK; k++)
    {
      r = ncg_cuda_status (cudaEventRecord (b->ev_br[k], b->sbr[k]), "record");

      if (r == NCG_OK)
        r = ncg_cuda_status (cudaStreamWaitEvent (b->s1, b->ev_br[k], 0), "wait");
    }

    free (ord);

    return r;
  }
}

/* the launch sequence of a plan: the tensor-core problems on their streams,
 * the persistent launch(es) on s1 (and s2 for the second launch); or the
 * branch schedule */
static ncg_status_t
_enqueue (ncg_batch_t *b, ncg_bplan_t *P, int mixed, const double *dX, double *dout)
{
  ncg_status_t r;

  if (P->prm.tc == 2)
    return _enqueue_branches (b, P, dX, dout);

  if ((r = _enqueue_tc (b, P, dX, dout)) != NCG_OK)
    return r;

  if (P->nitems[0] + (P->nlaunch > 1 ? P->nitems[1] : 0) == 0)
    return NCG_OK;

  if (P->nlaunch == 1)
  {
    CK (ncg_launch_batch_eval (mixed, P->set[0], P->dp, P->ditems, P->nitems[0], P->dcounter, dX, dout, P->grid[0],
                               b->s1), "batch eval");

    return NCG_OK;
  }

  CK (cudaEventRecord (b->ev_fork, b->s1), "record");
  CK (cudaStreamWaitEvent (b->s2, b->ev_fork, 0), "wait");
  CK (ncg_launch_batch_eval (mixed, P->set[0], P->dp, P->ditems, P->nitems[0], P->dcounter, dX, dout, P->grid[0],
                             b->s1), "batch eval");
  CK (ncg_launch_batch_eval (mixed, P->set[1], P->dp, P->ditems + 2 * (size_t) P->nitems[0], P->nitems[1],
                             P->dcounter + 1, dX, dout, P->grid[1], b->s2), "batch eval");
  CK (cudaEventRecord (b->ev_join, b->s2), "record");
  CK (cudaStreamWaitEvent (b->s1, b->ev_join, 0), "wait");

  return NCG_OK;
}

static int
_stale (ncg_batch_t *b, const ncg_bplan_t *P)
{
  if (!P->valid)
    return 1;

  for (int i = 0; i < b->n; i++)
    if (b->sd[i]->gen != b->gen[i] || !b->sd[i]->prepared)
      return 1;

  return 0;
}

static ncg_status_t
_capture (ncg_batch_t *b, ncg_bplan_t *P, int mixed, const double *dX, double *dout)
{
  cudaGraph_t g = NULL;
  ncg_status_t r;

  _plan_release (P);
  CK (cudaStreamBeginCapture (b->s1, cudaStreamCaptureModeRelaxed), "begin capture");
  r = _enqueue (b, P, mixed, dX, dout);

  {
    cudaError_t e = cudaStreamEndCapture (b->s1, &g);

    if (r != NCG_OK)
    {
      if (g)
        cudaGraphDestroy (g);

      return r;
    }

    CK (e, "end capture");
  }

  {
    cudaError_t e = cudaGraphInstantiate (&P->ge, g, 0);

    cudaGraphDestroy (g);
    CK (e, "graph instantiate");
  }

  P->gX   = dX;
  P->gout = dout;
  P->captures++;

  return NCG_OK;
}

static int
_prec_index (int32_t precision, ncg_status_t *r)
{
  *r = NCG_OK;

  if (precision == NCG_PREC_FP64)
    return BP_FP64;

  if (precision == NCG_PREC_MIXED || precision == NCG_PREC_MIXED_SIMT)
    return BP_MIXED;

  *r = NCG_ERR_INVALID_ARG;

  return 0;
}

ncg_status_t
ncg_batch_eval_m2lnp_device (ncg_batch_t *b, int32_t precision, const double *d_X, double *d_out, void *stream)
{
  ncg_status_t r;
  const int k = _prec_index (precision, &r);

  if (b == NULL || r != NCG_OK || (b->n > 0 && (d_X == NULL || d_out == NULL)))
    return NCG_ERR_INVALID_ARG;

  if (b->n == 0)
    return NCG_OK;

  ncg_bplan_t *P = &b->plan[k];
  cudaStream_t us = (cudaStream_t) stream;

  CK (cudaSetDevice (b->device), "cudaSetDevice");

  if (_stale (b, P) && (r = _build_plan (b, k)) != NCG_OK)
    return r;

  if (P->ge == NULL || P->gX != d_X || P->gout != d_out)
    if ((r = _capture (b, P, k, d_X, d_out)) != NCG_OK)
      return r;

  /* stream order: the user's stream -> the graph on s1 -> the user's stream */
  CK (cudaEventRecord (b->ev_in, us), "record");
  CK (cudaStreamWaitEvent (b->s1, b->ev_in, 0), "wait");
  CK (cudaGraphLaunch (P->ge, b->s1), "graph launch");
  CK (cudaEventRecord (b->ev_out, b->s1), "record");
  CK (cudaStreamWaitEvent (us, b->ev_out, 0), "wait");
  P->launches++;

  return NCG_OK;
}

ncg_status_t
ncg_batch_eval_m2lnp (ncg_batch_t *b, int32_t precision, const double *X, double *out)
{
  ncg_status_t r;

  if (b == NULL || (b->n > 0 && (X == NULL || out == NULL)))
    return NCG_ERR_INVALID_ARG;

  if (b->n == 0)
    return NCG_OK;

  CK (cudaSetDevice (b->device), "cudaSetDevice");

  if ((r = ncg_dev_reserve ((void **) &b->dX, &b->cap_dX, sizeof (double) * (size_t) b->x_total)) != NCG_OK)
    return r;

  if ((r = ncg_dev_reserve ((void **) &b->dout, &b->cap_dout, sizeof (double) * (size_t) b->out_total)) != NCG_OK)
    return r;

  CK (cudaMemcpyAsync (b->dX, X, sizeof (double) * (size_t) b->x_total, cudaMemcpyHostToDevice, b->s1), "H2D points");

  if ((r = ncg_batch_eval_m2lnp_device (b, precision, b->dX, b->dout, b->s1)) != NCG_OK)
    return r;

  CK (cudaMemcpyAsync (out, b->dout, sizeof (double) * (size_t) b->out_total, cudaMemcpyDeviceToHost, b->s1),
      "D2H m2lnp");
  CK (cudaStreamSynchronize (b->s1), "sync");

  /* the tensor-core launches report a bounded-wait timeout through their
   * handle's mapped error word */
  {
    const ncg_bplan_t *P = &b->plan[(precision == NCG_PREC_FP64) ? BP_FP64 : BP_MIXED];

    for (int k = 0; k < P->ntcp; k++)
      if (*(volatile int32_t *) b->sd[P->tcp[k]]->h_flag != 0)
      {
        ncg_set_error ("ncg_batch: the tensor-core eval of problem %d timed out", P->tcp[k]);

        return NCG_ERR_TIMEOUT;
      }
  }

  return NCG_OK;
}

ncg_status_t
ncg_batch_set_params (ncg_batch_t *b, int32_t precision, const ncg_batch_params_t *p)
{
  ncg_status_t r;
  const int k = _prec_index (precision, &r);

  if (b == NULL || p == NULL || r != NCG_OK || !(p->items_per_cta >= 1.0) || p->ctas_per_sm < 0 ||
      p->order < 0 || p->order > 1 || p->split < 0 || p->split > 1 || p->tc < 0 || p->tc > 2)
    return NCG_ERR_INVALID_ARG;

  cudaSetDevice (b->device);
  cudaStreamSynchronize (b->s1);
  b->plan[k].prm   = *p;
  b->plan[k].valid = 0;
  _plan_release (&b->plan[k]);

  return NCG_OK;
}

ncg_status_t
ncg_batch_get_params (ncg_batch_t *b, int32_t precision, ncg_batch_params_t *p)
{
  ncg_status_t r;
  const int k = _prec_index (precision, &r);

  if (b == NULL || p == NULL || r != NCG_OK)
    return NCG_ERR_INVALID_ARG;

  *p = b->plan[k].prm;

  return NCG_OK;
}

/* time one launch sequence of the current plan (no graph), best of reps */
static ncg_status_t
_time_plan (ncg_batch_t *b, int k, int reps, float *best)
{
  ncg_bplan_t *P = &b->plan[k];
  ncg_status_t r;

  *best = INFINITY;

  if ((r = _build_plan (b, k)) != NCG_OK)
    return r;

  for (int t = 0; t < reps + 1; t++)
  {
    float ms = 0.0f;

    CK (cudaEventRecord (b->t0, b->s1), "record");

    if ((r = _enqueue (b, P, k, b->dX, b->dout)) != NCG_OK)
      return r;

    CK (cudaEventRecord (b->t1, b->s1), "record");
    CK (cudaEventSynchronize (b->t1), "sync");
    CK (cudaEventElapsedTime (&ms, b->t0, b->t1), "elapsed");

    if (t > 0 && ms < *best)   /* the first run warms the caches */
      *best = ms;
  }

  return NCG_OK;
}

/* Coordinate search over the plan parameters: items per CTA, then resident
 * CTAs per SM, then the item order, then one or two launches, then (mixed)
 * whether VKDE problems go to the tensor-core kernel; each
 * candidate timed on the device (best of reps after one warm-up run) with
 * the batch's own point buffer (zeros).  The best parameters stay with the
 * batch for that precision. */
ncg_status_t
ncg_batch_autotune (ncg_batch_t *b, int32_t precision, int32_t reps, double *best_ms)
{
  static const double ipc[] = { 2.0, 4.0, 8.0, 16.0, 32.0 };
  ncg_status_t r;
  const int k = _prec_index (precision, &r);

  if (b == NULL || r != NCG_OK || reps < 1)
    return NCG_ERR_INVALID_ARG;

  if (b->n == 0)
    return NCG_OK;

  CK (cudaSetDevice (b->device), "cudaSetDevice");

  if ((r = ncg_dev_reserve ((void **) &b->dX, &b->cap_dX, sizeof (double) * (size_t) b->x_total)) != NCG_OK)
    return r;

  if ((r = ncg_dev_reserve ((void **) &b->dout, &b->cap_dout, sizeof (double) * (size_t) b->out_total)) != NCG_OK)
    return r;

  CK (cudaMemsetAsync (b->dX, 0, sizeof (double) * (size_t) b->x_total, b->s1), "memset");

  ncg_bplan_t *P = &b->plan[k];
  ncg_batch_params_t best = P->prm, cand;
  float tbest, t;

  if ((r = _time_plan (b, k, reps, &tbest)) != NCG_OK)
    return r;

  /* items per CTA */
  for (size_t i = 0; i < sizeof (ipc) / sizeof (ipc[0]); i++)
  {
    cand               = best;
    cand.items_per_cta = ipc[i];
    P->prm             = cand;

    if ((r = _time_plan (b, k, reps, &t)) != NCG_OK)
      return r;

    if (t < tbest)
    {
      tbest = t;
      best  = cand;
    }
  }

  /* resident CTAs per SM: as many as fit, or fewer */
  {
    const int occ = ncg_batch_ctas_per_sm (k, best.split ? NCG_BSET_SMALL : NCG_BSET_ALL);

    for (int c = 1; c <= occ; c++)
    {
      cand             = best;
      cand.ctas_per_sm = (c == occ) ? 0 : c;
      P->prm           = cand;

      if ((r = _time_plan (b, k, reps, &t)) != NCG_OK)
        return r;

      if (t < tbest)
      {
        tbest = t;
        best  = cand;
      }
    }
  }

  /* item order, one launch or two, then the routing: (mixed) the tensor-core
   * kernel for the problems it serves, and the branch schedule */
  for (int pass = 0; pass < 4; pass++)
  {
    cand = best;

    if (pass == 0)
      cand.order = 1 - best.order;
    else if (pass == 1)
      cand.split = 1 - best.split;
    else if (pass == 2)
    {
      if (k != BP_MIXED || best.tc == 2)
        continue;

      cand.tc = 1 - best.tc;
    }
    else
      cand.tc = 2;

    P->prm = cand;

    if ((r = _time_plan (b, k, reps, &t)) != NCG_OK)
      return r;

    if (t < tbest)
    {
      tbest = t;
      best  = cand;
    }
  }

  P->prm   = best;
  P->tuned = 1;

  if ((r = _build_plan (b, k)) != NCG_OK)
    return r;

  if (best_ms)
    *best_ms = tbest;

  return NCG_OK;
}

ncg_status_t
ncg_batch_get_stats (ncg_batch_t *b, int32_t precision, int64_t stats[7])
{
  ncg_status_t r;
  const int k = _prec_index (precision, &r);

  if (b == NULL || stats == NULL || r != NCG_OK)
    return NCG_ERR_INVALID_ARG;

  const ncg_bplan_t *P = &b->plan[k];

  stats[0] = P->valid ? (int64_t) P->nitems[0] + (P->nlaunch > 1 ? P->nitems[1] : 0) : 0;
  stats[1] = (P->valid && P->prm.tc != 2) ? P->nlaunch : 0;
  stats[2] = P->n_fp64_tiles;
  stats[3] = P->pairs;
  stats[4] = P->captures;
  stats[5] = P->launches;
  stats[6] = P->valid ? P->ntcp : 0;

  return NCG_OK;
}

/* ------------------------------------------------- prepare many at once */

/* Every problem's prepare (or prepare_interp) issued from a pool of host
 * threads, each handle on its own stream, so the problems' device work
 * overlaps: the reference prepares one NcmStatsDist at a time
 * (ncm_stats_dist.c:703-789, 878-1094); each handle's result is the one its
 * own call gives (the calls are independent and deterministic). */
typedef struct
{
  ncg_batch_t *b;
  int interp;
  const double *m2lnp;
  const int64_t *off;
  int next, failed_at;
  ncg_status_t status;
  char detail[256];
  pthread_mutex_t mu;
} _bprep_t;

static void *
_bprep_worker (void *arg)
{
  _bprep_t *j = arg;

  for (;;)
  {
    int i;

    pthread_mutex_lock (&j->mu);
    i = (j->status == NCG_OK && j->next < j->b->n) ? j->next++ : -1;
    pthread_mutex_unlock (&j->mu);

    if (i < 0)
      break;

    const ncg_status_t r = j->interp ? ncg_sd_prepare_interp (j->b->sd[i], j->m2lnp + j->off[i])
                                     : ncg_sd_prepare (j->b->sd[i]);

    if (r != NCG_OK)
    {
      pthread_mutex_lock (&j->mu);

      if (j->status == NCG_OK || i < j->failed_at)
      {
        j->status    = r;
        j->failed_at = i;
        snprintf (j->detail, sizeof (j->detail), "%s", ncg_last_error ());
      }

      pthread_mutex_unlock (&j->mu);
    }
  }

  return NULL;
}

static ncg_status_t
_bprep_run (ncg_batch_t *b, int interp, const double *m2lnp, int32_t nthreads)
{
  _bprep_t j;
  int64_t *off = NULL;
  pthread_t th[64];
  int nt = nthreads;

  if (b == NULL || (interp && m2lnp == NULL))
    return NCG_ERR_INVALID_ARG;

  if (b->n == 0)
    return NCG_OK;

  if (interp)
  {
    off = malloc (sizeof (int64_t) * (size_t) b->n);

    if (off == NULL)
      return NCG_ERR_OUT_OF_MEMORY;

    for (int i = 0, acc = 0; i < b->n; i++)
    {
      off[i] = acc;
      acc   += (int) b->sd[i]->n;
    }
  }

  if (nt <= 0)
  {
    const long nc = sysconf (_SC_NPROCESSORS_ONLN);

    nt = (nc > 0) ? (int) nc : 8;
  }

  nt = (nt > 64) ? 64 : nt;
  nt = (nt > b->n) ? b->n : nt;

  /* every handle's prepare buffers first, one at a time: the threads' prepares
   * then allocate nothing, and no cudaMalloc serialises the device under them */
  for (int i = 0; i < b->n; i++)
  {
    if (interp)
      ncg_sd_interp_reserve (b->sd[i]);
    else
      ncg_sd_prepare_reserve (b->sd[i]);
  }

  memset (&j, 0, sizeof (j));
  j.b         = b;
  j.interp    = interp;
  j.m2lnp     = m2lnp;
  j.off       = off;
  j.status    = NCG_OK;
  j.failed_at = b->n;
  pthread_mutex_init (&j.mu, NULL);

  int started = 0;

  for (; started < nt; started++)
    if (pthread_create (&th[started], NULL, _bprep_worker, &j) != 0)
      break;

  if (started == 0)
    _bprep_worker (&j);

  for (int t = 0; t < started; t++)
    pthread_join (th[t], NULL);

  pthread_mutex_destroy (&j.mu);
  free (off);
  _invalidate (b);

  if (j.status != NCG_OK)
    ncg_set_error ("problem %d: %s", j.failed_at, j.detail);

  return j.status;
}

ncg_status_t
ncg_batch_prepare (ncg_batch_t *b, int32_t nthreads)
{
  return _bprep_run (b, 0, NULL, nthreads);
}

ncg_status_t
ncg_batch_prepare_interp (ncg_batch_t *b, const double *m2lnp, int32_t nthreads)
{
  return _bprep_run (b, 1, m2lnp, nthreads);
}
