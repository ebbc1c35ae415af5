/*
 * Flat driver over NumCosmo's vendored kd-tree, linked only into
 * oracle/_ref/libkdtree_ref.so (test infrastructure).  It mirrors the call
 * sequence of _ncm_stats_dist_vkde_build_cov_array_kdtree
 * (numcosmo/ncm/stats/ncm_stats_dist_vkde.c:363-451): insert every whitened
 * row, rebuild, then for each row take its k nearest neighbours and walk the
 * result list in ascending (distance, index) order.
 */
#include <stddef.h>
#include "kdtree.h"
#include "rb_knn_list.h"

void
ref_kdtree_knn (const double *Y, int n, int d, int k, int *out)
{
  struct kdtree *tree = kdtree_init (d);
  int i;

  for (i = 0; i < n; i++)
    kdtree_insert (tree, (double *) (Y + (size_t) i * d));

  kdtree_rebuild (tree);

  for (i = 0; i < n; i++)
  {
    rb_knn_list_table_t *table = kdtree_knn_search (tree, (double *) (Y + (size_t) i * d), k);
    rb_knn_list_traverser_t trav;
    knn_list_t *p = rb_knn_list_t_first (&trav, table);
    int j = 0;

    while (p != NULL && j < k)
    {
      out[(size_t) i * k + j++] = (int) p->node->coord_index;
      p = rb_knn_list_t_next (&trav);
    }

    for (; j < k; j++)
      out[(size_t) i * k + j] = -1;

    rb_knn_list_destroy (table);
  }

  kdtree_destroy (tree);
}
