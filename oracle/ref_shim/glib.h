/*
 * Minimal stand-in for the few GLib names used by NumCosmo's vendored
 * kd-tree sources (numcosmo/external/misc/kdtree.c, rb_knn_list.c), so that
 * those two files compile unmodified into oracle/_ref for pinning the
 * oracle's exact kNN.  Test infrastructure only.
 */
#ifndef NCG_REF_SHIM_GLIB_H
#define NCG_REF_SHIM_GLIB_H
#include <stdlib.h>
typedef int gint;
#define g_slice_new(T) ((T *) malloc (sizeof (T)))
#define g_slice_new0(T) ((T *) calloc (1, sizeof (T)))
#define g_slice_free(T, p) free (p)
#ifndef MAX
#define MAX(a, b) (((a) > (b)) ? (a) : (b))
#endif
#endif
