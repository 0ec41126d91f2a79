/*
 * glib.h -- TEST INFRASTRUCTURE: the part of glib's API the reference's
 * operator layer (aran/aransphericalseriesd*.c, aranwigner*.c,
 * aransphericalharmonic.c, aranlegendre.c, aranbinomial.c, the generated
 * coefficient buffers, arandevelopment{2,3}d.c, aranlaurentseriesd.c) uses,
 * written for this repository from glib's documented behaviour so those
 * files compile unmodified where they lie.  Only the oracle's reference
 * build (oracle/ref_build.py) uses it.
 */
#ifndef ORACLE_SHIM_GLIB_H
#define ORACLE_SHIM_GLIB_H

#include <alloca.h>
#include <float.h>
#include <limits.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef char gchar;
typedef int gint;
typedef unsigned int guint;
typedef signed char gint8;
typedef unsigned char guint8;
typedef short gint16;
typedef unsigned short guint16;
typedef long glong;
typedef unsigned long gulong;
typedef double gdouble;
typedef float gfloat;
typedef void *gpointer;
typedef const void *gconstpointer;
typedef int gboolean;
typedef size_t gsize;

#ifndef TRUE
#define TRUE 1
#endif
#ifndef FALSE
#define FALSE 0
#endif

#define G_PI 3.1415926535897932384626433832795028841971693993751
#define G_MAXDOUBLE DBL_MAX
#define G_MAXUINT UINT_MAX
#define G_BEGIN_DECLS
#define G_END_DECLS
#define G_UNLIKELY(e) (__builtin_expect (!!(e), 0))
#define G_LIKELY(e) (__builtin_expect (!!(e), 1))
#define G_GNUC_CONST __attribute__ ((const))
#ifndef MAX
#define MAX(a, b) (((a) > (b)) ? (a) : (b))
#endif
#ifndef MIN
#define MIN(a, b) (((a) < (b)) ? (a) : (b))
#endif
#ifndef ABS
#define ABS(a) (((a) < 0) ? -(a) : (a))
#endif

void shim_check_failed (const char *expr, const char *file, int line);

#define g_return_if_fail(expr)                                          \
  do { if (!(expr)) { shim_check_failed (#expr, __FILE__, __LINE__); return; } } while (0)
#define g_return_val_if_fail(expr, val)                                 \
  do { if (!(expr)) { shim_check_failed (#expr, __FILE__, __LINE__); return (val); } } while (0)
#define g_assert(expr)                                                  \
  do { if (!(expr)) { shim_check_failed (#expr, __FILE__, __LINE__); abort (); } } while (0)
#define g_alloca(n) alloca (n)
#define g_new(T, n) ((T *) g_malloc (sizeof (T) * (n)))
#define g_new0(T, n) ((T *) g_malloc0 (sizeof (T) * (n)))

gpointer g_malloc (gsize n);
gpointer g_malloc0 (gsize n);
gpointer g_realloc (gpointer p, gsize n);
void g_free (gpointer p);
gpointer g_memdup (gconstpointer p, guint n);
void g_warning (const gchar *fmt, ...);
void g_critical (const gchar *fmt, ...);
void g_printerr (const gchar *fmt, ...);
gint g_atexit (void (*func) (void));

typedef struct _GSList GSList;
struct _GSList
{
  gpointer data;
  GSList *next;
};

typedef gint (*GCompareDataFunc) (gconstpointer a, gconstpointer b, gpointer user_data);
typedef void (*GDestroyNotify) (gpointer data);
typedef struct _GTree GTree;

GTree *g_tree_new_full (GCompareDataFunc compare, gpointer compare_data,
                        GDestroyNotify key_destroy, GDestroyNotify value_destroy);
gpointer g_tree_lookup (GTree *tree, gconstpointer key);
void g_tree_insert (GTree *tree, gpointer key, gpointer value);
gboolean g_tree_remove (GTree *tree, gconstpointer key);
gboolean g_tree_steal (GTree *tree, gconstpointer key);
void g_tree_destroy (GTree *tree);

#endif
