/*
 * aranglib.h -- the few glib types LibAran's public headers use (glib is not
 * needed to build or use the GPU library).  Same names and meaning as glib's.
 */
#ifndef ARAN_GLIB_COMPAT_H
#define ARAN_GLIB_COMPAT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define G_BEGIN_DECLS extern "C" {
#define G_END_DECLS }
#else
#define G_BEGIN_DECLS
#define G_END_DECLS
#endif

typedef int gint;
typedef unsigned int guint;
typedef signed char gint8;
typedef unsigned char guint8;
typedef long glong;
typedef double gdouble;
typedef float gfloat;
typedef void *gpointer;
typedef const void *gconstpointer;
typedef int gboolean;
typedef size_t GType;
typedef char gchar;

#ifndef FALSE
#define FALSE 0
#endif
#ifndef TRUE
#define TRUE 1
#endif
#define G_MAXUINT 0xffffffffU

typedef struct _GSList GSList;
struct _GSList
{
  gpointer data;
  GSList *next;
};

typedef void (*GFunc) (gpointer data, gpointer user_data);

/* orders of a tree traversal (glib's GTraverseType) */
typedef enum
{
  G_IN_ORDER,
  G_PRE_ORDER,
  G_POST_ORDER,
  G_LEVEL_ORDER
} GTraverseType;

#endif
