/* glib-object.h -- TEST INFRASTRUCTURE (see glib.h of this directory): the
 * boxed-type registry arandevelopment{2,3}d.c use. */
#ifndef ORACLE_SHIM_GLIB_OBJECT_H
#define ORACLE_SHIM_GLIB_OBJECT_H
#include <glib.h>

typedef gsize GType;
#define G_TYPE_NONE ((GType) 4)
typedef gpointer (*GBoxedCopyFunc) (gpointer boxed);
typedef void (*GBoxedFreeFunc) (gpointer boxed);

GType g_boxed_type_register_static (const gchar *name, GBoxedCopyFunc copy,
                                    GBoxedFreeFunc free_func);
gpointer g_boxed_copy (GType type, gconstpointer src);
void g_boxed_free (GType type, gpointer boxed);
void g_type_init (void);
#endif
