/*
 * shim.c -- TEST INFRASTRUCTURE: implementations behind the glib and libvsg
 * shim headers of this directory (allocation, messages, an ordered tree for
 * the Wigner repository, the boxed-type registry, vector functions), linked
 * with the reference's operator sources into oracle/_ref/libaranref.so.
 */
#include <glib.h>
#include <glib-object.h>
#include <vsg/vsgd.h>

#include <math.h>
#include <stdarg.h>

static int shim_verbose (void)
{
  static int v = -1;
  if (v < 0)
    v = getenv ("ORACLE_REF_VERBOSE") != NULL;
  return v;
}

void shim_check_failed (const char *expr, const char *file, int line)
{
  fprintf (stderr, "reference check failed: %s (%s:%d)\n", expr, file, line);
}

gpointer g_malloc (gsize n)
{
  gpointer p = n ? malloc (n) : NULL;
  if (n && !p)
    abort ();
  return p;
}

gpointer g_malloc0 (gsize n)
{
  gpointer p = n ? calloc (1, n) : NULL;
  if (n && !p)
    abort ();
  return p;
}

gpointer g_realloc (gpointer p, gsize n)
{
  gpointer q;
  if (!n)
    {
      free (p);
      return NULL;
    }
  q = realloc (p, n);
  if (!q)
    abort ();
  return q;
}

void g_free (gpointer p)
{
  free (p);
}

gpointer g_memdup (gconstpointer p, guint n)
{
  gpointer q;
  if (!p || !n)
    return NULL;
  q = g_malloc (n);
  memcpy (q, p, n);
  return q;
}

static void vmsg (const char *kind, const gchar *fmt, va_list ap)
{
  if (!shim_verbose ())
    return;
  fprintf (stderr, "%s", kind);
  vfprintf (stderr, fmt, ap);
  fputc ('\n', stderr);
}

void g_warning (const gchar *fmt, ...)
{
  va_list ap;
  va_start (ap, fmt);
  vmsg ("reference warning: ", fmt, ap);
  va_end (ap);
}

void g_critical (const gchar *fmt, ...)
{
  va_list ap;
  va_start (ap, fmt);
  vmsg ("reference critical: ", fmt, ap);
  va_end (ap);
}

void g_printerr (const gchar *fmt, ...)
{
  va_list ap;
  if (!shim_verbose ())
    return;
  va_start (ap, fmt);
  vfprintf (stderr, fmt, ap);
  va_end (ap);
}

gint g_atexit (void (*func) (void))
{
  return atexit (func);
}

/* ------------------------------------------------- ordered tree (GTree) */
typedef struct TNode
{
  gpointer key, value;
  struct TNode *left, *right;
} TNode;

struct _GTree
{
  TNode *root;
  GCompareDataFunc cmp;
  gpointer cmp_data;
  GDestroyNotify kd, vd;
};

GTree *g_tree_new_full (GCompareDataFunc compare, gpointer compare_data,
                        GDestroyNotify key_destroy, GDestroyNotify value_destroy)
{
  GTree *t = g_malloc0 (sizeof (GTree));
  t->cmp = compare;
  t->cmp_data = compare_data;
  t->kd = key_destroy;
  t->vd = value_destroy;
  return t;
}

gpointer g_tree_lookup (GTree *t, gconstpointer key)
{
  TNode *n = t->root;
  while (n)
    {
      gint c = t->cmp (key, n->key, t->cmp_data);
      if (c == 0)
        return n->value;
      n = c < 0 ? n->left : n->right;
    }
  return NULL;
}

void g_tree_insert (GTree *t, gpointer key, gpointer value)
{
  TNode **at = &t->root;
  while (*at)
    {
      gint c = t->cmp (key, (*at)->key, t->cmp_data);
      if (c == 0)
        {
          if (t->vd)
            t->vd ((*at)->value);
          if (t->kd)
            t->kd (key);
          (*at)->value = value;
          return;
        }
      at = c < 0 ? &(*at)->left : &(*at)->right;
    }
  *at = g_malloc0 (sizeof (TNode));
  (*at)->key = key;
  (*at)->value = value;
}

static gboolean tree_unlink (GTree *t, gconstpointer key, gboolean notify)
{
  TNode **at = &t->root, *n;
  while (*at)
    {
      gint c = t->cmp (key, (*at)->key, t->cmp_data);
      if (c == 0)
        break;
      at = c < 0 ? &(*at)->left : &(*at)->right;
    }
  n = *at;
  if (!n)
    return FALSE;
  if (notify)
    {
      if (t->kd)
        t->kd (n->key);
      if (t->vd)
        t->vd (n->value);
    }
  if (!n->left)
    *at = n->right;
  else if (!n->right)
    *at = n->left;
  else
    {
      /* the smallest of the right subtree takes the node's place */
      TNode **m = &n->right, *s;
      while ((*m)->left)
        m = &(*m)->left;
      s = *m;
      *m = s->right;
      s->left = n->left;
      s->right = n->right;
      *at = s;
    }
  g_free (n);
  return TRUE;
}

gboolean g_tree_remove (GTree *t, gconstpointer key)
{
  return tree_unlink (t, key, TRUE);
}

gboolean g_tree_steal (GTree *t, gconstpointer key)
{
  return tree_unlink (t, key, FALSE);
}

static void tree_free_nodes (GTree *t, TNode *n)
{
  if (!n)
    return;
  tree_free_nodes (t, n->left);
  tree_free_nodes (t, n->right);
  if (t->kd)
    t->kd (n->key);
  if (t->vd)
    t->vd (n->value);
  g_free (n);
}

void g_tree_destroy (GTree *t)
{
  if (!t)
    return;
  tree_free_nodes (t, t->root);
  g_free (t);
}

/* ------------------------------------------------------- boxed types */
#define MAX_BOXED 16
static struct
{
  GBoxedCopyFunc copy;
  GBoxedFreeFunc free_func;
} g_boxed_tab[MAX_BOXED];
static int g_nboxed = 0;

GType g_boxed_type_register_static (const gchar *name, GBoxedCopyFunc copy,
                                    GBoxedFreeFunc free_func)
{
  (void) name;
  g_boxed_tab[g_nboxed].copy = copy;
  g_boxed_tab[g_nboxed].free_func = free_func;
  return (GType) (0x100 + g_nboxed++);
}

gpointer g_boxed_copy (GType type, gconstpointer src)
{
  return g_boxed_tab[type - 0x100].copy ((gpointer) src);
}

void g_boxed_free (GType type, gpointer boxed)
{
  g_boxed_tab[type - 0x100].free_func (boxed);
}

void g_type_init (void)
{
}

/* ------------------------------------------------------------ vectors */
void vsg_vector3d_sub (const VsgVector3d *a, const VsgVector3d *b, VsgVector3d *res)
{
  res->x = a->x - b->x;
  res->y = a->y - b->y;
  res->z = a->z - b->z;
}

void vsg_vector3d_scalp (const VsgVector3d *a, gdouble s, VsgVector3d *res)
{
  res->x = a->x * s;
  res->y = a->y * s;
  res->z = a->z * s;
}

void vsg_vector3d_to_spherical_internal (const VsgVector3d *v, gdouble *r, gdouble *cost,
                                         gdouble *sint, gdouble *cosp, gdouble *sinp)
{
  double rho2 = v->x * v->x + v->y * v->y;
  double rho = sqrt (rho2);
  double rr = sqrt (rho2 + v->z * v->z);
  *r = rr;
  *cost = rr > 0. ? v->z / rr : 1.;
  *sint = rr > 0. ? rho / rr : 0.;
  *cosp = rho > 0. ? v->x / rho : 1.;
  *sinp = rho > 0. ? v->y / rho : 0.;
}

void vsg_vector3d_to_spherical (const VsgVector3d *v, gdouble *r, gdouble *theta, gdouble *phi)
{
  double rho2 = v->x * v->x + v->y * v->y;
  double rr = sqrt (rho2 + v->z * v->z);
  *r = rr;
  *theta = rr > 0. ? acos (v->z / rr) : 0.;
  *phi = rho2 > 0. ? atan2 (v->y, v->x) : 0.;
}
