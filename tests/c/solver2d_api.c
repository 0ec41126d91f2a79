/*
 * solver2d_api.c -- the rest of LibAran's serial 2D solver API
 * (aran/aransolver2d.h) on the GPU library, written the way a LibAran
 * program calls it (the Cauchy-kernel setting of tests/dummypot.c).
 * Self-checking: prints "FAIL <what>" for every failed check and exits 1 if
 * there was one, else prints "ok" and exits 0.
 *
 *   solver2d_api host    get_functions_full, insert_point_local, the costs
 *                        db_profile_operators reads from $ARAN_PROFILE_DB
 *   solver2d_api gpu     traverse in the four orders on the GPU quadtree,
 *                        Hilbert children order, foreach_point_custom with a
 *                        disc, set_nf_isleaf virtual leaves against the
 *                        equivalent leaf capacity, profile_operators
 */
#include <complex.h>
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <aran/aranprofiledb.h>
#include <aran/aransolver2d.h>
#include <aran_gpu.h>

typedef struct
{
  VsgVector2d vector;
  gdouble density;
  gcomplex128 accum;
} Point2;

static int g_fail = 0;
#define CHECK(cond, what)                                                       \
  do                                                                            \
    {                                                                           \
      if (!(cond))                                                              \
        {                                                                       \
          printf ("FAIL %s (line %d)\n", what, __LINE__);                       \
          g_fail = 1;                                                           \
        }                                                                       \
    }                                                                           \
  while (0)

static void pt_p2p (VsgPoint2 src, VsgPoint2 dst) { (void) src; (void) dst; }
static void pt_p2m (VsgPoint2 src, const VsgPRTree2dNodeInfo *n, gpointer d)
{ (void) src; (void) n; (void) d; }
static void pt_l2p (const VsgPRTree2dNodeInfo *n, gpointer s, VsgPoint2 dst)
{ (void) n; (void) s; (void) dst; }

static double uniform01 (unsigned long long *state)
{
  unsigned long long z = (*state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double) (z >> 11) * (1.0 / 9007199254740992.0);
}

static AranSolver2d *new_solver (guint maxbox, int order)
{
  VsgVector2d lb = { -1., -1. }, ub = { 1., 1. };
  VsgPRTree2d *tree = vsg_prtree2d_new_full (&lb, &ub,
                                             (VsgPoint2dLocFunc) vsg_vector2d_vector2d_locfunc,
                                             (VsgPoint2dDistFunc) vsg_vector2d_dist, NULL, maxbox);
  AranSolver2d *s = aran_solver2d_new (tree, ARAN_TYPE_DEVELOPMENT2D,
                                       aran_development2d_new (0, order),
                                       (AranZeroFunc) aran_development2d_set_zero);
  aran_solver2d_set_functions (s, pt_p2p, pt_p2m,
                               (AranMultipole2MultipoleFunc2d) aran_development2d_m2m,
                               (AranMultipole2LocalFunc2d) aran_development2d_m2l,
                               (AranLocal2LocalFunc2d) aran_development2d_l2l, pt_l2p);
  aran_solver2d_set_cauchy_layout (s, offsetof (Point2, vector), offsetof (Point2, density),
                                   offsetof (Point2, accum));
  return s;
}

static Point2 *make_points (int n, unsigned long long seed)
{
  Point2 *b = calloc (n, sizeof (Point2));
  int i;
  for (i = 0; i < n; i++)
    {
      double f = i % 3 == 0 ? 1.0 : 0.2;
      b[i].vector.x = f * (2 * uniform01 (&seed) - 1);
      b[i].vector.y = f * (2 * uniform01 (&seed) - 1);
      b[i].density = 2 * uniform01 (&seed) - 1;
    }
  return b;
}

static int host_checks (void)
{
  AranSolver2d *s = new_solver (8, 10);
  AranParticle2ParticleFunc2d p2p = (AranParticle2ParticleFunc2d) 0x1;
  AranParticle2MultipoleFunc2d p2m = NULL;
  AranMultipole2LocalFunc2d m2l = NULL;
  guint thr = 3;
  Point2 p = { { 0.1, 0.2 }, 1., 0. };

  aran_solver2d_set_functions_full (s, pt_p2p, pt_p2m,
                                    (AranMultipole2MultipoleFunc2d) aran_development2d_m2m,
                                    (AranMultipole2LocalFunc2d) aran_development2d_m2l,
                                    (AranLocal2LocalFunc2d) aran_development2d_l2l, pt_l2p,
                                    NULL, NULL, 17);
  aran_solver2d_get_functions_full (s, &p2p, &p2m, NULL, &m2l, NULL, NULL, NULL, NULL, &thr);
  CHECK (p2p == (AranParticle2ParticleFunc2d) 0x1, "get_functions_full wrote p2p");
  CHECK (p2m == pt_p2m, "get_functions_full p2m");
  CHECK (m2l == (AranMultipole2LocalFunc2d) aran_development2d_m2l, "get_functions_full m2l");
  CHECK (thr == 17, "get_functions_full threshold");
  CHECK (aran_solver2d_insert_point_local (s, &p), "insert_point_local");
  CHECK (aran_solver2d_point_count (s) == 1, "point_count");
  aran_profile_db_set_verbose (FALSE);
  CHECK (aran_profile_db_read_file (NULL, NULL), "read $ARAN_PROFILE_DB");
  CHECK (fabs (aran_profile_db_address_eval ((gpointer) aran_development2d_m2l, 10.) - 3e-6) < 1e-18,
         "2D operator cost by address");
  aran_solver2d_db_profile_operators (s, 10.);
  CHECK (aran_solver2d_optimal_semifar_threshold (s) == G_MAXUINT, "no p2l/m2p: G_MAXUINT");
  aran_solver2d_free (s);
  return g_fail;
}

typedef struct
{
  int nodes, points, bad_list, bad_father, level_ok;
  guint last_depth;
  gcomplex128 root_a1;
} Walk2;

static void walk2 (const VsgPRTree2dNodeInfo *info, gpointer data)
{
  Walk2 *w = (Walk2 *) data;
  w->nodes++;
  if (info->depth < w->last_depth)
    w->level_ok = 0;
  w->last_depth = info->depth;
  if ((info->father_info && info->father_info->depth + 1 != info->depth) ||
      (!info->father_info && info->depth != 0))
    w->bad_father++;
  if (info->isleaf)
    {
      guint k = 0;
      GSList *l;
      for (l = info->point_list; l; l = l->next)
        {
          Point2 *b = (Point2 *) l->data;
          if (b->vector.x < info->lbound.x || b->vector.x > info->ubound.x ||
              b->vector.y < info->lbound.y || b->vector.y > info->ubound.y)
            w->bad_list++;
          k++;
        }
      if (k != info->point_count)
        w->bad_list++;
      w->points += k;
    }
  if (info->depth == 0)
    w->root_a1 = *aran_laurent_seriesd_get_term (((AranDevelopment2d *) info->user_data)->multipole, -1);
}

typedef struct
{
  guint ids[8];
  int n;
} Kids2;

static void kids2 (const VsgPRTree2dNodeInfo *info, gpointer data)
{
  Kids2 *k = (Kids2 *) data;
  if (info->depth == 1 && k->n < 8)
    k->ids[k->n++] = info->id;
}

typedef struct
{
  VsgVector2d c;
  double r;
} Disc;

static vsgrloc2 disc_loc (const VsgRegion2 region, const VsgPoint2 point)
{
  const Disc *d = (const Disc *) region;
  const Point2 *p = (const Point2 *) point;
  return vsg_vector2d_dist (&d->c, &p->vector) <= d->r ? VSG_RLOC2_MASK : 0;
}

static void count2 (gpointer point, gpointer data)
{
  (void) point;
  (*(int *) data)++;
}

static gboolean virtual_maxbox2 (const VsgPRTree2dNodeInfo *info, gpointer vmax)
{
  if (VSG_PRTREE2D_NODE_INFO_IS_SHARED (info))
    return FALSE;
  return info->point_count <= *(guint *) vmax;
}

static int gpu_checks (void)
{
  const int n = 20000, order = 12;
  Point2 *b = make_points (n, 3), *b2 = make_points (n, 3);
  AranSolver2d *s = new_solver (24, order), *s1 = new_solver (1, order);
  GTraverseType orders[4] = { G_PRE_ORDER, G_POST_ORDER, G_IN_ORDER, G_LEVEL_ORDER };
  Walk2 w[4];
  double qsum = 0.;
  guint vmax = 24;
  int i, rc;

  for (i = 0; i < n; i++)
    {
      aran_solver2d_insert_point (s, &b[i]);
      aran_solver2d_insert_point (s1, &b2[i]);
      qsum += b[i].density;
    }
  rc = aran_solver2d_solve_try (s);
  CHECK (rc == ARAN_OK, "solve");
  for (i = 0; i < 4; i++)
    {
      memset (&w[i], 0, sizeof (Walk2));
      w[i].level_ok = 1;
      aran_solver2d_traverse (s, orders[i], walk2, &w[i]);
      CHECK (w[i].nodes == w[0].nodes && w[i].nodes > 1, "same node count in every order");
      CHECK (w[i].points == n, "every point in one leaf list");
      CHECK (w[i].bad_list == 0, "leaf lists: lengths and bounds");
      CHECK (w[i].bad_father == 0, "father links");
    }
  CHECK (w[3].level_ok, "level order");
  /* a_{-1} = sum q (arandevelopment2d.c:167-189) */
  CHECK (cabs (w[0].root_a1 - qsum) < 1e-9 * (1. + fabs (qsum)), "root multipole a_-1");
  {
    Kids2 d = { { 0 }, 0 }, h = { { 0 }, 0 };
    int j, k, same = 1;
    aran_solver2d_traverse (s, G_PRE_ORDER, kids2, &d);
    aran_solver2d_set_children_order_hilbert (s);
    aran_solver2d_traverse (s, G_PRE_ORDER, kids2, &h);
    aran_solver2d_set_children_order_default (s);
    CHECK (d.n == 4 && h.n == 4, "four depth-1 nodes");
    for (j = 0; j < 4; j++)
      {
        int hit = 0;
        for (k = 0; k < 4; k++)
          hit += d.ids[j] == h.ids[k];
        CHECK (hit == 1, "Hilbert order is a permutation");
        same &= d.ids[j] == h.ids[j];
      }
    CHECK (!same, "Hilbert order differs from the quadrant order");
  }
  {
    Disc dc = { { 0.05, -0.03 }, 0.12 };
    int got = 0, brute = 0;
    aran_solver2d_foreach_point_custom (s, &dc, disc_loc, count2, &got);
    for (i = 0; i < n; i++)
      brute += vsg_vector2d_dist (&dc.c, &b[i].vector) <= dc.r;
    CHECK (got == brute && brute > 0, "foreach_point_custom selects the disc's points");
  }
  aran_solver2d_set_nf_isleaf (s1, virtual_maxbox2, &vmax);
  rc = aran_solver2d_solve_try (s1);
  CHECK (rc == ARAN_OK, "solve with virtual leaves");
  {
    double num = 0., den = 0.;
    for (i = 0; i < n; i++)
      {
        num += cabs (b[i].accum - b2[i].accum) * cabs (b[i].accum - b2[i].accum);
        den += cabs (b[i].accum) * cabs (b[i].accum);
      }
    CHECK (sqrt (num / den) < 1e-13, "virtual leaves equal the capacity-24 tree");
  }
  aran_solver2d_profile_operators (s, NULL, NULL, NULL);
  CHECK (aran_solver2d_optimal_semifar_threshold (s) == G_MAXUINT,
         "2D: no semifar pass, threshold stays G_MAXUINT");
  aran_solver2d_free (s);
  aran_solver2d_free (s1);
  free (b);
  free (b2);
  return g_fail;
}

int main (int argc, char **argv)
{
  int rc;
  aran_init ();
  if (argc < 2)
    {
      fprintf (stderr, "usage: %s host|gpu\n", argv[0]);
      return 2;
    }
  rc = strcmp (argv[1], "gpu") == 0 ? gpu_checks () : host_checks ();
  if (!rc)
    printf ("ok\n");
  return rc ? 1 : 0;
}
