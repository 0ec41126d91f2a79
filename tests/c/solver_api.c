/*
 * solver_api.c -- the rest of LibAran's serial 3D solver API
 * (aran/aransolver3d.h:118-214) on the GPU library, written the way a
 * LibAran program calls it.  Self-checking: prints "FAIL <what>" for every
 * failed check and exits 1 if there was one, else prints "ok" and exits 0.
 *
 *   solver_api host      checks that need no GPU: get_functions_full (its
 *                        p2p quirk), insert_point_local, find_point with and
 *                        without a tolerance, the profile database
 *                        (db_profile_operators from $ARAN_PROFILE_DB, the
 *                        semifar threshold it implies)
 *   solver_api gpu       traverse in the four orders (node count, leaf point
 *                        lists, father links, the root multipole's degree-0
 *                        term, Hilbert children order), foreach_point_custom
 *                        with a sphere, set_nf_isleaf virtual leaves against
 *                        the equivalent leaf capacity, profile_operators
 */
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <aran/aranprofiledb.h>
#include <aran/aransolver3d.h>
#include <aran_gpu.h>

typedef struct
{
  VsgVector3d pos;
  gdouble charge;
  gcomplex128 pot;
} Body;

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

static void body_p2p (VsgPoint3 src, VsgPoint3 dst) { (void) src; (void) dst; }
static void body_p2m (VsgPoint3 src, const VsgPRTree3dNodeInfo *n, gpointer d)
{ (void) src; (void) n; (void) d; }
static void body_l2p (const VsgPRTree3dNodeInfo *n, gpointer s, VsgPoint3 dst)
{ (void) n; (void) s; (void) dst; }
static void body_p2l (VsgPoint3 src, const VsgPRTree3dNodeInfo *n, gpointer d)
{ (void) src; (void) n; (void) d; }
static void body_m2p (const VsgPRTree3dNodeInfo *n, gpointer s, VsgPoint3 dst)
{ (void) n; (void) s; (void) dst; }

static double uniform01 (unsigned long long *state)
{
  unsigned long long z = (*state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double) (z >> 11) * (1.0 / 9007199254740992.0);
}

static AranSolver3d *new_solver (guint maxbox, int order)
{
  VsgVector3d lb = { -1., -1., -1. }, ub = { 1., 1., 1. };
  VsgPRTree3d *tree = vsg_prtree3d_new_full (&lb, &ub,
                                             (VsgPoint3dLocFunc) vsg_vector3d_vector3d_locfunc,
                                             (VsgPoint3dDistFunc) vsg_vector3d_dist, NULL, maxbox);
  AranSolver3d *s = aran_solver3d_new (tree, ARAN_TYPE_DEVELOPMENT3D,
                                       aran_development3d_new (0, order),
                                       (AranZeroFunc) aran_development3d_set_zero);
  aran_solver3d_set_functions (s, body_p2p, body_p2m,
                               (AranMultipole2MultipoleFunc3d) aran_development3d_m2m_rotate,
                               (AranMultipole2LocalFunc3d) aran_development3d_m2l_rotate,
                               (AranLocal2LocalFunc3d) aran_development3d_l2l_rotate, body_l2p);
  aran_solver3d_set_newton_layout (s, ARAN_NEWTON_POTENTIAL, offsetof (Body, pos),
                                   offsetof (Body, charge), offsetof (Body, pot));
  return s;
}

static Body *make_bodies (int n, unsigned long long seed)
{
  Body *b = calloc (n, sizeof (Body));
  int i;
  for (i = 0; i < n; i++)
    {
      /* a cluster and a uniform background: a tree of uneven depth */
      double f = i % 3 == 0 ? 1.0 : 0.15;
      b[i].pos.x = f * (2 * uniform01 (&seed) - 1);
      b[i].pos.y = f * (2 * uniform01 (&seed) - 1);
      b[i].pos.z = f * (2 * uniform01 (&seed) - 1);
      b[i].charge = uniform01 (&seed);
    }
  return b;
}

/* ------------------------------------------------------------------ host */
static int host_checks (void)
{
  AranSolver3d *s = new_solver (10, 6);
  AranParticle2ParticleFunc3d p2p = (AranParticle2ParticleFunc3d) 0x1;
  AranParticle2MultipoleFunc3d p2m = NULL;
  AranMultipole2LocalFunc3d m2l = NULL;
  AranParticle2LocalFunc3d p2l = NULL;
  AranMultipole2ParticleFunc3d m2p = NULL;
  guint thr = 7;
  unsigned long long seed = 11;
  int i, n = 2000, kept = 0;
  Body *b = calloc (n, sizeof (Body));

  /* get_functions_full: every member but p2p (aran/aransolver3d.c:676-684) */
  aran_solver3d_set_functions_full (s, body_p2p, body_p2m,
                                    (AranMultipole2MultipoleFunc3d) aran_development3d_m2m_rotate,
                                    (AranMultipole2LocalFunc3d) aran_development3d_m2l_rotate,
                                    (AranLocal2LocalFunc3d) aran_development3d_l2l_rotate,
                                    body_l2p, body_p2l, body_m2p, 42);
  aran_solver3d_get_functions_full (s, &p2p, &p2m, NULL, &m2l, NULL, NULL, &p2l, &m2p, &thr);
  CHECK (p2p == (AranParticle2ParticleFunc3d) 0x1, "get_functions_full wrote p2p");
  CHECK (p2m == body_p2m, "get_functions_full p2m");
  CHECK (m2l == (AranMultipole2LocalFunc3d) aran_development3d_m2l_rotate, "get_functions_full m2l");
  CHECK (p2l == body_p2l && m2p == body_m2p, "get_functions_full p2l/m2p");
  CHECK (thr == 42, "get_functions_full threshold");

  /* find_point with the tolerance of tests/newtonfield3.c:495-541: points
   * within 1e-2 of an inserted one merge into it */
  aran_solver3d_set_tolerance (s, 1e-2);
  for (i = 0; i < n; i++)
    {
      Body *found;
      b[kept].pos.x = 0.2 * (2 * uniform01 (&seed) - 1);
      b[kept].pos.y = 0.2 * (2 * uniform01 (&seed) - 1);
      b[kept].pos.z = 0.2 * (2 * uniform01 (&seed) - 1);
      b[kept].charge = 1.;
      found = aran_solver3d_find_point (s, &b[kept]);
      if (found)
        {
          double d = vsg_vector3d_dist (&found->pos, &b[kept].pos);
          int j, brute = 0;
          CHECK (d <= 1e-2, "find_point returned a point beyond the tolerance");
          for (j = 0; j < kept; j++)
            brute |= vsg_vector3d_dist (&b[j].pos, &b[kept].pos) <= 1e-2;
          CHECK (brute, "find_point found a point where none is");
          found->charge += 1.;
        }
      else
        {
          int j;
          for (j = 0; j < kept; j++)
            CHECK (vsg_vector3d_dist (&b[j].pos, &b[kept].pos) > 1e-2,
                   "find_point missed a point within the tolerance");
          CHECK (aran_solver3d_insert_point_local (s, &b[kept]), "insert_point_local");
          kept++;
        }
    }
  CHECK (aran_solver3d_point_count (s) == (guint) kept, "point_count after merging");
  CHECK (kept < n, "some points merged");
  /* exact match with tolerance 0, and after a removal */
  aran_solver3d_set_tolerance (s, 0.);
  {
    Body probe = b[5];
    CHECK (aran_solver3d_find_point (s, &probe) == &b[5], "exact find_point");
    probe.pos.x += 1e-12;
    CHECK (aran_solver3d_find_point (s, &probe) == NULL, "exact find_point beside a point");
    CHECK (aran_solver3d_remove_point (s, &b[5]), "remove_point");
    probe = b[5];
    CHECK (aran_solver3d_find_point (s, &probe) == NULL, "find_point after remove");
  }

  /* profile database: costs of the registered operators at order 6, the
   * l2p cost looked up under the p2p address as in the reference */
  {
    double t;
    guint opt;
    aran_profile_db_set_verbose (FALSE);
    CHECK (aran_profile_db_read_file (NULL, NULL), "read $ARAN_PROFILE_DB");
    t = aran_profile_db_name_eval ("aran_development3d_m2l_rotate", 6.);
    CHECK (fabs (t - 6e-6) < 1e-18, "name_eval of a sample");
    t = aran_profile_db_address_eval ((gpointer) aran_development3d_m2l_rotate, 6.);
    CHECK (fabs (t - 6e-6) < 1e-18, "address_eval of a sample");
    t = aran_profile_db_address_eval ((gpointer) aran_development3d_m2l_rotate, 7.);
    CHECK (fabs (t - (1e-7 + 2e-7 * 7 + 3e-8 * 49)) < 1e-15, "address_eval of the polynomial");
    CHECK (isnan (aran_profile_db_address_eval ((gpointer) &kept, 1.)), "unknown address is NaN");
    CHECK (aran_profile_db_get_by_name ("aran_development3d_m2l_rotate") ==
           aran_profile_db_get_by_address ((gpointer) aran_development3d_m2l_rotate),
           "lookup by name and by address agree");
    aran_solver3d_set_functions_full (s, body_p2p, body_p2m,
                                      (AranMultipole2MultipoleFunc3d) aran_development3d_m2m_rotate,
                                      (AranMultipole2LocalFunc3d) aran_development3d_m2l_rotate,
                                      (AranLocal2LocalFunc3d) aran_development3d_l2l_rotate,
                                      body_l2p, (AranParticle2LocalFunc3d) aran_development3d_p2l,
                                      (AranMultipole2ParticleFunc3d) aran_development3d_m2pv, 0);
    CHECK (aran_solver3d_optimal_semifar_threshold (s) == G_MAXUINT, "no costs: G_MAXUINT");
    aran_solver3d_db_profile_operators (s, 6.);
    opt = aran_solver3d_optimal_semifar_threshold (s);
    /* p2l 4e-6 and m2pv 2e-6 at order 6, p2p (the test's callback) unknown */
    CHECK (opt == G_MAXUINT, "threshold without a p2p cost");
  }
  free (b);
  aran_solver3d_free (s);
  return g_fail;
}

/* ------------------------------------------------------------------- gpu */
typedef struct
{
  int nodes, leaves, points, bad_list, bad_father, max_depth;
  guint last_depth;
  int level_order_ok;
  gcomplex128 root_m00;
  int root_seen;
} Walk;

static void walk_cb (const VsgPRTree3dNodeInfo *info, gpointer data)
{
  Walk *w = (Walk *) data;
  w->nodes++;
  if (info->depth < w->last_depth)
    w->level_order_ok = 0;
  w->last_depth = info->depth;
  if ((int) info->depth > w->max_depth)
    w->max_depth = info->depth;
  if (info->father_info && info->father_info->depth + 1 != info->depth)
    w->bad_father++;
  if (!info->father_info && info->depth != 0)
    w->bad_father++;
  if (info->isleaf)
    {
      guint k = 0;
      GSList *l;
      for (l = info->point_list; l; l = l->next)
        {
          Body *b = (Body *) l->data;
          if (b->pos.x < info->lbound.x || b->pos.x > info->ubound.x)
            w->bad_list++;
          k++;
        }
      if (k != info->point_count)
        w->bad_list++;
      w->leaves++;
      w->points += k;
    }
  if (info->depth == 0)
    {
      AranDevelopment3d *d = (AranDevelopment3d *) info->user_data;
      w->root_m00 = *aran_spherical_seriesd_get_term (d->multipole, -1, 0);
      w->root_seen = 1;
    }
}

typedef struct
{
  guint first[16];
  int n;
} FirstKids;

static void kids_cb (const VsgPRTree3dNodeInfo *info, gpointer data)
{
  FirstKids *f = (FirstKids *) data;
  if (info->depth == 1 && f->n < 16)
    f->first[f->n++] = info->id;
}

typedef struct
{
  VsgVector3d c;
  double r;
} Sphere;

static vsgrloc3 sphere_loc (const VsgRegion3 region, const VsgPoint3 point)
{
  const Sphere *s = (const Sphere *) region;
  const Body *b = (const Body *) point;
  return vsg_vector3d_dist (&s->c, &b->pos) <= s->r ? VSG_RLOC3_MASK : 0;
}

static void count_cb (gpointer point, gpointer data)
{
  (void) point;
  (*(int *) data)++;
}

static gboolean virtual_maxbox (const VsgPRTree3dNodeInfo *info, gpointer vmax)
{
  if (VSG_PRTREE3D_NODE_INFO_IS_SHARED (info))
    return FALSE;
  return info->point_count <= *(guint *) vmax;
}

static int gpu_checks (void)
{
  const int n = 20000, order = 8;
  Body *b = make_bodies (n, 5), *b2 = make_bodies (n, 5);
  AranSolver3d *s = new_solver (16, order);
  AranSolver3d *s1 = new_solver (1, order);
  int i, rc;
  double qsum = 0.;
  guint vmax = 16;
  GTraverseType orders[4] = { G_PRE_ORDER, G_POST_ORDER, G_IN_ORDER, G_LEVEL_ORDER };
  Walk w[4];

  for (i = 0; i < n; i++)
    {
      aran_solver3d_insert_point (s, &b[i]);
      aran_solver3d_insert_point (s1, &b2[i]);
      qsum += b[i].charge;
    }
  /* traverse before any solve: the tree of the inserted points, zero
   * developments */
  memset (&w[0], 0, sizeof (Walk));
  w[0].level_order_ok = 1;
  aran_solver3d_traverse (s, G_PRE_ORDER, walk_cb, &w[0]);
  CHECK (w[0].points == n, "traverse before solve: points in leaves");
  CHECK (w[0].root_seen && cabs (w[0].root_m00) == 0., "traverse before solve: zero developments");
  rc = aran_solver3d_solve_try (s);
  CHECK (rc == ARAN_OK, "solve");
  for (i = 0; i < 4; i++)
    {
      memset (&w[i], 0, sizeof (Walk));
      w[i].level_order_ok = 1;
      aran_solver3d_traverse (s, orders[i], walk_cb, &w[i]);
      CHECK (w[i].nodes == w[0].nodes && w[i].nodes > 1, "same node count in every order");
      CHECK (w[i].points == n, "every point in one leaf list");
      CHECK (w[i].bad_list == 0, "leaf lists: lengths and bounds");
      CHECK (w[i].bad_father == 0, "father links");
    }
  CHECK (w[3].level_order_ok, "level order visits depths in order");
  /* M_0^0 = sum_i q_i 4 pi conj(Y_0^0) = sqrt(4 pi) sum q (arandevelopment3d.c:192-213) */
  CHECK (fabs (creal (w[0].root_m00) - sqrt (4. * M_PI) * qsum) < 1e-9 * qsum,
         "root multipole degree 0 after the solve");
  /* Hilbert children order: a permutation of the default one, and a
   * different one somewhere */
  {
    FirstKids d = { { 0 }, 0 }, h = { { 0 }, 0 };
    int j, k, same = 1;
    aran_solver3d_traverse (s, G_PRE_ORDER, kids_cb, &d);
    aran_solver3d_set_children_order_hilbert (s);
    aran_solver3d_traverse (s, G_PRE_ORDER, kids_cb, &h);
    aran_solver3d_set_children_order_default (s);
    CHECK (d.n == 8 && h.n == 8, "eight depth-1 nodes");
    for (j = 0; j < 8; j++)
      {
        int hit = 0;
        for (k = 0; k < 8; k++)
          hit += d.first[j] == h.first[k];
        CHECK (hit == 1, "Hilbert order is a permutation");
        same &= d.first[j] == h.first[j];
      }
    CHECK (!same, "Hilbert order differs from the octant order");
  }
  /* foreach_point_custom: points inside a sphere */
  {
    Sphere sp = { { 0.05, -0.02, 0.03 }, 0.1 };
    int got = 0, brute = 0;
    aran_solver3d_foreach_point_custom (s, &sp, sphere_loc, count_cb, &got);
    for (i = 0; i < n; i++)
      brute += vsg_vector3d_dist (&sp.c, &b[i].pos) <= sp.r;
    CHECK (got == brute && brute > 0, "foreach_point_custom selects the sphere's points");
  }
  /* virtual leaves: leaf capacity 1 with leaves of up to 16 points in the
   * near/far traversal gives the tree of capacity 16, so the same result */
  aran_solver3d_set_nf_isleaf (s1, virtual_maxbox, &vmax);
  rc = aran_solver3d_solve_try (s1);
  CHECK (rc == ARAN_OK, "solve with virtual leaves");
  {
    double num = 0., den = 0.;
    glong p2p_a, p2p_b, m2l_a, m2l_b;
    for (i = 0; i < n; i++)
      {
        double d = creal (b[i].pot) - creal (b2[i].pot);
        num += d * d;
        den += creal (b[i].pot) * creal (b[i].pot);
      }
    CHECK (sqrt (num / den) < 1e-13, "virtual leaves equal the capacity-16 tree");
    aran_solver3d_get_stats (s, NULL, &p2p_a, NULL, NULL, &m2l_a, NULL, NULL, NULL, NULL, NULL, NULL);
    aran_solver3d_get_stats (s1, NULL, &p2p_b, NULL, NULL, &m2l_b, NULL, NULL, NULL, NULL, NULL, NULL);
    CHECK (p2p_a == p2p_b && m2l_a == m2l_b, "virtual leaves: same p2p and m2l counts");
  }
  /* GPU-timed operator costs and the semifar threshold they give */
  aran_solver3d_set_functions_full (s, body_p2p, body_p2m,
                                    (AranMultipole2MultipoleFunc3d) aran_development3d_m2m_rotate,
                                    (AranMultipole2LocalFunc3d) aran_development3d_m2l_rotate,
                                    (AranLocal2LocalFunc3d) aran_development3d_l2l_rotate,
                                    body_l2p, body_p2l, body_m2p, 0);
  aran_solver3d_profile_operators (s, NULL, NULL, NULL);
  {
    guint t = aran_solver3d_optimal_semifar_threshold (s);
    printf ("profiled semifar threshold %u\n", t);
    CHECK (t != G_MAXUINT && t > 0, "threshold from GPU-timed costs");
    for (i = 0; i < n; i++)
      b[i].pot = 0.;
    rc = aran_solver3d_solve_try (s);
    CHECK (rc == ARAN_OK, "semifar solve with the profiled threshold");
  }
  aran_solver3d_free (s);
  aran_solver3d_free (s1);
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
