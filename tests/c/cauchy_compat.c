/*
 * cauchy_compat.c -- a LibAran-style 2D program built against the GPU
 * library's compatibility headers and linked with libaran_gpu.so.
 *
 * Part 1 follows the call sequence of the reference's tests/dummypot.c:
 * points on a circle of radius 0.9 (or uniform in [-0.9, 0.9]^2), unit
 * densities, vsg_prtree2d_new_full on [-1, 1]^2, aran_development2d_new
 * (0, p), set_functions with the aran_development2d operators, solve, and
 * a check of every point against the direct sum with dummypot's error
 * measure |acc - sum| / max(|acc|, |sum|).  The added call is
 * aran_solver2d_set_cauchy_layout.
 *
 * Part 2 runs the Laurent-series operators the way tests/laurent.c does
 * (the series of 1/(z - 1), translated and re-expanded) and P2L the way
 * tests/p2l2.c does; these calls run on the GPU one launch each.
 *
 *   cauchy_compat N ORDER MAXBOX circle|random
 *
 * Prints "maxerr=... laurent=... translate=... taylor=... p2l=... p2p=..."
 * and exits 0, or "error: ..." and exits 2.
 */
#include <complex.h>
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <aran/aransolver2d.h>
#include <aran_gpu.h>

typedef struct
{
  VsgVector2d vector;
  gdouble density;
  gcomplex128 accum;
  guint id;
} Point;

static int g_host_calls = 0;

static void point_p2p (VsgPoint2 a, VsgPoint2 b)
{
  (void) a;
  (void) b;
  g_host_calls++;
}

static void point_p2m (VsgPoint2 p, const VsgPRTree2dNodeInfo *node, gpointer dev)
{
  (void) p;
  (void) node;
  (void) dev;
  g_host_calls++;
}

static void point_l2p (const VsgPRTree2dNodeInfo *node, gpointer dev, VsgPoint2 p)
{
  (void) node;
  (void) dev;
  (void) p;
  g_host_calls++;
}

static double uniform01 (unsigned long long *state)
{
  unsigned long long z = (*state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double) (z >> 11) * (1.0 / 9007199254740992.0);
}

static double rel (double complex ref, double complex res)
{
  double complex d = ref - res;
  if (ref != 0.)
    d /= ref;
  return cabs (d);
}

/* worst relative error of a series against 1/(z - 1) on rings (inner: disk) */
static double ring_check (AranLaurentSeriesd *s, double complex center, double radius, int inner)
{
  double worst = 0.;
  int i, j;
  if (inner)
    worst = rel (1. / (center - 1.), aran_laurent_seriesd_evaluate (s, 0.));
  for (i = 0; i <= 10; i++)
    {
      double r = i * radius / 10 + (inner ? 0. : radius);
      for (j = 0; j < i; j++)
        {
          double complex z = r * cexp (I * 2. * j * M_PI / i);
          double e = rel (1. / (z + center - 1.), aran_laurent_seriesd_evaluate (s, z));
          if (e > worst)
            worst = e;
        }
    }
  return worst;
}

int main (int argc, char **argv)
{
  if (argc < 5)
    {
      fprintf (stderr, "usage: %s N ORDER MAXBOX circle|random\n", argv[0]);
      return 64;
    }
  const int np = atoi (argv[1]);
  const int order = atoi (argv[2]);
  const int maxbox = atoi (argv[3]);
  const int circle = strcmp (argv[4], "circle") == 0;

  aran_init ();

  /* ---- part 1: the solver ---- */
  VsgVector2d lb = {-1., -1.}, ub = {1., 1.};
  VsgPRTree2d *tree = vsg_prtree2d_new_full (&lb, &ub,
                                             (VsgPoint2dLocFunc) vsg_vector2d_vector2d_locfunc,
                                             (VsgPoint2dDistFunc) vsg_vector2d_dist, NULL, maxbox);
  AranSolver2d *solver = aran_solver2d_new (tree, ARAN_TYPE_DEVELOPMENT2D,
                                            aran_development2d_new (0, (guint8) order),
                                            (AranZeroFunc) aran_development2d_set_zero);
  aran_solver2d_set_functions (solver, point_p2p, point_p2m,
                               (AranMultipole2MultipoleFunc2d) aran_development2d_m2m,
                               (AranMultipole2LocalFunc2d) aran_development2d_m2l,
                               (AranLocal2LocalFunc2d) aran_development2d_l2l, point_l2p);
  aran_solver2d_set_cauchy_layout (solver, offsetof (Point, vector), offsetof (Point, density),
                                   offsetof (Point, accum));
  Point *pts = (Point *) calloc ((size_t) np, sizeof (Point));
  unsigned long long seed = 7ULL;
  for (int i = 0; i < np; i++)
    {
      if (circle)
        {
          pts[i].vector.x = 0.9 * cos (2. * M_PI * i / np);
          pts[i].vector.y = 0.9 * sin (2. * M_PI * i / np);
        }
      else
        {
          pts[i].vector.x = -0.9 + 1.8 * uniform01 (&seed);
          pts[i].vector.y = -0.9 + 1.8 * uniform01 (&seed);
        }
      pts[i].density = 1.;
      pts[i].id = (guint) i;
      aran_solver2d_insert_point (solver, &pts[i]);
    }
  int rc = aran_solver2d_solve_try (solver);
  if (rc != ARAN_OK)
    {
      printf ("error: %s\n", aran_gpu_last_error ());
      return 2;
    }
  double maxerr = 0.;
  for (int i = 0; i < np; i++)
    {
      double complex sum = 0.;
      for (int j = 0; j < np; j++)
        if (i != j)
          sum += pts[j].density / ((pts[i].vector.x + I * pts[i].vector.y) -
                                   (pts[j].vector.x + I * pts[j].vector.y));
      double complex acc = pts[i].accum;
      double e = cabs (acc - sum) / fmax (cabs (acc), cabs (sum));
      if (e > maxerr || !isfinite (e))
        maxerr = e;
    }
  glong zero, p2p, p2m, m2m, m2l, l2l, l2p, p2l, m2p, r1, r2;
  aran_solver2d_get_stats (solver, &zero, &p2p, &p2m, &m2m, &m2l, &l2l, &l2p, &p2l, &m2p, &r1, &r2);
  aran_solver2d_free (solver);
  free (pts);

  /* ---- part 2: series operators (tests/laurent.c, tests/p2l2.c) ---- */
  const int so = 24;
  AranLaurentSeriesd *als = aran_laurent_seriesd_new (0, so);
  for (int i = 1; i <= so; i++)
    *aran_laurent_seriesd_get_term (als, -i) = 1.;
  double e_laurent = ring_check (als, 0., 2., 0);
  AranLaurentSeriesd *alst = aran_laurent_seriesd_new (0, so);
  aran_laurent_seriesd_translate (als, 0., alst, I * 2.);
  double e_translate = ring_check (alst, I * 2., 4., 0);
  AranLaurentSeriesd *alstt = aran_laurent_seriesd_new (so, 0);
  aran_laurent_seriesd_to_taylor (als, 0., alstt, I * 6.);
  double e_taylor = ring_check (alstt, I * 6., 2., 1);

  AranDevelopment2d *dev = aran_development2d_new (29, 0);
  VsgVector2d src = {3., -1.};
  VsgPRTree2dNodeInfo node;
  memset (&node, 0, sizeof (node));
  node.center.x = 5.;
  node.center.y = 0.;
  aran_development2d_p2l (&src, 1., &node, dev);
  double e_p2l = 0.;
  for (int j = 0; j < 10; j++)
    for (int k = 0; k < 10; k++)
      {
        double t = M_PI * j / 9., r = k / 9.;
        VsgVector2d pos = {5. + r * cos (t), r * sin (t)};
        double complex ref = 1. / ((pos.x + I * pos.y) - (src.x + I * src.y));
        double e = rel (ref, aran_development2d_local_evaluate (&node, dev, &pos));
        if (e > e_p2l)
          e_p2l = e;
      }
  aran_laurent_seriesd_free (als);
  aran_laurent_seriesd_free (alst);
  aran_laurent_seriesd_free (alstt);
  aran_development2d_free (dev);

  printf ("maxerr=%.3e laurent=%.3e translate=%.3e taylor=%.3e p2l=%.3e p2p=%ld m2l=%ld "
          "p2m=%ld l2p=%ld host_calls=%d\n", maxerr, e_laurent, e_translate, e_taylor, e_p2l,
          (long) p2p, (long) m2l, (long) p2m, (long) l2p, g_host_calls);
  return 0;
}
