/*
 * newton_compat.c -- a LibAran-style Newton program built against the
 * GPU library's compatibility headers (include/aran, include/vsg) and
 * linked with libaran_gpu.so.
 *
 * It is written the way a LibAran user writes one (the call sequence of the
 * reference's tests/newtonfield3.c and tests/newtonpot3.c): a point struct,
 * p2p/p2m/l2p callbacks, a tree from vsg_prtree3d_new_full, a development
 * from aran_development3d_new (0, p), set_functions, insert_point for every
 * particle, solve, get_stats, free.  The only added call is
 * aran_solver3d_set_newton_layout.
 *
 *   newton_compat N ORDER rotate|kkylin|normal|mixops pot|field fp64|mixed [twice|nolayout]
 *
 * "mixops" hands m2m/l2l of the rotate flavour with the kkylin m2l, which the
 * GPU path refuses.
 *
 * Prints one line "maxerr=<max relative error vs direct sum> p2p=... m2l=..."
 * and exits 0, or prints "error: <aran_gpu_last_error()>" and exits 2 when
 * the solve was refused (the points are then untouched).
 */
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <aran/aransolver3d.h>
#include <aran_gpu.h>

typedef struct
{
  VsgVector3d pos;
  gdouble charge;
  VsgVector3d field;
  gcomplex128 pot;
} Body;

/* the callbacks a LibAran program registers; the GPU path runs its own Newton
 * kernels in their place, so none of these is called */
static int g_host_calls = 0;

static void body_p2p (VsgPoint3 src, VsgPoint3 dst)
{
  (void) src;
  (void) dst;
  g_host_calls++;
}

static void body_p2m (VsgPoint3 src, const VsgPRTree3dNodeInfo *dst_node, gpointer dst)
{
  (void) src;
  (void) dst_node;
  (void) dst;
  g_host_calls++;
}

static void body_l2p (const VsgPRTree3dNodeInfo *src_node, gpointer src, VsgPoint3 dst)
{
  (void) src_node;
  (void) src;
  (void) dst;
  g_host_calls++;
}

/* splitmix64 -> uniform [0, 1) */
static double uniform01 (unsigned long long *state)
{
  unsigned long long z = (*state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double) (z >> 11) * (1.0 / 9007199254740992.0);
}

int main (int argc, char **argv)
{
  if (argc < 6)
    {
      fprintf (stderr, "usage: %s N ORDER rotate|kkylin|normal|mixops pot|field fp64|mixed [twice|nolayout]\n",
               argv[0]);
      return 64;
    }
  const int n = atoi (argv[1]);
  const int order = atoi (argv[2]);
  const char *flavour = argv[3];
  const int field = strcmp (argv[4], "field") == 0;
  const int mixed = strcmp (argv[5], "mixed") == 0;
  const char *extra = argc > 6 ? argv[6] : "";
  const int passes = strcmp (extra, "twice") == 0 ? 2 : 1;

  aran_init ();

  VsgVector3d lb = {-1., -1., -1.};
  VsgVector3d ub = {1., 1., 1.};
  VsgPRTree3d *tree = vsg_prtree3d_new_full (&lb, &ub,
                                             (VsgPoint3dLocFunc) vsg_vector3d_vector3d_locfunc,
                                             (VsgPoint3dDistFunc) vsg_vector3d_dist, NULL, 32);
  AranSolver3d *solver = aran_solver3d_new (tree, ARAN_TYPE_DEVELOPMENT3D,
                                            aran_development3d_new (0, (guint8) order),
                                            (AranZeroFunc) aran_development3d_set_zero);

  AranMultipole2MultipoleFunc3d m2m = (AranMultipole2MultipoleFunc3d) aran_development3d_m2m;
  AranMultipole2LocalFunc3d m2l = (AranMultipole2LocalFunc3d) aran_development3d_m2l;
  AranLocal2LocalFunc3d l2l = (AranLocal2LocalFunc3d) aran_development3d_l2l;
  if (strcmp (flavour, "rotate") == 0)
    {
      m2m = (AranMultipole2MultipoleFunc3d) aran_development3d_m2m_rotate;
      m2l = (AranMultipole2LocalFunc3d) aran_development3d_m2l_rotate;
      l2l = (AranLocal2LocalFunc3d) aran_development3d_l2l_rotate;
    }
  else if (strcmp (flavour, "mixops") == 0)
    {
      m2m = (AranMultipole2MultipoleFunc3d) aran_development3d_m2m_rotate;
      m2l = (AranMultipole2LocalFunc3d) aran_development3d_m2l_kkylin;
      l2l = (AranLocal2LocalFunc3d) aran_development3d_l2l_rotate;
    }
  else if (strcmp (flavour, "kkylin") == 0)
    {
      m2m = (AranMultipole2MultipoleFunc3d) aran_development3d_m2m_kkylin;
      m2l = (AranMultipole2LocalFunc3d) aran_development3d_m2l_kkylin;
      l2l = (AranLocal2LocalFunc3d) aran_development3d_l2l_kkylin;
    }
  aran_solver3d_set_functions (solver, body_p2p, body_p2m, m2m, m2l, l2l, body_l2p);
  if (strcmp (extra, "nolayout") != 0)
    aran_solver3d_set_newton_layout (solver, field ? ARAN_NEWTON_FIELD : ARAN_NEWTON_POTENTIAL,
                                     offsetof (Body, pos), offsetof (Body, charge),
                                     field ? offsetof (Body, field) : offsetof (Body, pot));
  aran_solver3d_set_precision (solver, mixed ? ARAN_PRECISION_MIXED : ARAN_PRECISION_FP64);

  Body *bodies = (Body *) calloc ((size_t) n, sizeof (Body));
  unsigned long long seed = 20240611ULL;
  for (int i = 0; i < n; i++)
    {
      bodies[i].pos.x = 2. * uniform01 (&seed) - 1.;
      bodies[i].pos.y = 2. * uniform01 (&seed) - 1.;
      bodies[i].pos.z = 2. * uniform01 (&seed) - 1.;
      bodies[i].charge = 1. / n;
      aran_solver3d_insert_point (solver, &bodies[i]);
    }
  if ((int) aran_solver3d_point_count (solver) != n)
    {
      printf ("error: point_count %u != %d\n", aran_solver3d_point_count (solver), n);
      return 3;
    }

  aran_solver3d_reinit_stats (solver);
  for (int k = 0; k < passes; k++)
    aran_solver3d_solve (solver);

  int touched = 0;
  for (int i = 0; i < n && !touched; i++)
    touched = field ? (bodies[i].field.x != 0. || bodies[i].field.y != 0. || bodies[i].field.z != 0.)
                    : creal (bodies[i].pot) != 0.;
  if (!touched)
    {
      printf ("error: %s\n", aran_gpu_last_error ());
      aran_solver3d_free (solver);
      free (bodies);
      return 2;
    }

  /* direct sum in double: potential sum q/r and its gradient
   * sum -q (xi - xj)/r^3 (the "field" of tests/newtonfield3.c) */
  double maxerr = 0.;
  for (int i = 0; i < n; i++)
    {
      double phi = 0., fx = 0., fy = 0., fz = 0.;
      for (int j = 0; j < n; j++)
        {
          if (j == i)
            continue;
          double dx = bodies[i].pos.x - bodies[j].pos.x;
          double dy = bodies[i].pos.y - bodies[j].pos.y;
          double dz = bodies[i].pos.z - bodies[j].pos.z;
          double r2 = dx * dx + dy * dy + dz * dz;
          double inv = 1. / sqrt (r2);
          phi += bodies[j].charge * inv;
          double c = -bodies[j].charge * inv * inv * inv;
          fx += c * dx;
          fy += c * dy;
          fz += c * dz;
        }
      double err;
      if (field)
        {
          double ex = bodies[i].field.x / passes - fx;
          double ey = bodies[i].field.y / passes - fy;
          double ez = bodies[i].field.z / passes - fz;
          err = sqrt (ex * ex + ey * ey + ez * ez) / sqrt (fx * fx + fy * fy + fz * fz);
        }
      else
        err = fabs (creal (bodies[i].pot) / passes - phi) / fabs (phi);
      if (err > maxerr)
        maxerr = err;
    }

  glong zero, p2p, p2m, m2m_c, m2l_c, l2l_c, l2p, p2l, m2p, p2p_r, m2l_r;
  aran_solver3d_get_stats (solver, &zero, &p2p, &p2m, &m2m_c, &m2l_c, &l2l_c, &l2p, &p2l, &m2p,
                           &p2p_r, &m2l_r);
  printf ("maxerr=%.3e p2p=%ld p2m=%ld m2m=%ld m2l=%ld l2l=%ld l2p=%ld depth=%u host_calls=%d\n",
          maxerr, (long) p2p, (long) p2m, (long) m2m_c, (long) m2l_c, (long) l2l_c, (long) l2p,
          aran_solver3d_depth (solver), g_host_calls);
  aran_solver3d_free (solver);
  free (bodies);
  return 0;
}
