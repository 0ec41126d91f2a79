/*
 * or_translate.c -- Wigner rotations and the three translation flavours
 * (normal O(p^4), kkylin O(p^3), rotate "point and shoot" O(p^3)) of the
 * oracle.  TEST INFRASTRUCTURE ONLY (see aran_oracle.h).
 */
#include "or_internal.h"

#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define TRI(l, m) (((l) * ((l) + 1)) / 2 + (m))
#define PHASE(m) (((m) % 2 == 0) ? 1. : -1.)

/* ------------------------------------------------------------------------
 * Wigner D matrices: aran/aranwigner.c:37-313
 * Terms D_l^{m,m'} = e^{-i m alpha} d_l^{m,m'}(beta) e^{-i m' gamma} stored
 * packed as [l][m'][l+m] (aran/aranwigner-private.h:36-38).
 * ---------------------------------------------------------------------- */
typedef struct
{
  double alpha, beta, gamma;
  int lmax;
  double complex *t;
} OrWigner;

static int wig_off (int l)
{
  return (l * (l + 1) * (4 * l - 1)) / 6;
}

int or_wigner_size (int lmax)
{
  return ((lmax + 1) * (lmax + 2) * (4 * lmax + 3)) / 6;
}

#define WT(aw, l, mp, m) ((aw)->t[wig_off (l) + (mp) * (2 * (l) + 1) + (l) + (m)])

/* d_l^{m,m'}(beta) by the ten recurrence blocks of
 * aran/aranwigner.c:83-246 */
static void wigner_d (OrWigner *aw, int lmax)
{
  int l, mp, m;
  double cb = cos (aw->beta), sb = sin (aw->beta);
  double cb2 = cos (aw->beta * 0.5), sb2 = sin (aw->beta * 0.5);
  double tb2 = sb2 / cb2;
  double complex d100, d111, d11m1;

  WT (aw, 0, 0, 0) = 1.;
  if (lmax == 0)
    return;
  WT (aw, 1, 0, 0) = cb;
  WT (aw, 1, 1, -1) = sb2 * sb2;
  WT (aw, 1, 1, 0) = sb / sqrt (2.);
  WT (aw, 1, 1, 1) = cb2 * cb2;
  WT (aw, 1, 0, -1) = WT (aw, 1, 1, 0);
  WT (aw, 1, 0, 1) = -WT (aw, 1, 1, 0);
  if (lmax <= 1)
    return;
  d100 = WT (aw, 1, 0, 0);
  d111 = WT (aw, 1, 1, 1);
  d11m1 = WT (aw, 1, 1, -1);

  for (l = 2; l <= lmax; l++)
    {
      double two_l_m_1 = l + l - 1.;
      double sq_l = l * l;
      double sq_l_m_1 = (l - 1.) * (l - 1.);

      /* block 1: three-term recurrence in l */
      for (mp = 0; mp <= l - 2; mp++)
        {
          double sq_mp = mp * mp;
          for (m = -mp; m <= mp; m++)
            {
              double sq_m = m * m;
              double a = (l * two_l_m_1) / sqrt ((sq_l - sq_mp) * (sq_l - sq_m));
              double complex b = (d100 - ((mp * m) / (l * (l - 1.))));
              double c = sqrt ((sq_l_m_1 - sq_mp) * (sq_l_m_1 - sq_m)) /
                ((l - 1.) * two_l_m_1);
              WT (aw, l, mp, m) = a * (b * WT (aw, l - 1, mp, m) -
                                       c * WT (aw, l - 2, mp, m));
            }
        }
      /* blocks 2-3: corner terms */
      WT (aw, l, l, l) = d111 * WT (aw, l - 1, l - 1, l - 1);
      WT (aw, l, l - 1, l - 1) = (l * d100 - l + 1.) *
        WT (aw, l - 1, l - 1, l - 1);
      WT (aw, l, l, -l) = d11m1 * WT (aw, l - 1, l - 1, -(l - 1));
      WT (aw, l, l - 1, -(l - 1)) = (l * d100 + l - 1.) *
        WT (aw, l - 1, l - 1, -(l - 1));
      /* block 4: last column */
      for (mp = l; mp >= 1; mp--)
        WT (aw, l, mp - 1, l) = -sqrt ((l + mp) / (l - mp + 1.)) * tb2 *
          WT (aw, l, mp, l);
      /* block 5: penultimate column */
      for (mp = l - 1; mp >= 1; mp--)
        {
          double a = sqrt (((double) l + mp) / (((double) l + l) * (l - mp + 1.)));
          WT (aw, l, mp - 1, l - 1) = (l * cb - mp + 1.) * a *
            WT (aw, l, mp, l) / d111;
        }
      /* block 6: last rows by symmetry */
      for (mp = l - 1; mp <= l; mp++)
        for (m = 0; m < mp; m++)
          WT (aw, l, mp, m) = PHASE (mp + m) * WT (aw, l, m, mp);
      /* block 7 */
      for (m = 0; m < l; m++)
        WT (aw, l, l, -m - 1) = sqrt ((l - m) / (l + m + 1.)) * tb2 *
          WT (aw, l, l, -m);
      /* block 8 */
      for (m = 0; m < l; m++)
        {
          double a = sqrt (((double) l - m) / (((double) l + l) * (l + m + 1.)));
          WT (aw, l, l - 1, -m - 1) = (l * cb + m + 1.) * a *
            WT (aw, l, l, -m) / d111;
        }
      /* block 10: remaining terms by symmetry */
      for (mp = 0; mp <= l; mp++)
        for (m = mp + 1; m <= l; m++)
          {
            WT (aw, l, mp, m) = PHASE (m + mp) * WT (aw, l, m, mp);
            WT (aw, l, mp, -m) = WT (aw, l, m, -mp);
          }
    }
}

/* phases: aran/aranwigner.c:256-313 */
static void wigner_require (OrWigner *aw, int lmax)
{
  int l, mp, m;
  if (lmax <= aw->lmax)
    return;
  free (aw->t);
  aw->t = (double complex *) calloc (or_wigner_size (lmax),
                                     sizeof (double complex));
  wigner_d (aw, lmax);
  if (fabs (aw->alpha) >= 1.e-5)
    {
      double complex expa = cos (aw->alpha) - I * sin (aw->alpha);
      double complex *e = (double complex *) alloca ((lmax + 1) *
                                                     sizeof (double complex));
      e[0] = 1.;
      for (mp = 1; mp <= lmax; mp++)
        e[mp] = e[mp - 1] * expa;
      for (l = 0; l <= lmax; l++)
        for (mp = 0; mp <= l; mp++)
          {
            for (m = l; m >= 1; m--)
              WT (aw, l, mp, -m) *= conj (e[m]);
            for (m = 0; m <= l; m++)
              WT (aw, l, mp, m) *= e[m];
          }
    }
  if (fabs (aw->gamma) >= 1.e-5)
    {
      double complex expg = cos (aw->gamma) - I * sin (aw->gamma);
      double complex *e = (double complex *) alloca ((lmax + 1) *
                                                     sizeof (double complex));
      e[0] = 1.;
      for (mp = 1; mp <= lmax; mp++)
        e[mp] = e[mp - 1] * expg;
      for (l = 0; l <= lmax; l++)
        for (mp = 0; mp <= l; mp++)
          for (m = -l; m <= l; m++)
            WT (aw, l, mp, m) *= e[mp];
    }
  aw->lmax = lmax;
}

/* Rotation cache.  The reference keeps one AranWigner per angle triple in a
 * process-global GTree matched within 1e-3 (aran/aranwignerrepo.c:30-82).
 * Octree translations only ever produce angle triples that are either equal
 * up to rounding or differ by far more than 1e-3, so the oracle keys its
 * cache on the angles rounded to 1e-9. */
#define WCACHE 4096
static struct
{
  int used;
  int ready;          /* entry complete (published with release order) */
  int64_t k[3];
  OrWigner w;
} g_wc[WCACHE];

/* While several threads share the cache (or_wigner_cache_share), entries are
 * built under g_wc_mu to at least degree g_wc_floor and never change or go
 * away afterwards, so complete entries are read without the lock. */
static pthread_mutex_t g_wc_mu = PTHREAD_MUTEX_INITIALIZER;
static int g_wc_shared = 0;
static int g_wc_floor = 0;

void or_wigner_cache_clear (void)
{
  int i;
  for (i = 0; i < WCACHE; i++)
    if (g_wc[i].used)
      {
        free (g_wc[i].w.t);
        g_wc[i].used = 0;
        g_wc[i].ready = 0;
      }
}

void or_wigner_cache_share (int lmax)
{
  or_wigner_cache_clear ();
  g_wc_floor = lmax;
  g_wc_shared = 1;
}

void or_wigner_cache_unshare (void)
{
  g_wc_shared = 0;
  g_wc_floor = 0;
}

static void wc_key (double a, double b, double g, int64_t k[3], int *slot)
{
  uint64_t h;
  k[0] = llround (a * 1e9);
  k[1] = llround (b * 1e9);
  k[2] = llround (g * 1e9);
  h = (uint64_t) k[0] * 0x9E3779B97F4A7C15ull ^
    (uint64_t) k[1] * 0xC2B2AE3D27D4EB4Full ^ (uint64_t) k[2] * 0x165667B19E3779F9ull;
  *slot = (int) (h % WCACHE);
}

static int wigner_lookup (double a, double b, double g)
{
  int64_t k[3];
  int i, slot;
  wc_key (a, b, g, k, &slot);
  for (i = 0; i < WCACHE; i++)
    {
      int s = (slot + i) % WCACHE;
      if (!g_wc[s].used)
        {
          g_wc[s].used = 1;
          memcpy (g_wc[s].k, k, sizeof (k));
          g_wc[s].w.alpha = a;
          g_wc[s].w.beta = b;
          g_wc[s].w.gamma = g;
          g_wc[s].w.lmax = -1;
          g_wc[s].w.t = NULL;
          return s;
        }
      if (memcmp (g_wc[s].k, k, sizeof (k)) == 0)
        return s;
    }
  if (g_wc_shared)
    {
      fprintf (stderr, "oracle: Wigner cache full while shared\n");
      abort ();
    }
  /* cache full: start over */
  or_wigner_cache_clear ();
  return wigner_lookup (a, b, g);
}

/* the rotation of angles (a, b, g) up to degree lmax: aran_wigner_repo_lookup
 * + aran_wigner_require (aran/aranwignerrepo.c:57-82, aran/aranwigner.c:256-313) */
static const OrWigner *wigner_get (double a, double b, double g, int lmax)
{
  int s;
  if (g_wc_shared)
    {
      int64_t k[3];
      int i, slot;
      wc_key (a, b, g, k, &slot);
      for (i = 0; i < WCACHE; i++)
        {
          int e = (slot + i) % WCACHE;
          if (!__atomic_load_n (&g_wc[e].ready, __ATOMIC_ACQUIRE))
            break;
          if (memcmp (g_wc[e].k, k, sizeof (k)) == 0 && g_wc[e].w.lmax >= lmax)
            return &g_wc[e].w;
        }
      pthread_mutex_lock (&g_wc_mu);
    }
  s = wigner_lookup (a, b, g);
  if (g_wc_shared && g_wc[s].ready && g_wc[s].w.lmax < lmax)
    {
      fprintf (stderr, "oracle: shared Wigner entry below the requested degree\n");
      abort ();
    }
  wigner_require (&g_wc[s].w, lmax > g_wc_floor ? lmax : g_wc_floor);
  __atomic_store_n (&g_wc[s].ready, 1, __ATOMIC_RELEASE);
  if (g_wc_shared)
    pthread_mutex_unlock (&g_wc_mu);
  return &g_wc[s].w;
}

void or_wigner (double alpha, double beta, double gamma, int lmax,
                double *terms)
{
  OrWigner aw = { alpha, beta, gamma, -1, NULL };
  wigner_require (&aw, lmax);
  memcpy (terms, aw.t, or_wigner_size (lmax) * sizeof (double complex));
  free (aw.t);
}

/* per-degree rotation of a triangular block: aran/aransphericalseriesd-rotate.c:34-80 */
static void buffer_rotate (const OrWigner *aw, int deg,
                           const double complex *src, double complex *dst)
{
  double complex *sl = (double complex *) alloca ((deg + 1) *
                                                  sizeof (double complex));
  double complex *sln = (double complex *) alloca ((deg + 1) *
                                                   sizeof (double complex));
  int l, mp, m;
  for (l = 0; l <= deg; l++)
    {
      int o = TRI (l, 0);
      for (m = 0; m <= l; m++)
        {
          sl[m] = src[o + m];
          sln[m] = or_sph_sym (sl[m], m);
        }
      for (mp = 0; mp <= l; mp++)
        {
          double complex sum = 0.;
          for (m = -l; m < 0; m++)
            sum += WT (aw, l, mp, m) * sln[-m];
          for (m = 0; m <= l; m++)
            sum += WT (aw, l, mp, m) * sl[m];
          dst[o + mp] += sum;
        }
    }
}

static int imin (int a, int b) { return a < b ? a : b; }
static int imax (int a, int b) { return a > b ? a : b; }

/* aran/aransphericalseriesd-rotate.c:93-115 */
static void rotate_series (const OrSeries *src, double a, double b, double g,
                           OrSeries *dst)
{
  int nd = imin (dst->negdeg, src->negdeg);
  int pd = imin (dst->posdeg, src->posdeg);
  const OrWigner *aw = wigner_get (a, b, g, imax (pd + 1, nd));
  buffer_rotate (aw, src->posdeg, or_pos (src, 0, 0), or_pos (dst, 0, 0));
  if (src->negdeg > 0)
    buffer_rotate (aw, src->negdeg - 1, or_neg (src, 0, 0),
                   or_neg (dst, 0, 0));
}

/* aran/aransphericalseriesd-rotate.c:130-153 */
static void rotate_inverse_series (const OrSeries *src, double a, double b,
                                   double g, OrSeries *dst)
{
  int nd = imin (dst->negdeg, src->negdeg);
  int pd = imin (dst->posdeg, src->posdeg);
  const OrWigner *aw = wigner_get (-g, -b, -a, imax (pd + 1, nd));
  buffer_rotate (aw, pd, or_pos (src, 0, 0), or_pos (dst, 0, 0));
  if (nd > 0)
    buffer_rotate (aw, nd - 1, or_neg (src, 0, 0), or_neg (dst, 0, 0));
}

void or_rotate (int sp, int sn, const double *src, double alpha, double beta,
                double gamma, int dp, int dn, double *dst)
{
  OrSeries s = { sp, sn, (double complex *) src };
  OrSeries d = { dp, dn, (double complex *) dst };
  rotate_series (&s, alpha, beta, gamma, &d);
}

void or_rotate_inverse (int sp, int sn, const double *src, double alpha,
                        double beta, double gamma, int dp, int dn,
                        double *dst)
{
  OrSeries s = { sp, sn, (double complex *) src };
  OrSeries d = { dp, dn, (double complex *) dst };
  rotate_inverse_series (&s, alpha, beta, gamma, &d);
}

/* ------------------------------------------------------------------------
 * Vertical (z-axis) translations
 * ---------------------------------------------------------------------- */

/* L2L along z: aran/aransphericalseriesd-translate.c:301-364 */
static void local_translate_vertical (const OrSeries *src, OrSeries *dst,
                                      double r, double cost)
{
  int l, m, n;
  double *rpow = (double *) alloca ((src->posdeg + 1) * sizeof (double));
  double pw = 1.;
  for (l = 0; l <= src->posdeg; l++)
    {
      rpow[l] = pw;
      pw *= r;
    }
  for (l = 0; l <= dst->posdeg; l++)
    for (m = 0; m <= l; m++)
      {
        double complex *d = or_pos (dst, l, m);
        for (n = l; n <= src->posdeg; n++)
          {
            double normaliz = or_betal_over_betan (l, n);
            const double complex *s = or_pos (src, n, 0);
            double factor = or_alpha (n - l, 0) * or_alpha (l, m) /
              or_alpha (n, m);
            double h = ((n - l) % 2 == 0) ? 1. : cost;
            *d += h * s[m] * factor * normaliz * rpow[n - l];
          }
      }
}

/* M2M along z: aran/aransphericalseriesd-translate.c:445-505 */
static void multipole_translate_vertical (const OrSeries *src, OrSeries *dst,
                                          double r, double cost)
{
  int l, m, n;
  double *rpow = (double *) alloca ((dst->negdeg + 1) * sizeof (double));
  double pw = 1.;
  for (l = 0; l < dst->negdeg; l++)
    {
      rpow[l] = pw;
      pw *= r;
      for (m = 0; m <= l; m++)
        {
          double complex *d = or_neg (dst, l, m);
          for (n = m; n <= imin (l, src->negdeg - 1); n++)
            {
              double normaliz = or_betal_over_betan (l, n);
              const double complex *s = or_neg (src, n, 0);
              double factor = or_alpha (l - n, 0) * or_alpha (n, m) /
                or_alpha (l, m);
              double h = ((l - n) % 2 == 0) ? 1. : cost;
              *d += h * s[m] * factor * normaliz * rpow[l - n];
            }
        }
    }
}

/* aran/aransphericalseriesd-translate.c:581-594 */
static void translate_vertical (const OrSeries *src, OrSeries *dst, double r,
                                double cost)
{
  local_translate_vertical (src, dst, r, cost);
  if (src->negdeg > 0)
    multipole_translate_vertical (src, dst, r, -cost);
}

/* M2L along z with the precomputed table:
 * aran/aransphericalseriesd-translate.c:609-676 */
static void multipole_to_local_vertical (const OrSeries *src, OrSeries *dst,
                                         double r, double cost)
{
  int l, m, n;
  int d = dst->posdeg + src->negdeg;
  double *rpow = (double *) alloca ((d + 1) * sizeof (double));
  double pw = 1., inv_r = 1. / r;
  for (l = 0; l <= d; l++)
    {
      rpow[l] = pw;
      if (l % 2 == 0)
        rpow[l] *= cost;
      pw *= inv_r;
    }
  for (l = 0; l <= dst->posdeg; l++)
    for (m = 0; m <= l; m++)
      {
        double complex sum = 0.;
        double complex *dt = or_pos (dst, l, m);
        for (n = m; n < src->negdeg; n++)
          {
            double complex s = *or_neg (src, n, m);
            double tf = or_vertical_factor (l, m, n);
            sum += s * (rpow[l + n + 1] * tf);
          }
        sum = ((l + m) % 2 == 0) ? sum : -sum;
        *dt += sum;
      }
}

/* ------------------------------------------------------------------------
 * Normal flavour, O(p^4)
 * ---------------------------------------------------------------------- */

/* aran/aransphericalseriesd-translate.c:366-443 */
static void local_translate (const OrSeries *src, OrSeries *dst, double r,
                             double cost, double sint, double cosp,
                             double sinp)
{
  int l, m, n, o;
  int d = imax (src->posdeg, dst->posdeg);
  double *rpow = (double *) alloca ((src->posdeg + 1) * sizeof (double));
  double complex *h = (double complex *) alloca (TRI (d + 1, 0) *
                                                 sizeof (double complex));
  double pw = 1.;
  or_harmonics_c (src->posdeg, cost, sint, cosp + I * sinp, h);
  for (l = 0; l <= src->posdeg; l++)
    {
      rpow[l] = pw;
      pw *= r;
    }
  for (l = 0; l <= dst->posdeg; l++)
    for (m = 0; m <= l; m++)
      {
        double complex *dt = or_pos (dst, l, m);
        for (n = l; n <= src->posdeg; n++)
          {
            double normaliz = or_beta (n - l) * or_betal_over_betan (l, n);
            double complex sum = 0.;
            const double complex *s = or_pos (src, n, 0);
            const double complex *ht = h + TRI (n - l, 0);
            for (o = l + m - n; o <= m + n - l; o++)
              {
                int omm = o - m;
                int aomm = abs (omm);
                double factor = or_alpha (n - l, aomm) * or_alpha (l, m) /
                  or_alpha (n, abs (o));
                double complex hh = ht[aomm];
                if (omm < 0)
                  hh = or_sph_sym (hh, aomm);
                if (o >= 0)
                  hh *= s[o];
                else
                  hh *= or_sph_sym (s[-o], -o);
                sum += hh * factor;
              }
            *dt += sum * (normaliz * rpow[n - l]);
          }
      }
}

/* aran/aransphericalseriesd-translate.c:507-579 */
static void multipole_translate (const OrSeries *src, OrSeries *dst, double r,
                                 double cost, double sint, double cosp,
                                 double sinp)
{
  int l, m, n, o;
  int d = imax (src->negdeg, dst->negdeg) - 1;
  double *rpow = (double *) alloca ((dst->negdeg + 1) * sizeof (double));
  double complex *h = (double complex *) alloca (TRI (d + 2, 0) *
                                                 sizeof (double complex));
  double pw = 1.;
  or_harmonics_c (dst->negdeg - 1, cost, sint, cosp + I * sinp, h);
  for (l = 0; l < dst->negdeg; l++)
    {
      rpow[l] = pw;
      pw *= r;
      for (m = 0; m <= l; m++)
        {
          double complex *dt = or_neg (dst, l, m);
          for (n = 0; n <= imin (l, src->negdeg - 1); n++)
            {
              double normaliz = or_beta (l - n) * or_betal_over_betan (l, n);
              double complex sum = 0.;
              const double complex *s = or_neg (src, n, 0);
              const double complex *ht = h + TRI (l - n, 0);
              for (o = imax (-n, m + n - l); o <= imin (n, l + m - n); o++)
                {
                  int ammo = abs (m - o);
                  double factor = or_alpha (l - n, ammo) * or_alpha (n, abs (o)) /
                    or_alpha (l, abs (m));
                  double complex hh = conj (ht[ammo]);
                  if ((m - o) < 0)
                    hh = or_sph_sym (hh, ammo);
                  if (o >= 0)
                    hh *= s[o];
                  else
                    hh *= or_sph_sym (s[-o], -o);
                  sum += hh * factor;
                }
              *dt += sum * normaliz * rpow[l - n];
            }
        }
    }
}

/* aran/aransphericalseriesd-translate.c:678-773 */
static void multipole_to_local (const OrSeries *src, OrSeries *dst, double r,
                                double cost, double sint, double cosp,
                                double sinp)
{
  int l, m, n, o;
  int d = dst->posdeg + src->negdeg;
  double *rpow = (double *) alloca ((d + 1) * sizeof (double));
  double complex *h;
  double pw = 1., inv_r, sign;

  if (fabs (sint) < 1.e-5)
    {
      multipole_to_local_vertical (src, dst, r, cost);
      return;
    }
  h = (double complex *) alloca (TRI (d + 1, 0) * sizeof (double complex));
  or_harmonics_c (d, cost, sint, cosp + I * sinp, h);
  inv_r = 1. / r;
  for (l = 0; l <= d; l++)
    {
      rpow[l] = pw;
      pw *= inv_r;
    }
  sign = 1.;
  for (l = 0; l <= dst->posdeg; l++)
    {
      for (m = 0; m <= l; m++)
        {
          double complex *dt = or_pos (dst, l, m);
          for (n = 0; n < src->negdeg; n++)
            {
              double normaliz = or_beta (l + n) * or_betal_over_betan (l, n);
              double complex sum;
              const double complex *s = or_neg (src, n, 0);
              const double complex *ht = h + TRI (l + n, 0);
              sum = or_alpha (l, m) * or_alpha (n, 0) / or_alpha (l + n, m) *
                ht[m] * s[0];
              for (o = 1; o <= n; o++)
                {
                  int mpo = m + o;
                  double factor = or_alpha (l, m) * or_alpha (n, o);
                  double complex hh = ht[mpo];
                  sum += hh * s[o] * factor / or_alpha (l + n, mpo);
                  mpo = abs (m - o);
                  hh = ht[mpo];
                  if ((m - o) < 0)
                    hh = or_sph_sym (hh, mpo);
                  sum += hh * or_sph_sym (s[o], o) * factor /
                    or_alpha (l + n, mpo);
                }
              *dt += conj (sum) * sign * normaliz * rpow[l + n + 1];
            }
        }
      sign = -sign;
    }
}

/* ------------------------------------------------------------------------
 * kkylin flavour, O(p^3): aran/aransphericalseriesd-kkylin.c
 * ---------------------------------------------------------------------- */

/* aran/aransphericalseriesd-kkylin.c:32-209 */
static void multipole_translate_kkylin (const OrSeries *src, OrSeries *dst,
                                        double r, double cost, double sint,
                                        double cosp, double sinp)
{
  int l, m, n, o;
  int d = imax (src->negdeg, dst->negdeg) - 1;
  double *rpow;
  double complex *h, *buf1, *buf2, *partial, *partial_m_1, *flip;
  double complex expp = cosp + I * sinp;
  double complex f_sint_expp;
  double pw;
  const double complex *s;
  double complex *dt;
  int W = d + 1;

  if (src->negdeg > dst->negdeg || dst->negdeg == 0)
    return;
  rpow = (double *) alloca ((dst->negdeg + 1) * sizeof (double));
  h = (double complex *) alloca (TRI (d + 1, 0) * sizeof (double complex));
  buf1 = (double complex *) alloca (W * W * sizeof (double complex));
  buf2 = (double complex *) alloca (W * W * sizeof (double complex));
  partial = buf1;
  partial_m_1 = buf2;
#define P(a, mm, nn) ((a)[(mm) * W + (nn)])

  or_harmonics_c (dst->negdeg - 1, cost, sint, expp, h);
  pw = 1.;
  rpow[0] = pw;
  pw *= r;
  s = or_neg (src, 0, 0);
  P (partial, 0, 0) = conj (h[0]) * s[0];
  dt = or_neg (dst, 0, 0);
  dt[0] += P (partial, 0, 0) * or_beta (0);

  for (l = 1; l < dst->negdeg; l++)
    {
      double fact;
      rpow[l] = pw;
      pw *= r;
      flip = partial;
      partial = partial_m_1;
      partial_m_1 = flip;
      dt = or_neg (dst, l, 0);
      for (n = 0; n <= l - 1; n++)
        {
          const double complex *ht = h + TRI (l - n, 0);
          s = or_neg (src, n, 0);
          fact = or_beta (l - n) / or_beta (n);
          P (partial, 0, n) = 0.;
          for (o = imax (-n, n - l); o <= imin (n, l - n); o++)
            {
              int ao = abs (o);
              double complex hh = ht[ao];
              double complex ss = s[ao];
              if (o > 0)
                hh = or_sph_sym (hh, ao);
              else if (o < 0)
                ss = or_sph_sym (ss, ao);
              P (partial, 0, n) += (rpow[l - n] * or_alpha (n, ao) *
                                    or_alpha (l - n, ao)) * conj (hh) * ss;
            }
          P (partial, 0, n) *= fact;
          if (l > 1)
            {
              P (partial, l - 1, n) = 0.;
              for (o = imax (-n, n - 1); o <= imin (n, l + l - 1 - n); o++)
                {
                  int ao = abs (o);
                  double complex hh = ht[abs (l - o - 1)];
                  double complex ss = s[ao];
                  if ((l - o - 1) < 0)
                    hh = or_sph_sym (hh, abs (l - o - 1));
                  if (o < 0)
                    ss = or_sph_sym (ss, ao);
                  P (partial, l - 1, n) +=
                    (rpow[l - n] * or_alpha (n, ao) *
                     or_alpha (l - n, abs (l - o - 1))) * conj (hh) * ss;
                }
              P (partial, l - 1, n) *= fact;
            }
          P (partial, l, n) = 0.;
          for (o = imax (-n, n); o <= imin (n, l + l - n); o++)
            {
              int ao = abs (o);
              double complex hh = ht[abs (l - o)];
              double complex ss = s[ao];
              if ((l - o) < 0)
                hh = or_sph_sym (hh, abs (l - o));
              if (o < 0)
                ss = or_sph_sym (ss, ao);
              P (partial, l, n) += (rpow[l - n] * or_alpha (n, ao) *
                                    or_alpha (l - n, abs (l - o))) *
                conj (hh) * ss;
            }
          P (partial, l, n) *= fact;
          fact = 0.5 * r / (l - n);
          f_sint_expp = fact * sint * expp;
          fact *= 2. * cost;
          for (m = 1; m < l - 1; m++)
            P (partial, m, n) = f_sint_expp * P (partial_m_1, m + 1, n) -
              conj (f_sint_expp) * P (partial_m_1, m - 1, n) +
              fact * P (partial_m_1, m, n);
        }
      fact = or_beta (0) / or_beta (l);
      for (m = 0; m <= l; m++)
        P (partial, m, l) = (or_alpha (l, m) * fact) * conj (h[0]) *
          *or_neg (src, l, m);
      for (m = 0; m <= l; m++)
        {
          double complex sum = 0.;
          for (n = 0; n <= l; n++)
            sum += P (partial, m, n);
          dt[m] += sum * (or_beta (l) / or_alpha (l, m));
        }
    }
#undef P
}

/* aran/aransphericalseriesd-kkylin.c:211-362 */
static void local_translate_kkylin (const OrSeries *src, OrSeries *dst,
                                    double r, double cost, double sint,
                                    double cosp, double sinp)
{
  int l, m, n, o;
  int d = imax (src->posdeg, dst->posdeg);
  int W = d + 1;
  double *rpow = (double *) alloca ((src->posdeg + 1) * sizeof (double));
  double complex *h = (double complex *) alloca (TRI (d + 1, 0) *
                                                 sizeof (double complex));
  double complex *buf1 = (double complex *) alloca (W * W * sizeof (double complex));
  double complex *buf2 = (double complex *) alloca (W * W * sizeof (double complex));
  double complex *partial = buf1, *partial_p_1 = buf2, *flip;
  double complex expp = cosp + I * sinp;
  double complex f_sint_expp, y00;
  double pw;

  if (src->posdeg > dst->posdeg)
    return;
#define P(a, mm, nn) ((a)[(mm) * W + (nn)])
  or_harmonics_c (src->posdeg, cost, sint, expp, h);
  y00 = h[0];
  pw = 1.;
  for (l = 0; l <= src->posdeg; l++)
    {
      rpow[l] = pw;
      pw *= r;
    }
  for (l = dst->posdeg; l >= 0; l--)
    {
      double fact;
      double complex *dt = or_pos (dst, l, 0);
      if (l <= src->posdeg)
        {
          const double complex *s = or_pos (src, l, 0);
          fact = or_beta (0) / or_beta (l);
          for (m = 0; m <= l; m++)
            P (partial, m, l) = fact / or_alpha (l, m) * conj (y00 * s[m]);
        }
      for (n = l + 1; n <= src->posdeg; n++)
        {
          const double complex *ht = h + TRI (n - l, 0);
          const double complex *s = or_pos (src, n, 0);
          fact = or_beta (n - l) / or_beta (n);
          P (partial, 0, n) = 0.;
          for (o = imax (-n, l - n); o <= imin (n, n - l); o++)
            {
              int ao = abs (o);
              double complex hh = ht[ao];
              double complex ss = s[ao];
              if (o < 0)
                {
                  hh = or_sph_sym (hh, ao);
                  ss = or_sph_sym (ss, ao);
                }
              P (partial, 0, n) += (rpow[n - l] * or_alpha (n - l, ao) /
                                    or_alpha (n, ao)) * conj (hh * ss);
            }
          P (partial, 0, n) *= fact;
          if (l > 0)
            {
              P (partial, l, n) = 0.;
              for (o = imax (-n, l + l - n); o <= n; o++)
                {
                  int ao = abs (o);
                  double complex hh = ht[abs (o - l)];
                  double complex ss = s[ao];
                  if ((o - l) < 0)
                    hh = or_sph_sym (hh, abs (o - l));
                  if (o < 0)
                    ss = or_sph_sym (ss, ao);
                  P (partial, l, n) += (rpow[n - l] *
                                        or_alpha (n - l, abs (o - l)) /
                                        or_alpha (n, ao)) * conj (hh * ss);
                }
              P (partial, l, n) *= fact;
            }
          fact = 0.5 * r / (n - l);
          f_sint_expp = fact * sint * expp;
          fact *= 2. * cost;
          for (m = 1; m < l; m++)
            P (partial, m, n) = f_sint_expp * P (partial_p_1, m - 1, n) -
              conj (f_sint_expp) * P (partial_p_1, m + 1, n) +
              fact * P (partial_p_1, m, n);
        }
      for (m = 0; m <= l; m++)
        {
          double complex sum = 0.;
          for (n = l; n <= src->posdeg; n++)
            sum += P (partial, m, n);
          dt[m] += conj (sum) * (or_beta (l) * or_alpha (l, m));
        }
      flip = partial;
      partial = partial_p_1;
      partial_p_1 = flip;
    }
#undef P
}

/* aran/aransphericalseriesd-kkylin.c:364-517 */
static void multipole_to_local_kkylin (const OrSeries *src, OrSeries *dst,
                                       double r, double cost, double sint,
                                       double cosp, double sinp)
{
  int l, m, n, o;
  int d = dst->posdeg + src->negdeg;
  int W = d + 1;
  double *rpow;
  double complex *h, *buf1, *buf2, *partial, *partial_m_1, *flip;
  double complex expp = cosp + I * sinp;
  double complex two_cott_expp, exp2p, tl;
  double pw, inv_r, sign;

  if (src->negdeg - 1 > dst->posdeg)
    return;
  if (fabs (sint) < 1.e-5)
    {
      multipole_to_local_vertical (src, dst, r, cost);
      return;
    }
#define P(a, mm, nn) ((a)[(mm) * W + (nn)])
  rpow = (double *) alloca ((d + 1) * sizeof (double));
  h = (double complex *) alloca (TRI (d + 1, 0) * sizeof (double complex));
  buf1 = (double complex *) alloca (W * W * sizeof (double complex));
  buf2 = (double complex *) alloca (W * W * sizeof (double complex));
  partial = buf1;
  partial_m_1 = buf2;
  or_harmonics_c (d, cost, sint, expp, h);
  inv_r = 1. / r;
  pw = 1.;
  for (l = 0; l <= d; l++)
    {
      rpow[l] = pw;
      pw *= inv_r;
    }
  sign = 1.;
  for (l = 0; l <= dst->posdeg; l++)
    {
      double fact;
      double complex *dt = or_pos (dst, l, 0);
      for (n = 0; n < src->negdeg; n++)
        {
          const double complex *ht = h + TRI (l + n, 0);
          const double complex *s = or_neg (src, n, 0);
          fact = rpow[l + n + 1] * or_beta (l + n) / or_beta (n);
          P (partial, 0, n) = 0.;
          for (o = -n; o <= n; o++)
            {
              int ao = abs (o);
              double complex hh = ht[ao];
              double complex ss = s[ao];
              if (o < 0)
                {
                  hh = or_sph_sym (hh, ao);
                  ss = or_sph_sym (ss, ao);
                }
              P (partial, 0, n) += (or_alpha (n, ao) / or_alpha (l + n, ao)) *
                hh * ss;
            }
          P (partial, 0, n) *= fact;
          if (l > 0)
            {
              P (partial, 1, n) = 0.;
              for (o = -n; o <= n; o++)
                {
                  int ao = abs (o);
                  double complex hh = ht[abs (o + 1)];
                  double complex ss = s[ao];
                  if ((o + 1) < 0)
                    hh = or_sph_sym (hh, abs (o + 1));
                  if (o < 0)
                    ss = or_sph_sym (ss, ao);
                  P (partial, 1, n) += (or_alpha (n, ao) /
                                        or_alpha (l + n, abs (o + 1))) * hh * ss;
                }
              P (partial, 1, n) *= fact;
            }
          two_cott_expp = 2. * cost / sint * expp;
          exp2p = expp * expp;
          tl = 2. * (l + n) * inv_r / sint * expp;
          for (m = 2; m <= l; m++)
            P (partial, m, n) = two_cott_expp * P (partial, m - 1, n) +
              exp2p * P (partial, m - 2, n) - tl * P (partial_m_1, m - 1, n);
        }
      fact = or_beta (l) * sign;
      for (m = 0; m <= l; m++)
        {
          double complex sum = 0.;
          for (n = 0; n < src->negdeg; n++)
            sum += P (partial, m, n);
          dt[m] += conj (sum) * (or_alpha (l, m) * fact);
        }
      flip = partial;
      partial = partial_m_1;
      partial_m_1 = flip;
      sign = -sign;
    }
#undef P
}

/* ------------------------------------------------------------------------
 * Flavour dispatch
 * ---------------------------------------------------------------------- */

static OrSeries series_tmp (int posdeg, int negdeg)
{
  OrSeries s;
  s.posdeg = posdeg;
  s.negdeg = negdeg;
  s.c = (double complex *) calloc (or_series_size (posdeg, negdeg),
                                   sizeof (double complex));
  return s;
}

/* M2M / L2L: aran_spherical_seriesd_translate{,_kkylin,_rotate}
 * (aran/aransphericalseriesd-translate.c:786-804,
 *  aran/aransphericalseriesd-kkylin.c:530-548,
 *  aran/aransphericalseriesd-rotate.c:219-263) */
void or_translate_series (int flavour, const OrSeries *src, const double xs[3],
                          OrSeries *dst, const double xd[3])
{
  double v[3] = { xd[0] - xs[0], xd[1] - xs[1], xd[2] - xs[2] };
  if (flavour == OR_ROTATE)
    {
      double r, theta, phi, cost = 1.;
      OrSeries rot = series_tmp (src->posdeg, src->negdeg);
      OrSeries trans = series_tmp (dst->posdeg, dst->negdeg);
      if (v[2] < 0.)
        {
          cost = -1.;
          v[0] = -v[0];
          v[1] = -v[1];
          v[2] = -v[2];
        }
      or_to_spherical_angles (v, &r, &theta, &phi);
      rotate_series (src, -phi, theta, 0., &rot);
      translate_vertical (&rot, &trans, r, cost);
      rotate_inverse_series (&trans, -phi, theta, 0., dst);
      free (rot.c);
      free (trans.c);
      return;
    }
  {
    double r, cost, sint, cosp, sinp;
    or_to_spherical_internal (v, &r, &cost, &sint, &cosp, &sinp);
    if (flavour == OR_KKYLIN)
      {
        local_translate_kkylin (src, dst, r, cost, sint, cosp, sinp);
        if (src->negdeg > 0)
          multipole_translate_kkylin (src, dst, r, -cost, sint, -cosp, -sinp);
      }
    else
      {
        local_translate (src, dst, r, cost, sint, cosp, sinp);
        if (src->negdeg > 0)
          multipole_translate (src, dst, r, -cost, sint, -cosp, -sinp);
      }
  }
}

/* M2L: aran_spherical_seriesd_to_local{,_kkylin,_rotate}
 * (aran/aransphericalseriesd-translate.c:816-834,
 *  aran/aransphericalseriesd-kkylin.c:561-579,
 *  aran/aransphericalseriesd-rotate.c:165-207) */
void or_to_local_series (int flavour, const OrSeries *src, const double xs[3],
                         OrSeries *dst, const double xd[3])
{
  double v[3] = { xd[0] - xs[0], xd[1] - xs[1], xd[2] - xs[2] };
  if (flavour == OR_ROTATE)
    {
      double r, theta, phi, cost = 1.;
      OrSeries rot = series_tmp (src->posdeg, src->negdeg);
      OrSeries trans = series_tmp (dst->posdeg, dst->negdeg);
      if (v[2] < 0.)
        {
          cost = -1.;
          v[0] = -v[0];
          v[1] = -v[1];
          v[2] = -v[2];
        }
      or_to_spherical_angles (v, &r, &theta, &phi);
      rotate_series (src, -phi, theta, 0., &rot);
      multipole_to_local_vertical (&rot, &trans, r, cost);
      rotate_inverse_series (&trans, -phi, theta, 0., dst);
      free (rot.c);
      free (trans.c);
      return;
    }
  {
    double r, cost, sint, cosp, sinp;
    or_to_spherical_internal (v, &r, &cost, &sint, &cosp, &sinp);
    if (flavour == OR_KKYLIN)
      {
        local_translate_kkylin (src, dst, r, cost, sint, cosp, sinp);
        if (src->negdeg > 0)
          multipole_to_local_kkylin (src, dst, r, cost, sint, cosp, sinp);
      }
    else
      {
        local_translate (src, dst, r, cost, sint, cosp, sinp);
        if (src->negdeg > 0)
          multipole_to_local (src, dst, r, cost, sint, cosp, sinp);
      }
  }
}

void or_translate (int flavour, int sp, int sn, const double *src,
                   const double xs[3], int dp, int dn, double *dst,
                   const double xd[3])
{
  OrSeries s = { sp, sn, (double complex *) src };
  OrSeries d = { dp, dn, (double complex *) dst };
  or_translate_series (flavour, &s, xs, &d, xd);
}

void or_to_local (int flavour, int sp, int sn, const double *src,
                  const double xs[3], int dp, int dn, double *dst,
                  const double xd[3])
{
  OrSeries s = { sp, sn, (double complex *) src };
  OrSeries d = { dp, dn, (double complex *) dst };
  or_to_local_series (flavour, &s, xs, &d, xd);
}
