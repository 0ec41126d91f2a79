/*
 * or_series.c -- tables, Legendre functions, spherical harmonics and the
 * particle <-> series operators of the oracle (TEST INFRASTRUCTURE ONLY; see
 * aran_oracle.h).
 */
#include "or_internal.h"

#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------
 * Tables.  The reference grows each table lazily by doubling
 * (aran/aranbinomialbuffer@t@.c:107-139, arancoefficientbuffer@t@.c:93-116);
 * the recurrences do not depend on the allocated size, so the oracle fills
 * them once up to OR_TMAX.
 * ---------------------------------------------------------------------- */
static double *g_beta;      /* [OR_TMAX+1] */
static double *g_alpha;     /* triangular [(OR_TMAX+1)(OR_TMAX+2)/2] */
static double *g_hnorm;     /* triangular */
static int g_ready = 0;

#define TRI(l, m) (((l) * ((l) + 1)) / 2 + (m))

static void tables_init (void)
{
  int l, m;
  if (g_ready)
    return;
  g_beta = (double *) malloc ((OR_TMAX + 1) * sizeof (double));
  g_alpha = (double *) malloc (TRI (OR_TMAX + 1, 0) * sizeof (double));
  g_hnorm = (double *) malloc (TRI (OR_TMAX + 1, 0) * sizeof (double));

  /* beta_l = sqrt(4 pi / (2l+1)): aran/aransphericalseriesd.c:40-43 */
  for (l = 0; l <= OR_TMAX; l++)
    g_beta[l] = sqrt ((4. * OR_PI) / (l + l + 1.));

  /* alpha_l^m = 1/sqrt((l-m)!(l+m)!) by the recurrence of
   * aran/aransphericalseriesd.c:45-60 */
  for (l = 0; l <= OR_TMAX; l++)
    for (m = 0; m <= l; m++)
      {
        double v;
        if (l == 0)
          v = 1.;
        else if (m == 0)
          v = g_alpha[TRI (l - 1, 0)] / l;
        else if (l == m)
          v = g_alpha[TRI (l - 1, l - 1)] / sqrt ((l + l - 1.) * (l + l));
        else
          v = sqrt ((l - m + 1.) / (l + m)) * g_alpha[TRI (l, m - 1)];
        g_alpha[TRI (l, m)] = v;
      }

  /* Y_l^m normalisation sqrt((2l+1)/4pi (l-m)!/(l+m)!):
   * aran/aransphericalharmonic.c:31-38 (integer product under the sqrt) */
  for (l = 0; l <= OR_TMAX; l++)
    for (m = 0; m <= l; m++)
      {
        double v;
        if (m == 0)
          v = sqrt ((l + l + 1.) / (4. * OR_PI));
        else
          v = g_hnorm[TRI (l, m - 1)] /
            sqrt ((double) ((unsigned) (l - m + 1) * (unsigned) (l + m)));
        g_hnorm[TRI (l, m)] = v;
      }
  g_ready = 1;
}

void or_series_init (void)
{
  tables_init ();
}

double or_beta (int l)
{
  tables_init ();
  return g_beta[l];
}

double or_alpha (int l, int m)
{
  tables_init ();
  return g_alpha[TRI (l, m)];
}

double or_harmonic_norm (int l, int m)
{
  tables_init ();
  return g_hnorm[TRI (l, m)];
}

/* beta(l)/beta(n): aran/aransphericalseriesd-translate.c:119-123 */
double or_betal_over_betan (int l, int n)
{
  tables_init ();
  return g_beta[l] / g_beta[n];
}

/* T(l,m,n) = beta_l/beta_n alpha_l^m alpha_n^m / alpha_{l+n}^0:
 * aran/aransphericalseriesd-translate.c:259-268 */
double or_vertical_factor (int l, int m, int n)
{
  double normaliz = or_betal_over_betan (l, n);
  double factor = or_alpha (l, m) * or_alpha (n, m);
  return normaliz * factor / or_alpha (l + n, 0);
}

/* ------------------------------------------------------------------------
 * Associated Legendre functions with the Condon-Shortley phase:
 * aran/aranlegendre.c:135-169
 * ---------------------------------------------------------------------- */
void or_legendre_multiple (int l, double x, double s, double *res)
{
  int i, j;
  res[0] = 1.;
  if (l <= 0)
    return;
  res[TRI (1, 0)] = x;
  res[TRI (1, 1)] = -s;
  for (i = 2; i <= l; i++)
    {
      double *p = res + TRI (i, 0);
      const double *p1 = res + TRI (i - 1, 0);
      const double *p2 = res + TRI (i - 2, 0);
      for (j = 0; j < i - 1; j++)
        p[j] = ((i + i - 1) * x * p1[j] - (i + j - 1) * p2[j]) / (i - j);
      p[i - 1] = (i + i - 1) * x * p1[i - 1];
      p[i] = -(i + i - 1) * s * p1[i - 1];
    }
}

/* "special" Legendre values P_l^m / sin(theta) used by the gradient:
 * aran/aranlegendre.c:204-264 */
void or_legendre_special (int l, double x, double s, const double *leg,
                          double *spec)
{
  int i, j;
  double factor = DBL_MAX;
  const double *p;
  double *sp, *sp1, *sp2;

  if (s != 0.)
    factor = 1. / s;

  p = leg;
  sp = spec;
  sp[0] = p[0] * factor;
  if (l < 1)
    return;

  sp1 = sp;
  sp = spec + TRI (1, 0);
  sp[1] = -p[0];
  p = leg + TRI (1, 0);
  sp[0] = p[0] * factor;
  sp2 = NULL;
  for (i = 2; i <= l; i++)
    {
      sp2 = sp1;
      sp1 = sp;
      sp = spec + TRI (i, 0);
      sp[i] = -(i + i - 1.) * p[i - 1];
      p = leg + TRI (i, 0);
      sp[0] = p[0] * factor;
      for (j = 1; j < i - 1; j++)
        sp[j] = ((i + i - 1.) * x * sp1[j] - (i + j - 1.) * sp2[j]) / (i - j);
      sp[i - 1] = (i + i - 1.) * x * sp1[i - 1];
    }
}

/* Y_l^m for 0<=m<=l<=n: aran/aransphericalharmonic.c:149-184 */
void or_harmonics_c (int l, double cost, double sint, double complex expp,
                     double complex *res)
{
  int i, j;
  double *leg = (double *) alloca (TRI (l + 1, 0) * sizeof (double));
  double complex *epow = (double complex *) alloca ((l + 1) *
                                                    sizeof (double complex));
  double complex pw = 1.;
  const double *lp;
  const double *nrm;

  tables_init ();
  or_legendre_multiple (l, cost, sint, leg);
  lp = leg;
  nrm = g_hnorm;
  for (i = 0; i <= l; i++)
    {
      epow[i] = pw;
      for (j = 0; j <= i; j++)
        {
          *res = epow[j] * (*lp) * (*nrm);
          lp++;
          res++;
          nrm++;
        }
      pw *= expp;
    }
}

void or_harmonics (int l, double cost, double sint, double cosp, double sinp,
                   double *res)
{
  or_harmonics_c (l, cost, sint, cosp + I * sinp, (double complex *) res);
}

/* harmonics plus special harmonics for the gradient:
 * aran/aransphericalharmonic.c:229-276 */
void or_pre_gradient_c (int l, double cost, double sint, double complex expp,
                        double complex *h, double complex *sh)
{
  int i, j;
  double *leg = (double *) alloca (TRI (l + 1, 0) * sizeof (double));
  double *sleg = (double *) alloca (TRI (l + 1, 0) * sizeof (double));
  double complex *epow = (double complex *) alloca ((l + 1) *
                                                    sizeof (double complex));
  double complex pw = 1.;
  int k = 0;

  tables_init ();
  or_legendre_multiple (l, cost, sint, leg);
  or_legendre_special (l, cost, sint, leg, sleg);
  for (i = 0; i <= l; i++)
    {
      epow[i] = pw;
      for (j = 0; j <= i; j++)
        {
          double complex t = epow[j] * g_hnorm[k];
          h[k] = t * leg[k];
          sh[k] = t * sleg[k];
          k++;
        }
      pw *= expp;
    }
}

/* ------------------------------------------------------------------------
 * Spherical coordinates.  libvsg's vsg_vector3d_to_spherical_internal is not
 * vendored with the reference; this restates it from its use
 * (r, cos/sin theta, cos/sin phi) with the conventions: r = 0 gives
 * theta = 0; rho = sqrt(x^2+y^2) = 0 gives phi = 0.
 * ---------------------------------------------------------------------- */
void or_to_spherical_internal (const double v[3], double *r, double *cost,
                               double *sint, double *cosp, double *sinp)
{
  double rho2 = v[0] * v[0] + v[1] * v[1];
  double rho = sqrt (rho2);
  double rr = sqrt (rho2 + v[2] * v[2]);
  *r = rr;
  if (rr > 0.)
    {
      *cost = v[2] / rr;
      *sint = rho / rr;
    }
  else
    {
      *cost = 1.;
      *sint = 0.;
    }
  if (rho > 0.)
    {
      *cosp = v[0] / rho;
      *sinp = v[1] / rho;
    }
  else
    {
      *cosp = 1.;
      *sinp = 0.;
    }
}

/* angles version (vsg_vector3d_to_spherical, used by the rotate flavour) */
void or_to_spherical_angles (const double v[3], double *r, double *theta,
                             double *phi)
{
  double rho2 = v[0] * v[0] + v[1] * v[1];
  double rr = sqrt (rho2 + v[2] * v[2]);
  *r = rr;
  *theta = (rr > 0.) ? acos (v[2] / rr) : 0.;
  *phi = (rho2 > 0.) ? atan2 (v[1], v[0]) : 0.;
}

void or_to_spherical (const double v[3], double out[5])
{
  or_to_spherical_internal (v, out, out + 1, out + 2, out + 3, out + 4);
}

/* ------------------------------------------------------------------------
 * Series layout: aran/aransphericalseriesd-private.h:38-99
 * ---------------------------------------------------------------------- */
int or_series_size (int posdeg, int negdeg)
{
  return ((posdeg + 1) * (posdeg + 2) + negdeg * (negdeg + 1)) / 2;
}

double complex *or_pos (const OrSeries *s, int l, int m)
{
  return s->c + TRI (l, m);
}

double complex *or_neg (const OrSeries *s, int l, int m)
{
  return s->c + ((s->posdeg + 1) * (s->posdeg + 2) + l * (l + 1)) / 2 + m;
}

double complex or_sph_sym (double complex z, int m)
{
  z = conj (z);
  return (m % 2 != 0) ? -z : z;
}

/* ------------------------------------------------------------------------
 * P2M: aran/arandevelopment3d.c:169-216
 * M_l^m += q (4 pi/(2l+1)) r^l conj(Y_l^m), l < deg
 * ---------------------------------------------------------------------- */
void or_p2m_series (const double x[3], double q, const double center[3],
                    OrSeries *dst)
{
  int deg = dst->negdeg;
  int l, m;
  double tmp[3] = { x[0] - center[0], x[1] - center[1], x[2] - center[2] };
  double r, cost, sint, cosp, sinp, fact;
  double complex *h = (double complex *) alloca (TRI (deg + 1, 0) *
                                                 sizeof (double complex));

  or_to_spherical_internal (tmp, &r, &cost, &sint, &cosp, &sinp);
  or_harmonics_c (deg, cost, sint, cosp + I * sinp, h);
  *or_pos (dst, 0, 0) += 0.;
  fact = q;
  for (l = 0; l < deg; l++)
    {
      double complex *ptr = or_neg (dst, l, 0);
      for (m = 0; m <= l; m++)
        {
          double complex term = fact * (4. * OR_PI / (l + l + 1.)) *
            h[TRI (l, m)];
          ptr[m] += conj (term);
        }
      fact *= r;
    }
}

void or_p2m (const double x[3], double q, const double center[3], int deg,
             double *mult)
{
  OrSeries s = { 0, deg, (double complex *) mult };
  or_p2m_series (x, q, center, &s);
}

/* P2L: aran/arandevelopment3d.c:227-277
 * L_l^m += q (4 pi/(2l+1)) r^{-(l+1)} conj(Y_l^m), l <= deg */
void or_p2l_series (const double x[3], double q, const double center[3],
                    OrSeries *dst)
{
  int deg = dst->posdeg;
  int l, m;
  double tmp[3] = { x[0] - center[0], x[1] - center[1], x[2] - center[2] };
  double r, cost, sint, cosp, sinp, fact, inv_r;
  double complex *h = (double complex *) alloca (TRI (deg + 1, 0) *
                                                 sizeof (double complex));

  or_to_spherical_internal (tmp, &r, &cost, &sint, &cosp, &sinp);
  or_harmonics_c (deg, cost, sint, cosp + I * sinp, h);
  *or_pos (dst, 0, 0) += 0.;
  inv_r = 1. / r;
  fact = q * inv_r;
  for (l = 0; l <= deg; l++)
    {
      double complex *ptr = or_pos (dst, l, 0);
      for (m = 0; m <= l; m++)
        {
          double complex term = fact * (4. * OR_PI / (l + l + 1.)) *
            h[TRI (l, m)];
          ptr[m] += conj (term);
        }
      fact *= inv_r;
    }
}

void or_p2l (const double x[3], double q, const double center[3], int deg,
             double *local)
{
  OrSeries s = { deg, 0, (double complex *) local };
  or_p2l_series (x, q, center, &s);
}

/* ------------------------------------------------------------------------
 * Evaluation: aran/aransphericalseriesd.c:312-371
 * ---------------------------------------------------------------------- */
double complex or_evaluate_internal (const OrSeries *s, double r, double cost,
                                     double sint, double cosp, double sinp)
{
  int l, m;
  int n = s->posdeg > s->negdeg - 1 ? s->posdeg : s->negdeg - 1;
  double complex *h = (double complex *) alloca (TRI (n + 1, 0) *
                                                 sizeof (double complex));
  double complex res = 0.;

  or_harmonics_c (n, cost, sint, cosp + I * sinp, h);
  for (l = s->posdeg; l >= 0; l--)
    {
      double complex sum = 0.;
      const double complex *c = or_pos (s, l, 0);
      const double complex *ht = h + TRI (l, 0);
      for (m = 1; m <= l; m++)
        sum += creal (c[m] * ht[m]);
      sum = 2. * sum + c[0] * ht[0];
      res = res * r + sum;
    }
  if (s->negdeg != 0)
    {
      double complex negres = 0.;
      double invr = 1. / r;
      for (l = s->negdeg - 1; l >= 0; l--)
        {
          double complex sum = 0.;
          const double complex *c = or_neg (s, l, 0);
          const double complex *ht = h + TRI (l, 0);
          for (m = 1; m <= l; m++)
            sum += creal (c[m] * ht[m]);
          sum = 2. * sum + c[0] * ht[0];
          negres = (negres + sum) * invr;
        }
      res += negres;
    }
  return res;
}

void or_series_evaluate (int posdeg, int negdeg, const double *c,
                         const double xrel[3], double out[2])
{
  OrSeries s = { posdeg, negdeg, (double complex *) c };
  double r, cost, sint, cosp, sinp;
  double complex v;
  or_to_spherical_internal (xrel, &r, &cost, &sint, &cosp, &sinp);
  v = or_evaluate_internal (&s, r, cost, sint, cosp, sinp);
  out[0] = creal (v);
  out[1] = cimag (v);
}

/* gradient in spherical components: aran/aransphericalseriesd.c:419-519 */
void or_gradient_internal (const OrSeries *s, double r, double cost,
                           double sint, double cosp, double sinp,
                           double complex *dr, double complex *dt,
                           double complex *dp)
{
  int l, m;
  int n = s->posdeg > s->negdeg ? s->posdeg : s->negdeg;
  double complex expp = cosp + I * sinp;
  double complex *h = (double complex *) alloca (TRI (n + 1, 0) *
                                                 sizeof (double complex));
  double complex *sh = (double complex *) alloca (TRI (n + 1, 0) *
                                                  sizeof (double complex));

  or_pre_gradient_c (n, cost, sint, expp, h, sh);
  *dr = 0.;
  *dt = 0.;
  *dp = 0.;
  for (l = s->posdeg; l >= 1; l--)
    {
      double complex sumr = 0., sumt = 0., sump = 0.;
      const double complex *ht = h + TRI (l, 0);
      const double complex *sht = sh + TRI (l, 0);
      const double complex *c = or_pos (s, l, 0);
      for (m = 1; m <= l; m++)
        {
          sumr += creal (ht[m] * c[m]);
          sumt += creal (sht[m] * c[m]) * (cost * m);
          sump += cimag (sht[m] * c[m]) * m;
        }
      for (m = 1; m <= l - 1; m++)
        sumt += creal (ht[m + 1] * c[m] * conj (expp)) *
          sqrt ((double) ((l - m) * (l + m + 1)));
      sumr = 2. * sumr + creal (ht[0] * c[0]);
      sumt = 2. * sumt + creal (ht[1] * c[0] * conj (expp)) *
        sqrt ((double) (l * (l + 1)));
      sump *= -2.;
      *dr = (*dr) * r + sumr * l;
      *dt = (*dt) * r + sumt;
      *dp = (*dp) * r + sump;
    }
  if (s->negdeg > 0)
    {
      double dr2 = 0., dt2 = 0., dp2 = 0.;
      double invr = 1. / r;
      for (l = s->negdeg - 1; l >= 1; l--)
        {
          double complex sumr = 0., sumt = 0., sump = 0.;
          const double complex *ht = h + TRI (l, 0);
          const double complex *sht = sh + TRI (l, 0);
          const double complex *c = or_neg (s, l, 0);
          for (m = 1; m <= l; m++)
            {
              sumr += creal (ht[m] * c[m]);
              sumt += creal (sht[m] * c[m]) * (cost * m);
              sump += cimag (sht[m] * c[m]) * m;
            }
          for (m = 1; m <= l - 1; m++)
            sumt += creal (ht[m + 1] * c[m] * conj (expp)) *
              sqrt ((double) ((l - m) * (l + m + 1)));
          sumr = 2. * sumr + creal (ht[0] * c[0]);
          sumt = 2. * sumt + creal (ht[1] * c[0] * conj (expp)) *
            sqrt ((double) (l * (l + 1)));
          sump *= -2.;
          dr2 = dr2 * invr + creal (sumr) * (l + 1);
          dt2 = dt2 * invr + creal (sumt);
          dp2 = dp2 * invr + creal (sump);
        }
      {
        const double complex *c = or_neg (s, 0, 0);
        *dr += -invr * invr * (dr2 * invr + h[0] * c[0]);
        *dt += dt2 * invr * invr * invr;
        *dp += dp2 * invr * invr * invr;
      }
    }
}

/* Cartesian gradient: aran/aransphericalseriesd.c:394-403,530-546 */
void or_gradient_xyz (const OrSeries *s, const double xrel[3], double g[3])
{
  double r, cost, sint, cosp, sinp;
  double complex dr, dt, dp;
  double a, b, c;
  or_to_spherical_internal (xrel, &r, &cost, &sint, &cosp, &sinp);
  or_gradient_internal (s, r, cost, sint, cosp, sinp, &dr, &dt, &dp);
  a = creal (dr);
  b = creal (dt);
  c = creal (dp);
  g[0] = sint * cosp * a + cost * cosp * b - sinp * c;
  g[1] = sint * sinp * a + cost * sinp * b + cosp * c;
  g[2] = cost * a - sint * b;
}

void or_series_gradient (int posdeg, int negdeg, const double *c,
                         const double xrel[3], double grad[3])
{
  OrSeries s = { posdeg, negdeg, (double complex *) c };
  or_gradient_xyz (&s, xrel, grad);
}
