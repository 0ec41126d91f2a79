/* or_internal.h -- private declarations of the oracle (TEST INFRASTRUCTURE
 * ONLY; see aran_oracle.h). */
#ifndef OR_INTERNAL_H
#define OR_INTERNAL_H

#include "aran_oracle.h"

#include <alloca.h>
#include <complex.h>
#include <float.h>
#include <math.h>

#define OR_PI 3.1415926535897932384626433832795028841971693993751
#define OR_TMAX 160

typedef struct
{
  int posdeg;
  int negdeg;
  double complex *c;
} OrSeries;

double or_betal_over_betan (int l, int n);
void or_harmonics_c (int l, double cost, double sint, double complex expp,
                     double complex *res);
void or_pre_gradient_c (int l, double cost, double sint, double complex expp,
                        double complex *h, double complex *sh);
void or_to_spherical_internal (const double v[3], double *r, double *cost,
                               double *sint, double *cosp, double *sinp);
void or_to_spherical_angles (const double v[3], double *r, double *theta,
                             double *phi);
double complex *or_pos (const OrSeries *s, int l, int m);
double complex *or_neg (const OrSeries *s, int l, int m);
double complex or_sph_sym (double complex z, int m);
void or_p2m_series (const double x[3], double q, const double center[3],
                    OrSeries *dst);
void or_p2l_series (const double x[3], double q, const double center[3],
                    OrSeries *dst);
double complex or_evaluate_internal (const OrSeries *s, double r, double cost,
                                     double sint, double cosp, double sinp);
void or_gradient_xyz (const OrSeries *s, const double xrel[3], double g[3]);
void or_translate_series (int flavour, const OrSeries *src, const double xs[3],
                          OrSeries *dst, const double xd[3]);
void or_to_local_series (int flavour, const OrSeries *src, const double xs[3],
                         OrSeries *dst, const double xd[3]);
void or_wigner_cache_clear (void);
/* several threads are about to share the rotation cache: cleared, entries
 * built to at least degree lmax from now on (unshare: back to one thread) */
void or_wigner_cache_share (int lmax);
void or_wigner_cache_unshare (void);
void or_series_init (void);

#endif
