/*
 * aranpoly1d.h -- LibAran's polynomial in one variable (aran/aranpoly1d.h),
 * the cost model of the profile database: terms[i] is the coefficient of
 * x^i, evaluated by Horner's scheme.
 */
#ifndef ARAN_COMPAT_POLY1D_H
#define ARAN_COMPAT_POLY1D_H

#include <stdio.h>

#include <aran/aranglib.h>

G_BEGIN_DECLS

typedef struct _AranPoly1d AranPoly1d;
struct _AranPoly1d
{
  guint degree;
  gdouble *terms;
};

#define aran_poly1d_term(a, i) ((a)->terms[i])

AranPoly1d *aran_poly1d_new (guint deg);
AranPoly1d *aran_poly1d_new_with_terms (int degree, const double *terms);
void aran_poly1d_free (AranPoly1d *ap1d);
void aran_poly1d_write (AranPoly1d *ap1d, FILE *file);
void aran_poly1d_add (AranPoly1d *one, AranPoly1d *other, AranPoly1d *ret);
void aran_poly1d_sub (AranPoly1d *one, AranPoly1d *other, AranPoly1d *ret);
void aran_poly1d_scalp (AranPoly1d *ap1d, gdouble factor, AranPoly1d *ret);
gdouble aran_poly1d_eval (AranPoly1d *ap1d, gdouble x);

G_END_DECLS

#endif
