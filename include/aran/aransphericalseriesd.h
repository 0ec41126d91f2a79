/*
 * aransphericalseriesd.h -- LibAran's spherical-harmonic series
 * (aran/aransphericalseriesd.h:42-131) on the GPU library.
 *
 * A series of degrees (posdeg, negdeg) holds the local terms (l, m),
 * 0 <= m <= l <= posdeg, at l(l+1)/2 + m, then the multipole terms of degree
 * -(l+1), 0 <= m <= l < negdeg, at (posdeg+1)(posdeg+2)/2 + l(l+1)/2 + m
 * (aran/aransphericalseriesd-private.h:38-70); get_term (ass, i, j) returns
 * the term of degree i (i < 0: multipole degree -i-1) and order j >= 0, or
 * NULL outside the series.  The containers live in host memory; evaluate,
 * gradient, rotate, translate and to_local run on the GPU, one launch per
 * call, FP64.  All three translation flavours apply their operators through
 * the rotation factorisation (rotate, translate along z, rotate back), which
 * equals the normal and kkylin formulas to FP64 rounding.  Without a usable
 * GPU the computing calls leave their outputs untouched (return 0) and set
 * aran_gpu_last_error().
 */
#ifndef ARAN_COMPAT_SPHERICAL_SERIESD_H
#define ARAN_COMPAT_SPHERICAL_SERIESD_H

#include <stdio.h>

#include <aran/aran.h>
#include <vsg/vsgd.h>

G_BEGIN_DECLS

typedef struct _AranSphericalSeriesd AranSphericalSeriesd;

AranSphericalSeriesd *aran_spherical_seriesd_new (guint8 posdeg, guint8 negdeg);
void aran_spherical_seriesd_free (AranSphericalSeriesd *ass);
void aran_spherical_seriesd_copy (const AranSphericalSeriesd *src, AranSphericalSeriesd *dst);
AranSphericalSeriesd *aran_spherical_seriesd_clone (const AranSphericalSeriesd *src);
gcomplex128 *aran_spherical_seriesd_get_term (AranSphericalSeriesd *ass, gint i, gint j);
guint8 aran_spherical_seriesd_get_posdeg (const AranSphericalSeriesd *ass);
guint8 aran_spherical_seriesd_get_negdeg (const AranSphericalSeriesd *ass);
void aran_spherical_seriesd_set_zero (AranSphericalSeriesd *ass);
void aran_spherical_seriesd_write (const AranSphericalSeriesd *ass, FILE *file);
gcomplex128 aran_spherical_seriesd_evaluate_internal (const AranSphericalSeriesd *ass, gdouble r,
                                                      gdouble cost, gdouble sint,
                                                      gdouble cosp, gdouble sinp);
gcomplex128 aran_spherical_seriesd_evaluate (const AranSphericalSeriesd *ass,
                                             const VsgVector3d *x);
void aran_spherical_seriesd_gradient_evaluate_internal (const AranSphericalSeriesd *ass,
                                                        gdouble r, gdouble cost, gdouble sint,
                                                        gdouble cosp, gdouble sinp,
                                                        gcomplex128 *dr, gcomplex128 *dt,
                                                        gcomplex128 *dp);
void aran_spherical_seriesd_gradient_evaluate (const AranSphericalSeriesd *ass,
                                               const VsgVector3d *x, VsgVector3d *grad);
void aran_spherical_seriesd_add (AranSphericalSeriesd *one, AranSphericalSeriesd *other,
                                 AranSphericalSeriesd *result);
void aran_spherical_seriesd_translate (const AranSphericalSeriesd *src, const VsgVector3d *xsrc,
                                       AranSphericalSeriesd *dst, const VsgVector3d *xdst);
void aran_spherical_seriesd_to_local (const AranSphericalSeriesd *src, const VsgVector3d *xsrc,
                                      AranSphericalSeriesd *dst, const VsgVector3d *xdst);
void aran_spherical_seriesd_translate_kkylin (const AranSphericalSeriesd *src,
                                              const VsgVector3d *xsrc,
                                              AranSphericalSeriesd *dst,
                                              const VsgVector3d *xdst);
void aran_spherical_seriesd_to_local_kkylin (const AranSphericalSeriesd *src,
                                             const VsgVector3d *xsrc,
                                             AranSphericalSeriesd *dst,
                                             const VsgVector3d *xdst);
void aran_spherical_seriesd_rotate (const AranSphericalSeriesd *src, gdouble alpha,
                                    gdouble beta, gdouble gamma, AranSphericalSeriesd *dst);
void aran_spherical_seriesd_rotate_inverse (const AranSphericalSeriesd *src, gdouble alpha,
                                            gdouble beta, gdouble gamma,
                                            AranSphericalSeriesd *dst);
void aran_spherical_seriesd_translate_rotate (const AranSphericalSeriesd *src,
                                              const VsgVector3d *xsrc,
                                              AranSphericalSeriesd *dst,
                                              const VsgVector3d *xdst);
void aran_spherical_seriesd_to_local_rotate (const AranSphericalSeriesd *src,
                                             const VsgVector3d *xsrc,
                                             AranSphericalSeriesd *dst,
                                             const VsgVector3d *xdst);

G_END_DECLS

#endif
