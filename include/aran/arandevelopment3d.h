/*
 * arandevelopment3d.h -- LibAran's 3D development (multipole + local pair) and
 * its operators, as the GPU library exposes them.
 *
 * The development object is the template a program hands to
 * aran_solver3d_new (aran_development3d_new (0, p) fixes the order p,
 * aran/arandevelopment3d.c:64-73).  The operator functions are the callbacks
 * of the reference (aran/arandevelopment3d.c:169-552); with the GPU library
 * their addresses select what aran_solver3d_solve runs on the device (the
 * rotate or the kkylin flavour of M2M/M2L/L2L, the Newton P2M and L2P).
 * Calling an operator directly on host developments is not supported: it
 * leaves its output untouched and sets aran_gpu_last_error().
 */
#ifndef ARAN_COMPAT_DEVELOPMENT3D_H
#define ARAN_COMPAT_DEVELOPMENT3D_H

#include <stdio.h>

#include <aran/aran.h>
#include <vsg/vsgd.h>

G_BEGIN_DECLS

#define ARAN_TYPE_DEVELOPMENT3D (aran_development3d_get_type ())

typedef struct _AranDevelopment3d AranDevelopment3d;
struct _AranDevelopment3d
{
  guint8 posdeg;          /* multipole series: aran_spherical_seriesd_new (posdeg, negdeg) */
  guint8 negdeg;
  gcomplex128 *multipole; /* LibAran layout, ((posdeg+1)(posdeg+2)+negdeg(negdeg+1))/2 terms */
  gcomplex128 *local;     /* degree max (posdeg, negdeg) */
};

GType aran_development3d_get_type (void);
AranDevelopment3d *aran_development3d_new (guint8 posdeg, guint8 negdeg);
void aran_development3d_free (AranDevelopment3d *ad);
void aran_development3d_copy (const AranDevelopment3d *src, AranDevelopment3d *dst);
AranDevelopment3d *aran_development3d_clone (AranDevelopment3d *src);
void aran_development3d_set_zero (AranDevelopment3d *ad);
void aran_development3d_write (AranDevelopment3d *ad, FILE *file);

void aran_development3d_p2m (const VsgVector3d *position, const gdouble charge,
                             const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst);
void aran_development3d_p2l (const VsgVector3d *position, const gdouble charge,
                             const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst);
void aran_development3d_m2m (const VsgPRTree3dNodeInfo *src_node, AranDevelopment3d *src,
                             const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst);
void aran_development3d_m2l (const VsgPRTree3dNodeInfo *src_node, AranDevelopment3d *src,
                             const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst);
void aran_development3d_l2l (const VsgPRTree3dNodeInfo *src_node, AranDevelopment3d *src,
                             const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst);
void aran_development3d_m2m_kkylin (const VsgPRTree3dNodeInfo *src_node, AranDevelopment3d *src,
                                    const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst);
void aran_development3d_m2l_kkylin (const VsgPRTree3dNodeInfo *src_node, AranDevelopment3d *src,
                                    const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst);
void aran_development3d_l2l_kkylin (const VsgPRTree3dNodeInfo *src_node, AranDevelopment3d *src,
                                    const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst);
void aran_development3d_m2m_rotate (const VsgPRTree3dNodeInfo *src_node, AranDevelopment3d *src,
                                    const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst);
void aran_development3d_m2l_rotate (const VsgPRTree3dNodeInfo *src_node, AranDevelopment3d *src,
                                    const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst);
void aran_development3d_l2l_rotate (const VsgPRTree3dNodeInfo *src_node, AranDevelopment3d *src,
                                    const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst);
gcomplex128 aran_development3d_local_evaluate (const VsgPRTree3dNodeInfo *devel_node,
                                               AranDevelopment3d *devel, const VsgVector3d *pos);
void aran_development3d_local_gradient_evaluate (const VsgPRTree3dNodeInfo *devel_node,
                                                 AranDevelopment3d *devel,
                                                 const VsgVector3d *pos, VsgVector3d *grad);

G_END_DECLS

#endif
