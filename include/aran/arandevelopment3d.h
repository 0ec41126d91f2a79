/*
 * arandevelopment3d.h -- LibAran's 3D development (multipole + local pair) and
 * its operators (aran/arandevelopment3d.h:38-150) on the GPU library.
 *
 * The development object is the template a program hands to
 * aran_solver3d_new (aran_development3d_new (0, p) fixes the order p,
 * aran/arandevelopment3d.c:64-73).  Handed to aran_solver3d_set_functions the
 * operator addresses select what aran_solver3d_solve runs on the device (the
 * normal, kkylin or rotate flavour of M2M/M2L/L2L; the Newton P2M and L2P).
 * Called directly on host developments the operators run on the GPU one
 * launch per call (see aransphericalseriesd.h).
 */
#ifndef ARAN_COMPAT_DEVELOPMENT3D_H
#define ARAN_COMPAT_DEVELOPMENT3D_H

#include <stdio.h>

#include <aran/aran.h>
#include <aran/aransphericalseriesd.h>
#include <vsg/vsgd.h>

G_BEGIN_DECLS

#define ARAN_TYPE_DEVELOPMENT3D (aran_development3d_get_type ())

typedef struct _AranDevelopment3d AranDevelopment3d;
struct _AranDevelopment3d
{
  AranSphericalSeriesd *multipole;   /* series (posdeg, negdeg) */
  AranSphericalSeriesd *local;       /* series (max (posdeg, negdeg), 0) */
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
gcomplex128 aran_development3d_multipole_evaluate (const VsgPRTree3dNodeInfo *devel_node,
                                                   AranDevelopment3d *devel,
                                                   const VsgVector3d *pos);
gcomplex128 aran_development3d_local_evaluate (const VsgPRTree3dNodeInfo *devel_node,
                                               AranDevelopment3d *devel, const VsgVector3d *pos);
gcomplex128 aran_development3d_m2p (const VsgPRTree3dNodeInfo *devel_node,
                                    AranDevelopment3d *devel, const VsgVector3d *pos);
gcomplex128 aran_development3d_l2p (const VsgPRTree3dNodeInfo *devel_node,
                                    AranDevelopment3d *devel, const VsgVector3d *pos);
void aran_development3d_multipole_gradient_evaluate (const VsgPRTree3dNodeInfo *devel_node,
                                                     AranDevelopment3d *devel,
                                                     const VsgVector3d *pos, VsgVector3d *grad);
void aran_development3d_local_gradient_evaluate (const VsgPRTree3dNodeInfo *devel_node,
                                                 AranDevelopment3d *devel,
                                                 const VsgVector3d *pos, VsgVector3d *grad);
void aran_development3d_m2pv (const VsgPRTree3dNodeInfo *devel_node, AranDevelopment3d *devel,
                              const VsgVector3d *pos, VsgVector3d *grad);
void aran_development3d_l2pv (const VsgPRTree3dNodeInfo *devel_node, AranDevelopment3d *devel,
                              const VsgVector3d *pos, VsgVector3d *grad);

G_END_DECLS

#endif
