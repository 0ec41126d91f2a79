/*
 * arandevelopment2d.h -- LibAran's 2D development (multipole + local Laurent
 * series) and its operators (aran/arandevelopment2d.h:31-100) on the GPU
 * library.
 *
 * aran_development2d_new (0, p) is the template a program hands to
 * aran_solver2d_new (aran/arandevelopment2d.c:64-73).  The operators are
 * the callbacks of the reference; handed to aran_solver2d_set_functions
 * their addresses select the GPU 2D solve, and called directly they run on
 * the GPU one launch at a time (see aranlaurentseriesd.h).
 */
#ifndef ARAN_COMPAT_DEVELOPMENT2D_H
#define ARAN_COMPAT_DEVELOPMENT2D_H

#include <stdio.h>

#include <aran/aran.h>
#include <aran/aranlaurentseriesd.h>
#include <vsg/vsgd.h>

G_BEGIN_DECLS

#define ARAN_TYPE_DEVELOPMENT2D (aran_development2d_get_type ())

typedef struct _AranDevelopment2d AranDevelopment2d;
struct _AranDevelopment2d
{
  AranLaurentSeriesd *multipole;   /* laurent (posdeg, negdeg) */
  AranLaurentSeriesd *local;       /* laurent (max (posdeg, negdeg), 0) */
};

GType aran_development2d_get_type (void);
AranDevelopment2d *aran_development2d_new (guint8 posdeg, guint8 negdeg);
void aran_development2d_free (AranDevelopment2d *ad);
void aran_development2d_copy (const AranDevelopment2d *src, AranDevelopment2d *dst);
AranDevelopment2d *aran_development2d_clone (AranDevelopment2d *src);
void aran_development2d_set_zero (AranDevelopment2d *ad);
void aran_development2d_write (AranDevelopment2d *ad, FILE *file);

void aran_development2d_p2m (VsgVector2d *position, gdouble charge,
                             const VsgPRTree2dNodeInfo *dst_node, AranDevelopment2d *dst);
void aran_development2d_p2l (VsgVector2d *position, gdouble charge,
                             const VsgPRTree2dNodeInfo *dst_node, AranDevelopment2d *dst);
void aran_development2d_m2m (const VsgPRTree2dNodeInfo *src_node, AranDevelopment2d *src,
                             const VsgPRTree2dNodeInfo *dst_node, AranDevelopment2d *dst);
void aran_development2d_m2l (const VsgPRTree2dNodeInfo *src_node, AranDevelopment2d *src,
                             const VsgPRTree2dNodeInfo *dst_node, AranDevelopment2d *dst);
void aran_development2d_l2l (const VsgPRTree2dNodeInfo *src_node, AranDevelopment2d *src,
                             const VsgPRTree2dNodeInfo *dst_node, AranDevelopment2d *dst);
gcomplex128 aran_development2d_multipole_evaluate (const VsgPRTree2dNodeInfo *devel_node,
                                                   AranDevelopment2d *devel,
                                                   const VsgVector2d *pos);
gcomplex128 aran_development2d_local_evaluate (const VsgPRTree2dNodeInfo *devel_node,
                                               AranDevelopment2d *devel, const VsgVector2d *pos);
gcomplex128 aran_development2d_m2p (const VsgPRTree2dNodeInfo *devel_node,
                                    AranDevelopment2d *devel, const VsgVector2d *pos);
gcomplex128 aran_development2d_l2p (const VsgPRTree2dNodeInfo *devel_node,
                                    AranDevelopment2d *devel, const VsgVector2d *pos);

G_END_DECLS

#endif
