/*
 * vsgd.h -- the libvsg types and tree constructor LibAran's 3D solver API
 * takes (libvsg is not used: the GPU library builds its own octree).  The
 * reference programs create the tree with vsg_prtree3d_new_full
 * (tests/newtonfield3.c:615-619) and hand it to aran_solver3d_new.
 */
#ifndef ARAN_VSG_COMPAT_H
#define ARAN_VSG_COMPAT_H

#include <aran/aranglib.h>

G_BEGIN_DECLS

typedef struct _VsgVector3d VsgVector3d;
struct _VsgVector3d
{
  gdouble x, y, z;
};

/* a particle: any struct whose first member is a VsgVector3d */
typedef gpointer VsgPoint3;
typedef gpointer VsgRegion3;

typedef struct _VsgPRTree3d VsgPRTree3d;

/* the node view LibAran's operator callbacks receive
 * (fields read by aran/aransolver3d.c:254-490) */
typedef struct _VsgPRTree3dNodeInfo VsgPRTree3dNodeInfo;
struct _VsgPRTree3dNodeInfo
{
  VsgVector3d center;
  VsgVector3d lbound;
  VsgVector3d ubound;
  GSList *point_list;
  guint point_count;
  gboolean isleaf;
  guint depth;
  gpointer user_data;
  VsgPRTree3dNodeInfo *father_info;
  guint id;
};

typedef gint (*VsgPoint3dLocFunc) (const VsgPoint3 candidate, const VsgVector3d *center);
typedef gdouble (*VsgPoint3dDistFunc) (const VsgPoint3 one, const VsgPoint3 other);
typedef gint (*VsgRegion3dLocFunc) (const VsgRegion3 region, const VsgVector3d *center);

/* Creates the tree description the solver will build on the GPU: bounding
 * box and leaf capacity (vsg_prtree3d_new_full in libvsg; the location and
 * distance callbacks are accepted for source compatibility, the GPU tree
 * places VsgVector3d positions by their coordinates). */
VsgPRTree3d *vsg_prtree3d_new_full (const VsgVector3d *lbound,
                                    const VsgVector3d *ubound,
                                    VsgPoint3dLocFunc locfunc,
                                    VsgPoint3dDistFunc dist,
                                    VsgRegion3dLocFunc region_locfunc,
                                    guint maxbox);
void vsg_prtree3d_free (VsgPRTree3d *prtree);

/* the default location/distance functions of libvsg (identity tokens) */
gint vsg_vector3d_vector3d_locfunc (const VsgVector3d *candidate, const VsgVector3d *center);
gdouble vsg_vector3d_dist (const VsgVector3d *one, const VsgVector3d *other);

G_END_DECLS

#endif
