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

/* Serial trees share no node with another process. */
#define VSG_PRTREE3D_NODE_INFO_IS_SHARED(node_info) (FALSE)

/* Octant mask: bit o set when a region reaches octant o (x + 2y + 4z, a bit
 * set on the upper side) around a point; all eight bits: the region
 * surrounds the point. */
typedef guint8 vsgrloc3;
#define VSG_RLOC3_MASK ((vsgrloc3) 0xff)

typedef gint (*VsgPoint3dLocFunc) (const VsgPoint3 candidate, const VsgVector3d *center);
/* where a region lies around a point, as an octant mask */
typedef vsgrloc3 (*VsgRegion3Point3LocFunc) (const VsgRegion3 region, const VsgPoint3 point);
/* node visitor of aran_solver3d_traverse */
typedef void (*VsgPRTree3dFunc) (const VsgPRTree3dNodeInfo *node_info, gpointer user_data);
/* near/far traversal's is-leaf callback (aran_solver3d_set_nf_isleaf) */
typedef gboolean (*VsgPRTree3dNFIsleafFunc) (const VsgPRTree3dNodeInfo *node_info,
                                             gpointer user_data);
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

/* ---- 2D (the quadtree of aran/aransolver2d.c) ---- */
typedef struct _VsgVector2d VsgVector2d;
struct _VsgVector2d
{
  gdouble x, y;
};

typedef gpointer VsgPoint2;
typedef gpointer VsgRegion2;
typedef struct _VsgPRTree2d VsgPRTree2d;

typedef struct _VsgPRTree2dNodeInfo VsgPRTree2dNodeInfo;
struct _VsgPRTree2dNodeInfo
{
  VsgVector2d center;
  VsgVector2d lbound;
  VsgVector2d ubound;
  GSList *point_list;
  guint point_count;
  gboolean isleaf;
  guint depth;
  gpointer user_data;
  VsgPRTree2dNodeInfo *father_info;
  guint id;
};

#define VSG_PRTREE2D_NODE_INFO_IS_SHARED(node_info) (FALSE)

/* Quadrant mask: bit o set when a region reaches quadrant o (x + 2y, a bit
 * set on the upper side) around a point; all four bits: the region
 * surrounds the point. */
typedef guint8 vsgrloc2;
#define VSG_RLOC2_MASK ((vsgrloc2) 0xf)

typedef gint (*VsgPoint2dLocFunc) (const VsgPoint2 candidate, const VsgVector2d *center);
typedef vsgrloc2 (*VsgRegion2Point2LocFunc) (const VsgRegion2 region, const VsgPoint2 point);
typedef void (*VsgPRTree2dFunc) (const VsgPRTree2dNodeInfo *node_info, gpointer user_data);
typedef gboolean (*VsgPRTree2dNFIsleafFunc) (const VsgPRTree2dNodeInfo *node_info,
                                             gpointer user_data);
typedef gdouble (*VsgPoint2dDistFunc) (const VsgPoint2 one, const VsgPoint2 other);
typedef gint (*VsgRegion2dLocFunc) (const VsgRegion2 region, const VsgVector2d *center);

/* The 2D tree description (bounding box and leaf capacity) the solver
 * builds on the GPU (tests/dummypot.c:420-424). */
VsgPRTree2d *vsg_prtree2d_new_full (const VsgVector2d *lbound,
                                    const VsgVector2d *ubound,
                                    VsgPoint2dLocFunc locfunc,
                                    VsgPoint2dDistFunc dist,
                                    VsgRegion2dLocFunc region_locfunc,
                                    guint maxbox);
void vsg_prtree2d_free (VsgPRTree2d *prtree);
gint vsg_vector2d_vector2d_locfunc (const VsgVector2d *candidate, const VsgVector2d *center);
gdouble vsg_vector2d_dist (const VsgVector2d *one, const VsgVector2d *other);

G_END_DECLS

#endif
