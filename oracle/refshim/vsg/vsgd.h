/*
 * vsg/vsgd.h -- TEST INFRASTRUCTURE: the libvsg types and vector functions
 * the reference's operator layer uses (libvsg is not vendored with the
 * reference).  The spherical conversions follow the oracle's documented
 * conventions (oracle/or_series.c: r = 0 gives theta = 0, rho = 0 gives
 * phi = 0).
 */
#ifndef ORACLE_SHIM_VSGD_H
#define ORACLE_SHIM_VSGD_H
#include <glib.h>

typedef struct _VsgVector3d VsgVector3d;
struct _VsgVector3d
{
  gdouble x, y, z;
};
typedef struct _VsgVector2d VsgVector2d;
struct _VsgVector2d
{
  gdouble x, y;
};
typedef gpointer VsgPoint3;
typedef gpointer VsgPoint2;
typedef struct _VsgPRTree3d VsgPRTree3d;
typedef struct _VsgPRTree2d VsgPRTree2d;

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

void vsg_vector3d_sub (const VsgVector3d *a, const VsgVector3d *b, VsgVector3d *res);
void vsg_vector3d_scalp (const VsgVector3d *a, gdouble s, VsgVector3d *res);
void vsg_vector3d_to_spherical (const VsgVector3d *v, gdouble *r, gdouble *theta,
                                gdouble *phi);
void vsg_vector3d_to_spherical_internal (const VsgVector3d *v, gdouble *r, gdouble *cost,
                                         gdouble *sint, gdouble *cosp, gdouble *sinp);
#endif
