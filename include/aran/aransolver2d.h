/*
 * aransolver2d.h -- LibAran's 2D solver API (aran/aransolver2d.h, serial
 * part) on the GPU library: the twin of aransolver3d.h.
 *
 * A program written against LibAran (tests/dummypot.c:410-450) keeps its
 * calls and adds aran_solver2d_set_cauchy_layout, which tells the library
 * where position, density and accumulator sit in its point struct.  With
 * m2m/m2l/l2l the aran_development2d_* operators, aran_solver2d_solve runs
 * the Cauchy-kernel FMM (acc_i += sum_j q_j / (z_i - z_j), the p2p of
 * tests/dummypot.c:62-76) on the GPU and adds the result into each point's
 * accumulator.  Anything else is refused with aran_gpu_last_error() set and
 * the points untouched; there is no CPU fallback.
 */
#ifndef ARAN_COMPAT_SOLVER2D_H
#define ARAN_COMPAT_SOLVER2D_H

#include <aran/aran.h>
#include <aran/arandevelopment2d.h>
#include <vsg/vsgd.h>

G_BEGIN_DECLS

typedef struct _AranSolver2d AranSolver2d;

typedef void (*AranParticleInitFunc2d) (VsgPoint2 particle);
typedef void (*AranParticle2ParticleFunc2d) (VsgPoint2 src, VsgPoint2 dst);
typedef void (*AranParticle2MultipoleFunc2d) (VsgPoint2 src, const VsgPRTree2dNodeInfo *dst_node,
                                              gpointer dst);
typedef AranParticle2MultipoleFunc2d AranParticle2LocalFunc2d;
typedef void (*AranLocal2ParticleFunc2d) (const VsgPRTree2dNodeInfo *src_node, gpointer src,
                                          VsgPoint2 dst);
typedef AranLocal2ParticleFunc2d AranMultipole2ParticleFunc2d;
typedef void (*AranMultipole2MultipoleFunc2d) (const VsgPRTree2dNodeInfo *src_node, gpointer src,
                                                const VsgPRTree2dNodeInfo *dst_node, gpointer dst);
typedef void (*AranMultipole2LocalFunc2d) (const VsgPRTree2dNodeInfo *src_node, gpointer src,
                                           const VsgPRTree2dNodeInfo *dst_node, gpointer dst);
typedef void (*AranLocal2LocalFunc2d) (const VsgPRTree2dNodeInfo *src_node, gpointer src,
                                       const VsgPRTree2dNodeInfo *dst_node, gpointer dst);

AranSolver2d *aran_solver2d_new (VsgPRTree2d *prtree, GType devel_type, gpointer devel,
                                 AranZeroFunc zero);
void aran_solver2d_free (AranSolver2d *solver);
void aran_solver2d_set_development (AranSolver2d *solver, GType devel_type, gpointer devel,
                                    AranZeroFunc zero);
void aran_solver2d_set_functions (AranSolver2d *solver, AranParticle2ParticleFunc2d p2p,
                                  AranParticle2MultipoleFunc2d p2m,
                                  AranMultipole2MultipoleFunc2d m2m,
                                  AranMultipole2LocalFunc2d m2l, AranLocal2LocalFunc2d l2l,
                                  AranLocal2ParticleFunc2d l2p);
void aran_solver2d_set_functions_full (AranSolver2d *solver, AranParticle2ParticleFunc2d p2p,
                                       AranParticle2MultipoleFunc2d p2m,
                                       AranMultipole2MultipoleFunc2d m2m,
                                       AranMultipole2LocalFunc2d m2l, AranLocal2LocalFunc2d l2l,
                                       AranLocal2ParticleFunc2d l2p, AranParticle2LocalFunc2d p2l,
                                       AranMultipole2ParticleFunc2d m2p, guint semifar_threshold);
void aran_solver2d_reinit_stats (AranSolver2d *solver);
void aran_solver2d_get_stats (AranSolver2d *solver, glong *zero_count, glong *p2p_count,
                              glong *p2m_count, glong *m2m_count, glong *m2l_count,
                              glong *l2l_count, glong *l2p_count, glong *p2l_count,
                              glong *m2p_count, glong *p2p_remote_count,
                              glong *m2l_remote_count);
gdouble aran_solver2d_get_tolerance (AranSolver2d *solver);
void aran_solver2d_set_tolerance (AranSolver2d *solver, gdouble tolerance);
void aran_solver2d_get_bounds (AranSolver2d *solver, VsgVector2d *lbound, VsgVector2d *ubound);
guint aran_solver2d_depth (const AranSolver2d *solver);
guint aran_solver2d_point_count (const AranSolver2d *solver);
void aran_solver2d_insert_point (AranSolver2d *solver, VsgPoint2 point);
gboolean aran_solver2d_remove_point (AranSolver2d *solver, VsgPoint2 point);
void aran_solver2d_foreach_point (AranSolver2d *solver, GFunc func, gpointer user_data);
void aran_solver2d_solve (AranSolver2d *solver);

/* The rest of aran/aransolver2d.h (serial), with the meaning of the 3D twins
 * in aran/aransolver3d.h: get_functions_full leaves *p2p unwritten;
 * db_profile_operators reads the costs of the registered operators from the
 * profile database (the l2p cost under the p2p address);
 * profile_operators times them on the GPU (a calibration solve of 100,000
 * uniform particles in the tree's box; p2l/m2p stay unknown: the 2D GPU
 * path has no semifar pass); the optimal semifar threshold is
 * (p2l + m2p) / p2p of those costs, G_MAXUINT while one is unknown;
 * foreach_point_custom visits the points for which locfunc returns
 * VSG_RLOC2_MASK; traverse walks the GPU quadtree (children in quadrant
 * order x + 2y or along the Hilbert curve); set_nf_isleaf keeps nodes about
 * to be split as leaves. */
void aran_solver2d_get_functions_full (AranSolver2d *solver, AranParticle2ParticleFunc2d *p2p,
                                       AranParticle2MultipoleFunc2d *p2m,
                                       AranMultipole2MultipoleFunc2d *m2m,
                                       AranMultipole2LocalFunc2d *m2l, AranLocal2LocalFunc2d *l2l,
                                       AranLocal2ParticleFunc2d *l2p, AranParticle2LocalFunc2d *p2l,
                                       AranMultipole2ParticleFunc2d *m2p,
                                       guint *semifar_threshold);
void aran_solver2d_db_profile_operators (AranSolver2d *solver, gdouble order);
void aran_solver2d_profile_operators (AranSolver2d *solver, AranParticleInitFunc2d point_init,
                                      gpointer p1, gpointer p2);
guint aran_solver2d_optimal_semifar_threshold (AranSolver2d *solver);
gboolean aran_solver2d_insert_point_local (AranSolver2d *solver, VsgPoint2 point);
void aran_solver2d_foreach_point_custom (AranSolver2d *solver, VsgRegion2 selector,
                                         VsgRegion2Point2LocFunc locfunc, GFunc func,
                                         gpointer user_data);
void aran_solver2d_traverse (AranSolver2d *solver, GTraverseType order, VsgPRTree2dFunc func,
                             gpointer user_data);
void aran_solver2d_set_children_order_hilbert (AranSolver2d *solver);
void aran_solver2d_set_children_order_default (AranSolver2d *solver);
void aran_solver2d_set_nf_isleaf (AranSolver2d *solver, VsgPRTree2dNFIsleafFunc isleaf,
                                  gpointer user_data);

/* Additive: where the Cauchy-kernel data sits in the caller's point struct
 * (position: VsgVector2d at pos_offset, density: gdouble at
 * density_offset, accumulator: gcomplex128 at accum_offset). */
void aran_solver2d_set_cauchy_layout (AranSolver2d *solver, size_t pos_offset,
                                      size_t density_offset, size_t accum_offset);
/* Additive: aran_solver2d_solve returning its status (ARAN_OK or a
 * negative ARAN_ERR_* code of aran_gpu.h). */
int aran_solver2d_solve_try (AranSolver2d *solver);

G_END_DECLS

#endif
