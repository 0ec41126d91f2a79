/*
 * aransolver3d.h -- LibAran's 3D solver API (aran/aransolver3d.h:33-214,
 * serial part) on the GPU library.
 *
 * A program written against LibAran keeps its calls: vsg_prtree3d_new_full,
 * aran_solver3d_new (..., aran_development3d_new (0, p), ...),
 * aran_solver3d_set_functions (p2p, p2m, m2m, m2l, l2l, l2p),
 * aran_solver3d_insert_point x N, aran_solver3d_solve,
 * aran_solver3d_get_stats, aran_solver3d_free.  It adds one call,
 * aran_solver3d_set_newton_layout, that tells the library where position,
 * charge and result sit in its point struct; the per-pair/per-particle user
 * callbacks are then replaced by the GPU Newton kernels (potential as in
 * tests/newtonpot3.c, field as in tests/newtonfield3.c) and the m2m/m2l/l2l
 * addresses select the flavour (normal and rotate run the rotation
 * kernels, kkylin its own).  aran_solver3d_solve adds
 * the result into each point's result member, as the reference's callbacks
 * accumulate.  Anything the GPU path cannot run (unknown operator
 * callbacks, no layout) makes aran_solver3d_solve return without touching
 * the points and sets aran_gpu_last_error(); there is no CPU fallback.
 */
#ifndef ARAN_COMPAT_SOLVER3D_H
#define ARAN_COMPAT_SOLVER3D_H

#include <aran/aran.h>
#include <aran/arandevelopment3d.h>
#include <vsg/vsgd.h>

G_BEGIN_DECLS

typedef struct _AranSolver3d AranSolver3d;

typedef void (*AranParticleInitFunc3d) (VsgPoint3 particle);
typedef void (*AranParticle2ParticleFunc3d) (VsgPoint3 src, VsgPoint3 dst);
typedef void (*AranParticle2MultipoleFunc3d) (VsgPoint3 src, const VsgPRTree3dNodeInfo *dst_node,
                                              gpointer dst);
typedef AranParticle2MultipoleFunc3d AranParticle2LocalFunc3d;
typedef void (*AranLocal2ParticleFunc3d) (const VsgPRTree3dNodeInfo *src_node, gpointer src,
                                          VsgPoint3 dst);
typedef AranLocal2ParticleFunc3d AranMultipole2ParticleFunc3d;
typedef void (*AranMultipole2MultipoleFunc3d) (const VsgPRTree3dNodeInfo *src_node, gpointer src,
                                                const VsgPRTree3dNodeInfo *dst_node, gpointer dst);
typedef void (*AranMultipole2LocalFunc3d) (const VsgPRTree3dNodeInfo *src_node, gpointer src,
                                           const VsgPRTree3dNodeInfo *dst_node, gpointer dst);
typedef void (*AranLocal2LocalFunc3d) (const VsgPRTree3dNodeInfo *src_node, gpointer src,
                                       const VsgPRTree3dNodeInfo *dst_node, gpointer dst);

/* result kinds of aran_solver3d_set_newton_layout */
#define ARAN_NEWTON_POTENTIAL 0  /* result is a gcomplex128 accumulator (newtonpot3) */
#define ARAN_NEWTON_FIELD 1      /* result is a VsgVector3d field (newtonfield3) */

AranSolver3d *aran_solver3d_new (VsgPRTree3d *prtree, GType devel_type, gpointer devel,
                                 AranZeroFunc zero);
void aran_solver3d_free (AranSolver3d *solver);
void aran_solver3d_set_development (AranSolver3d *solver, GType devel_type, gpointer devel,
                                    AranZeroFunc zero);
void aran_solver3d_set_functions (AranSolver3d *solver, AranParticle2ParticleFunc3d p2p,
                                  AranParticle2MultipoleFunc3d p2m,
                                  AranMultipole2MultipoleFunc3d m2m,
                                  AranMultipole2LocalFunc3d m2l, AranLocal2LocalFunc3d l2l,
                                  AranLocal2ParticleFunc3d l2p);
void aran_solver3d_set_functions_full (AranSolver3d *solver, AranParticle2ParticleFunc3d p2p,
                                       AranParticle2MultipoleFunc3d p2m,
                                       AranMultipole2MultipoleFunc3d m2m,
                                       AranMultipole2LocalFunc3d m2l, AranLocal2LocalFunc3d l2l,
                                       AranLocal2ParticleFunc3d l2p, AranParticle2LocalFunc3d p2l,
                                       AranMultipole2ParticleFunc3d m2p, guint semifar_threshold);
void aran_solver3d_reinit_stats (AranSolver3d *solver);
void aran_solver3d_get_stats (AranSolver3d *solver, glong *zero_count, glong *p2p_count,
                              glong *p2m_count, glong *m2m_count, glong *m2l_count,
                              glong *l2l_count, glong *l2p_count, glong *p2l_count,
                              glong *m2p_count, glong *p2p_remote_count,
                              glong *m2l_remote_count);
gdouble aran_solver3d_get_tolerance (AranSolver3d *solver);
void aran_solver3d_set_tolerance (AranSolver3d *solver, gdouble tolerance);
void aran_solver3d_get_bounds (AranSolver3d *solver, VsgVector3d *lbound, VsgVector3d *ubound);
guint aran_solver3d_depth (const AranSolver3d *solver);
guint aran_solver3d_point_count (const AranSolver3d *solver);
void aran_solver3d_insert_point (AranSolver3d *solver, VsgPoint3 point);
gboolean aran_solver3d_remove_point (AranSolver3d *solver, VsgPoint3 point);
void aran_solver3d_foreach_point (AranSolver3d *solver, GFunc func, gpointer user_data);
void aran_solver3d_solve (AranSolver3d *solver);
/* the semifar threshold used when set_functions_full was given 0
 * (aran/aransolver3d.c:1090-1127): (p2l + m2p) / p2p of the operator costs
 * set by aran_solver3d_db_profile_operators or _profile_operators; G_MAXUINT
 * without p2l/m2p or without costs */
guint aran_solver3d_optimal_semifar_threshold (AranSolver3d *solver);

/* aran/aransolver3d.c:663-685; like the reference, *p2p is not written */
void aran_solver3d_get_functions_full (AranSolver3d *solver, AranParticle2ParticleFunc3d *p2p,
                                       AranParticle2MultipoleFunc3d *p2m,
                                       AranMultipole2MultipoleFunc3d *m2m,
                                       AranMultipole2LocalFunc3d *m2l, AranLocal2LocalFunc3d *l2l,
                                       AranLocal2ParticleFunc3d *l2p, AranParticle2LocalFunc3d *p2l,
                                       AranMultipole2ParticleFunc3d *m2p,
                                       guint *semifar_threshold);
/* operator costs of the registered callbacks from the profile database
 * (aran_profile_db_address_eval at `order`, p2p at 0; as the reference,
 * aran/aransolver3d.c:687-740, the l2p cost is looked up under the p2p
 * address), printed to stderr */
void aran_solver3d_db_profile_operators (AranSolver3d *solver, gdouble order);
/* operator costs measured on the GPU (aran/aransolver3d.c:742-770 times
 * the callbacks on the host): a calibration solve of the solver's
 * configuration with semifar interactions on, each stage's CUDA-event time
 * divided by its operation count (p2p per directed pair, p2m/l2p per
 * particle, m2m/l2l per node, m2l per translation, p2l/m2p per particle).
 * point_init, p1 and p2 are accepted for source compatibility and unused. */
void aran_solver3d_profile_operators (AranSolver3d *solver, AranParticleInitFunc3d point_init,
                                      gpointer p1, gpointer p2);
/* serial: the same as aran_solver3d_insert_point; TRUE */
gboolean aran_solver3d_insert_point_local (AranSolver3d *solver, VsgPoint3 point);
/* a point whose position (the VsgVector3d at the start of the point) lies
 * within the tolerance (aran_solver3d_set_tolerance; 0: the same position)
 * of the selector's, or NULL (aran/aransolver3d.c:1024-1030) */
VsgPoint3 aran_solver3d_find_point (AranSolver3d *solver, VsgPoint3 selector);
/* func on every point for which locfunc (selector, point) returns
 * VSG_RLOC3_MASK, in tree order (aran/aransolver3d.c:1077-1088) */
void aran_solver3d_foreach_point_custom (AranSolver3d *solver, VsgRegion3 selector,
                                         VsgRegion3Point3LocFunc locfunc, GFunc func,
                                         gpointer user_data);
/* func on every node of the tree of the inserted points, in the given order
 * (G_IN_ORDER: first child, node, other children, as glib's n-ary trees)
 * (aran/aransolver3d.c:1057-1066).  The tree is the one the GPU builds;
 * user_data is the node's development (after a solve with the same points:
 * its multipole and local expansions, else zero); point_list holds a leaf's
 * points.  The node infos live for the duration of the call. */
void aran_solver3d_traverse (AranSolver3d *solver, GTraverseType order, VsgPRTree3dFunc func,
                             gpointer user_data);
/* children visited in Hilbert-curve order (J. Skilling's transpose
 * algorithm) or in the default octant order x + 2y + 4z by
 * aran_solver3d_traverse and foreach_point_custom; solve results do not
 * depend on it (aran/aransolver3d.c:1204-1217) */
void aran_solver3d_set_children_order_hilbert (AranSolver3d *solver);
void aran_solver3d_set_children_order_default (AranSolver3d *solver);
/* virtual leaves (aran/aransolver3d.c:1272-1279): a node about to be split
 * stays a leaf of the near/far interactions when isleaf (node_info,
 * user_data) is TRUE; node_info carries center, bounds, point_count and
 * depth.  See aran_gpu_solver3d_set_leaf_predicate. */
void aran_solver3d_set_nf_isleaf (AranSolver3d *solver, VsgPRTree3dNFIsleafFunc isleaf,
                                  gpointer user_data);

/* Additive: where the Newton data sits in the caller's point struct
 * (position: VsgVector3d at pos_offset, charge: gdouble at charge_offset,
 * result: gcomplex128 or VsgVector3d at result_offset, by kind). */
void aran_solver3d_set_newton_layout (AranSolver3d *solver, int kind, size_t pos_offset,
                                      size_t charge_offset, size_t result_offset);
/* Additive: aran_solver3d_solve returning its status (ARAN_OK or a negative
 * ARAN_ERR_* code of aran_gpu.h; the message is in aran_gpu_last_error()). */
int aran_solver3d_solve_try (AranSolver3d *solver);
/* Additive: ARAN_PRECISION_FP64 (default) or ARAN_PRECISION_MIXED of aran_gpu.h. */
void aran_solver3d_set_precision (AranSolver3d *solver, int precision);

G_END_DECLS

#endif
