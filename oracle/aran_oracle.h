/*
 * aran_oracle.h -- CPU restatement of LibAran's 3D (and 2D) FMM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The GPU path is tested against this library:
 * only the parity tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it.  It is never linked into, called by, or shipped with the
 * GPU product library.
 *
 * Every function restates the reference algorithm it names (file:line in the
 * pigay/aran source tree).  All arithmetic is FP64 / complex128 as in the
 * reference.  Series coefficients use the reference layout
 * (aran/aransphericalseriesd-private.h:38-70): positive (local) terms (l,m),
 * 0<=m<=l<=posdeg at l(l+1)/2+m, then negative (multipole) terms of degree
 * -(l+1), 0<=m<=l<negdeg, at (posdeg+1)(posdeg+2)/2 + l(l+1)/2 + m.  Complex
 * values cross this C ABI as interleaved (re, im) doubles.
 *
 * The octree and near/far traversal restate libvsg's PR-octree semantics
 * (libvsg itself is not vendored with the reference, so this part is
 * "parity unpinned": it follows the behaviour the reference solver relies on,
 * aran/aransolver3d.c:254-490, with the criteria documented below).
 */
#ifndef ARAN_ORACLE_H
#define ARAN_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* translation flavours: aran_development3d_{m2m,m2l,l2l}{,_kkylin,_rotate} */
enum { OR_NORMAL = 0, OR_KKYLIN = 1, OR_ROTATE = 2 };

/* ---- tables and special functions ---------------------------------- */
double or_beta (int l);
double or_alpha (int l, int m);
double or_harmonic_norm (int l, int m);
double or_vertical_factor (int l, int m, int n);
void or_legendre_multiple (int l, double x, double s, double *res);
void or_legendre_special (int l, double x, double s, const double *leg,
                          double *spec);
void or_harmonics (int l, double cost, double sint, double cosp, double sinp,
                   double *res);
void or_to_spherical (const double v[3], double out[5]);

/* ---- series operators (interleaved complex) --------------------------- */
int or_series_size (int posdeg, int negdeg);
void or_p2m (const double x[3], double q, const double center[3], int deg,
             double *mult /* series(0,deg) */);
void or_p2l (const double x[3], double q, const double center[3], int deg,
             double *local /* series(deg,0) */);
void or_series_evaluate (int posdeg, int negdeg, const double *c,
                         const double xrel[3], double out[2]);
void or_series_gradient (int posdeg, int negdeg, const double *c,
                         const double xrel[3], double grad[3]);
/* dst += T(src), src centred at xs, dst centred at xd (translate) */
void or_translate (int flavour, int sp, int sn, const double *src,
                   const double xs[3], int dp, int dn, double *dst,
                   const double xd[3]);
/* dst(local) += M2L(src) */
void or_to_local (int flavour, int sp, int sn, const double *src,
                  const double xs[3], int dp, int dn, double *dst,
                  const double xd[3]);
void or_rotate (int sp, int sn, const double *src, double alpha, double beta,
                double gamma, int dp, int dn, double *dst);
void or_rotate_inverse (int sp, int sn, const double *src, double alpha,
                        double beta, double gamma, int dp, int dn,
                        double *dst);
/* D_l^{m,m'} for l<=lmax, m'<=l, -l<=m<=l, stored [l][m'][l+m] packed */
int or_wigner_size (int lmax);
void or_wigner (double alpha, double beta, double gamma, int lmax,
                double *terms);

/* ---- octree, near/far traversal, solve --------------------------------- */
typedef struct
{
  int n;              /* particle count */
  int maxbox;         /* leaf capacity ('-s' / vsg maxbox) */
  int order;          /* p: multipole degrees 0..p-1, local degrees 0..p */
  int flavour;        /* OR_NORMAL / OR_KKYLIN / OR_ROTATE */
  int field;          /* 0: potential (newtonpot3), 1: field (newtonfield3) */
  int max_depth;      /* <= 21 */
  double lb[3], ub[3];
  int semifar_threshold;  /* <= 0: off; > 0: semifar P2L/M2P for nodes
                             holding more points (aransolver3d.c:357-396) */
} OrSolveConfig;

/* Counters in the order of aran_solver3d_get_stats
 * (aran/aransolver3d.c:566-586): zero, p2p, p2m, m2m, m2l, l2l, l2p, p2l,
 * m2p, p2p_remote, m2l_remote. */
#define OR_NSTATS 11

/* A node about to be split, as a leaf predicate sees it. */
typedef struct
{
  double center[3];
  double lbound[3];
  double ubound[3];
  int64_t point_count;
  int depth;
} OrNodeView;

/* Non-zero keeps the node as a leaf ("virtual leaf" of the near/far
 * traversal, aran_solver3d_set_nf_isleaf, aran/aransolver3d.c:1272-1279). */
typedef int (*OrLeafPredicate) (const OrNodeView *node, void *user_data);

/* Sets (or clears, with NULL) the leaf predicate of every later tree build;
 * process-global, for the tests. */
void or_set_leaf_predicate (OrLeafPredicate pred, void *user_data);

/* Builds the tree, runs the solve, writes potential (n) or field (3n). */
int or_solve (const OrSolveConfig *cfg, const double *xyz, const double *q,
              double *pot, double *field, int64_t stats[OR_NSTATS]);

/* The same solve with the per-node and per-leaf work spread over nthreads
 * host threads (<= 0: the host core count).  Every target (node local,
 * particle) receives its terms in the order of the single-threaded solve;
 * results agree to rounding (angle triples within 1e-9 share one cached
 * rotation, built by whichever call asked first).  A near pair is evaluated
 * from both of its leaves (the single-threaded solve updates both sides at
 * once).  Semifar solves run single-threaded. */
int or_solve_threaded (const OrSolveConfig *cfg, const double *xyz,
                       const double *q, double *pot, double *field,
                       int64_t stats[OR_NSTATS], int nthreads);

/* Tree/list description for bit-exact parity with the device tree.
 * Node id = (1 << 3*depth) | morton_key(depth).  Returns counts; arrays may
 * be NULL to query sizes.  Far pairs are unordered (a<b by id), near pairs
 * are unordered leaf pairs including (a,a). */
int or_tree_lists (const OrSolveConfig *cfg, const double *xyz,
                   int64_t *n_nodes, uint64_t *node_ids, int32_t *node_begin,
                   int32_t *node_end, uint8_t *node_leaf,
                   int64_t *n_far, uint64_t *far_pairs,
                   int64_t *n_near, uint64_t *near_pairs,
                   int32_t *perm);

/* quantised 21-bit Morton key of one point, as the device computes it */
uint64_t or_morton_key (const double x[3], const double lb[3],
                        const double ub[3]);

/* FP64 direct sum (Neumaier-compensated) over all sources for the given
 * targets: potential sum_j q_j/|xi-xj| (j != i) and field
 * sum_j -q_j (xi-xj)/|xi-xj|^3 with the |xi-xj| > 1e-5 guard of
 * tests/newtonfield3.c:58-89.  nthreads <= 0 picks the host core count. */
void or_direct (int n, const double *xyz, const double *q, int nt,
                const int32_t *targets, double *pot, double *field,
                int nthreads);

/* ---- 2D: Laurent series and the Cauchy-kernel solve --------------------
 * A Laurent series of degrees (posdeg, negdeg) holds posdeg + negdeg + 1
 * complex terms (interleaved re, im); the term of degree i,
 * -negdeg <= i <= posdeg, sits at index posdeg - i
 * (aran/aranlaurentseriesd.c:37-43).  A 2D development is a multipole
 * laurent(0, p) and a local laurent(p, 0) (aran/arandevelopment2d.c:64-73). */
void or2_p2m (double x, double y, double q, double cx, double cy, int negdeg,
              double *mult);
void or2_p2l (double x, double y, double q, double cx, double cy, int posdeg,
              double *loc);
void or2_translate (int sp, int sn, const double *src, double zsx, double zsy,
                    int dp, int dn, double *dst, double zdx, double zdy);
void or2_to_taylor (int sp, int sn, const double *src, double zsx, double zsy,
                    int dp, int dn, double *dst, double zdx, double zdy);
void or2_evaluate (int pd, int nd, const double *s, double zx, double zy,
                   double out[2]);

typedef struct
{
  int maxbox;         /* leaf capacity */
  int order;          /* p: aran_development2d_new (0, p) */
  int max_depth;      /* <= 21 (0: 21) */
} Or2Config;

/* Solves nsys independent 2D systems (system s holds particles
 * offs[s]..offs[s+1]-1 in the box box[4s..4s+3] = lbx, lby, ubx, uby):
 * acc_i = sum_j q_j / (z_i - z_j), j != i, the kernel of tests/dummypot.c,
 * as the reference solver computes it (P2P, P2M, M2M, M2L, L2L, L2P over a
 * quadtree with the traversal rules of the 3D oracle).  acc holds 2 doubles
 * per particle; stats are summed over the systems. */
int or2_solve (const Or2Config *cfg, int nsys, const int64_t *offs,
               const double *xy, const double *q, const double *box,
               double *acc, int64_t stats[OR_NSTATS]);
/* FP64 direct sum of the same kernel for the listed targets of one system */
void or2_direct (int n, const double *xy, const double *q, int nt,
                 const int32_t *targets, double *acc);

#ifdef __cplusplus
}
#endif

#endif
