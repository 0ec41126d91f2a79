/*
 * aran_gpu.h -- C ABI of the GB300 FMM library (libaran_gpu.so).
 *
 * The library replaces the hot path behind LibAran's aran_solver3d_solve()
 * (aran/aransolver3d.c:1135-1202): tree construction (libvsg's PR-octree in
 * the reference), the clear/up/near-far/down passes and the operator
 * callbacks aran_development3d_{p2m,m2m*,m2l*,l2l*,local_gradient_evaluate}
 * (aran/arandevelopment3d.c:169-552) together with the user P2P kernels of
 * tests/newtonpot3.c:61-78 and tests/newtonfield3.c:91-119.  Everything runs
 * on one GPU; there is no CPU fallback: a call that cannot run on the GPU
 * returns an error code and leaves the outputs untouched.
 *
 * Plain pointers and sizes only.  Particle positions are AoS xyz triples
 * (the VsgVector3d at offset 0 of the reference's point structs), charges
 * and outputs are FP64.
 */
#ifndef ARAN_GPU_H
#define ARAN_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define ARAN_OK 0
#define ARAN_ERR_INVALID (-1)      /* bad argument / configuration */
#define ARAN_ERR_CUDA (-2)         /* CUDA runtime failure */
#define ARAN_ERR_NO_DEVICE (-3)    /* no usable GPU: the library never falls back to the CPU */
#define ARAN_ERR_OOM (-4)          /* device memory exhausted */
#define ARAN_ERR_TIMEOUT (-5)      /* a bounded device-side wait gave up */
#define ARAN_ERR_UNSUPPORTED (-6)
#define ARAN_ERR_CANCELLED (-7)    /* a queued request was cancelled */

/* M2M/M2L/L2L flavours: aran_development3d_{m2l,m2l_kkylin,m2l_rotate}
 * (aran/arandevelopment3d.c:306-313,362-369,423-430).  NORMAL applies the
 * same operators as ROTATE and runs its kernels. */
#define ARAN_FLAVOUR_NORMAL 0
#define ARAN_FLAVOUR_KKYLIN 1
#define ARAN_FLAVOUR_ROTATE 2

/* arithmetic of the solve */
#define ARAN_PRECISION_FP64 0      /* every pass in FP64 (the plain path) */
#define ARAN_PRECISION_MIXED 1     /* FP32 bulk, FP64 tables/centres/final sums */

/* pointer location for solve calls */
#define ARAN_MEM_HOST 0
#define ARAN_MEM_DEVICE 1

typedef struct
{
  double lb[3];        /* tree bounding box (vsg_prtree3d_new_full lbound) */
  double ub[3];        /* (ubound) */
  int maxbox;          /* leaf capacity: vsg_prtree3d_new_full 'maxbox' */
  int order;           /* p of aran_development3d_new (0, p) */
  int flavour;         /* ARAN_FLAVOUR_* */
  int field;           /* 0: potential only (newtonpot3); 1: potential + field (newtonfield3) */
  int precision;       /* ARAN_PRECISION_* */
  int max_depth;       /* tree depth limit, 1..21 (0 = 21) */
  int semifar_threshold; /* <= 0: off; > 0: a coarse leaf against a deeper,
                            non-touching node holding more points takes P2L/M2P
                            instead of P2P (aran/aransolver3d.c:357-396) */
} AranGpuConfig3d;

typedef struct AranGpuSolver3d AranGpuSolver3d;

/* Creates a solver bound to the current CUDA device and builds the operator
 * tables for cfg->order.  Replaces aran_solver3d_new + set_functions
 * (aran/aransolver3d.c:509-661). */
int aran_gpu_solver3d_create (const AranGpuConfig3d *cfg,
                              AranGpuSolver3d **out);
void aran_gpu_solver3d_destroy (AranGpuSolver3d *s);

/* One full solve: tree build, lists, up/near-far/down passes.  xyz is 3n
 * doubles (AoS), q is n doubles; pot (n) and field (3n, AoS) receive the
 * potential sum_j q_j/|xi-xj| and field sum_j -q_j (xi-xj)/|xi-xj|^3 of
 * every particle (either may be NULL).  mem selects host or device pointers;
 * with host pointers the copies are part of the call.  A point outside the
 * box [lbound, ubound] is placed in the nearest boundary cell (FP64 solves
 * evaluate it there); a mixed-precision solve returns ARAN_ERR_INVALID,
 * before any output is written, for a point more than one finest cell
 * (box / 2^21) outside it, as for a NaN or infinite coordinate or charge.  Replaces
 * aran_solver3d_insert_point x n + aran_solver3d_solve
 * (aran/aransolver3d.c:972-978,1135-1202). */
int aran_gpu_solver3d_solve (AranGpuSolver3d *s, int64_t n, const double *xyz,
                             const double *q, double *pot, double *field,
                             int mem);

/* nsys independent systems in one solve (a forest: one octree per system,
 * each level's kernels run over the nodes of every system at once).
 * System k holds particles offsets[k] .. offsets[k+1]-1 (offsets: nsys+1
 * host int64, offsets[0] = 0, non-decreasing; n = offsets[nsys]) in the box
 * boxes[6k .. 6k+5] = (lbx, lby, lbz, ubx, uby, ubz) (host).  Every box
 * must have the solver's extents (ub - lb per axis, compared exactly): the
 * operator tables are made for them; its origin is free.  xyz, q, pot and
 * field as for aran_gpu_solver3d_solve over the n particles; each system's
 * results equal those of a solve of that system alone in its box (up to the
 * order of FP64 additions), and the counters are summed over the systems.
 * The batched form of calling aran_solver3d_solve once per system
 * (aran/aransolver3d.c:1135-1202). */
int aran_gpu_solver3d_solve_forest (AranGpuSolver3d *s, int nsys, const int64_t *offsets,
                                    const double *boxes, const double *xyz, const double *q,
                                    double *pot, double *field, int mem);

/* M2L kernel of the FP32 part of mixed solves (rotation flavours):
 * ARAN_M2L_AUTO: the lane-parallel kernel at orders 4, 8 and 12, else the
 * sibling kernel with the library's table slots and parents per CTA;
 * ARAN_M2L_LANES / ARAN_M2L_SIBLING: that kernel (nst table slots in {1, 2,
 * 3} and g parents per CTA in {1, 2}; 0 and 0 = the library's choice);
 * ARAN_M2L_TENSOR: the tcgen05 kernel at orders 8 and 12 (TF32 products with
 * a hi/lo split, the accumulator drained into FP32 registers per offset;
 * about twice the FP32 kernels' rounding error, 5e-7 against 3e-7 relative
 * at order 12).  Where the chosen kernel does not
 * serve the order the next one in the order tensor, lanes, sibling does.
 * Without a call, $ARAN_M2L_KERNEL ("lanes", "sibling", "tc") picks. */
#define ARAN_M2L_AUTO 0
#define ARAN_M2L_LANES 1
#define ARAN_M2L_SIBLING 2
#define ARAN_M2L_TENSOR 3
int aran_gpu_solver3d_set_m2l_kernel (AranGpuSolver3d *s, int kernel, int nst, int g);

/* ---- autotuner ---------------------------------------------------------
 * With db_path it also stores, in the operator-cost group ($ARAN_PROFILE_GROUP
 * or "aran-profile"), samples at x = order of the amortised GPU cost of one
 * call of every development operator under the reference's names
 * (aran_development3d_p2m, _m2m_rotate, _m2l_rotate, _l2l_rotate, _l2p;
 * the flavour's suffix), from a solve of the chosen configuration: what
 * aran_solver3d_db_profile_operators and aran_profile_db_* read.
 * Times solves of a sample (n particles, host or device pointers by mem)
 * with cfg's box, order, flavour, precision and field for every leaf
 * capacity of maxboxes (NULL: 16, 24, 32, 48, 64, 96, 128) and every M2L
 * kernel that serves the order (lane-parallel, sibling configurations;
 * mixed precision only; the tensor-core kernel is no candidate, as it
 * trades accuracy for time),
 * reps timed solves each after one untimed, and keeps the fastest device
 * time.  The choice goes to *out and, when db_path is not NULL, into the
 * profile database file (profiledb.ini syntax, group [aran-gpu-tune], key
 * p<order>-<precision>-<flavour>-<field|pot>, with the timed samples under
 * samples-<key>; other groups and keys of the file are kept).  LibAran
 * times operators for its cost model (aran/aranprofile.c:11-60,
 * aran/aranprofiledb.c:158-200); this tunes the GPU solve itself. */
typedef struct
{
  int maxbox;
  int m2l_kernel;      /* ARAN_M2L_* */
  int m2l_nst, m2l_g;  /* sibling configuration (0: the library's) */
  double ms;           /* device time of one solve of the sample */
  int candidates;      /* configurations timed */
} AranGpuTuneResult;

int aran_gpu_autotune3d (const AranGpuConfig3d *cfg, int64_t n, const double *xyz,
                         const double *q, int mem, const int *maxboxes, int nmaxbox,
                         int reps, const char *db_path, AranGpuTuneResult *out);
/* The tuned choice for cfg's order, precision, flavour and field from the
 * database (db_path, else $ARAN_PROFILE_DB, else profiledb.ini beside
 * libaran_gpu.so): 1 and *out filled when found, 0 when not, negative on a
 * malformed entry.  Host only.  A solver created with cfg->maxbox == 0
 * takes its leaf capacity and M2L kernel from here (64 and the automatic
 * kernel when there is no entry). */
int aran_gpu_tune_lookup (const char *db_path, const AranGpuConfig3d *cfg,
                          AranGpuTuneResult *out);

/* Call counters of the last solve in the order of aran_solver3d_get_stats
 * (aran/aransolver3d.c:566-586): zero, p2p, p2m, m2m, m2l, l2l, l2p, p2l,
 * m2p, p2p_remote, m2l_remote. */
int aran_gpu_solver3d_get_stats (AranGpuSolver3d *s, int64_t stats[11]);

/* Sizes of the last tree: nodes, directed far (M2L) entries, directed near
 * (P2P) leaf entries, non-empty leaves, depth. */
int aran_gpu_solver3d_tree_info (AranGpuSolver3d *s, int64_t info[5]);

/* Copies the last tree out for parity checks.  Node id =
 * (1 << 3*depth) | morton key.  far: (target id, source id) per directed
 * M2L; near: (target leaf id, source leaf id) per directed P2P block.
 * perm: sorted position -> input index.  Any pointer may be NULL. */
int aran_gpu_solver3d_tree_lists (AranGpuSolver3d *s, uint64_t *node_ids,
                                  int32_t *node_begin, int32_t *node_end,
                                  uint8_t *node_leaf, uint64_t *far_pairs,
                                  uint64_t *near_pairs, int32_t *perm);

/* Copies the scaled device expansions of the last solve (debug/parity):
 * per node, multipole then local coefficients (m >= 0) as interleaved
 * complex FP64, in LibAran order; unscaled to physical units. */
int aran_gpu_solver3d_expansions (AranGpuSolver3d *s, double *mult,
                                  double *local);

/* Stage times of the last solve in ms (CUDA events on the solve stream):
 * [0] total, [1] keys+sort, [2] tree, [3] lists, [4] p2m, [5] m2m, [6] m2l
 * (semifar P2L included), [7] l2l, [8] l2p (semifar M2P included), [9] p2p
 * (its own stream), [10] h2d, [11] d2h, [12] semifar p2l, [13] semifar m2p. */
int aran_gpu_solver3d_timings (AranGpuSolver3d *s, double ms[16]);

/* Number of GPU kernel launches issued by the last solve. */
int64_t aran_gpu_solver3d_launches (AranGpuSolver3d *s);

/* The view of a tree node a leaf predicate receives. */
typedef struct
{
  double center[3];
  double lbound[3];
  double ubound[3];
  int64_t point_count;   /* particles below the node */
  int depth;
} AranGpuNodeView;

/* Returns non-zero when a node that holds more than maxbox particles is to be
 * a leaf all the same (a "virtual leaf": its particles take P2P as one leaf
 * and no M2L runs below it). */
typedef int (*AranGpuLeafPredicate) (const AranGpuNodeView *node, void *user_data);

/* Sets (pred != NULL) or clears the leaf predicate: while the tree of a solve
 * is subdivided level by level, every node about to be split is shown to
 * pred and stays a leaf when it answers non-zero.  Replaces the near/far
 * traversal's is-leaf callback of aran_solver3d_set_nf_isleaf
 * (aran/aransolver3d.c:1272-1279, libvsg's vsg_prtree3d_set_nf_isleaf): the
 * reference keeps the nodes below a virtual leaf for its up and down passes,
 * here they are not made, which changes only the rounding (M2M and L2L are
 * exact on truncated expansions) and the zero/m2m/l2l counters. */
int aran_gpu_solver3d_set_leaf_predicate (AranGpuSolver3d *s, AranGpuLeafPredicate pred,
                                          void *user_data);

/* Mixed precision only: nodes of depth <= depth keep FP64 expansions, so
 * M2M into them and M2L and L2L at them run in FP64 (the coarse levels,
 * whose translations span the widest range of powers of the distance at
 * high order: aran/aransphericalseriesd-translate.c:609-676).  -1 turns it
 * off.  A mixed solver starts with depth 3 when its order is >= 16 and -1
 * below; the kkylin flavour ignores it.  No counterpart in the reference
 * (all FP64 there).  ARAN_ERR_INVALID outside [-1, 21] or on an FP64 solver. */
int aran_gpu_solver3d_set_fp64_root_depth (AranGpuSolver3d *s, int depth);

/* Allocation-free Newton near field: every pair of n <= 131072 particles
 * (potential, and field when d_field is not NULL, with the same rules as the
 * solver's single-leaf P2P), FP64, device pointers, AoS xyz.  No counterpart
 * in the reference: it exists for callers that may not allocate device
 * memory during a call (a host that owns all device memory, or a loop that
 * must not meet cudaMalloc's implicit synchronisation).  Its scratch is a
 * static 4 MiB device array of the library's device code, placed on a GPU
 * when that code is loaded there (lazily, at the first call on the device,
 * unless CUDA_MODULE_LOADING=EAGER) and kept until exit: make one warm-up
 * call per device before the no-allocation region and before any stream
 * capture.  The kernels run on, and the call synchronises, the legacy
 * default stream: finish writing d_xyz and d_q first.  Calls share the
 * array, so calls that overlap on the GPU race.  Returns ARAN_ERR_INVALID
 * for n outside [1, 131072]. */
int aran_gpu_p2p_direct_noalloc (int64_t n, const double *d_xyz,
                                 const double *d_q, double *d_pot,
                                 double *d_field);

/* ---- request loop (continuous batching of independent solves) ---------
 * No counterpart in the reference (which solves one system per call); it
 * serves many aran_solver3d_solve-equivalent requests on one GPU. */

typedef struct
{
  AranGpuConfig3d cfg;
  int64_t n;
  const double *xyz;   /* host, 3n, valid until the request completes */
  const double *q;     /* host, n */
  double *pot;         /* host, n (or NULL) */
  double *field;       /* host, 3n (or NULL) */
  double tolerance;    /* > 0: requested relative L2 error of the potential
                          against the direct sum; the server then picks
                          cfg.precision, and cfg.order too when it is 0
                          (aran_gpu_plan_for_tolerance).  <= 0: cfg as given */
} AranGpuRequest3d;

typedef struct
{
  int status;          /* ARAN_OK or the request's error code */
  double submit_s;     /* seconds since the server was created */
  double start_s;
  double end_s;
  int slot;
  int64_t footprint_bytes;
  int order;           /* order and precision the request ran at */
  int precision;
} AranGpuRequestInfo;

/* Picks the cheapest (order, precision) whose relative L2 potential error
 * against the FP64 direct sum, measured on GB300 over uniform and Plummer
 * draws of 2e4-3e5 particles at leaf capacity 64, is at most tol / 2:
 * mixed precision wherever it reaches that, FP64 otherwise.  cfg->order > 0
 * keeps the order and picks only the precision.  Returns the table's error
 * estimate for the pick (tolerances below what order 30 in FP64 reaches get
 * order 30, FP64, and an estimate above tol / 2). */
double aran_gpu_plan_for_tolerance (double tol, AranGpuConfig3d *cfg);

typedef struct AranGpuServer AranGpuServer;

/* Estimated device memory of one solve (particles, tree, lists, expansions). */
int64_t aran_gpu_footprint_bytes (const AranGpuConfig3d *cfg, int64_t n);

/* nslots concurrent solves (host worker threads with their own streams and
 * resident solvers) under an HBM admission budget (<= 0: 80% of free). */
int aran_gpu_server_create (int nslots, double hbm_budget_bytes,
                            AranGpuServer **out);
/* Queues a request; it starts when a slot is free and its footprint fits the
 * budget next to the running ones (first fit in arrival order).  A request
 * larger than the whole budget is refused with ARAN_ERR_OOM. */
int aran_gpu_server_submit (AranGpuServer *sv, const AranGpuRequest3d *req,
                            int64_t *ticket);
/* Waits for a request (timeout_s < 0: forever); returns its status and
 * fills info.  A ticket can be waited for once. */
int aran_gpu_server_wait (AranGpuServer *sv, int64_t ticket, double timeout_s,
                          AranGpuRequestInfo *info);
/* Cancels a request that has not started (ARAN_ERR_CANCELLED for waiters). */
int aran_gpu_server_cancel (AranGpuServer *sv, int64_t ticket);
/* Finishes running requests, cancels queued ones, frees everything. */
void aran_gpu_server_destroy (AranGpuServer *sv);

/* ---- 2D: Cauchy-kernel FMM over a batch of independent systems --------
 * Replaces aran_solver2d_solve (aran/aransolver2d.c:1137-1204) with the
 * operators aran_development2d_{p2m,m2m,m2l,l2l,local_evaluate}
 * (aran/arandevelopment2d.c:167-346: Laurent multipole laurent(0, p), Taylor
 * local laurent(p, 0)) and the P2P kernel of tests/dummypot.c:62-76:
 * acc_i = sum_{j != i} q_j / (z_i - z_j), complex, FP64.  One call solves
 * nsys systems at once (a forest: one quadtree per system). */

typedef struct
{
  int maxbox;          /* leaf capacity (vsg_prtree2d_new_full maxbox) */
  int order;           /* p of aran_development2d_new (0, p), 1..64 */
  int max_depth;       /* quadtree depth limit, 1..21 (0 = 21) */
  int precision;       /* ARAN_PRECISION_FP64 (0), or ARAN_PRECISION_MIXED: FP32
                          expansions scaled by the node size and FP32 near-field
                          arithmetic on FP64 differences, FP64 centres and sums */
} AranGpuConfig2d;

typedef struct AranGpuSolver2d AranGpuSolver2d;

int aran_gpu_solver2d_create (const AranGpuConfig2d *cfg, AranGpuSolver2d **out);
void aran_gpu_solver2d_destroy (AranGpuSolver2d *s);

/* System s holds particles offs[s] .. offs[s+1]-1 (offs: nsys+1 host
 * int64, offs[0] = 0, non-decreasing) in the box box[4s .. 4s+3] = (lbx,
 * lby, ubx, uby) (host).  xy is 2n doubles (AoS), q n doubles, acc receives
 * 2n doubles (re, im per particle).  mem selects host or device pointers for
 * xy, q and acc.  ARAN_ERR_INVALID, before anything is written, for a NaN or
 * infinite coordinate or charge, and in mixed precision for a point more
 * than one finest cell outside its system's box (FP64 places it in the
 * nearest boundary cell). */
int aran_gpu_solver2d_solve (AranGpuSolver2d *s, int nsys, const int64_t *offs,
                             const double *box, const double *xy, const double *q,
                             double *acc, int mem);
/* Leaf predicate of the 2D forest (z components of the view are 0): the
 * twin of aran_gpu_solver3d_set_leaf_predicate for
 * aran_solver2d_set_nf_isleaf (aran/aransolver2d.c). */
int aran_gpu_solver2d_set_leaf_predicate (AranGpuSolver2d *s, AranGpuLeafPredicate pred,
                                          void *user_data);
/* Call counters of the last solve, summed over its systems, in the order
 * of aran_solver2d_get_stats (aran/aransolver2d.c:868-896). */
int aran_gpu_solver2d_get_stats (AranGpuSolver2d *s, int64_t stats[11]);
/* Stage times of the last solve in ms, same slots as the 3D solver. */
int aran_gpu_solver2d_timings (AranGpuSolver2d *s, double ms[16]);
/* Sizes of the last forest: nodes, directed far entries, near ranges,
 * non-empty leaves, depth. */
int aran_gpu_solver2d_tree_info (AranGpuSolver2d *s, int64_t info[5]);
int64_t aran_gpu_solver2d_launches (AranGpuSolver2d *s);

/* Last error message of the calling thread. */
const char *aran_gpu_last_error (void);

/* Library version string. */
const char *aran_gpu_version (void);

#ifdef __cplusplus
}
#endif

#endif
