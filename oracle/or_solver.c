/*
 * or_solver.c -- octree, near/far traversal, FMM solve and FP64 direct sum
 * of the oracle.  TEST INFRASTRUCTURE ONLY (see aran_oracle.h).
 *
 * Tree semantics (restating the libvsg PR-octree the reference solver runs
 * on; libvsg is not vendored with the reference, so these criteria are the
 * documented contract, "parity unpinned" against libvsg itself):
 *  - the root box is the caller's [lb, ub]; a point belongs to the node its
 *    21-bit quantised coordinates fall in (or_morton_key);
 *  - a node is subdivided into its 8 octants iff it holds more than maxbox
 *    points and its depth is below max_depth; all 8 octants exist as nodes;
 *  - node centres are obtained by halving the parent box;
 *  - near/far pairs come from a dual traversal starting at (root, root):
 *    same-depth nodes that are not adjacent (|di|,|dj|,|dk| not all <= 1)
 *    are FAR (2 M2L, aran/aransolver3d.c:333-354); adjacent leaves are NEAR
 *    (P2P, :254-324); a leaf against an adjacent internal node is NEAR with
 *    every non-empty leaf below that node; empty nodes take no part.
 *  - semifar (only with p2l/m2p and a threshold T > 0): a leaf A against an
 *    adjacent internal node walks that node's subtree instead; a descendant
 *    D adjacent to A (touching A's box) is walked further (near if it is a
 *    leaf), a descendant D not adjacent to A takes P2L of A's points into
 *    D's local and M2P of D's multipole to A's points when D holds more than
 *    T points (semifar_func, aran/aransolver3d.c:357-396; "beyond this
 *    number of particles", :622-623), and is near with every leaf below it
 *    otherwise.
 */
#include "or_internal.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define OR_KEYBITS 21

typedef struct
{
  uint64_t id;        /* (1 << 3 depth) | key */
  int depth;
  int32_t ijk[3];
  int begin, end;     /* range in sorted order */
  int leaf;
  int child[8];       /* -1 when leaf */
  int father;
  double center[3];
} OrNode;

typedef struct
{
  OrNode *nodes;
  int nn, cap;
  int32_t *perm;      /* sorted position -> original index */
  uint64_t *keys;     /* sorted keys */
  int n;
} OrTree;

/* ------------------------------------------------------------------ keys */
static uint64_t spread3 (uint64_t v)
{
  uint64_t r = 0;
  int b;
  for (b = 0; b < OR_KEYBITS; b++)
    r |= ((v >> b) & 1ull) << (3 * b);
  return r;
}

static int64_t quantise (double x, double lb, double scale)
{
  double t = (x - lb) * scale;
  int64_t i = (int64_t) floor (t);
  if (i < 0)
    i = 0;
  if (i > (1 << OR_KEYBITS) - 1)
    i = (1 << OR_KEYBITS) - 1;
  return i;
}

static void key_scales (const double lb[3], const double ub[3], double s[3])
{
  int a;
  for (a = 0; a < 3; a++)
    s[a] = (double) (1 << OR_KEYBITS) / (ub[a] - lb[a]);
}

uint64_t or_morton_key (const double x[3], const double lb[3],
                        const double ub[3])
{
  double s[3];
  key_scales (lb, ub, s);
  return spread3 ((uint64_t) quantise (x[0], lb[0], s[0])) |
    (spread3 ((uint64_t) quantise (x[1], lb[1], s[1])) << 1) |
    (spread3 ((uint64_t) quantise (x[2], lb[2], s[2])) << 2);
}

/* centre of the node with integer coordinates ijk at depth d: repeated
 * halving of the root box (the same sequence of FP64 operations the device
 * uses) */
static void node_center (const double lb0[3], const double ub0[3], int d,
                         const int32_t ijk[3], double c[3])
{
  int a, b;
  for (a = 0; a < 3; a++)
    {
      double lo = lb0[a], hi = ub0[a];
      for (b = d - 1; b >= 0; b--)
        {
          double mid = (lo + hi) * 0.5;
          if ((ijk[a] >> b) & 1)
            lo = mid;
          else
            hi = mid;
        }
      c[a] = (lo + hi) * 0.5;
    }
}

typedef struct
{
  uint64_t k;
  int32_t i;
} KeyIdx;

static int cmp_keyidx (const void *a, const void *b)
{
  const KeyIdx *x = (const KeyIdx *) a, *y = (const KeyIdx *) b;
  if (x->k != y->k)
    return x->k < y->k ? -1 : 1;
  return x->i - y->i;
}

static int push_node (OrTree *t)
{
  if (t->nn == t->cap)
    {
      t->cap = t->cap ? 2 * t->cap : 1024;
      t->nodes = (OrNode *) realloc (t->nodes, t->cap * sizeof (OrNode));
    }
  return t->nn++;
}

static OrLeafPredicate g_leaf_pred = NULL;
static void *g_leaf_data = NULL;

void or_set_leaf_predicate (OrLeafPredicate pred, void *user_data)
{
  g_leaf_pred = pred;
  g_leaf_data = user_data;
}

/* a node the predicate keeps as a leaf; its cell by halving the root box */
static int virtual_leaf (const OrSolveConfig *cfg, const OrNode *nd)
{
  OrNodeView v;
  int a, b;
  if (!g_leaf_pred)
    return 0;
  for (a = 0; a < 3; a++)
    {
      double lo = cfg->lb[a], hi = cfg->ub[a];
      for (b = nd->depth - 1; b >= 0; b--)
        {
          double mid = (lo + hi) * 0.5;
          if ((nd->ijk[a] >> b) & 1)
            lo = mid;
          else
            hi = mid;
        }
      v.lbound[a] = lo;
      v.ubound[a] = hi;
      v.center[a] = (lo + hi) * 0.5;
    }
  v.point_count = nd->end - nd->begin;
  v.depth = nd->depth;
  return g_leaf_pred (&v, g_leaf_data) != 0;
}

static void tree_build (OrTree *t, const OrSolveConfig *cfg,
                        const double *xyz)
{
  int i, d, maxd = cfg->max_depth > 0 ? cfg->max_depth : OR_KEYBITS;
  KeyIdx *ki = (KeyIdx *) malloc ((size_t) cfg->n * sizeof (KeyIdx));
  int lvl_begin, lvl_end;

  if (maxd > OR_KEYBITS)
    maxd = OR_KEYBITS;
  memset (t, 0, sizeof (*t));
  t->n = cfg->n;
  for (i = 0; i < cfg->n; i++)
    {
      ki[i].k = or_morton_key (xyz + 3 * i, cfg->lb, cfg->ub);
      ki[i].i = i;
    }
  qsort (ki, cfg->n, sizeof (KeyIdx), cmp_keyidx);
  t->perm = (int32_t *) malloc ((size_t) cfg->n * sizeof (int32_t));
  t->keys = (uint64_t *) malloc ((size_t) cfg->n * sizeof (uint64_t));
  for (i = 0; i < cfg->n; i++)
    {
      t->perm[i] = ki[i].i;
      t->keys[i] = ki[i].k;
    }
  free (ki);

  /* root */
  {
    int r = push_node (t);
    OrNode *nd = &t->nodes[r];
    memset (nd, 0, sizeof (*nd));
    nd->id = 1;
    nd->depth = 0;
    nd->begin = 0;
    nd->end = cfg->n;
    nd->father = -1;
    node_center (cfg->lb, cfg->ub, 0, nd->ijk, nd->center);
  }
  /* level-by-level subdivision */
  lvl_begin = 0;
  lvl_end = 1;
  for (d = 0; lvl_begin < lvl_end; d++)
    {
      int nb;
      for (nb = lvl_begin; nb < lvl_end; nb++)
        {
          OrNode *nd = &t->nodes[nb];
          int c, pos;
          if (nd->end - nd->begin <= cfg->maxbox || d >= maxd || virtual_leaf (cfg, nd))
            {
              nd->leaf = 1;
              for (c = 0; c < 8; c++)
                nd->child[c] = -1;
              continue;
            }
          nd->leaf = 0;
          pos = nd->begin;
          for (c = 0; c < 8; c++)
            {
              int ci = push_node (t);
              OrNode *ch;
              int shift = 3 * (OR_KEYBITS - d - 1);
              int e = pos;
              nd = &t->nodes[nb];
              while (e < nd->end && (int) ((t->keys[e] >> shift) & 7ull) == c)
                e++;
              ch = &t->nodes[ci];
              memset (ch, 0, sizeof (*ch));
              ch->id = (nd->id << 3) | (uint64_t) c;
              ch->depth = d + 1;
              ch->ijk[0] = (nd->ijk[0] << 1) | (c & 1);
              ch->ijk[1] = (nd->ijk[1] << 1) | ((c >> 1) & 1);
              ch->ijk[2] = (nd->ijk[2] << 1) | ((c >> 2) & 1);
              ch->begin = pos;
              ch->end = e;
              ch->father = nb;
              node_center (cfg->lb, cfg->ub, d + 1, ch->ijk, ch->center);
              nd->child[c] = ci;
              pos = e;
            }
        }
      /* children of this level were appended contiguously */
      nb = lvl_end;
      lvl_begin = lvl_end;
      lvl_end = t->nn;
      (void) nb;
    }
}

static void tree_free (OrTree *t)
{
  free (t->nodes);
  free (t->perm);
  free (t->keys);
}

static int adjacent (const OrNode *a, const OrNode *b)
{
  int k;
  for (k = 0; k < 3; k++)
    {
      int d = a->ijk[k] - b->ijk[k];
      if (d > 1 || d < -1)
        return 0;
    }
  return 1;
}

/* ------------------------------------------------------------- traversal */
typedef struct
{
  void (*far) (void *ctx, int a, int b);
  void (*near) (void *ctx, int a, int b);
  void (*semifar) (void *ctx, int leaf, int node);   /* may be NULL */
  int threshold;                                     /* semifar: > 0 */
  void *ctx;
  const OrTree *t;
} Traversal;

static int cnt (const OrNode *n)
{
  return n->end - n->begin;
}

static void near_leaves_below (const Traversal *tv, int leaf, int node)
{
  const OrNode *nd = &tv->t->nodes[node];
  int c;
  if (cnt (nd) == 0)
    return;
  if (nd->leaf)
    {
      tv->near (tv->ctx, leaf, node);
      return;
    }
  for (c = 0; c < 8; c++)
    near_leaves_below (tv, leaf, nd->child[c]);
}

/* box of node b (depth >= depth of a) touches box of a */
static int adjacent_ml (const OrNode *a, const OrNode *b)
{
  int k, sh = b->depth - a->depth;
  for (k = 0; k < 3; k++)
    {
      int64_t lo = ((int64_t) a->ijk[k] << sh) - 1;
      int64_t hi = ((int64_t) (a->ijk[k] + 1) << sh);
      if (b->ijk[k] < lo || b->ijk[k] > hi)
        return 0;
    }
  return 1;
}

/* leaf against the subtree of an adjacent internal node, semifar on */
static void semifar_walk (const Traversal *tv, int leaf, int node)
{
  const OrNode *A = &tv->t->nodes[leaf], *C = &tv->t->nodes[node];
  int c;
  for (c = 0; c < 8; c++)
    {
      int d = C->child[c];
      const OrNode *D = &tv->t->nodes[d];
      if (cnt (D) == 0)
        continue;
      if (adjacent_ml (A, D))
        {
          if (D->leaf)
            tv->near (tv->ctx, leaf, d);
          else
            semifar_walk (tv, leaf, d);
        }
      else if (cnt (D) > tv->threshold)
        tv->semifar (tv->ctx, leaf, d);
      else
        near_leaves_below (tv, leaf, d);
    }
}

static void leaf_vs_node (const Traversal *tv, int leaf, int node)
{
  if (tv->semifar && tv->threshold > 0)
    semifar_walk (tv, leaf, node);
  else
    near_leaves_below (tv, leaf, node);
}

static void pair_traverse (const Traversal *tv, int a, int b)
{
  const OrNode *A = &tv->t->nodes[a], *B = &tv->t->nodes[b];
  int i, j;
  if (cnt (A) == 0 || cnt (B) == 0)
    return;
  if (a == b)
    {
      if (A->leaf)
        {
          tv->near (tv->ctx, a, a);
          return;
        }
      for (i = 0; i < 8; i++)
        for (j = i; j < 8; j++)
          pair_traverse (tv, A->child[i], A->child[j]);
      return;
    }
  if (A->leaf && B->leaf)
    {
      tv->near (tv->ctx, a, b);
      return;
    }
  if (A->leaf)
    {
      leaf_vs_node (tv, a, b);
      return;
    }
  if (B->leaf)
    {
      leaf_vs_node (tv, b, a);
      return;
    }
  for (i = 0; i < 8; i++)
    for (j = 0; j < 8; j++)
      {
        int ca = A->child[i], cb = B->child[j];
        const OrNode *CA = &tv->t->nodes[ca], *CB = &tv->t->nodes[cb];
        if (cnt (CA) == 0 || cnt (CB) == 0)
          continue;
        if (adjacent (CA, CB))
          pair_traverse (tv, ca, cb);
        else
          tv->far (tv->ctx, ca, cb);
      }
}

/* ------------------------------------------------------------------ solve */
typedef struct
{
  const OrSolveConfig *cfg;
  const OrTree *t;
  const double *xyz, *q;
  double *acc;            /* potential accumulators (sorted order) */
  double *fld;            /* field accumulators (sorted order, 3 per) */
  OrSeries *mult, *loc;   /* per node */
  int64_t *stats;
} SolveCtx;

static void p2p_pair (SolveCtx *s, int i, int j)
{
  /* i, j are sorted positions; both sides updated (tests/newtonpot3.c:61-78,
   * tests/newtonfield3.c:91-119) */
  const double *xi = s->xyz + 3 * s->t->perm[i];
  const double *xj = s->xyz + 3 * s->t->perm[j];
  double qi = s->q[s->t->perm[i]], qj = s->q[s->t->perm[j]];
  double d[3] = { xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2] };
  double r = sqrt (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  if (!s->cfg->field)
    {
      /* coincident distinct points: the reference divides by zero
       * (tests/newtonpot3.c:72); here, as on the GPU, the pair is skipped */
      if (r > 0.)
        {
          double inv_r = 1. / r;
          s->acc[i] += inv_r * qj;
          s->acc[j] += inv_r * qi;
        }
    }
  else if (r > 1.e-5)
    {
      double inv_r = 1. / r, inv_r3 = inv_r * inv_r * inv_r;
      int k;
      for (k = 0; k < 3; k++)
        {
          s->fld[3 * i + k] += d[k] * (-inv_r3 * qj);
          s->fld[3 * j + k] += d[k] * (inv_r3 * qi);
        }
    }
}

static void cb_near (void *ctx, int a, int b)
{
  SolveCtx *s = (SolveCtx *) ctx;
  const OrNode *A = &s->t->nodes[a], *B = &s->t->nodes[b];
  int i, j;
  if (a == b)
    {
      /* reflexive: triangle including i == j (aran/aransolver3d.c:285-314) */
      for (i = A->begin; i < A->end; i++)
        for (j = i + 1; j < A->end; j++)
          p2p_pair (s, i, j);
      s->stats[1] += (int64_t) cnt (A) * (cnt (A) + 1) / 2;
      return;
    }
  for (i = A->begin; i < A->end; i++)
    for (j = B->begin; j < B->end; j++)
      p2p_pair (s, i, j);
  s->stats[1] += (int64_t) cnt (A) * cnt (B);
}

static void cb_far (void *ctx, int a, int b)
{
  SolveCtx *s = (SolveCtx *) ctx;
  const OrNode *A = &s->t->nodes[a], *B = &s->t->nodes[b];
  /* both ways: aran/aransolver3d.c:333-354 */
  or_to_local_series (s->cfg->flavour, &s->mult[a], A->center, &s->loc[b],
                      B->center);
  or_to_local_series (s->cfg->flavour, &s->mult[b], B->center, &s->loc[a],
                      A->center);
  s->stats[4] += 2;
}

/* semifar_func (aran/aransolver3d.c:357-396): every point of the coarse
 * leaf goes into the deep node's local (p2l, tests/newtonpot3.c:93-97) and
 * takes the deep node's multipole (m2p: potential tests/newtonpot3.c:99-104,
 * field = multipole gradient tests/newtonfield3.c:145-151) */
static void cb_semifar (void *ctx, int leaf, int node)
{
  SolveCtx *s = (SolveCtx *) ctx;
  const OrNode *A = &s->t->nodes[leaf], *D = &s->t->nodes[node];
  int i;
  for (i = A->begin; i < A->end; i++)
    {
      int o = s->t->perm[i];
      const double *x = s->xyz + 3 * o;
      double rel[3] = { x[0] - D->center[0], x[1] - D->center[1], x[2] - D->center[2] };
      or_p2l_series (x, s->q[o], D->center, &s->loc[node]);
      if (s->cfg->field)
        {
          double g[3];
          or_gradient_xyz (&s->mult[node], rel, g);
          s->fld[3 * i] += g[0];
          s->fld[3 * i + 1] += g[1];
          s->fld[3 * i + 2] += g[2];
        }
      else
        {
          double r, cost, sint, cosp, sinp;
          or_to_spherical_internal (rel, &r, &cost, &sint, &cosp, &sinp);
          s->acc[i] += creal (or_evaluate_internal (&s->mult[node], r, cost, sint, cosp,
                                                    sinp));
        }
    }
  s->stats[7] += cnt (A);
  s->stats[8] += cnt (A);
}

/* up pass, post order: aran/aransolver3d.c:412-450 */
static void up (SolveCtx *s, int nb)
{
  const OrNode *nd = &s->t->nodes[nb];
  int c, i;
  if (!nd->leaf)
    for (c = 0; c < 8; c++)
      up (s, nd->child[c]);
  if (nd->leaf)
    for (i = nd->begin; i < nd->end; i++)
      {
        int o = s->t->perm[i];
        or_p2m_series (s->xyz + 3 * o, s->q[o], nd->center, &s->mult[nb]);
        s->stats[2]++;
      }
  if (cnt (nd) != 0 && nd->father >= 0)
    {
      const OrNode *f = &s->t->nodes[nd->father];
      or_translate_series (s->cfg->flavour, &s->mult[nb], nd->center,
                           &s->mult[nd->father], f->center);
      s->stats[3]++;
    }
}

/* down pass, pre order: aran/aransolver3d.c:452-490 */
static void down (SolveCtx *s, int nb)
{
  const OrNode *nd = &s->t->nodes[nb];
  int c, i;
  if (cnt (nd) != 0 && nd->father >= 0)
    {
      const OrNode *f = &s->t->nodes[nd->father];
      or_translate_series (s->cfg->flavour, &s->loc[nd->father], f->center,
                           &s->loc[nb], nd->center);
      s->stats[5]++;
    }
  if (nd->leaf)
    {
      for (i = nd->begin; i < nd->end; i++)
        {
          int o = s->t->perm[i];
          const double *x = s->xyz + 3 * o;
          double rel[3] = { x[0] - nd->center[0], x[1] - nd->center[1],
            x[2] - nd->center[2] };
          if (s->cfg->field)
            {
              double g[3];
              or_gradient_xyz (&s->loc[nb], rel, g);
              s->fld[3 * i] += g[0];
              s->fld[3 * i + 1] += g[1];
              s->fld[3 * i + 2] += g[2];
            }
          else
            {
              double r, cost, sint, cosp, sinp;
              or_to_spherical_internal (rel, &r, &cost, &sint, &cosp, &sinp);
              s->acc[i] += creal (or_evaluate_internal (&s->loc[nb], r, cost,
                                                        sint, cosp, sinp));
            }
          s->stats[6]++;
        }
      return;
    }
  for (c = 0; c < 8; c++)
    down (s, nd->child[c]);
}

int or_solve (const OrSolveConfig *cfg, const double *xyz, const double *q,
              double *pot, double *field, int64_t stats[OR_NSTATS])
{
  OrTree t;
  SolveCtx s;
  Traversal tv;
  int i, p = cfg->order;
  int ms = or_series_size (0, p), ls = or_series_size (p, 0);
  double complex *mstore, *lstore;

  if (cfg->n <= 0 || p <= 0)
    return -1;
  tree_build (&t, cfg, xyz);
  memset (stats, 0, OR_NSTATS * sizeof (int64_t));
  s.cfg = cfg;
  s.t = &t;
  s.xyz = xyz;
  s.q = q;
  s.stats = stats;
  s.acc = (double *) calloc ((size_t) cfg->n, sizeof (double));
  s.fld = (double *) calloc ((size_t) cfg->n * 3, sizeof (double));
  s.mult = (OrSeries *) malloc (t.nn * sizeof (OrSeries));
  s.loc = (OrSeries *) malloc (t.nn * sizeof (OrSeries));
  mstore = (double complex *) calloc ((size_t) t.nn * ms, sizeof (double complex));
  lstore = (double complex *) calloc ((size_t) t.nn * ls, sizeof (double complex));
  /* aran_development3d_new (0, p): multipole (0,p), local (p,0)
   * (aran/arandevelopment3d.c:64-73); clear pass zeroes them */
  for (i = 0; i < t.nn; i++)
    {
      s.mult[i].posdeg = 0;
      s.mult[i].negdeg = p;
      s.mult[i].c = mstore + (size_t) i * ms;
      s.loc[i].posdeg = p;
      s.loc[i].negdeg = 0;
      s.loc[i].c = lstore + (size_t) i * ls;
    }
  stats[0] = t.nn;

  up (&s, 0);
  tv.far = cb_far;
  tv.near = cb_near;
  tv.semifar = cb_semifar;
  tv.threshold = cfg->semifar_threshold;
  tv.ctx = &s;
  tv.t = &t;
  pair_traverse (&tv, 0, 0);
  down (&s, 0);

  for (i = 0; i < cfg->n; i++)
    {
      int o = t.perm[i];
      if (cfg->field)
        {
          if (field)
            {
              field[3 * o] = s.fld[3 * i];
              field[3 * o + 1] = s.fld[3 * i + 1];
              field[3 * o + 2] = s.fld[3 * i + 2];
            }
        }
      else if (pot)
        pot[o] = s.acc[i];
    }
  free (s.acc);
  free (s.fld);
  free (s.mult);
  free (s.loc);
  free (mstore);
  free (lstore);
  tree_free (&t);
  return 0;
}

/* ------------------------------------------------------- threaded solve */
typedef struct
{
  void (*fn) (void *ctx, int i);
  void *ctx;
  int n, chunk;
  int next;
} ParFor;

static void *par_worker (void *arg)
{
  ParFor *p = (ParFor *) arg;
  for (;;)
    {
      int i0 = __atomic_fetch_add (&p->next, p->chunk, __ATOMIC_RELAXED), i;
      if (i0 >= p->n)
        break;
      for (i = i0; i < p->n && i < i0 + p->chunk; i++)
        p->fn (p->ctx, i);
    }
  return NULL;
}

/* fn (ctx, i) for i in [0, n), dynamically scheduled over nthreads threads */
static void par_for (int n, int nthreads, int chunk, void (*fn) (void *, int), void *ctx)
{
  ParFor p = { fn, ctx, n, chunk > 0 ? chunk : 1, 0 };
  pthread_t th[256];
  int k, nt = nthreads < 256 ? nthreads : 256;
  if (n <= 0)
    return;
  if (nt > (n + p.chunk - 1) / p.chunk)
    nt = (n + p.chunk - 1) / p.chunk;
  for (k = 1; k < nt; k++)
    pthread_create (&th[k], NULL, par_worker, &p);
  par_worker (&p);
  for (k = 1; k < nt; k++)
    pthread_join (th[k], NULL);
}

typedef struct
{
  SolveCtx *s;
  int lvl_begin;
  int *far_off, *far_src;     /* per target node: sources in traversal order */
  int *near_off, *near_src;   /* per target leaf: source leaves in traversal order */
  int64_t nfar, capfar, nnear, capnear;
  int *farp, *nearp;          /* collected pairs (a, b) */
} ThrCtx;

static void push2 (int **arr, int64_t *n, int64_t *cap, int a, int b)
{
  if (*n == *cap)
    {
      *cap = *cap ? 2 * *cap : 4096;
      *arr = (int *) realloc (*arr, (size_t) *cap * 2 * sizeof (int));
    }
  (*arr)[2 * *n] = a;
  (*arr)[2 * *n + 1] = b;
  (*n)++;
}

static void th_far (void *ctx, int a, int b)
{
  ThrCtx *c = (ThrCtx *) ctx;
  push2 (&c->farp, &c->nfar, &c->capfar, a, b);
  c->s->stats[4] += 2;
}

static void th_near (void *ctx, int a, int b)
{
  ThrCtx *c = (ThrCtx *) ctx;
  const OrNode *A = &c->s->t->nodes[a], *B = &c->s->t->nodes[b];
  push2 (&c->nearp, &c->nnear, &c->capnear, a, b);
  c->s->stats[1] += a == b ? (int64_t) cnt (A) * (cnt (A) + 1) / 2
    : (int64_t) cnt (A) * cnt (B);
}

/* per-target CSR of directed pairs: (a, b) gives b the source a and, unless
 * a == b, a the source b; the order within a target is the pair order */
static void csr_targets (int nn, const int *pairs, int64_t np, int **off_out, int **src_out)
{
  int *off = (int *) calloc ((size_t) nn + 1, sizeof (int));
  int *fill = (int *) malloc ((size_t) nn * sizeof (int));
  int *src;
  int64_t k;
  int i;
  for (k = 0; k < np; k++)
    {
      off[pairs[2 * k + 1] + 1]++;
      if (pairs[2 * k] != pairs[2 * k + 1])
        off[pairs[2 * k] + 1]++;
    }
  for (i = 0; i < nn; i++)
    off[i + 1] += off[i];
  src = (int *) malloc ((size_t) (off[nn] + 1) * sizeof (int));
  memcpy (fill, off, (size_t) nn * sizeof (int));
  for (k = 0; k < np; k++)
    {
      int a = pairs[2 * k], b = pairs[2 * k + 1];
      src[fill[b]++] = a;
      if (a != b)
        src[fill[a]++] = b;
    }
  free (fill);
  *off_out = off;
  *src_out = src;
}

static void th_p2m (void *ctx, int nb)
{
  SolveCtx *s = ((ThrCtx *) ctx)->s;
  const OrNode *nd = &s->t->nodes[nb];
  int i;
  if (!nd->leaf)
    return;
  for (i = nd->begin; i < nd->end; i++)
    {
      int o = s->t->perm[i];
      or_p2m_series (s->xyz + 3 * o, s->q[o], nd->center, &s->mult[nb]);
    }
}

/* M2M into one parent: its children in child order, as up() adds them */
static void th_m2m (void *ctx, int k)
{
  ThrCtx *c = (ThrCtx *) ctx;
  SolveCtx *s = c->s;
  int nb = c->lvl_begin + k, ch;
  const OrNode *nd = &s->t->nodes[nb];
  if (nd->leaf)
    return;
  for (ch = 0; ch < 8; ch++)
    {
      const OrNode *cn = &s->t->nodes[nd->child[ch]];
      if (cnt (cn) != 0)
        or_translate_series (s->cfg->flavour, &s->mult[nd->child[ch]], cn->center,
                             &s->mult[nb], nd->center);
    }
}

static void th_m2l (void *ctx, int nb)
{
  ThrCtx *c = (ThrCtx *) ctx;
  SolveCtx *s = c->s;
  const OrNode *B = &s->t->nodes[nb];
  int k;
  for (k = c->far_off[nb]; k < c->far_off[nb + 1]; k++)
    {
      int a = c->far_src[k];
      or_to_local_series (s->cfg->flavour, &s->mult[a], s->t->nodes[a].center,
                          &s->loc[nb], B->center);
    }
}

/* target side of p2p_pair for every particle of one leaf */
static void th_p2p (void *ctx, int nb)
{
  ThrCtx *c = (ThrCtx *) ctx;
  SolveCtx *s = c->s;
  const OrNode *T = &s->t->nodes[nb];
  int i, k, j;
  for (i = T->begin; i < T->end; i++)
    {
      const double *xi = s->xyz + 3 * s->t->perm[i];
      for (k = c->near_off[nb]; k < c->near_off[nb + 1]; k++)
        {
          const OrNode *S = &s->t->nodes[c->near_src[k]];
          for (j = S->begin; j < S->end; j++)
            {
              const double *xj;
              double d[3], r, qj;
              if (j == i)
                continue;
              xj = s->xyz + 3 * s->t->perm[j];
              qj = s->q[s->t->perm[j]];
              d[0] = xi[0] - xj[0];
              d[1] = xi[1] - xj[1];
              d[2] = xi[2] - xj[2];
              r = sqrt (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
              if (!s->cfg->field)
                {
                  if (r > 0.)
                    s->acc[i] += (1. / r) * qj;
                }
              else if (r > 1.e-5)
                {
                  double inv_r = 1. / r, inv_r3 = inv_r * inv_r * inv_r;
                  s->fld[3 * i] += d[0] * (-inv_r3 * qj);
                  s->fld[3 * i + 1] += d[1] * (-inv_r3 * qj);
                  s->fld[3 * i + 2] += d[2] * (-inv_r3 * qj);
                }
            }
        }
    }
}

static void th_l2l (void *ctx, int k)
{
  ThrCtx *c = (ThrCtx *) ctx;
  SolveCtx *s = c->s;
  int nb = c->lvl_begin + k;
  const OrNode *nd = &s->t->nodes[nb];
  if (cnt (nd) != 0 && nd->father >= 0)
    {
      const OrNode *f = &s->t->nodes[nd->father];
      or_translate_series (s->cfg->flavour, &s->loc[nd->father], f->center, &s->loc[nb],
                           nd->center);
    }
}

static void th_l2p (void *ctx, int nb)
{
  SolveCtx *s = ((ThrCtx *) ctx)->s;
  const OrNode *nd = &s->t->nodes[nb];
  int i;
  if (!nd->leaf)
    return;
  for (i = nd->begin; i < nd->end; i++)
    {
      int o = s->t->perm[i];
      const double *x = s->xyz + 3 * o;
      double rel[3] = { x[0] - nd->center[0], x[1] - nd->center[1], x[2] - nd->center[2] };
      if (s->cfg->field)
        {
          double g[3];
          or_gradient_xyz (&s->loc[nb], rel, g);
          s->fld[3 * i] += g[0];
          s->fld[3 * i + 1] += g[1];
          s->fld[3 * i + 2] += g[2];
        }
      else
        {
          double r, cost, sint, cosp, sinp;
          or_to_spherical_internal (rel, &r, &cost, &sint, &cosp, &sinp);
          s->acc[i] += creal (or_evaluate_internal (&s->loc[nb], r, cost, sint, cosp, sinp));
        }
    }
}

int or_solve_threaded (const OrSolveConfig *cfg, const double *xyz, const double *q,
                       double *pot, double *field, int64_t stats[OR_NSTATS], int nthreads)
{
  OrTree t;
  SolveCtx s;
  ThrCtx c;
  Traversal tv;
  int i, d, p = cfg->order, nlev = 0;
  int ms = or_series_size (0, p), ls = or_series_size (p, 0);
  int *lvl;
  double complex *mstore, *lstore;

  if (nthreads <= 0)
    nthreads = (int) sysconf (_SC_NPROCESSORS_ONLN);
  if (nthreads <= 1 || cfg->semifar_threshold > 0)
    return or_solve (cfg, xyz, q, pot, field, stats);
  if (cfg->n <= 0 || p <= 0)
    return -1;
  tree_build (&t, cfg, xyz);
  memset (stats, 0, OR_NSTATS * sizeof (int64_t));
  memset (&c, 0, sizeof (c));
  s.cfg = cfg;
  s.t = &t;
  s.xyz = xyz;
  s.q = q;
  s.stats = stats;
  s.acc = (double *) calloc ((size_t) cfg->n, sizeof (double));
  s.fld = (double *) calloc ((size_t) cfg->n * 3, sizeof (double));
  s.mult = (OrSeries *) malloc (t.nn * sizeof (OrSeries));
  s.loc = (OrSeries *) malloc (t.nn * sizeof (OrSeries));
  mstore = (double complex *) calloc ((size_t) t.nn * ms, sizeof (double complex));
  lstore = (double complex *) calloc ((size_t) t.nn * ls, sizeof (double complex));
  for (i = 0; i < t.nn; i++)
    {
      s.mult[i].posdeg = 0;
      s.mult[i].negdeg = p;
      s.mult[i].c = mstore + (size_t) i * ms;
      s.loc[i].posdeg = p;
      s.loc[i].negdeg = 0;
      s.loc[i].c = lstore + (size_t) i * ls;
    }
  c.s = &s;
  /* level ranges: the tree is built level by level */
  lvl = (int *) malloc ((size_t) (t.nn + 2) * sizeof (int));
  lvl[0] = 0;
  for (i = 0; i < t.nn; i++)
    if (t.nodes[i].depth != nlev)
      lvl[++nlev] = i;
  lvl[++nlev] = t.nn;
  /* shared read-only tables from here on */
  or_series_init ();
  or_wigner_cache_share (p + 1);

  stats[0] = t.nn;
  stats[2] = cfg->n;
  stats[6] = cfg->n;
  for (i = 0; i < t.nn; i++)
    if (cnt (&t.nodes[i]) != 0 && t.nodes[i].father >= 0)
      {
        stats[3]++;
        stats[5]++;
      }
  /* up: P2M at the leaves, then M2M level by level, deepest parents first */
  par_for (t.nn, nthreads, 64, th_p2m, &c);
  for (d = nlev - 2; d >= 0; d--)
    {
      c.lvl_begin = lvl[d];
      par_for (lvl[d + 1] - lvl[d], nthreads, 8, th_m2m, &c);
    }
  /* near/far pairs in traversal order, then every target's sources */
  tv.far = th_far;
  tv.near = th_near;
  tv.semifar = NULL;
  tv.threshold = 0;
  tv.ctx = &c;
  tv.t = &t;
  pair_traverse (&tv, 0, 0);
  csr_targets (t.nn, c.farp, c.nfar, &c.far_off, &c.far_src);
  csr_targets (t.nn, c.nearp, c.nnear, &c.near_off, &c.near_src);
  par_for (t.nn, nthreads, 16, th_m2l, &c);
  par_for (t.nn, nthreads, 16, th_p2p, &c);
  /* down: L2L level by level, then L2P at the leaves */
  for (d = 1; d < nlev; d++)
    {
      c.lvl_begin = lvl[d];
      par_for (lvl[d + 1] - lvl[d], nthreads, 32, th_l2l, &c);
    }
  par_for (t.nn, nthreads, 64, th_l2p, &c);
  or_wigner_cache_unshare ();

  for (i = 0; i < cfg->n; i++)
    {
      int o = t.perm[i];
      if (cfg->field)
        {
          if (field)
            {
              field[3 * o] = s.fld[3 * i];
              field[3 * o + 1] = s.fld[3 * i + 1];
              field[3 * o + 2] = s.fld[3 * i + 2];
            }
        }
      else if (pot)
        pot[o] = s.acc[i];
    }
  free (lvl);
  free (c.farp);
  free (c.nearp);
  free (c.far_off);
  free (c.far_src);
  free (c.near_off);
  free (c.near_src);
  free (s.acc);
  free (s.fld);
  free (s.mult);
  free (s.loc);
  free (mstore);
  free (lstore);
  tree_free (&t);
  return 0;
}

/* ----------------------------------------------------------- tree lists */
typedef struct
{
  const OrTree *t;
  uint64_t *far;
  int64_t nfar, capfar;
  uint64_t *nearp;
  int64_t nnear, capnear;
} ListCtx;

static void push_pair (uint64_t **arr, int64_t *n, int64_t *cap, uint64_t a,
                       uint64_t b)
{
  if (*n == *cap)
    {
      *cap = *cap ? 2 * *cap : 4096;
      *arr = (uint64_t *) realloc (*arr, (size_t) *cap * 2 * sizeof (uint64_t));
    }
  if (a > b)
    {
      uint64_t t = a;
      a = b;
      b = t;
    }
  (*arr)[2 * *n] = a;
  (*arr)[2 * *n + 1] = b;
  (*n)++;
}

static void lc_far (void *ctx, int a, int b)
{
  ListCtx *c = (ListCtx *) ctx;
  push_pair (&c->far, &c->nfar, &c->capfar, c->t->nodes[a].id,
             c->t->nodes[b].id);
}

static void lc_near (void *ctx, int a, int b)
{
  ListCtx *c = (ListCtx *) ctx;
  push_pair (&c->nearp, &c->nnear, &c->capnear, c->t->nodes[a].id,
             c->t->nodes[b].id);
}

int or_tree_lists (const OrSolveConfig *cfg, const double *xyz,
                   int64_t *n_nodes, uint64_t *node_ids, int32_t *node_begin,
                   int32_t *node_end, uint8_t *node_leaf,
                   int64_t *n_far, uint64_t *far_pairs,
                   int64_t *n_near, uint64_t *near_pairs, int32_t *perm)
{
  OrTree t;
  ListCtx lc;
  Traversal tv;
  int i;
  tree_build (&t, cfg, xyz);
  memset (&lc, 0, sizeof (lc));
  lc.t = &t;
  tv.far = lc_far;
  tv.near = lc_near;
  tv.semifar = NULL;
  tv.threshold = 0;
  tv.ctx = &lc;
  tv.t = &t;
  pair_traverse (&tv, 0, 0);
  *n_nodes = t.nn;
  if (node_ids)
    for (i = 0; i < t.nn; i++)
      {
        node_ids[i] = t.nodes[i].id;
        node_begin[i] = t.nodes[i].begin;
        node_end[i] = t.nodes[i].end;
        node_leaf[i] = (uint8_t) t.nodes[i].leaf;
      }
  *n_far = lc.nfar;
  if (far_pairs)
    memcpy (far_pairs, lc.far, (size_t) lc.nfar * 2 * sizeof (uint64_t));
  *n_near = lc.nnear;
  if (near_pairs)
    memcpy (near_pairs, lc.nearp, (size_t) lc.nnear * 2 * sizeof (uint64_t));
  if (perm)
    memcpy (perm, t.perm, (size_t) cfg->n * sizeof (int32_t));
  free (lc.far);
  free (lc.nearp);
  tree_free (&t);
  return 0;
}

/* ------------------------------------------------------------ direct sum */
typedef struct
{
  int n, nt;
  const double *xyz, *q;
  const int32_t *targets;
  double *pot, *field;
  int t0, t1;
} DirectJob;

/* Neumaier compensated accumulation */
static void nsum (double *s, double *c, double v)
{
  double t = *s + v;
  if (fabs (*s) >= fabs (v))
    *c += (*s - t) + v;
  else
    *c += (v - t) + *s;
  *s = t;
}

static void *direct_worker (void *arg)
{
  DirectJob *j = (DirectJob *) arg;
  int ti, k;
  for (ti = j->t0; ti < j->t1; ti++)
    {
      int i = j->targets ? j->targets[ti] : ti;
      const double *xi = j->xyz + 3 * i;
      double ps = 0, pc = 0, fs[3] = { 0, 0, 0 }, fc[3] = { 0, 0, 0 };
      for (k = 0; k < j->n; k++)
        {
          const double *xk = j->xyz + 3 * k;
          double d[3], r;
          if (k == i)
            continue;
          d[0] = xi[0] - xk[0];
          d[1] = xi[1] - xk[1];
          d[2] = xi[2] - xk[2];
          r = sqrt (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
          if (r == 0.)
            continue;           /* coincident distinct points: skipped */
          nsum (&ps, &pc, j->q[k] / r);
          if (r > 1.e-5)
            {
              double f = -j->q[k] / (r * r * r);
              nsum (&fs[0], &fc[0], f * d[0]);
              nsum (&fs[1], &fc[1], f * d[1]);
              nsum (&fs[2], &fc[2], f * d[2]);
            }
        }
      if (j->pot)
        j->pot[ti] = ps + pc;
      if (j->field)
        {
          j->field[3 * ti] = fs[0] + fc[0];
          j->field[3 * ti + 1] = fs[1] + fc[1];
          j->field[3 * ti + 2] = fs[2] + fc[2];
        }
    }
  return NULL;
}

void or_direct (int n, const double *xyz, const double *q, int nt,
                const int32_t *targets, double *pot, double *field,
                int nthreads)
{
  int t;
  pthread_t th[256];
  DirectJob jobs[256];
  if (nthreads <= 0)
    nthreads = (int) sysconf (_SC_NPROCESSORS_ONLN);
  if (nthreads > 256)
    nthreads = 256;
  if (nthreads > nt)
    nthreads = nt > 0 ? nt : 1;
  for (t = 0; t < nthreads; t++)
    {
      jobs[t].n = n;
      jobs[t].nt = nt;
      jobs[t].xyz = xyz;
      jobs[t].q = q;
      jobs[t].targets = targets;
      jobs[t].pot = pot;
      jobs[t].field = field;
      jobs[t].t0 = (int) ((int64_t) nt * t / nthreads);
      jobs[t].t1 = (int) ((int64_t) nt * (t + 1) / nthreads);
      pthread_create (&th[t], NULL, direct_worker, &jobs[t]);
    }
  for (t = 0; t < nthreads; t++)
    pthread_join (th[t], NULL);
}
