/*
 * or_laurent.c -- 2D Laurent-series operators and the 2D (Cauchy kernel)
 * FMM solve of the oracle.  TEST INFRASTRUCTURE ONLY (see aran_oracle.h).
 *
 * The operators follow the reference's loops term by term, in the same
 * order of complex operations:
 *   P2M   aran/arandevelopment2d.c:167-189 (a_{-i} += q (zp-zm)^{i-1}, i < negdeg)
 *   P2L   aran/arandevelopment2d.c:200-221 (a_i += -q (zp-zl)^{-(i+1)}, i <= posdeg)
 *   M2M / L2L   aran_laurent_seriesd_translate, aran/aranlaurentseriesd.c:358-397,
 *         with aran_taylor_translate :47-73 for the non-negative part
 *   M2L   aran_laurent_seriesd_to_taylor :409-452
 *   L2P / M2P   aran_laurent_seriesd_evaluate :311-347
 * The binomial coefficients are the Pascal-triangle doubles of
 * aran/aranbinomial.c:44-51.
 *
 * The quadtree and its near/far traversal restate, for two dimensions, the
 * contract of the 3D oracle (or_solver.c): 21-bit quantised coordinates, a
 * node with more than maxbox points below max_depth gets all 4 quadrants,
 * same-depth non-adjacent children of adjacent nodes are FAR (M2L both
 * ways, aran/aransolver2d.c:334-357), adjacent leaves are NEAR, a leaf
 * against an adjacent internal node is NEAR with every leaf below it.
 * The P2P kernel is tests/dummypot.c:62-76: one->accum += q_other/(z_one -
 * z_other), other->accum -= q_one/(z_one - z_other).
 */
#include "or_internal.h"

#include <stdlib.h>
#include <string.h>

#define OR2_KEYBITS 21

typedef double complex cplx;

/* ------------------------------------------------------------- binomials */
static double *g_binom = NULL;
static int g_binom_n = -1;

static double binom (int n, int k)
{
  if (n > g_binom_n)
    {
      int nn = n + 16, i, j;
      double *t = (double *) calloc ((size_t) (nn + 1) * (nn + 1), sizeof (double));
      for (i = 0; i <= nn; i++)
        for (j = 0; j <= i; j++)
          t[i * (nn + 1) + j] = (j == 0 || j == i) ? 1. :
            t[(i - 1) * (nn + 1) + j] + t[(i - 1) * (nn + 1) + j - 1];
      free (g_binom);
      g_binom = t;
      g_binom_n = nn;
    }
  if (k < 0 || k > n)
    return 0.;
  return g_binom[n * (g_binom_n + 1) + k];
}

/* term of degree i of a series (posdeg, negdeg) */
#define TERM(s, posdeg, i) ((s) + ((posdeg) - (i)))

/* ------------------------------------------------------------- operators */
void or2_p2m (double x, double y, double q, double cx, double cy, int negdeg,
              double *mult)
{
  cplx *m = (cplx *) mult;    /* laurent (0, negdeg): m[i] is degree -i */
  cplx tmp = q;
  cplx d = (x + I * y) - (cx + I * cy);
  int i;
  m[0] += 0.;
  for (i = 1; i < negdeg; i++)
    {
      m[i] += tmp;
      tmp *= d;
    }
}

void or2_p2l (double x, double y, double q, double cx, double cy, int posdeg,
              double *loc)
{
  cplx *l = TERM ((cplx *) loc, posdeg, 0);
  cplx inv = 1. / ((x + I * y) - (cx + I * cy));
  cplx tmp = -q;
  int i;
  for (i = 0; i <= posdeg; i++)
    {
      tmp *= inv;
      *l += tmp;
      l--;
    }
}

/* aran_taylor_translate: non-negative part of src re-expanded at dst */
static void taylor_translate (int sp, const cplx *src, int dp, cplx *dst,
                              cplx zd_m_zs)
{
  int i, j;
  cplx *dt = TERM (dst, dp, dp);
  for (i = dp; i >= 0; i--)
    {
      const cplx *st = TERM (src, sp, sp);
      cplx sum = *st;
      for (j = sp - 1; j >= i; j--)
        {
          st++;
          sum = sum * zd_m_zs + binom (j, i) * (*st);
        }
      *dt += sum;
      dt++;
    }
}

void or2_translate (int sp, int sn, const double *src_, double zsx, double zsy,
                    int dp, int dn, double *dst_, double zdx, double zdy)
{
  const cplx *src = (const cplx *) src_;
  cplx *dst = (cplx *) dst_;
  cplx zd_m_zs = (zdx + I * zdy) - (zsx + I * zsy);
  int i, j;
  taylor_translate (sp, src, dp, dst, zd_m_zs);
  if (sn > 0)
    {
      cplx zs_m_zd = -zd_m_zs;
      cplx *dt = TERM (dst, dp, -1);
      for (i = 1; i <= dn; i++)
        {
          const cplx *st = TERM (src, sp, -1);
          cplx sum = 0.;
          int jmax = i < sn ? i : sn;
          for (j = 1; j < jmax; j++)
            {
              sum = (sum + binom (i - 1, j - 1) * (*st)) * zs_m_zd;
              st++;
            }
          *dt += sum + *st;
          dt++;
        }
    }
}

void or2_to_taylor (int sp, int sn, const double *src_, double zsx, double zsy,
                    int dp, int dn, double *dst_, double zdx, double zdy)
{
  const cplx *src = (const cplx *) src_;
  cplx *dst = (cplx *) dst_;
  cplx zd_m_zs = (zdx + I * zdy) - (zsx + I * zsy);
  int i, j;
  (void) dn;
  taylor_translate (sp, src, dp, dst, zd_m_zs);
  if (sn > 0)
    {
      cplx inv = 1. / zd_m_zs;
      cplx pw = 1.;
      cplx *dt = TERM (dst, dp, 0);
      for (i = 0; i <= dp; i++)
        {
          const cplx *st = TERM (src, sp, -sn + 1);
          cplx sum = 0.;
          for (j = sn - 1; j >= 1; j--)
            {
              sum = (sum + binom (i + j - 1, j - 1) * (*st)) * inv;
              st--;
            }
          *dt += sum * pw;
          dt--;
          pw *= -inv;
        }
    }
}

static cplx evaluate (int pd, int nd, const cplx *s, cplx z)
{
  const cplx *t = TERM (s, pd, pd);
  cplx pos = *t, neg = 0.;
  int i;
  for (i = 1; i <= pd; i++)
    {
      t++;
      pos = pos * z + *t;
    }
  if (nd != 0)
    {
      cplx invz = 1. / z;
      t = TERM (s, pd, -nd);
      neg = *t;
      for (i = nd - 1; i > 0; i--)
        {
          t--;
          neg = neg * invz + *t;
        }
      neg *= invz;
    }
  return pos + neg;
}

void or2_evaluate (int pd, int nd, const double *s, double zx, double zy,
                   double out[2])
{
  cplx v = evaluate (pd, nd, (const cplx *) s, zx + I * zy);
  out[0] = creal (v);
  out[1] = cimag (v);
}

/* ------------------------------------------------------------------ tree */
typedef struct
{
  int depth;
  int32_t ij[2];
  int begin, end;
  int leaf;
  int child[4];
  int father;
  double center[2];
} Or2Node;

typedef struct
{
  Or2Node *nodes;
  int nn, cap;
  int32_t *perm;       /* sorted position -> index within the system */
  uint64_t *keys;
  int n;
} Or2Tree;

static uint64_t spread2 (uint64_t v)
{
  uint64_t r = 0;
  int b;
  for (b = 0; b < OR2_KEYBITS; b++)
    r |= ((v >> b) & 1ull) << (2 * b);
  return r;
}

static int64_t quantise2 (double x, double lb, double scale)
{
  double t = (x - lb) * scale;
  int64_t i = (int64_t) floor (t);
  if (i < 0)
    i = 0;
  if (i > (1 << OR2_KEYBITS) - 1)
    i = (1 << OR2_KEYBITS) - 1;
  return i;
}

static double center_axis (double lo, double hi, int d, int32_t i)
{
  int b;
  for (b = d - 1; b >= 0; b--)
    {
      double mid = (lo + hi) * 0.5;
      if ((i >> b) & 1)
        lo = mid;
      else
        hi = mid;
    }
  return (lo + hi) * 0.5;
}

typedef struct
{
  uint64_t k;
  int32_t i;
} KeyIdx2;

static int cmp_ki2 (const void *a, const void *b)
{
  const KeyIdx2 *x = (const KeyIdx2 *) a, *y = (const KeyIdx2 *) b;
  if (x->k != y->k)
    return x->k < y->k ? -1 : 1;
  return x->i - y->i;
}

static int push2 (Or2Tree *t)
{
  if (t->nn == t->cap)
    {
      t->cap = t->cap ? 2 * t->cap : 256;
      t->nodes = (Or2Node *) realloc (t->nodes, t->cap * sizeof (Or2Node));
    }
  return t->nn++;
}

static void tree2_build (Or2Tree *t, const Or2Config *cfg, int n,
                         const double *xy, const double box[4])
{
  int i, d, maxd = cfg->max_depth > 0 ? cfg->max_depth : OR2_KEYBITS;
  double sx = (double) (1 << OR2_KEYBITS) / (box[2] - box[0]);
  double sy = (double) (1 << OR2_KEYBITS) / (box[3] - box[1]);
  KeyIdx2 *ki = (KeyIdx2 *) malloc ((size_t) (n > 0 ? n : 1) * sizeof (KeyIdx2));
  int lvl_begin, lvl_end;
  if (maxd > OR2_KEYBITS)
    maxd = OR2_KEYBITS;
  memset (t, 0, sizeof (*t));
  t->n = n;
  for (i = 0; i < n; i++)
    {
      ki[i].k = spread2 ((uint64_t) quantise2 (xy[2 * i], box[0], sx)) |
        (spread2 ((uint64_t) quantise2 (xy[2 * i + 1], box[1], sy)) << 1);
      ki[i].i = i;
    }
  qsort (ki, n, sizeof (KeyIdx2), cmp_ki2);
  t->perm = (int32_t *) malloc ((size_t) (n > 0 ? n : 1) * sizeof (int32_t));
  t->keys = (uint64_t *) malloc ((size_t) (n > 0 ? n : 1) * sizeof (uint64_t));
  for (i = 0; i < n; i++)
    {
      t->perm[i] = ki[i].i;
      t->keys[i] = ki[i].k;
    }
  free (ki);
  {
    int r = push2 (t);
    Or2Node *nd = &t->nodes[r];
    memset (nd, 0, sizeof (*nd));
    nd->end = n;
    nd->father = -1;
    nd->center[0] = center_axis (box[0], box[2], 0, 0);
    nd->center[1] = center_axis (box[1], box[3], 0, 0);
  }
  lvl_begin = 0;
  lvl_end = 1;
  for (d = 0; lvl_begin < lvl_end; d++)
    {
      int nb;
      for (nb = lvl_begin; nb < lvl_end; nb++)
        {
          Or2Node *nd = &t->nodes[nb];
          int c, pos;
          if (nd->end - nd->begin <= cfg->maxbox || d >= maxd)
            {
              nd->leaf = 1;
              for (c = 0; c < 4; c++)
                nd->child[c] = -1;
              continue;
            }
          nd->leaf = 0;
          pos = nd->begin;
          for (c = 0; c < 4; c++)
            {
              int ci = push2 (t);
              int shift = 2 * (OR2_KEYBITS - d - 1);
              int e = pos;
              Or2Node *ch;
              nd = &t->nodes[nb];
              while (e < nd->end && (int) ((t->keys[e] >> shift) & 3ull) == c)
                e++;
              ch = &t->nodes[ci];
              memset (ch, 0, sizeof (*ch));
              ch->depth = d + 1;
              ch->ij[0] = (nd->ij[0] << 1) | (c & 1);
              ch->ij[1] = (nd->ij[1] << 1) | ((c >> 1) & 1);
              ch->begin = pos;
              ch->end = e;
              ch->father = nb;
              ch->center[0] = center_axis (box[0], box[2], d + 1, ch->ij[0]);
              ch->center[1] = center_axis (box[1], box[3], d + 1, ch->ij[1]);
              nd->child[c] = ci;
              pos = e;
            }
        }
      lvl_begin = lvl_end;
      lvl_end = t->nn;
    }
}

static int cnt2 (const Or2Node *n)
{
  return n->end - n->begin;
}

static int adjacent2 (const Or2Node *a, const Or2Node *b)
{
  int k;
  for (k = 0; k < 2; k++)
    {
      int d = a->ij[k] - b->ij[k];
      if (d > 1 || d < -1)
        return 0;
    }
  return 1;
}

/* ----------------------------------------------------------------- solve */
typedef struct
{
  const Or2Config *cfg;
  const Or2Tree *t;
  const double *xy, *q;   /* this system's particles */
  cplx *acc;              /* sorted order */
  cplx *mult, *loc;       /* per node: (p + 1) terms each */
  int64_t *stats;
} Solve2;

static void p2p2 (Solve2 *s, int i, int j)
{
  /* tests/dummypot.c:62-76 with one = i, other = j */
  int oi = s->t->perm[i], oj = s->t->perm[j];
  cplx zd_m_zs = (s->xy[2 * oi] + I * s->xy[2 * oi + 1]) -
    (s->xy[2 * oj] + I * s->xy[2 * oj + 1]);
  cplx inv = 1. / zd_m_zs;
  s->acc[i] += inv * s->q[oj];
  s->acc[j] += -inv * s->q[oi];
}

static void near2 (Solve2 *s, int a, int b)
{
  const Or2Node *A = &s->t->nodes[a], *B = &s->t->nodes[b];
  int i, j;
  if (a == b)
    {
      for (i = A->begin; i < A->end; i++)
        for (j = i + 1; j < A->end; j++)
          p2p2 (s, i, j);
      s->stats[1] += (int64_t) cnt2 (A) * (cnt2 (A) + 1) / 2;
      return;
    }
  for (i = A->begin; i < A->end; i++)
    for (j = B->begin; j < B->end; j++)
      p2p2 (s, i, j);
  s->stats[1] += (int64_t) cnt2 (A) * cnt2 (B);
}

static void far2 (Solve2 *s, int a, int b)
{
  const Or2Node *A = &s->t->nodes[a], *B = &s->t->nodes[b];
  int p = s->cfg->order;
  or2_to_taylor (0, p, (double *) (s->mult + (size_t) a * (p + 1)), A->center[0],
                 A->center[1], p, 0, (double *) (s->loc + (size_t) b * (p + 1)),
                 B->center[0], B->center[1]);
  or2_to_taylor (0, p, (double *) (s->mult + (size_t) b * (p + 1)), B->center[0],
                 B->center[1], p, 0, (double *) (s->loc + (size_t) a * (p + 1)),
                 A->center[0], A->center[1]);
  s->stats[4] += 2;
}

static void near_below2 (Solve2 *s, int leaf, int node)
{
  const Or2Node *nd = &s->t->nodes[node];
  int c;
  if (cnt2 (nd) == 0)
    return;
  if (nd->leaf)
    {
      near2 (s, leaf, node);
      return;
    }
  for (c = 0; c < 4; c++)
    near_below2 (s, leaf, nd->child[c]);
}

static void traverse2 (Solve2 *s, int a, int b)
{
  const Or2Node *A = &s->t->nodes[a], *B = &s->t->nodes[b];
  int i, j;
  if (cnt2 (A) == 0 || cnt2 (B) == 0)
    return;
  if (a == b)
    {
      if (A->leaf)
        {
          near2 (s, a, a);
          return;
        }
      for (i = 0; i < 4; i++)
        for (j = i; j < 4; j++)
          traverse2 (s, A->child[i], A->child[j]);
      return;
    }
  if (A->leaf && B->leaf)
    {
      near2 (s, a, b);
      return;
    }
  if (A->leaf)
    {
      near_below2 (s, a, b);
      return;
    }
  if (B->leaf)
    {
      near_below2 (s, b, a);
      return;
    }
  for (i = 0; i < 4; i++)
    for (j = 0; j < 4; j++)
      {
        int ca = A->child[i], cb = B->child[j];
        const Or2Node *CA = &s->t->nodes[ca], *CB = &s->t->nodes[cb];
        if (cnt2 (CA) == 0 || cnt2 (CB) == 0)
          continue;
        if (adjacent2 (CA, CB))
          traverse2 (s, ca, cb);
        else
          far2 (s, ca, cb);
      }
}

/* up pass (aran/aransolver2d.c:414-452) */
static void up2 (Solve2 *s, int nb)
{
  const Or2Node *nd = &s->t->nodes[nb];
  int p = s->cfg->order, c, i;
  if (!nd->leaf)
    for (c = 0; c < 4; c++)
      up2 (s, nd->child[c]);
  if (nd->leaf)
    for (i = nd->begin; i < nd->end; i++)
      {
        int o = s->t->perm[i];
        or2_p2m (s->xy[2 * o], s->xy[2 * o + 1], s->q[o], nd->center[0], nd->center[1],
                 p, (double *) (s->mult + (size_t) nb * (p + 1)));
        s->stats[2]++;
      }
  if (cnt2 (nd) != 0 && nd->father >= 0)
    {
      const Or2Node *f = &s->t->nodes[nd->father];
      or2_translate (0, p, (double *) (s->mult + (size_t) nb * (p + 1)), nd->center[0],
                     nd->center[1], 0, p, (double *) (s->mult + (size_t) nd->father * (p + 1)),
                     f->center[0], f->center[1]);
      s->stats[3]++;
    }
}

/* down pass (aran/aransolver2d.c:454-492) */
static void down2 (Solve2 *s, int nb)
{
  const Or2Node *nd = &s->t->nodes[nb];
  int p = s->cfg->order, c, i;
  if (cnt2 (nd) != 0 && nd->father >= 0)
    {
      const Or2Node *f = &s->t->nodes[nd->father];
      or2_translate (p, 0, (double *) (s->loc + (size_t) nd->father * (p + 1)), f->center[0],
                     f->center[1], p, 0, (double *) (s->loc + (size_t) nb * (p + 1)),
                     nd->center[0], nd->center[1]);
      s->stats[5]++;
    }
  if (nd->leaf)
    {
      for (i = nd->begin; i < nd->end; i++)
        {
          int o = s->t->perm[i];
          cplx z = (s->xy[2 * o] + I * s->xy[2 * o + 1]) - (nd->center[0] + I * nd->center[1]);
          s->acc[i] += evaluate (p, 0, s->loc + (size_t) nb * (p + 1), z);
          s->stats[6]++;
        }
      return;
    }
  for (c = 0; c < 4; c++)
    down2 (s, nd->child[c]);
}

int or2_solve (const Or2Config *cfg, int nsys, const int64_t *offs,
               const double *xy, const double *q, const double *box,
               double *acc, int64_t stats[OR_NSTATS])
{
  int sys, p = cfg->order;
  if (p < 1 || cfg->maxbox < 1 || nsys < 0)
    return -1;
  memset (stats, 0, OR_NSTATS * sizeof (int64_t));
  for (sys = 0; sys < nsys; sys++)
    {
      int64_t o0 = offs[sys];
      int n = (int) (offs[sys + 1] - o0), i;
      Or2Tree t;
      Solve2 s;
      if (n <= 0)
        continue;
      tree2_build (&t, cfg, n, xy + 2 * o0, box + 4 * sys);
      s.cfg = cfg;
      s.t = &t;
      s.xy = xy + 2 * o0;
      s.q = q + o0;
      s.stats = stats;
      s.acc = (cplx *) calloc ((size_t) n, sizeof (cplx));
      s.mult = (cplx *) calloc ((size_t) t.nn * (p + 1), sizeof (cplx));
      s.loc = (cplx *) calloc ((size_t) t.nn * (p + 1), sizeof (cplx));
      stats[0] += t.nn;
      up2 (&s, 0);
      traverse2 (&s, 0, 0);
      down2 (&s, 0);
      for (i = 0; i < n; i++)
        {
          int o = t.perm[i];
          acc[2 * (o0 + o)] = creal (s.acc[i]);
          acc[2 * (o0 + o) + 1] = cimag (s.acc[i]);
        }
      free (s.acc);
      free (s.mult);
      free (s.loc);
      free (t.nodes);
      free (t.perm);
      free (t.keys);
    }
  return 0;
}

void or2_direct (int n, const double *xy, const double *q, int nt,
                 const int32_t *targets, double *acc)
{
  int k, j;
  for (k = 0; k < nt; k++)
    {
      int i = targets ? targets[k] : k;
      /* Neumaier-compensated sums of the real and imaginary parts */
      double sr = 0., cr = 0., si = 0., ci = 0.;
      for (j = 0; j < n; j++)
        {
          double dx, dy, r2, tr, ti, t;
          if (j == i)
            continue;
          dx = xy[2 * i] - xy[2 * j];
          dy = xy[2 * i + 1] - xy[2 * j + 1];
          r2 = dx * dx + dy * dy;
          tr = q[j] * dx / r2;
          ti = -q[j] * dy / r2;
          t = sr + tr;
          cr += fabs (sr) >= fabs (tr) ? (sr - t) + tr : (tr - t) + sr;
          sr = t;
          t = si + ti;
          ci += fabs (si) >= fabs (ti) ? (si - t) + ti : (ti - t) + si;
          si = t;
        }
      acc[2 * k] = sr + cr;
      acc[2 * k + 1] = si + ci;
    }
}
