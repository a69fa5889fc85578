/*
 * d3force_oracle.c -- CPU restatement (FP64) of d3-force-3d's CPU force simulation.
 *
 * TEST INFRASTRUCTURE ONLY (the checker); see d3force_oracle.h for what it restates and why.
 * Built with -ffp-contract=off so that every a*b+c rounds twice, as JavaScript does.
 */
#include "d3force_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define MAXF 32

typedef struct {
  int32_t type; /* 1 manyBody, 2 link, 3 collide, 4 center, 5 radial, 6 position */
  int32_t mode;
  int32_t iterations;
  double *a, *b, *c; /* per-node or per-link arrays (meaning per type) */
  double p[4];       /* scalars (meaning per type) */
  int32_t m, axis;
  int32_t *src, *dst;
} oforce;

typedef struct {
  int32_t kid[8]; /* internal: children (-1 = empty) */
  int32_t data;   /* leaf: node index; internal: -1 */
  int32_t next;   /* leaf chain (coincident points), newest first */
  double x[3], value, r;
} tnode;

typedef struct {
  tnode* a;
  int32_t len, cap, root, dims;
  double x0[3], x1[3];
} tree;

typedef struct {
  int32_t node;
  double x0[3], x1[3];
} quad;

struct osim {
  int32_t n, ndim;
  double *x, *v, *f; /* n*3 */
  uint8_t* fmask;
  double alpha, alpha_min, alpha_decay, alpha_target, vmul;
  uint32_t lcg;
  oforce forces[MAXF];
  int32_t nforces;
  tree t;
  quad* stack;
  int32_t stack_cap;
  double* coords; /* n*3 accessor values for the tree being built */
  int64_t stats[3];
};

/* ------------------------------------------------------------------ random (src/lcg.js:1-9) */

double ofl_random(osim* s) {
  /* s = (a * s + c) % m with a = 1664525, c = 1013904223, m = 2^32: exact in uint64 */
  s->lcg = (uint32_t)(((uint64_t)1664525u * s->lcg + 1013904223u) & 0xffffffffu);
  return (double)s->lcg / 4294967296.0;
}

/* src/jiggle.js:1-3 */
static double jiggle(osim* s) { return (ofl_random(s) - 0.5) * 1e-6; }

/* ------------------------------------------------------------------ d3 trees */

static void tree_reset(tree* t, int32_t dims) {
  t->len = 0;
  t->root = -1;
  t->dims = dims;
}

static int32_t tree_new(tree* t) {
  if (t->len == t->cap) {
    t->cap = t->cap ? 2 * t->cap : 1024;
    t->a = (tnode*)realloc(t->a, sizeof(tnode) * (size_t)t->cap);
  }
  tnode* q = &t->a[t->len];
  for (int k = 0; k < 8; ++k) q->kid[k] = -1;
  q->data = -1;
  q->next = -1;
  q->value = 0;
  q->r = 0;
  q->x[0] = q->x[1] = q->x[2] = 0;
  return t->len++;
}

static int internal(const tree* t, int32_t q) { return t->a[q].data < 0; }

/* cover(x) for the first point (extent NaN): x0 = floor(x), x1 = x0 + 1; then cover(max):
 * double the extent (the min corner stays, as max >= the first point) until it holds max. */
static void tree_cover(tree* t, const double* lo, const double* hi) {
  int d = t->dims;
  for (int k = 0; k < d; ++k) {
    t->x0[k] = floor(lo[k]);
    t->x1[k] = t->x0[k] + 1;
  }
  double z = t->x1[0] - t->x0[0];
  if (z == 0) z = 1;
  for (;;) {
    int inside = 1;
    for (int k = 0; k < d; ++k)
      if (t->x0[k] > hi[k] || hi[k] >= t->x1[k]) inside = 0;
    if (inside) break;
    z *= 2;
    for (int k = 0; k < d; ++k) t->x1[k] = t->x0[k] + z;
  }
}

/* add(tree, point di): midpoint descent; coincident -> chained (newest first); else split
 * until the old and new points separate. */
static void tree_add(tree* t, int32_t di, const double* P) {
  int d = t->dims;
  const double* p = &P[3 * (size_t)di];
  int32_t leaf = tree_new(t);
  t->a[leaf].data = di;
  if (t->root < 0) {
    t->root = leaf;
    return;
  }
  double x0[3], x1[3], xm;
  for (int k = 0; k < d; ++k) x0[k] = t->x0[k], x1[k] = t->x1[k];
  int32_t node = t->root, parent = -1;
  int i = 0;
  while (internal(t, node)) {
    int idx = 0;
    for (int k = 0; k < d; ++k) {
      xm = (x0[k] + x1[k]) / 2;
      if (p[k] >= xm) x0[k] = xm, idx |= 1 << k;
      else x1[k] = xm;
    }
    parent = node, i = idx;
    node = t->a[parent].kid[i];
    if (node < 0) {
      t->a[parent].kid[i] = leaf;
      return;
    }
  }
  const double* q = &P[3 * (size_t)t->a[node].data];
  int same = 1;
  for (int k = 0; k < d; ++k)
    if (p[k] != q[k]) same = 0;
  if (same) {
    t->a[leaf].next = node;
    if (parent >= 0) t->a[parent].kid[i] = leaf;
    else t->root = leaf;
    return;
  }
  int j, guard = 0;
  do {
    int32_t np = tree_new(t);
    if (parent >= 0) t->a[parent].kid[i] = np;
    else t->root = np;
    parent = np;
    int idx = 0, jdx = 0;
    for (int k = 0; k < d; ++k) {
      xm = (x0[k] + x1[k]) / 2;
      if (p[k] >= xm) x0[k] = xm, idx |= 1 << k;
      else x1[k] = xm;
      if (q[k] >= xm) jdx |= 1 << k;
    }
    i = idx, j = jdx;
  } while (i == j && ++guard < 2200);
  t->a[parent].kid[j] = node;
  t->a[parent].kid[i] = leaf;
}

/* d3's tree(nodes, accessors): extent of the points, cover, then add them in order. */
static void tree_build(osim* s, const double* P) {
  tree* t = &s->t;
  tree_reset(t, s->ndim);
  int d = s->ndim;
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  int any = 0;
  for (int32_t i = 0; i < s->n; ++i) {
    const double* p = &P[3 * (size_t)i];
    int bad = 0;
    for (int k = 0; k < d; ++k)
      if (isnan(p[k])) bad = 1;
    if (bad) continue;
    any = 1;
    for (int k = 0; k < d; ++k) {
      if (p[k] < lo[k]) lo[k] = p[k];
      if (p[k] > hi[k]) hi[k] = p[k];
    }
  }
  if (!any) return;
  tree_cover(t, lo, hi);
  for (int32_t i = 0; i < s->n; ++i) {
    const double* p = &P[3 * (size_t)i];
    int bad = 0;
    for (int k = 0; k < d; ++k)
      if (isnan(p[k])) bad = 1;
    if (!bad) tree_add(t, i, P);
  }
}

static void stack_push(osim* s, int32_t* sp, int32_t node, const double* x0, const double* x1) {
  if (*sp == s->stack_cap) {
    s->stack_cap = s->stack_cap ? 2 * s->stack_cap : 4096;
    s->stack = (quad*)realloc(s->stack, sizeof(quad) * (size_t)s->stack_cap);
  }
  quad* q = &s->stack[(*sp)++];
  q->node = node;
  for (int k = 0; k < 3; ++k) q->x0[k] = x0[k], q->x1[k] = x1[k];
}

/* Children of an internal node, with their bounds, pushed so that child 0 pops first. */
static void push_children(osim* s, int32_t* sp, const quad* q, int reverse) {
  const tree* t = &s->t;
  int d = t->dims, nk = 1 << d;
  double xm[3];
  for (int k = 0; k < d; ++k) xm[k] = (q->x0[k] + q->x1[k]) / 2;
  for (int c0 = 0; c0 < nk; ++c0) {
    int c = reverse ? nk - 1 - c0 : c0;
    int32_t child = t->a[q->node].kid[c];
    if (child < 0) continue;
    double x0[3] = {0, 0, 0}, x1[3] = {0, 0, 0};
    for (int k = 0; k < d; ++k) {
      if ((c >> k) & 1) x0[k] = xm[k], x1[k] = q->x1[k];
      else x0[k] = q->x0[k], x1[k] = xm[k];
    }
    stack_push(s, sp, child, x0, x1);
  }
}

/* visitAfter: post-order over the tree; children before their parent. */
typedef void (*after_fn)(osim* s, int32_t q);
static void visit_after(osim* s, after_fn fn) {
  tree* t = &s->t;
  if (t->root < 0) return;
  int32_t sp = 0;
  int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (size_t)t->len);
  int32_t no = 0;
  stack_push(s, &sp, t->root, t->x0, t->x1);
  while (sp > 0) {
    quad q = s->stack[--sp];
    if (internal(t, q.node)) push_children(s, &sp, &q, 0);
    order[no++] = q.node;
  }
  while (no > 0) fn(s, order[--no]);
  free(order);
}

/* ------------------------------------------------------------------ many-body (src/manyBody.js) */

static const double* g_strengths;

static void mb_accumulate(osim* s, int32_t qi) {
  tree* t = &s->t;
  tnode* q = &t->a[qi];
  int d = s->ndim;
  double strength = 0, weight = 0, x = 0, y = 0, z = 0, c;
  if (internal(t, qi)) {
    int nk = 1 << d;
    for (int i = 0; i < nk; ++i) {
      int32_t k = q->kid[i];
      if (k < 0) continue;
      const tnode* ch = &t->a[k];
      c = fabs(ch->value);
      if (!(c != 0)) continue; /* `c = Math.abs(q.value)` is falsy for 0 and NaN */
      strength += ch->value, weight += c;
      x += c * (isnan(ch->x[0]) ? 0 : ch->x[0]);
      y += c * (isnan(ch->x[1]) ? 0 : ch->x[1]);
      z += c * (isnan(ch->x[2]) ? 0 : ch->x[2]);
    }
    strength *= sqrt(4.0 / nk);
    q->x[0] = x / weight;
    if (d > 1) q->x[1] = y / weight;
    if (d > 2) q->x[2] = z / weight;
  } else {
    const double* p = &s->x[3 * (size_t)q->data];
    q->x[0] = p[0];
    if (d > 1) q->x[1] = p[1];
    if (d > 2) q->x[2] = p[2];
    int32_t l = qi;
    do strength += g_strengths[t->a[l].data];
    while ((l = t->a[l].next) >= 0);
  }
  q->value = strength;
}

/* apply() of src/manyBody.js:73-115 for one node: the d3 walk from the root of the tree the
 * caller built (tree_build + visit_after(mb_accumulate)), adding the node's velocity change to
 * acc[0..2]. */
static void mb_walk_node(osim* s, oforce* f, int32_t ni, double alpha, double* acc) {
  int d = s->ndim;
  double theta2 = f->p[2], dmin2 = f->p[0], dmax2 = f->p[1];
  tree* t = &s->t;
  const double* np = &s->x[3 * (size_t)ni];
  double* nv = acc;
  int32_t sp = 0;
  stack_push(s, &sp, t->root, t->x0, t->x1);
  while (sp > 0) {
    quad q = s->stack[--sp];
    tnode* tn = &t->a[q.node];
    /* apply(treeNode, x0, ..., x1, ...) */
    if (!(tn->value != 0)) continue; /* `!treeNode.value` (0 or NaN): skip the cell */
    double x = tn->x[0] - np[0];
    double y = d > 1 ? tn->x[1] - np[1] : 0;
    double z = d > 2 ? tn->x[2] - np[2] : 0;
    double w = q.x1[0] - q.x0[0];
    double l = x * x + y * y + z * z;
    int isint = internal(t, q.node);
    if (w * w / theta2 < l) {
      if (l < dmax2) {
        if (x == 0) x = jiggle(s), l += x * x;
        if (d > 1 && y == 0) y = jiggle(s), l += y * y;
        if (d > 2 && z == 0) z = jiggle(s), l += z * z;
        if (l < dmin2) l = sqrt(dmin2 * l);
        nv[0] += x * tn->value * alpha / l;
        if (d > 1) nv[1] += y * tn->value * alpha / l;
        if (d > 2) nv[2] += z * tn->value * alpha / l;
      }
      if (isint) s->stats[0]++;
      continue;
    }
    if (isint) {
      s->stats[2]++;
      push_children(s, &sp, &q, 1);
      continue;
    }
    if (l >= dmax2) continue;
    if (tn->data != ni || tn->next >= 0) {
      if (x == 0) x = jiggle(s), l += x * x;
      if (d > 1 && y == 0) y = jiggle(s), l += y * y;
      if (d > 2 && z == 0) z = jiggle(s), l += z * z;
      if (l < dmin2) l = sqrt(dmin2 * l);
    }
    int32_t li = q.node;
    do {
      if (t->a[li].data != ni) {
        w = g_strengths[t->a[li].data] * alpha / l;
        nv[0] += x * w;
        if (d > 1) nv[1] += y * w;
        if (d > 2) nv[2] += z * w;
        s->stats[1]++;
      }
    } while ((li = t->a[li].next) >= 0);
  }
}

/* The tree of force f over the current positions, with d3's cell values and centroids. */
static int mb_prepare(osim* s, oforce* f) {
  g_strengths = f->a;
  tree_build(s, s->x);
  visit_after(s, mb_accumulate);
  return s->t.root >= 0;
}

static void manybody_tree(osim* s, oforce* f, double alpha) {
  if (!mb_prepare(s, f)) return;
  for (int32_t ni = 0; ni < s->n; ++ni) mb_walk_node(s, f, ni, alpha, &s->v[3 * (size_t)ni]);
}

/* FP64 exact sum over all pairs for node i, with the same distanceMin / distanceMax rule. */
static void mb_exact_node(const osim* s, const oforce* f, int32_t i, double alpha, double* out3) {
  int d = s->ndim;
  int32_t n = s->n;
  double dmin2 = f->p[0], dmax2 = f->p[1];
  const double* pi = &s->x[3 * (size_t)i];
  double ax = 0, ay = 0, az = 0;
  for (int32_t j = 0; j < n; ++j) {
    if (j == i || f->a[j] == 0) continue;
    const double* pj = &s->x[3 * (size_t)j];
    double x = pj[0] - pi[0], y = d > 1 ? pj[1] - pi[1] : 0, z = d > 2 ? pj[2] - pi[2] : 0;
    double l = x * x + y * y + z * z;
    if (l >= dmax2 || l == 0) continue;
    if (l < dmin2) l = sqrt(dmin2 * l);
    double w = f->a[j] * alpha / l;
    ax += x * w, ay += y * w, az += z * w;
  }
  out3[0] = ax, out3[1] = d > 1 ? ay : 0, out3[2] = d > 2 ? az : 0;
}

static void manybody_exact(osim* s, oforce* f, double alpha) {
  int d = s->ndim;
  int32_t n = s->n;
  double* acc = (double*)calloc(3 * (size_t)n, sizeof(double));
  for (int32_t i = 0; i < n; ++i) mb_exact_node(s, f, i, alpha, &acc[3 * (size_t)i]);
  for (int32_t i = 0; i < n; ++i)
    for (int k = 0; k < d; ++k) s->v[3 * (size_t)i + k] += acc[3 * (size_t)i + k];
  free(acc);
}

typedef struct {
  const osim* s;
  const oforce* f;
  double alpha;
  const int32_t* targets;
  int32_t lo, hi;
  double* out3;
} probe_job;

static void* probe_exact_run(void* arg) {
  probe_job* j = (probe_job*)arg;
  for (int32_t k = j->lo; k < j->hi; ++k)
    mb_exact_node(j->s, j->f, j->targets[k], j->alpha, &j->out3[3 * (size_t)k]);
  return NULL;
}

int32_t ofl_manybody_probe(osim* s, int32_t k, double alpha, int32_t mode, int32_t count,
                           const int32_t* targets, int32_t threads, double* out3) {
  if (k < 0 || k >= s->nforces || s->forces[k].type != 1 || count < 0) return -1;
  oforce* f = &s->forces[k];
  for (int32_t i = 0; i < count; ++i)
    if (targets[i] < 0 || targets[i] >= s->n) return -1;
  memset(out3, 0, sizeof(double) * 3 * (size_t)count);
  if (mode != OFL_MODE_EXACT) {
    memset(s->stats, 0, sizeof(s->stats));
    if (!mb_prepare(s, f)) return 0;
    for (int32_t i = 0; i < count; ++i) mb_walk_node(s, f, targets[i], alpha, &out3[3 * (size_t)i]);
    return 0;
  }
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  if (threads > count) threads = count > 0 ? count : 1;
  pthread_t tid[256];
  probe_job jobs[256];
  for (int32_t t = 0; t < threads; ++t) {
    jobs[t].s = s, jobs[t].f = f, jobs[t].alpha = alpha, jobs[t].targets = targets;
    jobs[t].lo = (int32_t)((int64_t)count * t / threads);
    jobs[t].hi = (int32_t)((int64_t)count * (t + 1) / threads);
    jobs[t].out3 = out3;
  }
  int32_t started = 0;
  for (int32_t t = 1; t < threads; ++t) {
    if (pthread_create(&tid[t], NULL, probe_exact_run, &jobs[t]) != 0) break;
    started = t;
  }
  probe_exact_run(&jobs[0]);
  for (int32_t t = 1; t <= started; ++t) pthread_join(tid[t], NULL);
  for (int32_t t = started + 1; t < threads; ++t) probe_exact_run(&jobs[t]);  // not started
  return 0;
}

/* ------------------------------------------------------------------ link (src/link.js) */

static void link_force(osim* s, oforce* f, double alpha) {
  int d = s->ndim;
  double* snap = NULL;
  if (f->mode == OFL_MODE_JACOBI) snap = (double*)malloc(sizeof(double) * 3 * (size_t)s->n);
  for (int32_t k = 0; k < f->iterations; ++k) {
    if (snap)
      for (size_t i = 0; i < 3 * (size_t)s->n; ++i) snap[i] = s->x[i] + s->v[i];
    for (int32_t i = 0; i < f->m; ++i) {
      int32_t si = f->src[i], ti = f->dst[i];
      double *sp = &s->x[3 * (size_t)si], *sv = &s->v[3 * (size_t)si];
      double *tp = &s->x[3 * (size_t)ti], *tv = &s->v[3 * (size_t)ti];
      double x, y = 0, z = 0, l, b;
      if (snap) {
        double *a = &snap[3 * (size_t)ti], *c = &snap[3 * (size_t)si];
        x = a[0] - c[0];
        if (!(x != 0)) x = jiggle(s);
        if (d > 1) { y = a[1] - c[1]; if (!(y != 0)) y = jiggle(s); }
        if (d > 2) { z = a[2] - c[2]; if (!(z != 0)) z = jiggle(s); }
      } else {
        x = tp[0] + tv[0] - sp[0] - sv[0];
        if (!(x != 0)) x = jiggle(s);
        if (d > 1) { y = tp[1] + tv[1] - sp[1] - sv[1]; if (!(y != 0)) y = jiggle(s); }
        if (d > 2) { z = tp[2] + tv[2] - sp[2] - sv[2]; if (!(z != 0)) z = jiggle(s); }
      }
      l = sqrt(x * x + y * y + z * z);
      l = (l - f->a[i]) / l * alpha * f->b[i];
      x *= l, y *= l, z *= l;
      b = f->c[i];
      tv[0] -= x * b;
      if (d > 1) tv[1] -= y * b;
      if (d > 2) tv[2] -= z * b;
      b = 1 - b;
      sv[0] += x * b;
      if (d > 1) sv[1] += y * b;
      if (d > 2) sv[2] += z * b;
    }
  }
  free(snap);
}

/* ------------------------------------------------------------------ collide (src/collide.js) */

static const double* g_radii;

static void collide_prepare(osim* s, int32_t qi) {
  tree* t = &s->t;
  tnode* q = &t->a[qi];
  if (!internal(t, qi)) {
    q->r = g_radii[q->data];
    return;
  }
  q->r = 0;
  int nk = 1 << s->ndim;
  for (int i = 0; i < nk; ++i) {
    int32_t k = q->kid[i];
    if (k >= 0 && t->a[k].r > q->r) q->r = t->a[k].r;
  }
}

static void collide_tree(osim* s, oforce* f) {
  int d = s->ndim;
  int32_t n = s->n;
  double strength = f->p[0];
  g_radii = f->a;
  for (int32_t k = 0; k < f->iterations; ++k) {
    for (size_t i = 0; i < 3 * (size_t)n; ++i) s->coords[i] = s->x[i] + s->v[i];
    tree_build(s, s->coords);
    visit_after(s, collide_prepare);
    tree* t = &s->t;
    if (t->root < 0) continue;
    for (int32_t ni = 0; ni < n; ++ni) {
      double ri = g_radii[ni], ri2 = ri * ri;
      double* np = &s->x[3 * (size_t)ni];
      double* nv = &s->v[3 * (size_t)ni];
      double xi = np[0] + nv[0], yi = 0, zi = 0;
      if (d > 1) yi = np[1] + nv[1];
      if (d > 2) zi = np[2] + nv[2];
      int32_t sp = 0;
      stack_push(s, &sp, t->root, t->x0, t->x1);
      while (sp > 0) {
        quad q = s->stack[--sp];
        tnode* tn = &t->a[q.node];
        double rj = tn->r, r = ri + rj;
        if (!internal(t, q.node)) {
          int32_t di = tn->data;
          if (di > ni) {
            double* dp = &s->x[3 * (size_t)di];
            double* dv = &s->v[3 * (size_t)di];
            double x = xi - dp[0] - dv[0];
            double y = d > 1 ? yi - dp[1] - dv[1] : 0;
            double z = d > 2 ? zi - dp[2] - dv[2] : 0;
            double l = x * x + y * y + z * z;
            if (l < r * r) {
              if (x == 0) x = jiggle(s), l += x * x;
              if (d > 1 && y == 0) y = jiggle(s), l += y * y;
              if (d > 2 && z == 0) z = jiggle(s), l += z * z;
              l = sqrt(l);
              l = (r - l) / l * strength;
              rj *= rj;
              r = rj / (ri2 + rj);
              x *= l;
              nv[0] += x * r;
              if (d > 1) y *= l, nv[1] += y * r;
              if (d > 2) z *= l, nv[2] += z * r;
              r = 1 - r;
              dv[0] -= x * r;
              if (d > 1) dv[1] -= y * r;
              if (d > 2) dv[2] -= z * r;
            }
          }
          continue;
        }
        int prune = q.x0[0] > xi + r || q.x1[0] < xi - r ||
                    (d > 1 && (q.x0[1] > yi + r || q.x1[1] < yi - r)) ||
                    (d > 2 && (q.x0[2] > zi + r || q.x1[2] < zi - r));
        if (!prune) push_children(s, &sp, &q, 1);
      }
    }
  }
}

/* Every pair once against one snapshot of p + v; each node gets its own share. */
static void collide_jacobi(osim* s, oforce* f) {
  int d = s->ndim;
  int32_t n = s->n;
  double strength = f->p[0];
  double* acc = (double*)malloc(sizeof(double) * 3 * (size_t)n);
  for (int32_t k = 0; k < f->iterations; ++k) {
    for (size_t i = 0; i < 3 * (size_t)n; ++i) s->coords[i] = s->x[i] + s->v[i], acc[i] = 0;
    for (int32_t i = 0; i < n; ++i) {
      double ri = f->a[i], ri2 = ri * ri;
      const double* pi = &s->coords[3 * (size_t)i];
      for (int32_t j = i + 1; j < n; ++j) {
        const double* pj = &s->coords[3 * (size_t)j];
        double rj = f->a[j], r = ri + rj;
        double x = pi[0] - pj[0], y = d > 1 ? pi[1] - pj[1] : 0, z = d > 2 ? pi[2] - pj[2] : 0;
        double l = x * x + y * y + z * z;
        if (!(l < r * r) || l == 0) continue;
        l = sqrt(l);
        l = (r - l) / l * strength;
        double rj2 = rj * rj, w = rj2 / (ri2 + rj2);
        acc[3 * (size_t)i] += x * l * w, acc[3 * (size_t)i + 1] += y * l * w,
            acc[3 * (size_t)i + 2] += z * l * w;
        w = 1 - w;
        acc[3 * (size_t)j] -= x * l * w, acc[3 * (size_t)j + 1] -= y * l * w,
            acc[3 * (size_t)j + 2] -= z * l * w;
      }
    }
    for (int32_t i = 0; i < n; ++i)
      for (int kk = 0; kk < d; ++kk) s->v[3 * (size_t)i + kk] += acc[3 * (size_t)i + kk];
  }
  free(acc);
}

/* collide_jacobi's velocity change of target node t in one iteration, from the snapshot
 * coords = x + v: every pair (a, b), a < b, that holds t, with the same expressions as the loop
 * of collide_jacobi, and in its order (pairs (j, t) for j < t, then (t, j) for j > t), so the
 * same value. */
static void collide_jacobi_node(const osim* s, const oforce* f, const double* coords, int32_t t,
                                double* out3) {
  int d = s->ndim;
  int32_t n = s->n;
  double strength = f->p[0];
  double ax = 0, ay = 0, az = 0;
  for (int32_t j = 0; j < n; ++j) {
    if (j == t) continue;
    const int32_t a = j < t ? j : t, b = j < t ? t : j;
    const double* pa = &coords[3 * (size_t)a];
    const double* pb = &coords[3 * (size_t)b];
    double ra = f->a[a], rb = f->a[b], r = ra + rb;
    double x = pa[0] - pb[0], y = d > 1 ? pa[1] - pb[1] : 0, z = d > 2 ? pa[2] - pb[2] : 0;
    double l = x * x + y * y + z * z;
    if (!(l < r * r) || l == 0) continue;
    l = sqrt(l);
    l = (r - l) / l * strength;
    double ra2 = ra * ra, rb2 = rb * rb, w = rb2 / (ra2 + rb2);
    if (t == a) {
      ax += x * l * w, ay += y * l * w, az += z * l * w;
    } else {
      w = 1 - w;
      ax -= x * l * w, ay -= y * l * w, az -= z * l * w;
    }
  }
  out3[0] = ax, out3[1] = d > 1 ? ay : 0, out3[2] = d > 2 ? az : 0;
}

typedef struct {
  const osim* s;
  const oforce* f;
  const double* coords;
  const int32_t* targets;
  int32_t lo, hi;
  double* out3;
} collide_job;

static void* collide_probe_run(void* arg) {
  collide_job* j = (collide_job*)arg;
  for (int32_t k = j->lo; k < j->hi; ++k)
    collide_jacobi_node(j->s, j->f, j->coords, j->targets[k], &j->out3[3 * (size_t)k]);
  return NULL;
}

int32_t ofl_collide_probe(osim* s, int32_t k, int32_t count, const int32_t* targets,
                          int32_t threads, double* out3) {
  if (k < 0 || k >= s->nforces || s->forces[k].type != 3 || count < 0) return -1;
  const oforce* f = &s->forces[k];
  for (int32_t i = 0; i < count; ++i)
    if (targets[i] < 0 || targets[i] >= s->n) return -1;
  double* coords = (double*)malloc(sizeof(double) * 3 * (size_t)(s->n > 0 ? s->n : 1));
  for (size_t i = 0; i < 3 * (size_t)s->n; ++i) coords[i] = s->x[i] + s->v[i];
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  if (threads > count) threads = count > 0 ? count : 1;
  pthread_t tid[256];
  collide_job jobs[256];
  for (int32_t t = 0; t < threads; ++t) {
    jobs[t].s = s, jobs[t].f = f, jobs[t].coords = coords, jobs[t].targets = targets;
    jobs[t].lo = (int32_t)((int64_t)count * t / threads);
    jobs[t].hi = (int32_t)((int64_t)count * (t + 1) / threads);
    jobs[t].out3 = out3;
  }
  int32_t started = 0;
  for (int32_t t = 1; t < threads; ++t) {
    if (pthread_create(&tid[t], NULL, collide_probe_run, &jobs[t]) != 0) break;
    started = t;
  }
  collide_probe_run(&jobs[0]);
  for (int32_t t = 1; t <= started; ++t) pthread_join(tid[t], NULL);
  for (int32_t t = started + 1; t < threads; ++t) collide_probe_run(&jobs[t]);  /* not started */
  free(coords);
  return 0;
}

/* ------------------------------------------------------------------ center, radial, x/y/z */

static void center_force(osim* s, oforce* f) {
  int32_t n = s->n;
  double sx = 0, sy = 0, sz = 0, v;
  for (int32_t i = 0; i < n; ++i) {
    const double* p = &s->x[3 * (size_t)i];
    v = p[0], sx += (v != 0 && !isnan(v)) ? v : 0; /* `node.x || 0` */
    v = s->ndim > 1 ? p[1] : 0, sy += (v != 0 && !isnan(v)) ? v : 0;
    v = s->ndim > 2 ? p[2] : 0, sz += (v != 0 && !isnan(v)) ? v : 0;
  }
  double st = f->p[3];
  sx = (sx / n - f->p[0]) * st, sy = (sy / n - f->p[1]) * st, sz = (sz / n - f->p[2]) * st;
  /* Axes beyond numDimensions hold no value in the reference's nodes; they are left alone. */
  for (int32_t i = 0; i < n; ++i) {
    double* p = &s->x[3 * (size_t)i];
    if (sx != 0 && !isnan(sx)) p[0] -= sx;
    if (s->ndim > 1 && sy != 0 && !isnan(sy)) p[1] -= sy;
    if (s->ndim > 2 && sz != 0 && !isnan(sz)) p[2] -= sz;
  }
}

static double or1e6(double v) { return (v != 0 && !isnan(v)) ? v : 1e-6; }

static void radial_force(osim* s, oforce* f, double alpha) {
  int d = s->ndim;
  for (int32_t i = 0; i < s->n; ++i) {
    double* p = &s->x[3 * (size_t)i];
    double* v = &s->v[3 * (size_t)i];
    double dx = or1e6(p[0] - f->p[0]);
    double dy = or1e6((d > 1 ? p[1] : 0) - f->p[1]);
    double dz = or1e6((d > 2 ? p[2] : 0) - f->p[2]);
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    double k = (f->a[i] - r) * f->b[i] * alpha / r;
    v[0] += dx * k;
    if (d > 1) v[1] += dy * k;
    if (d > 2) v[2] += dz * k;
  }
}

static void position_force(osim* s, oforce* f, double alpha) {
  int ax = f->axis;
  if (ax >= s->ndim) return; /* the axis does not exist in this simulation */
  for (int32_t i = 0; i < s->n; ++i)
    s->v[3 * (size_t)i + ax] += (f->a[i] - s->x[3 * (size_t)i + ax]) * f->b[i] * alpha;
}

/* ------------------------------------------------------------------ simulation */

static const double kInitialRadius = 10;

osim* ofl_create(int32_t n, int32_t ndim, const double* xyz, const double* vxyz,
                 const double* fxyz, const uint8_t* fmask) {
  osim* s = (osim*)calloc(1, sizeof(osim));
  if (ndim < 1) ndim = 1;
  if (ndim > 3) ndim = 3;
  s->n = n, s->ndim = ndim;
  s->x = (double*)calloc(3 * (size_t)(n > 0 ? n : 1), sizeof(double));
  s->v = (double*)calloc(3 * (size_t)(n > 0 ? n : 1), sizeof(double));
  s->f = (double*)calloc(3 * (size_t)(n > 0 ? n : 1), sizeof(double));
  s->coords = (double*)calloc(3 * (size_t)(n > 0 ? n : 1), sizeof(double));
  s->fmask = (uint8_t*)calloc((size_t)(n > 0 ? n : 1), 1);
  s->alpha = 1, s->alpha_min = 0.001, s->alpha_decay = 1 - pow(0.001, 1.0 / 300);
  s->alpha_target = 0, s->vmul = 0.6, s->lcg = 1;
  double roll = M_PI * (3 - sqrt(5.0)), yaw = M_PI * 20 / (9 + sqrt(221.0));
  for (int32_t i = 0; i < n; ++i) {
    double* p = &s->x[3 * (size_t)i];
    double* v = &s->v[3 * (size_t)i];
    for (int k = 0; k < 3; ++k) {
      p[k] = xyz ? xyz[3 * (size_t)i + k] : NAN;
      v[k] = vxyz ? vxyz[3 * (size_t)i + k] : NAN;
    }
    uint8_t m = fmask ? fmask[i] : 0;
    s->fmask[i] = m;
    for (int k = 0; k < 3; ++k) {
      s->f[3 * (size_t)i + k] = fxyz ? fxyz[3 * (size_t)i + k] : 0;
      if (m & (1 << k)) p[k] = s->f[3 * (size_t)i + k];
    }
    if (isnan(p[0]) || (ndim > 1 && isnan(p[1])) || (ndim > 2 && isnan(p[2]))) {
      double radius = kInitialRadius * (ndim > 2 ? cbrt(0.5 + i) : (ndim > 1 ? sqrt(0.5 + i) : i));
      double ra = i * roll, ya = i * yaw;
      if (ndim == 1) {
        p[0] = radius;
      } else if (ndim == 2) {
        p[0] = radius * cos(ra);
        p[1] = radius * sin(ra);
      } else {
        p[0] = radius * sin(ra) * cos(ya);
        p[1] = radius * cos(ra);
        p[2] = radius * sin(ra) * sin(ya);
      }
    }
    if (isnan(v[0]) || (ndim > 1 && isnan(v[1])) || (ndim > 2 && isnan(v[2]))) {
      v[0] = 0;
      if (ndim > 1) v[1] = 0;
      if (ndim > 2) v[2] = 0;
    }
    /* axes beyond numDimensions: the reference leaves them undefined; here they hold 0 */
    for (int k = ndim; k < 3; ++k) {
      if (isnan(p[k])) p[k] = 0;
      if (isnan(v[k])) v[k] = 0;
    }
  }
  return s;
}

static void force_free(oforce* f) {
  free(f->a), free(f->b), free(f->c), free(f->src), free(f->dst);
  memset(f, 0, sizeof(*f));
}

void ofl_destroy(osim* s) {
  if (!s) return;
  ofl_clear_forces(s);
  free(s->x), free(s->v), free(s->f), free(s->fmask), free(s->coords);
  free(s->t.a), free(s->stack);
  free(s);
}

void ofl_set_params(osim* s, double alpha, double alpha_min, double alpha_decay,
                    double alpha_target, double velocity_multiplier) {
  s->alpha = alpha, s->alpha_min = alpha_min, s->alpha_decay = alpha_decay;
  s->alpha_target = alpha_target, s->vmul = velocity_multiplier;
}

void ofl_get_params(const osim* s, double* o) {
  o[0] = s->alpha, o[1] = s->alpha_min, o[2] = s->alpha_decay, o[3] = s->alpha_target,
  o[4] = s->vmul;
}

void ofl_set_pins(osim* s, const double* fxyz, const uint8_t* fmask) {
  for (int32_t i = 0; i < s->n; ++i) {
    s->fmask[i] = fmask ? fmask[i] : 0;
    for (int k = 0; k < 3; ++k) s->f[3 * (size_t)i + k] = fxyz ? fxyz[3 * (size_t)i + k] : 0;
  }
}

void ofl_get_state(const osim* s, double* xyz, double* vxyz) {
  if (xyz) memcpy(xyz, s->x, sizeof(double) * 3 * (size_t)s->n);
  if (vxyz) memcpy(vxyz, s->v, sizeof(double) * 3 * (size_t)s->n);
}

void ofl_set_state(osim* s, const double* xyz, const double* vxyz) {
  if (xyz) memcpy(s->x, xyz, sizeof(double) * 3 * (size_t)s->n);
  if (vxyz) memcpy(s->v, vxyz, sizeof(double) * 3 * (size_t)s->n);
}

uint32_t ofl_get_lcg(const osim* s) { return s->lcg; }
void ofl_set_lcg(osim* s, uint32_t state) { s->lcg = state; }

static double* dup(const double* a, size_t n, double fill) {
  double* out = (double*)malloc(sizeof(double) * (n ? n : 1));
  for (size_t i = 0; i < n; ++i) out[i] = a ? a[i] : fill;
  return out;
}

int32_t ofl_add_manybody(osim* s, const double* strengths, double dmin2, double dmax2,
                         double theta2, int32_t mode) {
  if (s->nforces == MAXF) return -1;
  oforce* f = &s->forces[s->nforces];
  f->type = 1, f->mode = mode;
  f->a = dup(strengths, (size_t)s->n, -30);
  f->p[0] = dmin2, f->p[1] = dmax2, f->p[2] = theta2;
  return s->nforces++;
}

int32_t ofl_add_link(osim* s, int32_t m, const int32_t* src, const int32_t* dst,
                     const double* dist, const double* str, int32_t iterations, int32_t mode) {
  if (s->nforces == MAXF) return -1;
  oforce* f = &s->forces[s->nforces];
  f->type = 2, f->mode = mode, f->m = m, f->iterations = iterations;
  f->src = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
  f->dst = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
  memcpy(f->src, src, sizeof(int32_t) * (size_t)m);
  memcpy(f->dst, dst, sizeof(int32_t) * (size_t)m);
  /* initialize(): count per node, bias = count[s] / (count[s] + count[t]) */
  double* count = (double*)calloc((size_t)(s->n ? s->n : 1), sizeof(double));
  for (int32_t i = 0; i < m; ++i) count[src[i]] += 1, count[dst[i]] += 1;
  f->c = (double*)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
  for (int32_t i = 0; i < m; ++i) f->c[i] = count[src[i]] / (count[src[i]] + count[dst[i]]);
  f->b = (double*)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
  for (int32_t i = 0; i < m; ++i) {
    double a = count[src[i]], b = count[dst[i]];
    f->b[i] = str ? str[i] : 1 / (a < b ? a : b);
  }
  f->a = dup(dist, (size_t)m, 30);
  free(count);
  return s->nforces++;
}

void ofl_link_params(const osim* s, int32_t k, double* bias, double* strength) {
  const oforce* f = &s->forces[k];
  if (bias) memcpy(bias, f->c, sizeof(double) * (size_t)f->m);
  if (strength) memcpy(strength, f->b, sizeof(double) * (size_t)f->m);
}

int32_t ofl_add_collide(osim* s, const double* radii, double strength, int32_t iterations,
                        int32_t mode) {
  if (s->nforces == MAXF) return -1;
  oforce* f = &s->forces[s->nforces];
  f->type = 3, f->mode = mode, f->iterations = iterations;
  f->a = dup(radii, (size_t)s->n, 1);
  f->p[0] = strength;
  return s->nforces++;
}

int32_t ofl_add_center(osim* s, double x, double y, double z, double strength) {
  if (s->nforces == MAXF) return -1;
  oforce* f = &s->forces[s->nforces];
  f->type = 4;
  f->p[0] = x, f->p[1] = y, f->p[2] = z, f->p[3] = strength;
  return s->nforces++;
}

int32_t ofl_add_radial(osim* s, const double* radiuses, const double* strengths, double x,
                       double y, double z) {
  if (s->nforces == MAXF) return -1;
  oforce* f = &s->forces[s->nforces];
  f->type = 5;
  f->a = dup(radiuses, (size_t)s->n, 0);
  f->b = dup(strengths, (size_t)s->n, 0.1);
  f->p[0] = x, f->p[1] = y, f->p[2] = z;
  return s->nforces++;
}

int32_t ofl_add_position(osim* s, int32_t axis, const double* targets, const double* strengths) {
  if (s->nforces == MAXF) return -1;
  oforce* f = &s->forces[s->nforces];
  f->type = 6, f->axis = axis;
  f->a = dup(targets, (size_t)s->n, 0);
  f->b = dup(strengths, (size_t)s->n, 0.1);
  return s->nforces++;
}

void ofl_clear_forces(osim* s) {
  for (int32_t i = 0; i < s->nforces; ++i) force_free(&s->forces[i]);
  s->nforces = 0;
}

void ofl_apply_force(osim* s, int32_t k, double alpha) {
  oforce* f = &s->forces[k];
  switch (f->type) {
    case 1:
      memset(s->stats, 0, sizeof(s->stats));
      if (f->mode == OFL_MODE_EXACT) manybody_exact(s, f, alpha);
      else manybody_tree(s, f, alpha);
      break;
    case 2: link_force(s, f, alpha); break;
    case 3:
      if (f->mode == OFL_MODE_JACOBI) collide_jacobi(s, f);
      else collide_tree(s, f);
      break;
    case 4: center_force(s, f); break;
    case 5: radial_force(s, f, alpha); break;
    case 6: position_force(s, f, alpha); break;
  }
}

void ofl_tick(osim* s, int32_t iterations) {
  int d = s->ndim;
  for (int32_t k = 0; k < iterations; ++k) {
    s->alpha += (s->alpha_target - s->alpha) * s->alpha_decay;
    for (int32_t j = 0; j < s->nforces; ++j) ofl_apply_force(s, j, s->alpha);
    for (int32_t i = 0; i < s->n; ++i) {
      double* p = &s->x[3 * (size_t)i];
      double* v = &s->v[3 * (size_t)i];
      const double* fx = &s->f[3 * (size_t)i];
      uint8_t m = s->fmask[i];
      for (int a = 0; a < d; ++a) {
        if (!(m & (1 << a))) v[a] *= s->vmul, p[a] += v[a];
        else p[a] = fx[a], v[a] = 0;
      }
    }
  }
}

void ofl_walk_stats(const osim* s, int64_t* out3) {
  out3[0] = s->stats[0], out3[1] = s->stats[1], out3[2] = s->stats[2];
}

/* ------------------------------------------------------------------ integer rebuilds */

static const int32_t kLevels[4] = {0, 24, 24, 21};

int32_t ofl_levels(int32_t ndim) { return kLevels[ndim < 1 ? 1 : ndim > 3 ? 3 : ndim]; }

int32_t ofl_cube(int32_t n, int32_t ndim, const float* pos4, double* out4) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int32_t i = 0; i < n; ++i)
    for (int k = 0; k < ndim; ++k) {
      double v = pos4[4 * (size_t)i + k];
      if (v < lo[k]) lo[k] = v;
      if (v > hi[k]) hi[k] = v;
    }
  double origin[3] = {0, 0, 0};
  for (int k = 0; k < ndim; ++k) origin[k] = floor(lo[k]);
  double size = 1;
  int32_t lg = 0;
  for (;;) {
    int inside = 1;
    for (int k = 0; k < ndim; ++k)
      if (!(hi[k] < origin[k] + size)) inside = 0;
    if (inside || lg >= 1100) break;
    size *= 2, ++lg;
  }
  out4[0] = origin[0], out4[1] = origin[1], out4[2] = origin[2], out4[3] = size;
  return lg;
}

void ofl_morton(int32_t n, int32_t ndim, const float* pos4, uint64_t* codes) {
  double cube[4];
  int32_t lg = ofl_cube(n, ndim, pos4, cube);
  int32_t L = ofl_levels(ndim);
  double top = (double)((1u << L) - 1);
  for (int32_t i = 0; i < n; ++i) {
    uint64_t q[3] = {0, 0, 0};
    for (int k = 0; k < ndim; ++k) {
      /* cell index at the finest level, floor((x - origin) * 2^e) with e = L - log2(size),
       * in exact arithmetic: for e >= 0 as floor(x * 2^e) - origin * 2^e (origin is an
       * integer), for e < 0 as floor((floor(x) - origin) * 2^e). Every step is exact in FP64. */
      double x = (double)pos4[4 * (size_t)i + k], c;
      int32_t e = L - lg;
      if (e >= 0) c = floor(ldexp(x, e)) - ldexp(cube[k], e);
      else c = floor(ldexp(floor(x) - cube[k], e));
      if (c < 0) c = 0;
      if (c > top) c = top;
      q[k] = (uint64_t)c;
    }
    uint64_t code = 0;
    for (int32_t lv = L - 1; lv >= 0; --lv)
      for (int k = ndim - 1; k >= 0; --k) code = (code << 1) | ((q[k] >> lv) & 1);
    codes[i] = code;
  }
}

static const uint64_t* g_codes;
static int cmp_perm(const void* a, const void* b) {
  uint32_t i = *(const uint32_t*)a, j = *(const uint32_t*)b;
  if (g_codes[i] != g_codes[j]) return g_codes[i] < g_codes[j] ? -1 : 1;
  return i < j ? -1 : (i > j ? 1 : 0);
}

void ofl_sort_perm(int32_t n, const uint64_t* codes, uint32_t* perm) {
  for (int32_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
  g_codes = codes;
  qsort(perm, (size_t)n, sizeof(uint32_t), cmp_perm); /* ties by index: a stable order */
}

static int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }

/* common prefix of sorted codes a, b (shifted so the code's top bit is bit 63), -1 if out of
 * range, 64 + clz(a ^ b) for equal codes */
static int kdelta(int32_t n, const uint64_t* k, int32_t a, int32_t b) {
  if (b < 0 || b >= n) return -1;
  if (k[a] != k[b]) return clz64(k[a] ^ k[b]);
  return 64 + __builtin_clz((uint32_t)a ^ (uint32_t)b);
}

void ofl_karras(int32_t n, int32_t ndim, const uint64_t* sorted_codes, uint32_t* left,
                uint32_t* right, int32_t* depth) {
  int32_t L = ofl_levels(ndim), bits = L * ndim;
  uint64_t* k = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(n > 0 ? n : 1));
  for (int32_t i = 0; i < n; ++i) k[i] = sorted_codes[i] << (64 - bits);
  for (int32_t i = 0; i + 1 < n; ++i) {
    int dn = kdelta(n, k, i, i - 1), up = kdelta(n, k, i, i + 1);
    int dir = up > dn ? 1 : -1;
    int dmin = dn < up ? dn : up;
    int64_t lmax = 2;
    while (kdelta(n, k, i, (int32_t)(i + lmax * dir)) > dmin) lmax *= 2;
    int64_t len = 0;
    for (int64_t t = lmax / 2; t >= 1; t /= 2)
      if (kdelta(n, k, i, (int32_t)(i + (len + t) * dir)) > dmin) len += t;
    int32_t j = (int32_t)(i + len * dir);
    int dnode = kdelta(n, k, i, j);
    int64_t s = 0, t = len;
    do {
      t = (t + 1) / 2;
      if (kdelta(n, k, i, (int32_t)(i + (s + t) * dir)) > dnode) s += t;
    } while (t > 1);
    int32_t split = (int32_t)(i + s * dir + (dir < 0 ? -1 : 0));
    int32_t first = i < j ? i : j, last = i < j ? j : i;
    left[i] = first == split ? (0x80000000u | (uint32_t)split) : (uint32_t)split;
    right[i] = last == split + 1 ? (0x80000000u | (uint32_t)(split + 1)) : (uint32_t)(split + 1);
    int dep = dnode >= bits ? L : dnode / ndim;
    depth[i] = dep > L ? L : dep;
  }
  free(k);
}

void ofl_csr(int32_t n, int32_t m, const int32_t* src, const int32_t* dst, int32_t* row_start,
             int32_t* other, int32_t* code) {
  for (int32_t i = 0; i <= n; ++i) row_start[i] = 0;
  for (int32_t k = 0; k < m; ++k) row_start[src[k] + 1]++, row_start[dst[k] + 1]++;
  for (int32_t i = 0; i < n; ++i) row_start[i + 1] += row_start[i];
  int32_t* cur = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  for (int32_t i = 0; i < n; ++i) cur[i] = row_start[i];
  for (int32_t k = 0; k < m; ++k) {
    int32_t a = cur[src[k]]++;
    other[a] = dst[k], code[a] = 2 * k;
    int32_t b = cur[dst[k]]++;
    other[b] = src[k], code[b] = 2 * k + 1;
  }
  free(cur);
}
