/*
 * vo_oracle.c -- CPU oracle for the Voroffset 3D dexel morphology path.
 *
 * TEST INFRASTRUCTURE ONLY (see vo_oracle.h). A plain-C restatement of the
 * reference (geometryprocessing/voroffset, src/vor3d); each function cites the
 * reference lines it follows. Parity of this restatement is pinned against the
 * reference compiled unmodified (oracle/_ref, ref_bridge.cpp) and against the
 * committed golden fixtures in tests/golden/.
 *
 * Separable dilation ("ours", VoronoiVorPower.cpp:24-96) is restated as the
 * exact set it computes:
 *   pass 1 (y sweep, Voronoi2D.cpp + radius-aware appendSegment,
 *           MorphologyOperators.cpp:37-95): every column gets pieces [a,b]
 *           labelled with d = min |dy| of a column (x, y+dy) covering them,
 *           carrying radius r(d) = d==0 ? R : sqrt(R*R - d*d)
 *           (Voronoi2D.cpp:699-723);
 *   pass 2 (x sweep, SeparatePower2D.cpp:295-341): the output column is the
 *           union of [a - h, b + h], h = sqrt(r*r - dx*dx), over pieces of
 *           columns (x+dx, y) still alive (floor(x_s + r) + 1 > i,
 *           SeparatePower2D.cpp:258-273), merged as closed intervals
 *           (appendSegment, MorphologyOperators.cpp:15-34: touching merges).
 * The Voronoi / power-diagram bookkeeping of the reference only discards
 * seeds whose contribution is covered by others, so the union is the same.
 */
#define _GNU_SOURCE
#include "vo_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------ util */

static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

typedef struct {
  double *v; /* pairs */
  int n;     /* number of pairs */
  int cap;   /* capacity in pairs */
} ivec;

static int ivec_reserve(ivec *a, int n) {
  if (n <= a->cap) return 0;
  int c = a->cap ? a->cap : 16;
  while (c < n) c *= 2;
  double *p = (double *)realloc(a->v, sizeof(double) * 2 * (size_t)c);
  if (!p) return -1;
  a->v = p;
  a->cap = c;
  return 0;
}

static int ivec_push(ivec *a, double lo, double hi) {
  if (ivec_reserve(a, a->n + 1)) return -1;
  a->v[2 * a->n] = lo;
  a->v[2 * a->n + 1] = hi;
  a->n++;
  return 0;
}

typedef struct {
  double *v; /* pairs */
  unsigned char *d;
  int n, cap;
} pvec; /* labelled pieces */

static int pvec_push(pvec *a, double lo, double hi, int d) {
  if (a->n + 1 > a->cap) {
    int c = a->cap ? a->cap * 2 : 32;
    double *p = (double *)realloc(a->v, sizeof(double) * 2 * (size_t)c);
    if (!p) return -1;
    a->v = p;
    unsigned char *q = (unsigned char *)realloc(a->d, (size_t)c);
    if (!q) return -1;
    a->d = q;
    a->cap = c;
  }
  a->v[2 * a->n] = lo;
  a->v[2 * a->n + 1] = hi;
  a->d[a->n] = (unsigned char)d;
  a->n++;
  return 0;
}

void vo_or_free(void *p) { free(p); }

/* ---------------------------------------------------------- radius tables */

typedef struct {
  double R;
  int Dy;       /* max pass-1 lattice distance */
  double *r1;   /* [Dy+1] pass-1 radius per label (Voronoi2D.cpp:704-712) */
  int *Dx;      /* [Dy+1] max pass-2 lattice distance per label */
  int W;        /* row stride of H: Dx[0] + 1 */
  double *H;    /* [(Dy+1)*W]: sqrt(r1*r1 - dx*dx) (SeparatePower2D.cpp:314) */
  double *HB;   /* [(Dy+1)*(Dy+1)] brute force sqrt(R*R - dx^2 - dy^2), NAN outside */
} tables;

static void tables_free(tables *t) {
  free(t->r1);
  free(t->Dx);
  free(t->H);
  free(t->HB);
  memset(t, 0, sizeof(*t));
}

/* kmax: the largest sweep index + 1 the tables must serve. Expiry in the
 * reference is floor(x_s + r) + 1 > i (Voronoi2D.cpp:619, SeparatePower2D.cpp:266)
 * evaluated at x_s = 0..kmax-1; a radius whose floor(x_s + r) is not
 * x_s + floor(r) for some x_s (r a hair below an integer) is rejected. */
static int tables_build(double R, int kmax, tables *t) {
  memset(t, 0, sizeof(*t));
  if (!(R >= 0.0) || R > 255.0) return VO_OR_EINVAL;
  t->R = R;
  t->Dy = (int)floor(R);
  for (int k = 0; k < kmax; ++k)
    if ((int)floor((double)k + R) != k + t->Dy) return VO_OR_ERADIUS;
  const int Dy = t->Dy;
  t->r1 = (double *)malloc(sizeof(double) * (Dy + 1));
  t->Dx = (int *)malloc(sizeof(int) * (Dy + 1));
  if (!t->r1 || !t->Dx) return VO_OR_ENOMEM;
  for (int d = 0; d <= Dy; ++d) {
    if (d == 0) {
      t->r1[d] = R;
    } else {
      double dd = (double)d < R ? (double)d : R;
      t->r1[d] = sqrt(R * R - dd * dd);
    }
    t->Dx[d] = (int)floor(t->r1[d]);
    for (int k = 0; k < kmax; ++k)
      if ((int)floor((double)k + t->r1[d]) != k + t->Dx[d]) {
        tables_free(t);
        return VO_OR_ERADIUS;
      }
  }
  t->W = t->Dx[0] + 1;
  t->H = (double *)malloc(sizeof(double) * (size_t)(Dy + 1) * t->W);
  t->HB = (double *)malloc(sizeof(double) * (size_t)(Dy + 1) * (Dy + 1));
  if (!t->H || !t->HB) return VO_OR_ENOMEM;
  for (int d = 0; d <= Dy; ++d)
    for (int dx = 0; dx < t->W; ++dx) {
      double r = t->r1[d];
      double x = (double)dx;
      t->H[d * t->W + dx] = dx <= t->Dx[d] ? sqrt(r * r - x * x) : NAN;
    }
  /* VoronoiBruteForce.cpp:41-52: pow(dx,2)+pow(dy,2) <= R*R, dz = sqrt(R*R - dx^2 - dy^2). */
  for (int dy = 0; dy <= Dy; ++dy)
    for (int dx = 0; dx <= Dy; ++dx) {
      double fx = (double)dx * dx, fy = (double)dy * dy;
      t->HB[dy * (Dy + 1) + dx] = (fx + fy <= R * R) ? sqrt(R * R - fx - fy) : NAN;
    }
  return VO_OR_OK;
}

/* --------------------------------------------------- closed-interval union */

/* Insert [lo,hi] into a sorted list of disjoint closed intervals, merging
 * overlapping or touching ones (same rule as appendSegment /
 * addSegmentAtTheEnd, MorphologyOperators.cpp:15-34, .hpp:7-20). */
static int union_insert(ivec *A, double lo, double hi) {
  int n = A->n;
  double *v = A->v;
  /* first i with A[i].hi >= lo */
  int l = 0, r = n;
  while (l < r) {
    int m = (l + r) >> 1;
    if (v[2 * m + 1] >= lo)
      r = m;
    else
      l = m + 1;
  }
  int i = l;
  if (i == n || v[2 * i] > hi) {
    if (ivec_reserve(A, n + 1)) return -1;
    v = A->v;
    memmove(v + 2 * (i + 1), v + 2 * i, sizeof(double) * 2 * (size_t)(n - i));
    v[2 * i] = lo;
    v[2 * i + 1] = hi;
    A->n = n + 1;
    return 0;
  }
  int j = i;
  while (j + 1 < n && v[2 * (j + 1)] <= hi) ++j;
  double nlo = v[2 * i] < lo ? v[2 * i] : lo;
  double nhi = v[2 * j + 1] > hi ? v[2 * j + 1] : hi;
  v[2 * i] = nlo;
  v[2 * i + 1] = nhi;
  if (j > i) {
    memmove(v + 2 * (i + 1), v + 2 * (j + 1), sizeof(double) * 2 * (size_t)(n - j - 1));
    A->n = n - (j - i);
  }
  return 0;
}

/* Union of two sorted disjoint lists (unionSegs, MorphologyOperators.cpp:117-158). */
static int union_two(const double *a, int na, const double *b, int nb, ivec *out) {
  out->n = 0;
  int i = 0, j = 0;
  while (i < na || j < nb) {
    double lo, hi;
    if (j < nb && (i >= na || b[2 * j] <= a[2 * i])) {
      lo = b[2 * j];
      hi = b[2 * j + 1];
      ++j;
    } else {
      lo = a[2 * i];
      hi = a[2 * i + 1];
      ++i;
    }
    if (out->n == 0 || out->v[2 * out->n - 1] < lo) {
      if (ivec_push(out, lo, hi)) return -1;
    } else if (hi > out->v[2 * out->n - 1]) {
      out->v[2 * out->n - 1] = hi;
    }
  }
  return 0;
}

/* ------------------------------------------------------------- pass 1 */

typedef struct {
  ivec M;
  pvec P, Q;
  ivec A;
} scratch;

static void scratch_free(scratch *s) {
  free(s->M.v);
  free(s->P.v);
  free(s->P.d);
  free(s->Q.v);
  free(s->Q.d);
  free(s->A.v);
  memset(s, 0, sizeof(*s));
}

/* Pieces of column (x,y): pass-1 output restated as the painter over lattice
 * distance d = 0..Dy. The level-d sources are columns (x, y-d) and (x, y+d);
 * the part of their union not yet covered gets label d. Result sorted by z. */
static int pass1_column(int nx, int ny, const vo_or_csr *in, const tables *t, int x, int y,
                        scratch *s) {
  pvec *P = &s->P, *Q = &s->Q;
  P->n = 0;
  for (int d = 0; d <= t->Dy; ++d) {
    const double *la = NULL, *lb = NULL;
    int na = 0, nb = 0;
    int ya = y - d, yb = y + d;
    if (ya >= 0) {
      int c = x + nx * ya;
      la = in->z + 2 * (size_t)in->offs[c];
      na = in->offs[c + 1] - in->offs[c];
    }
    if (d > 0 && yb < ny) {
      int c = x + nx * yb;
      lb = in->z + 2 * (size_t)in->offs[c];
      nb = in->offs[c + 1] - in->offs[c];
    }
    if (na + nb == 0) continue;
    if (union_two(la, na, lb, nb, &s->M)) return -1;
    const double *M = s->M.v;
    const int nm = s->M.n;
    Q->n = 0;
    int j = 0;
    const int np = P->n;
    for (int k = 0; k <= np; ++k) {
      if (k > 0 && pvec_push(Q, P->v[2 * (k - 1)], P->v[2 * (k - 1) + 1], P->d[k - 1])) return -1;
      const double g1 = k == 0 ? -INFINITY : P->v[2 * (k - 1) + 1];
      const double g2 = k == np ? INFINITY : P->v[2 * k];
      if (!(g1 < g2)) continue;
      while (j < nm && M[2 * j + 1] <= g1) ++j;
      int jj = j;
      while (jj < nm && M[2 * jj] < g2) {
        double lo = M[2 * jj] > g1 ? M[2 * jj] : g1;
        double hi = M[2 * jj + 1] < g2 ? M[2 * jj + 1] : g2;
        if (pvec_push(Q, lo, hi, d)) return -1;
        if (M[2 * jj + 1] >= g2) break;
        ++jj;
      }
      j = jj;
    }
    pvec tmp = *P;
    *P = *Q;
    *Q = tmp;
  }
  return 0;
}

/* ------------------------------------------------------------- pass 2 */

typedef struct {
  const int32_t *offs; /* per column, in pieces */
  const double *v;
  const unsigned char *d;
} pieces_csr;

/* Output column (x,y): union over dx of the dilated pieces of column (x+dx, y). */
static int pass2_column(int nx, const pieces_csr *pc, const tables *t, int x, int y, ivec *A) {
  A->n = 0;
  const int W = t->W;
  for (int adx = 0; adx < W; ++adx) {
    for (int sgn = -1; sgn <= 1; sgn += 2) {
      if (adx == 0 && sgn > 0) continue;
      int xs = x + sgn * adx;
      if (xs < 0 || xs >= nx) continue;
      int c = xs + nx * y;
      int b = pc->offs[c], e = pc->offs[c + 1];
      int open = 0;
      double glo = 0, ghi = 0;
      for (int k = b; k < e; ++k) {
        int d = pc->d[k];
        if (adx > t->Dx[d]) continue;
        double h = t->H[d * W + adx];
        double p1 = pc->v[2 * k], p2 = pc->v[2 * k + 1];
        if (p1 > p2) {
          /* An inverted pair (a complemented column whose values left
           * [zmin, zmax]) contributes its two endpoint circles
           * (SeparatePower2D.cpp:215-226, 321-335); the stadium between them is
           * empty or inside their union. */
          if (union_insert(A, p1 - h, p1 + h) || union_insert(A, p2 - h, p2 + h)) return -1;
          continue;
        }
        double lo = p1 - h, hi = p2 + h;
        if (open && lo <= ghi && hi >= glo) {
          if (lo < glo) glo = lo;
          if (hi > ghi) ghi = hi;
        } else {
          if (open && union_insert(A, glo, ghi)) return -1;
          open = 1;
          glo = lo;
          ghi = hi;
        }
      }
      if (open && union_insert(A, glo, ghi)) return -1;
    }
  }
  return 0;
}

/* --------------------------------------------------------- thread driver */

typedef struct {
  int ncols;
  int nthreads;
  int (*fn)(void *ctx, int c, scratch *s, pvec *outp, ivec *outi);
  void *ctx;
  int labelled; /* output carries labels (pvec) */
  /* per-thread results */
  pvec *tp;
  ivec *ti;
  int32_t *counts; /* per column */
  int err;
} pdriver;

typedef struct {
  pdriver *D;
  int tid;
} pworker;

static void *pworker_main(void *arg) {
  pworker *w = (pworker *)arg;
  pdriver *D = w->D;
  const int per = (D->ncols + D->nthreads - 1) / D->nthreads;
  const int c0 = w->tid * per;
  const int c1 = c0 + per < D->ncols ? c0 + per : D->ncols;
  scratch s;
  memset(&s, 0, sizeof(s));
  for (int c = c0; c < c1; ++c) {
    int before = D->labelled ? D->tp[w->tid].n : D->ti[w->tid].n;
    if (D->fn(D->ctx, c, &s, &D->tp[w->tid], &D->ti[w->tid])) {
      D->err = VO_OR_ENOMEM;
      break;
    }
    int after = D->labelled ? D->tp[w->tid].n : D->ti[w->tid].n;
    D->counts[c] = after - before;
  }
  scratch_free(&s);
  return NULL;
}

/* Runs fn over all columns on nthreads threads (contiguous column ranges) and
 * gathers the per-thread outputs into one CSR. */
static int pdrive(pdriver *D, int32_t **offs_out, double **v_out, unsigned char **d_out) {
  if (D->nthreads < 1) D->nthreads = 1;
  if (D->nthreads > D->ncols && D->ncols > 0) D->nthreads = D->ncols;
  if (D->ncols == 0) D->nthreads = 1;
  D->err = 0;
  D->tp = (pvec *)calloc(D->nthreads, sizeof(pvec));
  D->ti = (ivec *)calloc(D->nthreads, sizeof(ivec));
  D->counts = (int32_t *)calloc((size_t)D->ncols + 1, sizeof(int32_t));
  pworker *ws = (pworker *)calloc(D->nthreads, sizeof(pworker));
  pthread_t *th = (pthread_t *)calloc(D->nthreads, sizeof(pthread_t));
  int rc = VO_OR_OK;
  if (!D->tp || !D->ti || !D->counts || !ws || !th) {
    rc = VO_OR_ENOMEM;
    goto done;
  }
  for (int i = 0; i < D->nthreads; ++i) {
    ws[i].D = D;
    ws[i].tid = i;
  }
  if (D->nthreads == 1) {
    pworker_main(&ws[0]);
  } else {
    for (int i = 0; i < D->nthreads; ++i) pthread_create(&th[i], NULL, pworker_main, &ws[i]);
    for (int i = 0; i < D->nthreads; ++i) pthread_join(th[i], NULL);
  }
  if (D->err) {
    rc = D->err;
    goto done;
  }
  {
    int64_t total = 0;
    int32_t *offs = (int32_t *)malloc(sizeof(int32_t) * ((size_t)D->ncols + 1));
    if (!offs) {
      rc = VO_OR_ENOMEM;
      goto done;
    }
    offs[0] = 0;
    for (int c = 0; c < D->ncols; ++c) {
      total += D->counts[c];
      if (total > 2147483647LL) {
        free(offs);
        rc = VO_OR_ENOMEM;
        goto done;
      }
      offs[c + 1] = (int32_t)total;
    }
    double *v = (double *)malloc(sizeof(double) * 2 * (size_t)(total > 0 ? total : 1));
    unsigned char *dl = D->labelled ? (unsigned char *)malloc((size_t)(total > 0 ? total : 1)) : NULL;
    if (!v || (D->labelled && !dl)) {
      free(offs);
      free(v);
      free(dl);
      rc = VO_OR_ENOMEM;
      goto done;
    }
    int64_t k = 0;
    for (int i = 0; i < D->nthreads; ++i) {
      int n = D->labelled ? D->tp[i].n : D->ti[i].n;
      const double *src = D->labelled ? D->tp[i].v : D->ti[i].v;
      if (n) memcpy(v + 2 * k, src, sizeof(double) * 2 * (size_t)n);
      if (D->labelled && n) memcpy(dl + k, D->tp[i].d, (size_t)n);
      k += n;
    }
    *offs_out = offs;
    *v_out = v;
    if (d_out) *d_out = dl;
  }
done:
  if (D->tp)
    for (int i = 0; i < D->nthreads; ++i) {
      free(D->tp[i].v);
      free(D->tp[i].d);
    }
  if (D->ti)
    for (int i = 0; i < D->nthreads; ++i) free(D->ti[i].v);
  free(D->tp);
  free(D->ti);
  free(D->counts);
  free(ws);
  free(th);
  return rc;
}

typedef struct {
  int nx, ny;
  const vo_or_csr *in;
  const tables *t;
  const pieces_csr *pc;
} sep_ctx;

static int pass1_fn(void *vctx, int c, scratch *s, pvec *outp, ivec *outi) {
  (void)outi;
  sep_ctx *x = (sep_ctx *)vctx;
  if (pass1_column(x->nx, x->ny, x->in, x->t, c % x->nx, c / x->nx, s)) return -1;
  for (int k = 0; k < s->P.n; ++k)
    if (pvec_push(outp, s->P.v[2 * k], s->P.v[2 * k + 1], s->P.d[k])) return -1;
  return 0;
}

static int pass2_fn(void *vctx, int c, scratch *s, pvec *outp, ivec *outi) {
  (void)outp;
  sep_ctx *x = (sep_ctx *)vctx;
  if (pass2_column(x->nx, x->pc, x->t, c % x->nx, c / x->nx, &s->A)) return -1;
  for (int k = 0; k < s->A.n; ++k)
    if (ivec_push(outi, s->A.v[2 * k], s->A.v[2 * k + 1])) return -1;
  return 0;
}

static int kmax_of(const vo_or_grid *g) { return (g->nx > g->ny ? g->nx : g->ny) + 2; }

static int cmp_pair(const void *a, const void *b) {
  const double *x = (const double *)a, *y = (const double *)b;
  if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
  return x[1] < y[1] ? -1 : (x[1] > y[1] ? 1 : 0);
}

/* Inverted pairs [a, b], a > b, appear when erosion complements a column whose
 * values left [zmin, zmax] (negate_ray, MorphologyOperators.cpp:230-259). The
 * reference's pass 2 then only sees their two endpoint circles
 * (SeparatePower2D.cpp:215-226 inserts both endpoints as points), so they are
 * rewritten as the points [b, b] and [a, a]; columns that contain one are
 * re-sorted and merged as closed intervals. Columns without inverted pairs
 * are copied unchanged. Returns 1 if anything was rewritten (and fills out). */
static int normalize_inverted(int ncols, const vo_or_csr *in, vo_or_csr *out) {
  int64_t nseg = in->offs[ncols], ninv = 0;
  for (int64_t k = 0; k < nseg; ++k)
    if (in->z[2 * k] > in->z[2 * k + 1]) ++ninv;
  if (!ninv) return 0;
  out->offs = (int32_t *)malloc(sizeof(int32_t) * ((size_t)ncols + 1));
  out->z = (double *)malloc(sizeof(double) * 2 * (size_t)(nseg + ninv + 1));
  double *tmp = (double *)malloc(sizeof(double) * 2 * (size_t)(nseg + ninv + 1));
  if (!out->offs || !out->z || !tmp) {
    free(out->offs);
    free(out->z);
    free(tmp);
    return -1;
  }
  int64_t w = 0;
  out->offs[0] = 0;
  for (int c = 0; c < ncols; ++c) {
    int n = 0;
    for (int k = in->offs[c]; k < in->offs[c + 1]; ++k) {
      double a = in->z[2 * k], b = in->z[2 * k + 1];
      if (a > b) {
        tmp[2 * n] = b, tmp[2 * n + 1] = b, ++n;
        tmp[2 * n] = a, tmp[2 * n + 1] = a, ++n;
      } else {
        tmp[2 * n] = a, tmp[2 * n + 1] = b, ++n;
      }
    }
    qsort(tmp, n, 2 * sizeof(double), cmp_pair);
    int64_t c0 = w;
    for (int k = 0; k < n; ++k) {
      if (w > c0 && !(out->z[2 * w - 1] < tmp[2 * k])) {
        if (tmp[2 * k + 1] > out->z[2 * w - 1]) out->z[2 * w - 1] = tmp[2 * k + 1];
      } else {
        out->z[2 * w] = tmp[2 * k];
        out->z[2 * w + 1] = tmp[2 * k + 1];
        ++w;
      }
    }
    out->offs[c + 1] = (int32_t)w;
  }
  free(tmp);
  return 1;
}

/* VoronoiMorphoVorPower::dilation (VoronoiVorPower.cpp:24-96). */
int vo_or_dilate(const vo_or_grid *g, const vo_or_csr *in, double radius, int nthreads,
                 vo_or_csr *out, double *t1_ms, double *t2_ms) {
  if (!g || !in || !out || g->nx < 0 || g->ny < 0) return VO_OR_EINVAL;
  tables t;
  int rc = tables_build(radius, kmax_of(g), &t);
  if (rc) return rc;
  const int ncols = g->nx * g->ny;
  vo_or_csr norm = {0};
  int nrc = normalize_inverted(ncols, in, &norm);
  if (nrc < 0) {
    tables_free(&t);
    return VO_OR_ENOMEM;
  }
  if (nrc > 0) in = &norm;
  double t0 = now_ms();
  sep_ctx ctx = {g->nx, g->ny, in, &t, NULL};
  pdriver D1 = {ncols, nthreads, pass1_fn, &ctx, 1, NULL, NULL, NULL, 0};
  int32_t *poffs = NULL;
  double *pv = NULL;
  unsigned char *pd = NULL;
  rc = pdrive(&D1, &poffs, &pv, &pd);
  if (rc) {
    free(norm.offs);
    free(norm.z);
    tables_free(&t);
    return rc;
  }
  double t1 = now_ms();
  pieces_csr pc = {poffs, pv, pd};
  ctx.pc = &pc;
  pdriver D2 = {ncols, nthreads, pass2_fn, &ctx, 0, NULL, NULL, NULL, 0};
  rc = pdrive(&D2, &out->offs, &out->z, NULL);
  double t2 = now_ms();
  if (t1_ms) *t1_ms = t1 - t0;
  if (t2_ms) *t2_ms = t2 - t1;
  free(poffs);
  free(pv);
  free(pd);
  free(norm.offs);
  free(norm.z);
  tables_free(&t);
  return rc;
}

/* Separable dilation restricted to selected output columns: for each one, the
 * pass-1 pieces of the 2*Dx[0]+1 source columns of its row are built on the
 * fly, then pass 2 runs on that one-row window. Same arithmetic as
 * vo_or_dilate; used for exact checks of full-size GPU results on a sample. */
typedef struct {
  int nx, ny;
  const vo_or_csr *in;
  const tables *t;
  const int32_t *cols;
} sel_ctx;

static int sel_fn(void *vctx, int i, scratch *s, pvec *outp, ivec *outi) {
  (void)outp;
  sel_ctx *x = (sel_ctx *)vctx;
  const int c = x->cols[i];
  const int cx = c % x->nx, cy = c / x->nx, W = x->t->W;
  const int x0 = cx - (W - 1) < 0 ? 0 : cx - (W - 1);
  const int x1 = cx + (W - 1) > x->nx - 1 ? x->nx - 1 : cx + (W - 1);
  const int nw = x1 - x0 + 1;
  int32_t *woffs = (int32_t *)malloc(sizeof(int32_t) * (nw + 1));
  pvec all = {0};
  if (!woffs) return -1;
  woffs[0] = 0;
  for (int k = 0; k < nw; ++k) {
    if (pass1_column(x->nx, x->ny, x->in, x->t, x0 + k, cy, s)) {
      free(woffs);
      return -1;
    }
    for (int j = 0; j < s->P.n; ++j)
      if (pvec_push(&all, s->P.v[2 * j], s->P.v[2 * j + 1], s->P.d[j])) {
        free(woffs);
        return -1;
      }
    woffs[k + 1] = all.n;
  }
  pieces_csr pc = {woffs, all.v, all.d};
  int rc = pass2_column(nw, &pc, x->t, cx - x0, 0, &s->A);
  free(woffs);
  free(all.v);
  free(all.d);
  if (rc) return -1;
  for (int k = 0; k < s->A.n; ++k)
    if (ivec_push(outi, s->A.v[2 * k], s->A.v[2 * k + 1])) return -1;
  return 0;
}

int vo_or_dilate_columns(const vo_or_grid *g, const vo_or_csr *in, double radius, const int32_t *cols,
                         int ncols_sel, int nthreads, vo_or_csr *out) {
  if (!g || !in || !cols || !out || ncols_sel < 0) return VO_OR_EINVAL;
  for (int i = 0; i < ncols_sel; ++i)
    if (cols[i] < 0 || cols[i] >= g->nx * g->ny) return VO_OR_EINVAL;
  tables t;
  int rc = tables_build(radius, kmax_of(g), &t);
  if (rc) return rc;
  sel_ctx ctx = {g->nx, g->ny, in, &t, cols};
  pdriver D = {ncols_sel, nthreads, sel_fn, &ctx, 0, NULL, NULL, NULL, 0};
  rc = pdrive(&D, &out->offs, &out->z, NULL);
  tables_free(&t);
  return rc;
}

int64_t vo_or_pass1_pieces(const vo_or_grid *g, const vo_or_csr *in, double radius, int nthreads) {
  tables t;
  if (tables_build(radius, kmax_of(g), &t)) return -1;
  sep_ctx ctx = {g->nx, g->ny, in, &t, NULL};
  pdriver D1 = {g->nx * g->ny, nthreads, pass1_fn, &ctx, 1, NULL, NULL, NULL, 0};
  int32_t *poffs = NULL;
  double *pv = NULL;
  unsigned char *pd = NULL;
  int64_t total = -1;
  if (pdrive(&D1, &poffs, &pv, &pd) == 0) total = poffs[g->nx * g->ny];
  free(poffs);
  free(pv);
  free(pd);
  tables_free(&t);
  return total;
}

/* ---------------------------------------------------------- brute force */

typedef struct {
  int nx, ny;
  const vo_or_csr *in;
  const tables *t;
} brute_ctx;

/* VoronoiBruteForce.cpp:16-68 for one column: every lattice neighbour within
 * the disc contributes [z1 - dz, z2 + dz]; the union merges touching intervals. */
static int brute_fn(void *vctx, int c, scratch *s, pvec *outp, ivec *outi) {
  (void)outp;
  brute_ctx *b = (brute_ctx *)vctx;
  const tables *t = b->t;
  const int x = c % b->nx, y = c / b->nx, D = t->Dy;
  ivec *A = &s->A;
  A->n = 0;
  for (int dy = -D; dy <= D; ++dy) {
    int ys = y + dy;
    if (ys < 0 || ys >= b->ny) continue;
    for (int dx = -D; dx <= D; ++dx) {
      int xs = x + dx;
      if (xs < 0 || xs >= b->nx) continue;
      double dz = t->HB[(dy < 0 ? -dy : dy) * (D + 1) + (dx < 0 ? -dx : dx)];
      if (isnan(dz)) continue;
      int cs = xs + b->nx * ys;
      for (int k = b->in->offs[cs]; k < b->in->offs[cs + 1]; ++k)
        if (union_insert(A, b->in->z[2 * k] - dz, b->in->z[2 * k + 1] + dz)) return -1;
    }
  }
  for (int k = 0; k < A->n; ++k)
    if (ivec_push(outi, A->v[2 * k], A->v[2 * k + 1])) return -1;
  return 0;
}

int vo_or_dilate_brute(const vo_or_grid *g, const vo_or_csr *in, double radius, int nthreads,
                       vo_or_csr *out) {
  tables t;
  int rc = tables_build(radius, kmax_of(g), &t);
  if (rc) return rc;
  vo_or_csr norm = {0};
  int nrc = normalize_inverted(g->nx * g->ny, in, &norm);
  if (nrc < 0) {
    tables_free(&t);
    return VO_OR_ENOMEM;
  }
  brute_ctx ctx = {g->nx, g->ny, nrc > 0 ? &norm : in, &t};
  pdriver D = {g->nx * g->ny, nthreads, brute_fn, &ctx, 0, NULL, NULL, NULL, 0};
  rc = pdrive(&D, &out->offs, &out->z, NULL);
  free(norm.offs);
  free(norm.z);
  tables_free(&t);
  return rc;
}

/* ------------------------------------------------- erosion / complement */

/* negate_ray (MorphologyOperators.cpp:230-259) on one column; appends to out. */
static int negate_ray(const double *v, int n2, double ymin, double ymax, double *out) {
  /* n2: number of values (even). Returns number of values written. */
  if (n2 == 0) {
    out[0] = ymin;
    out[1] = ymax;
    return 2;
  }
  int w = 0, i = 0;
  if (v[0] == ymin)
    i = 1;
  else
    out[w++] = ymin;
  for (; i < n2; ++i) out[w++] = v[i];
  if (w > 0 && out[w - 1] == ymax)
    --w;
  else
    out[w++] = ymax;
  return w;
}

/* negate_ray_range (MorphologyOperators.cpp:282-315). */
static int negate_ray_range(const double *v, int n2, double ymin, double ymax, double *out) {
  if (n2 == 0) {
    out[0] = ymin;
    out[1] = ymax;
    return 2;
  }
  int b = 0, e = n2; /* working view v[b..e) */
  int count_first = 0, count_last = 0, w = 0;
  int front_ymin = 0;
  while (v[b] <= ymin) {
    ++b;
    ++count_first;
    if (b == e) break;
  }
  if (count_first % 2 == 0) front_ymin = 1;
  /* The view is now [ymin?] + v[b..e). Pop from the back while >= ymax. */
  int has_front = front_ymin;
  for (;;) {
    double back;
    if (e > b)
      back = v[e - 1];
    else if (has_front)
      back = ymin;
    else
      break;
    if (!(back >= ymax)) break;
    if (e > b)
      --e;
    else
      has_front = 0;
    ++count_last;
    if (e == b && !has_front) break;
  }
  if (has_front) out[w++] = ymin;
  for (int i = b; i < e; ++i) out[w++] = v[i];
  if (count_last % 2 == 0) out[w++] = ymax;
  return w;
}

static int csr_alloc(int ncols, int64_t nvals, vo_or_csr *o) {
  o->offs = (int32_t *)malloc(sizeof(int32_t) * ((size_t)ncols + 1));
  o->z = (double *)malloc(sizeof(double) * (size_t)(nvals > 0 ? nvals : 1));
  return (o->offs && o->z) ? 0 : -1;
}

/* VoronoiMorpho::negate (Voronoi.cpp:18-55): grid grows by one empty column on
 * every side, then every column is complemented within [zmin, zmax]. */
static int negate_grid(int nx, int ny, const vo_or_csr *in, double zmin, double zmax,
                       vo_or_csr *out) {
  const int NX = nx + 2, NY = ny + 2;
  const int64_t nin = 2 * (int64_t)in->offs[nx * ny];
  if (csr_alloc(NX * NY, nin + 4 * (int64_t)NX * NY, out)) return VO_OR_ENOMEM;
  int64_t w = 0;
  out->offs[0] = 0;
  for (int Y = 0; Y < NY; ++Y)
    for (int X = 0; X < NX; ++X) {
      const double *v = NULL;
      int n2 = 0;
      if (X >= 1 && X <= nx && Y >= 1 && Y <= ny) {
        int c = (X - 1) + nx * (Y - 1);
        v = in->z + 2 * (size_t)in->offs[c];
        n2 = 2 * (in->offs[c + 1] - in->offs[c]);
      }
      int k = negate_ray(v, n2, zmin, zmax, out->z + w);
      if (k % 2) return VO_OR_EINVAL;
      w += k;
      out->offs[X + NX * Y + 1] = (int32_t)(w / 2);
    }
  return VO_OR_OK;
}

/* VoronoiMorpho::negateInv (Voronoi.cpp:57-89): crop the border, then
 * negate_ray_range within [zmin, zmax]. */
static int negate_inv_grid(int nx, int ny, const vo_or_csr *in, double zmin, double zmax,
                           vo_or_csr *out) {
  const int NX = nx + 2;
  int64_t nin = 2 * (int64_t)in->offs[NX * (ny + 2)];
  if (csr_alloc(nx * ny, nin + 4 * (int64_t)nx * ny, out)) return VO_OR_ENOMEM;
  int64_t w = 0;
  out->offs[0] = 0;
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      int c = (x + 1) + NX * (y + 1);
      const double *v = in->z + 2 * (size_t)in->offs[c];
      int n2 = 2 * (in->offs[c + 1] - in->offs[c]);
      int k = negate_ray_range(v, n2, zmin, zmax, out->z + w);
      if (k % 2) return VO_OR_EINVAL;
      w += k;
      out->offs[x + nx * y + 1] = (int32_t)(w / 2);
    }
  return VO_OR_OK;
}

static int dilate_any(int method, const vo_or_grid *g, const vo_or_csr *in, double radius,
                      int nthreads, vo_or_csr *out) {
  if (method == 0) return vo_or_dilate(g, in, radius, nthreads, out, NULL, NULL);
  return vo_or_dilate_brute(g, in, radius, nthreads, out);
}

/* VoronoiMorpho::erosion (Voronoi.cpp:8-17). */
static int erode_any(int method, const vo_or_grid *g, const vo_or_csr *in, double radius,
                     int nthreads, vo_or_csr *out) {
  const double zmin = g->origin[2] / g->spacing - 1;
  const double zmax =
      g->origin[2] / g->spacing + 2 * g->padding + g->extent[2] / g->spacing + 1;
  vo_or_csr neg = {0}, dil = {0};
  int rc = negate_grid(g->nx, g->ny, in, zmin, zmax, &neg);
  if (rc) goto done;
  vo_or_grid g2 = *g;
  g2.nx += 2;
  g2.ny += 2;
  rc = dilate_any(method, &g2, &neg, radius, nthreads, &dil);
  if (rc) goto done;
  rc = negate_inv_grid(g->nx, g->ny, &dil, zmin + 1, zmax - 1, out);
done:
  free(neg.offs);
  free(neg.z);
  free(dil.offs);
  free(dil.z);
  return rc;
}

/* Operation chaining of app/cli3d/offset3d.cpp:116-136. */
int vo_or_morph(int method, int op, const vo_or_grid *g, const vo_or_csr *in, double radius,
                int nthreads, vo_or_csr *out) {
  if (!g || !in || !out || (method != 0 && method != 1)) return VO_OR_EINVAL;
  vo_or_csr tmp = {0};
  int rc;
  switch (op) {
    case 0:
      return dilate_any(method, g, in, radius, nthreads, out);
    case 1:
      return erode_any(method, g, in, radius, nthreads, out);
    case 2:
      rc = erode_any(method, g, in, radius, nthreads, &tmp);
      if (!rc) rc = dilate_any(method, g, &tmp, radius, nthreads, out);
      break;
    case 3:
      rc = dilate_any(method, g, in, radius, nthreads, &tmp);
      if (!rc) rc = erode_any(method, g, &tmp, radius, nthreads, out);
      break;
    default:
      return VO_OR_EINVAL;
  }
  free(tmp.offs);
  free(tmp.z);
  return rc;
}

/* --------------------------------------------------------------- selected columns of any op
 *
 * vo_or_morph_columns: the result of vo_or_morph (separable method) at selected
 * columns only, with the same arithmetic, so that full-size GPU results can be
 * checked exactly on a sample. Erosion complements the whole input (linear
 * work, Voronoi.cpp:18-55), dilates the complement at the selected columns only
 * and complements them back (Voronoi.cpp:57-89). Opening and closing evaluate
 * their first op on the selected columns' lattice neighbourhoods (the only
 * columns the second op reads) and their second op on the selected columns. */

static int dilate_cols_norm(const vo_or_grid *g, const vo_or_csr *in, double radius, const int32_t *cols,
                            int n, int nthreads, vo_or_csr *out) {
  vo_or_csr norm = {0};
  int nrc = normalize_inverted(g->nx * g->ny, in, &norm);
  if (nrc < 0) return VO_OR_ENOMEM;
  int rc = vo_or_dilate_columns(g, nrc > 0 ? &norm : in, radius, cols, n, nthreads, out);
  free(norm.offs);
  free(norm.z);
  return rc;
}

static int erode_cols(const vo_or_grid *g, const vo_or_csr *in, double radius, const int32_t *cols, int n,
                      int nthreads, vo_or_csr *out) {
  const double zmin = g->origin[2] / g->spacing - 1;
  const double zmax = g->origin[2] / g->spacing + 2 * g->padding + g->extent[2] / g->spacing + 1;
  vo_or_csr neg = {0}, dil = {0};
  int32_t *mcols = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  int rc = mcols ? negate_grid(g->nx, g->ny, in, zmin, zmax, &neg) : VO_OR_ENOMEM;
  if (rc) goto done;
  for (int i = 0; i < n; ++i) mcols[i] = (cols[i] % g->nx + 1) + (g->nx + 2) * (cols[i] / g->nx + 1);
  vo_or_grid g2 = *g;
  g2.nx += 2;
  g2.ny += 2;
  rc = dilate_cols_norm(&g2, &neg, radius, mcols, n, nthreads, &dil);
  if (rc) goto done;
  if (csr_alloc(n, 2 * (int64_t)dil.offs[n] + 4 * (int64_t)n, out)) {
    rc = VO_OR_ENOMEM;
    goto done;
  }
  {
    int64_t w = 0;
    out->offs[0] = 0;
    for (int i = 0; i < n; ++i) {
      int k = negate_ray_range(dil.z + 2 * (size_t)dil.offs[i], 2 * (dil.offs[i + 1] - dil.offs[i]), zmin + 1,
                               zmax - 1, out->z + w);
      if (k % 2) {
        rc = VO_OR_EINVAL;
        goto done;
      }
      w += k;
      out->offs[i + 1] = (int32_t)(w / 2);
    }
  }
done:
  free(mcols);
  free(neg.offs);
  free(neg.z);
  free(dil.offs);
  free(dil.z);
  return rc;
}

/* Columns within the lattice reach (|dy| <= floor(R), |dx| <= floor(R)) of the
 * selected ones, sorted and unique; *nb receives the count. */
static int32_t *neighbourhood(const vo_or_grid *g, double radius, const int32_t *cols, int n, int *nb) {
  const int D = (int)floor(radius), N = g->nx * g->ny;
  unsigned char *mark = (unsigned char *)calloc((size_t)N, 1);
  if (!mark) return NULL;
  int cnt = 0;
  for (int i = 0; i < n; ++i) {
    const int cx = cols[i] % g->nx, cy = cols[i] / g->nx;
    for (int y = cy - D; y <= cy + D; ++y)
      for (int x = cx - D; x <= cx + D; ++x)
        if (x >= 0 && x < g->nx && y >= 0 && y < g->ny && !mark[x + g->nx * y]) {
          mark[x + g->nx * y] = 1;
          ++cnt;
        }
  }
  int32_t *out = (int32_t *)malloc(sizeof(int32_t) * (size_t)(cnt > 0 ? cnt : 1));
  if (out) {
    int k = 0;
    for (int c = 0; c < N; ++c)
      if (mark[c]) out[k++] = c;
  }
  free(mark);
  *nb = cnt;
  return out;
}

/* A full-grid CSR holding `part` (results at the sorted columns `sel`) and empty
 * columns elsewhere. */
static int scatter_cols(const vo_or_grid *g, const int32_t *sel, int n, const vo_or_csr *part, vo_or_csr *out) {
  const int N = g->nx * g->ny;
  if (csr_alloc(N, 2 * (int64_t)part->offs[n], out)) return VO_OR_ENOMEM;
  memcpy(out->z, part->z, sizeof(double) * 2 * (size_t)part->offs[n]);
  out->offs[0] = 0;
  int k = 0;
  for (int c = 0; c < N; ++c) {
    if (k < n && sel[k] == c) ++k;
    out->offs[c + 1] = part->offs[k];
  }
  return VO_OR_OK;
}

int vo_or_morph_columns(int op, const vo_or_grid *g, const vo_or_csr *in, double radius, const int32_t *cols,
                        int ncols_sel, int nthreads, vo_or_csr *out) {
  if (!g || !in || !cols || !out || ncols_sel < 0) return VO_OR_EINVAL;
  for (int i = 0; i < ncols_sel; ++i)
    if (cols[i] < 0 || cols[i] >= g->nx * g->ny) return VO_OR_EINVAL;
  if (op == 0) return dilate_cols_norm(g, in, radius, cols, ncols_sel, nthreads, out);
  if (op == 1) return erode_cols(g, in, radius, cols, ncols_sel, nthreads, out);
  if (op != 2 && op != 3) return VO_OR_EINVAL;
  int nb = 0;
  int32_t *sel = neighbourhood(g, radius, cols, ncols_sel, &nb);
  if (!sel) return VO_OR_ENOMEM;
  vo_or_csr part = {0}, full = {0};
  int rc = op == 2 ? erode_cols(g, in, radius, sel, nb, nthreads, &part)
                   : dilate_cols_norm(g, in, radius, sel, nb, nthreads, &part);
  if (!rc) rc = scatter_cols(g, sel, nb, &part, &full);
  if (!rc)
    rc = op == 2 ? dilate_cols_norm(g, &full, radius, cols, ncols_sel, nthreads, out)
                 : erode_cols(g, &full, radius, cols, ncols_sel, nthreads, out);
  free(sel);
  free(part.offs);
  free(part.z);
  free(full.offs);
  free(full.z);
  return rc;
}

/* --------------------------------------------------------------- 2D images
 *
 * The reference's 2D library (src/vor2d): an image of `height` rows, each a
 * sorted list of half-open pixel spans as events [a0, b0, a1, b1, ...]
 * (CompressedImage.h:32-41). Restated as lattice unions:
 *
 * dilate (CompressedImage.cpp:608-616, Voronoi.cpp:749-759): row i is the union
 *   over rows i0 with t = |i - i0| <= floor(r) of the spans [a, b) of row i0
 *   widened to [max(a - dy, 0), min(b + dy, width)), dy = floor(sqrt(r*r - t*t));
 *   touching spans merge (appendSegment, MorphologyOperators.cpp:10-29).
 * erode (CompressedImage.cpp:620-630, Voronoi.h:126-150): the complement of the
 *   same dilation applied to the complement spans of every row with one
 *   border pixel on each side ([-1, a0 - 1], [b0, a1 - 1], ..., [b_last, width],
 *   inclusive) and a full extra row before the first and after the last row.
 * open / close: erode then dilate / dilate then erode (CompressedImage.cpp:634-647). */

static int32_t img_dy(double r, int t) { return (int32_t)floor(sqrt(r * r - (double)((long long)t * t))); }

/* Marks the union of [lo, hi) ranges in a difference array over [0, w]. */
static void img_add(int32_t *diff, int w, int64_t lo, int64_t hi) {
  if (lo < 0) lo = 0;
  if (hi > w) hi = w;
  if (lo >= hi) return;
  diff[lo] += 1;
  diff[hi] -= 1;
}

/* Covered pixels of row i under the dilation (erode = 0) or the dilation of the
 * bordered complement (erode = 1); returns their spans as events. */
static int img_row(int w, int h, const int32_t *offs, const int32_t *ev, double r, int erode, int i,
                   int32_t *diff, int32_t *out) {
  const int D = (int)floor(r);
  memset(diff, 0, sizeof(int32_t) * ((size_t)w + 1));
  for (int i0 = (i - D > -1 ? i - D : -1); i0 <= (i + D < h ? i + D : h); ++i0) {
    const int t = i0 < i ? i - i0 : i0 - i;
    if (erode && (i0 == -1 || i0 == h)) {
      img_add(diff, w, 0, w);  /* the extra full row */
      continue;
    }
    if (i0 < 0 || i0 >= h) continue;
    const int32_t dy = img_dy(r, t);
    const int32_t *e = ev + offs[i0];
    const int n = offs[i0 + 1] - offs[i0];
    if (!erode) {
      for (int k = 0; k + 1 < n; k += 2) img_add(diff, w, (int64_t)e[k] - dy, (int64_t)e[k + 1] + dy);
    } else {
      int64_t y1 = -1;
      for (int k = 0; k + 1 < n; k += 2) {
        img_add(diff, w, y1 - dy, (int64_t)e[k] - 1 + dy + 1);
        y1 = e[k + 1];
      }
      img_add(diff, w, y1 - dy, (int64_t)w + dy + 1);
    }
  }
  int k = 0, c = 0, prev = 0;
  for (int p = 0; p <= w; ++p) {
    c += diff[p];
    const int cov = p < w && c > 0;
    if (cov != prev) out[k++] = p;
    prev = cov;
  }
  return k;
}

static int img_apply(int op1, int w, int h, const int32_t *offs, const int32_t *ev, double r, int32_t **oo,
                     int32_t **oe) {
  int32_t *diff = (int32_t *)malloc(sizeof(int32_t) * ((size_t)w + 2));
  int32_t *row = (int32_t *)malloc(sizeof(int32_t) * ((size_t)w + 2));
  int32_t *ro = (int32_t *)malloc(sizeof(int32_t) * ((size_t)h + 1));
  int64_t cap = 16, used = 0;
  int32_t *re = (int32_t *)malloc(sizeof(int32_t) * cap);
  if (!diff || !row || !ro || !re) {
    free(diff); free(row); free(ro); free(re);
    return VO_OR_ENOMEM;
  }
  ro[0] = 0;
  for (int i = 0; i < h; ++i) {
    int n = img_row(w, h, offs, ev, r, op1, i, diff, row);
    if (op1) {  /* erosion: complement of the covered spans within [0, w) (negate, CompressedImage.cpp:366-397) */
      int m = 0;
      int32_t *neg = diff; /* reuse as scratch */
      if (n == 0) {
        neg[m++] = 0;
        neg[m++] = w;
      } else {
        if (row[0] != 0) neg[m++] = 0;
        for (int k = (row[0] == 0 ? 1 : 0); k < n; ++k) neg[m++] = row[k];
        if (row[n - 1] == w) --m;
        else neg[m++] = w;
      }
      memcpy(row, neg, sizeof(int32_t) * m);
      n = m;
    }
    if (used + n > cap) {
      while (used + n > cap) cap *= 2;
      int32_t *t = (int32_t *)realloc(re, sizeof(int32_t) * cap);
      if (!t) {
        free(diff); free(row); free(ro); free(re);
        return VO_OR_ENOMEM;
      }
      re = t;
    }
    memcpy(re + used, row, sizeof(int32_t) * n);
    used += n;
    ro[i + 1] = (int32_t)used;
  }
  free(diff);
  free(row);
  *oo = ro;
  *oe = re;
  return VO_OR_OK;
}

int vo_or_image_morph(int op, int width, int height, const int32_t *offs, const int32_t *events, double radius,
                      int32_t **out_offs, int32_t **out_events) {
  if (width < 0 || height < 0 || !offs || !out_offs || !out_events || !(radius >= 0) || op < 0 || op > 3)
    return VO_OR_EINVAL;
  int32_t *o1 = NULL, *e1 = NULL;
  int rc;
  switch (op) {
    case 0:
    case 1:
      return img_apply(op, width, height, offs, events, radius, out_offs, out_events);
    case 2:
      rc = img_apply(1, width, height, offs, events, radius, &o1, &e1);
      if (!rc) rc = img_apply(0, width, height, o1, e1, radius, out_offs, out_events);
      break;
    default:
      rc = img_apply(0, width, height, offs, events, radius, &o1, &e1);
      if (!rc) rc = img_apply(1, width, height, o1, e1, radius, out_offs, out_events);
      break;
  }
  free(o1);
  free(e1);
  return rc;
}

/* The FP64 twin (DoubleCompressedImage.cpp:680-720): rows of closed spans with
 * FP64 events in [0, width].
 * dilate: radius scaled by the row count, R = r * height; row i is the union
 *   over rows i0 with |i - i0| <= floor(R) of [y1 - dy, y2 + dy], dy =
 *   sqrt(R*R - t*t) (VoronoiMorphoF::getLine, DoubleVoronoi.cpp:713-726) — the
 *   3D dilation of a one-row grid — clamped to [0, width], intervals wholly
 *   outside dropped.
 * erode: radius as given; the complement spans [-1, a0], [b0, a1], ...,
 *   [b_last, width] of every row plus a full row [-1, width] before the first
 *   and after the last (voronoiF_half_erode, DoubleVoronoi.h:124-148), dilated,
 *   clamped the same way, then negate (DoubleCompressedImage.cpp:438-470). */

static int img64_dilate_rows(int nrows, const int32_t *soffs, const double *z, double R, vo_or_csr *out) {
  vo_or_grid g;
  memset(&g, 0, sizeof g);
  g.nx = nrows;
  g.ny = 1;
  g.spacing = 1.0;
  vo_or_csr in = {(int32_t *)soffs, (double *)z};
  return vo_or_dilate(&g, &in, R, 1, out, NULL, NULL);
}

/* Clamps row i (segments of rows[row0 + i]) to [0, w], optionally negates it, appends events. */
static int64_t img64_clip_row(const vo_or_csr *v, int row, double w, int negate, double *dst) {
  double tmp_lo, tmp_hi;
  int64_t k = 0;
  for (int s = v->offs[row]; s < v->offs[row + 1]; ++s) {
    tmp_lo = v->z[2 * s];
    tmp_hi = v->z[2 * s + 1];
    if (tmp_hi < 0 || tmp_lo > w) continue;
    dst[k++] = tmp_lo > 0 ? tmp_lo : 0;
    dst[k++] = tmp_hi < w ? tmp_hi : w;
  }
  if (!negate) return k;
  if (k == 0) {
    dst[0] = 0;
    dst[1] = w;
    return 2;
  }
  /* first event: drop a leading 0, else prepend 0; last: drop a trailing w, else append w */
  int64_t m = 0;
  double *o = dst + k + 1;  /* scratch after the clipped events */
  if (dst[0] != 0) o[m++] = 0;
  for (int64_t q = (dst[0] == 0 ? 1 : 0); q < k; ++q) o[m++] = dst[q];
  if (dst[k - 1] == w) --m;
  else o[m++] = w;
  memmove(dst, o, sizeof(double) * m);
  return m;
}

static int img64_apply(int erode, int w, int h, const int32_t *offs, const double *ev, double r, int32_t **oo,
                       double **oe) {
  const int nr = erode ? h + 2 : h;
  int32_t *so = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nr + 1));
  int64_t nval = erode ? (int64_t)offs[h] + 2 * (int64_t)h + 4 : (int64_t)offs[h];
  double *sz = (double *)malloc(sizeof(double) * (size_t)(nval + 2));
  if (!so || !sz) {
    free(so); free(sz);
    return VO_OR_ENOMEM;
  }
  so[0] = 0;
  int64_t q = 0;
  if (!erode) {
    memcpy(sz, ev, sizeof(double) * (size_t)offs[h]);
    for (int i = 0; i < h; ++i) so[i + 1] = offs[i + 1] / 2;
  } else {
    for (int rr = 0; rr < nr; ++rr) {
      if (rr == 0 || rr == nr - 1) {
        sz[q++] = -1;
        sz[q++] = w;
      } else {
        const int i = rr - 1;
        double y1 = -1;
        for (int k = offs[i]; k + 1 < offs[i + 1]; k += 2) {
          sz[q++] = y1;
          sz[q++] = ev[k];
          y1 = ev[k + 1];
        }
        sz[q++] = y1;
        sz[q++] = w;
      }
      so[rr + 1] = (int32_t)(q / 2);
    }
  }
  vo_or_csr dil = {0};
  int rc = img64_dilate_rows(nr, so, sz, erode ? r : r * h, &dil);
  free(so);
  free(sz);
  if (rc) return rc;
  int32_t *ro = (int32_t *)malloc(sizeof(int32_t) * ((size_t)h + 1));
  double *re = (double *)malloc(sizeof(double) * (size_t)(2 * (int64_t)dil.offs[nr] * 2 + 4 * (int64_t)h + 8));
  if (!ro || !re) {
    free(ro); free(re); free(dil.offs); free(dil.z);
    return VO_OR_ENOMEM;
  }
  int64_t used = 0;
  ro[0] = 0;
  for (int i = 0; i < h; ++i) {
    used += img64_clip_row(&dil, erode ? i + 1 : i, (double)w, erode, re + used);
    ro[i + 1] = (int32_t)used;
  }
  free(dil.offs);
  free(dil.z);
  *oo = ro;
  *oe = re;
  return VO_OR_OK;
}

int vo_or_image_morph_f64(int op, int width, int height, const int32_t *offs, const double *events, double radius,
                          int32_t **out_offs, double **out_events) {
  if (width < 0 || height < 0 || !offs || !out_offs || !out_events || !(radius >= 0) || op < 0 || op > 3)
    return VO_OR_EINVAL;
  int32_t *o1 = NULL;
  double *e1 = NULL;
  int rc;
  if (op == 0 || op == 1) return img64_apply(op, width, height, offs, events, radius, out_offs, out_events);
  rc = img64_apply(op == 2 ? 1 : 0, width, height, offs, events, radius, &o1, &e1);
  if (!rc) rc = img64_apply(op == 2 ? 0 : 1, width, height, o1, e1, radius, out_offs, out_events);
  free(o1);
  free(e1);
  return rc;
}

/* --------------------------------------------------------------- xor */

static int union_segs(const double *a, int na2, const double *b, int nb2, double *out) {
  /* unionSegs on flat value lists (MorphologyOperators.cpp:117-158) */
  ivec o = {0};
  int rc = union_two(a, na2 / 2, b, nb2 / 2, &o);
  int w = 0;
  if (!rc) {
    memcpy(out, o.v, sizeof(double) * 2 * (size_t)o.n);
    w = 2 * o.n;
  }
  free(o.v);
  return rc ? -1 : w;
}

/* calculate_ray_xor (MorphologyOperators.cpp:334-352) + removepoint (:364-374). */
static double ray_xor_length(const double *r1, int n1, const double *r2, int n2, double ymin,
                             double ymax) {
  size_t cap = (size_t)(n1 + n2 + 8) * 2;
  double *rec1 = (double *)malloc(sizeof(double) * cap);
  double *rec2 = (double *)malloc(sizeof(double) * cap);
  double *u1 = (double *)malloc(sizeof(double) * cap);
  double *u2 = (double *)malloc(sizeof(double) * cap);
  double *t1 = (double *)malloc(sizeof(double) * cap);
  double *t2 = (double *)malloc(sizeof(double) * cap);
  double *bp = (double *)malloc(sizeof(double) * cap * 2);
  double len = 0;
  int k1 = negate_ray(r1, n1, ymin, ymax, rec1);
  int k2 = negate_ray(r2, n2, ymin, ymax, rec2);
  int ku1 = union_segs(rec1, k1, r2, n2, u1);
  int ku2 = union_segs(rec2, k2, r1, n1, u2);
  int kt1 = negate_ray(u1, ku1, ymin, ymax, t1);
  int kt2 = negate_ray(u2, ku2, ymin, ymax, t2);
  int kb = union_segs(t1, kt1, t2, kt2, bp);
  for (int i = 0; i + 1 < kb; i += 2)
    if (!(bp[i + 1] - bp[i] < 1e-10)) len += bp[i + 1] - bp[i];
  free(rec1);
  free(rec2);
  free(u1);
  free(u2);
  free(t1);
  free(t2);
  free(bp);
  return len;
}

/* VoronoiMorpho::calculateXor (Voronoi.cpp:91-111) returning the xor volume. */
double vo_or_xor_volume(const vo_or_grid *g, const vo_or_csr *a, const vo_or_csr *b) {
  const double zmin = g->origin[2] / g->spacing;
  const double zmax = g->origin[2] / g->spacing + 2 * g->padding + g->extent[2] / g->spacing;
  const double h3 = g->spacing * g->spacing * g->spacing;
  double vol = 0;
  for (int x = 0; x < g->nx; ++x)
    for (int y = 0; y < g->ny; ++y) {
      int c = x + g->nx * y;
      double l = ray_xor_length(a->z + 2 * (size_t)a->offs[c], 2 * (a->offs[c + 1] - a->offs[c]),
                                b->z + 2 * (size_t)b->offs[c], 2 * (b->offs[c + 1] - b->offs[c]),
                                zmin, zmax);
      vol += h3 * l;
    }
  return vol;
}

/* CompressedVolume::get_volume (CompressedVolume.cpp:61-74). */
double vo_or_get_volume(const vo_or_grid *g, const vo_or_csr *a) {
  const double h = g->spacing;
  double vol = 0;
  for (int x = 0; x < g->nx; ++x)
    for (int y = 0; y < g->ny; ++y) {
      int c = x + g->nx * y;
      for (int k = a->offs[c]; k < a->offs[c + 1]; ++k)
        vol = vol + h * h * h * (a->z[2 * k + 1] - a->z[2 * k]);
    }
  return vol;
}

/* ------------------------------------------------------------ dexelize */

/* orientation (Dexelize.cpp:56-67): SOS-determined sign of twice the signed
 * area of (0,0)-(x1,y1)-(x2,y2). */
static int orientation(double x1, double y1, double x2, double y2, double *tsa) {
  *tsa = y1 * x2 - x1 * y2;
  if (*tsa > 0) return 1;
  if (*tsa < 0) return -1;
  if (y2 > y1) return 1;
  if (y2 < y1) return -1;
  if (x1 > x2) return 1;
  if (x1 < x2) return -1;
  return 0;
}

/* point_in_triangle_2d (Dexelize.cpp:73-92). */
static int point_in_triangle_2d(double x0, double y0, double x1, double y1, double x2, double y2,
                                double x3, double y3, double *a, double *b, double *c) {
  x1 -= x0;
  x2 -= x0;
  x3 -= x0;
  y1 -= y0;
  y2 -= y0;
  y3 -= y0;
  int signa = orientation(x2, y2, x3, y3, a);
  if (signa == 0) return 0;
  int signb = orientation(x3, y3, x1, y1, b);
  if (signb != signa) return 0;
  int signc = orientation(x1, y1, x2, y2, c);
  if (signc != signa) return 0;
  double sum = *a + *b + *c;
  *a /= sum;
  *b /= sum;
  *c /= sum;
  return 1;
}

/* intersect_ray_z (Dexelize.cpp:137-162): hit iff the SOS inside test passes
 * and the projected triangle orientation (orient_2d_inexact, :107-121) is
 * nonzero. */
static int intersect_ray_z(const double *p1, const double *p2, const double *p3, double qx,
                           double qy, double *z) {
  double u, v, w;
  if (point_in_triangle_2d(qx, qy, p1[0], p1[1], p2[0], p2[1], p3[0], p3[1], &u, &v, &w)) {
    *z = u * p1[2] + v * p2[2] + w * p3[2];
    double a11 = p2[0] - p1[0], a12 = p2[1] - p1[1];
    double a21 = p3[0] - p1[0], a22 = p3[1] - p1[1];
    double delta = a11 * a22 - a12 * a21;
    return delta > 0 ? 1 : (delta < 0 ? -1 : 0);
  }
  return 0;
}

static int cmp_double(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* create_dexels + compute_sign (Dexelize.cpp:166-274). The geogram AABB query
 * only filters facets whose bounding box contains the dexel centre (inclusive),
 * so an inclusive per-column bin of facet boxes gives the same candidate set. */
int vo_or_dexelize(const double *verts, int nv, const int32_t *tris, int nt, double *spacing,
                   int padding, int num_dexels, vo_or_grid *g, vo_or_csr *out) {
  if (nv <= 0 || nt < 0 || !spacing || !g || !out) return VO_OR_EINVAL;
  double mn[3], mx[3];
  for (int k = 0; k < 3; ++k) mn[k] = mx[k] = verts[k];
  for (int i = 1; i < nv; ++i)
    for (int k = 0; k < 3; ++k) {
      double v = verts[3 * i + k];
      if (v < mn[k]) mn[k] = v;
      if (v > mx[k]) mx[k] = v;
    }
  double ext[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
  if (num_dexels > 0) {
    double me = ext[0] > ext[1] ? ext[0] : ext[1];
    me = me > ext[2] ? me : ext[2];
    *spacing = me / num_dexels;
  }
  const double h = *spacing;
  if (!(h > 0)) return VO_OR_EINVAL;
  /* CompressedVolume ctor (CompressedVolume.cpp:11-23). */
  g->spacing = h;
  g->padding = padding;
  for (int k = 0; k < 3; ++k) {
    g->origin[k] = mn[k] - padding * h;
    g->extent[k] = ext[k];
  }
  g->nx = (int)(ceil(ext[0] / h) + 2 * padding);
  g->ny = (int)(ceil(ext[1] / h) + 2 * padding);
  const int nx = g->nx, ny = g->ny, ncols = nx * ny;
  /* Bin facets by the columns whose centre lies in their xy box. */
  int32_t *cnt = (int32_t *)calloc((size_t)ncols + 1, sizeof(int32_t));
  if (!cnt) return VO_OR_ENOMEM;
  int *bx0 = (int *)malloc(sizeof(int) * 4 * (size_t)(nt > 0 ? nt : 1));
  if (!bx0) {
    free(cnt);
    return VO_OR_ENOMEM;
  }
  for (int f = 0; f < nt; ++f) {
    const double *p[3] = {verts + 3 * tris[3 * f], verts + 3 * tris[3 * f + 1],
                          verts + 3 * tris[3 * f + 2]};
    double lo[2], hi[2];
    for (int k = 0; k < 2; ++k) {
      lo[k] = hi[k] = p[0][k];
      for (int j = 1; j < 3; ++j) {
        if (p[j][k] < lo[k]) lo[k] = p[j][k];
        if (p[j][k] > hi[k]) hi[k] = p[j][k];
      }
    }
    /* conservative index range, refined by the exact inclusive test below */
    int x0 = (int)floor((lo[0] - g->origin[0]) / h - 0.5) - 1;
    int x1 = (int)ceil((hi[0] - g->origin[0]) / h - 0.5) + 1;
    int y0 = (int)floor((lo[1] - g->origin[1]) / h - 0.5) - 1;
    int y1 = (int)ceil((hi[1] - g->origin[1]) / h - 0.5) + 1;
    if (x0 < 0) x0 = 0;
    if (y0 < 0) y0 = 0;
    if (x1 > nx - 1) x1 = nx - 1;
    if (y1 > ny - 1) y1 = ny - 1;
    bx0[4 * f] = x0;
    bx0[4 * f + 1] = x1;
    bx0[4 * f + 2] = y0;
    bx0[4 * f + 3] = y1;
    for (int y = y0; y <= y1; ++y)
      for (int x = x0; x <= x1; ++x) cnt[x + nx * y + 1]++;
  }
  for (int c = 0; c < ncols; ++c) cnt[c + 1] += cnt[c];
  int32_t *bin = (int32_t *)malloc(sizeof(int32_t) * (size_t)(cnt[ncols] > 0 ? cnt[ncols] : 1));
  int32_t *fill = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ncols > 0 ? ncols : 1));
  if (!bin || !fill) {
    free(cnt);
    free(bx0);
    free(bin);
    free(fill);
    return VO_OR_ENOMEM;
  }
  memcpy(fill, cnt, sizeof(int32_t) * (size_t)ncols);
  for (int f = 0; f < nt; ++f)
    for (int y = bx0[4 * f + 2]; y <= bx0[4 * f + 3]; ++y)
      for (int x = bx0[4 * f]; x <= bx0[4 * f + 1]; ++x) bin[fill[x + nx * y]++] = f;
  /* Ray casting per column. */
  int64_t cap = 1024, used = 0;
  double *z = (double *)malloc(sizeof(double) * cap);
  int32_t *offs = (int32_t *)malloc(sizeof(int32_t) * ((size_t)ncols + 1));
  double *hits = (double *)malloc(sizeof(double) * 64);
  int hcap = 64;
  int rc = VO_OR_OK;
  if (!z || !offs || !hits) rc = VO_OR_ENOMEM;
  if (!rc) offs[0] = 0;
  for (int y = 0; y < ny && !rc; ++y)
    for (int x = 0; x < nx && !rc; ++x) {
      const int c = x + nx * y;
      const double cx = (x + 0.5) * h + g->origin[0];
      const double cy = (y + 0.5) * h + g->origin[1];
      int nh = 0;
      for (int k = cnt[c]; k < cnt[c + 1]; ++k) {
        int f = bin[k];
        const double *p1 = verts + 3 * tris[3 * f], *p2 = verts + 3 * tris[3 * f + 1],
                     *p3 = verts + 3 * tris[3 * f + 2];
        double bl0 = fmin(p1[0], fmin(p2[0], p3[0])), bh0 = fmax(p1[0], fmax(p2[0], p3[0]));
        double bl1 = fmin(p1[1], fmin(p2[1], p3[1])), bh1 = fmax(p1[1], fmax(p2[1], p3[1]));
        if (cx < bl0 || cx > bh0 || cy < bl1 || cy > bh1) continue;
        double zz;
        if (intersect_ray_z(p1, p2, p3, cx, cy, &zz)) {
          if (nh == hcap) {
            hcap *= 2;
            double *nhp = (double *)realloc(hits, sizeof(double) * hcap);
            if (!nhp) {
              rc = VO_OR_ENOMEM;
              break;
            }
            hits = nhp;
          }
          hits[nh++] = zz / h;
        }
      }
      qsort(hits, nh, sizeof(double), cmp_double);
      nh &= ~1; /* an unpaired trailing hit is ignored (CompressedVolume::iterate pairs values) */
      if (used + nh > cap) {
        while (used + nh > cap) cap *= 2;
        double *nz = (double *)realloc(z, sizeof(double) * cap);
        if (!nz) {
          rc = VO_OR_ENOMEM;
          break;
        }
        z = nz;
      }
      memcpy(z + used, hits, sizeof(double) * nh);
      used += nh;
      offs[c + 1] = (int32_t)(used / 2);
    }
  free(cnt);
  free(bx0);
  free(bin);
  free(fill);
  free(hits);
  if (rc) {
    free(z);
    free(offs);
    return rc;
  }
  out->offs = offs;
  out->z = z;
  return VO_OR_OK;
}
