/*
 * FP64 CPU oracle for the 2-D (curve) Galerkin matrix fill -- TEST INFRASTRUCTURE ONLY.
 * Conventions, classes and rules: bem2d_oracle.h.
 *
 * Compile with -ffp-contract=off: the classification predicate must round exactly like the
 * library's device predicate (no fused multiply-add) on x86_64 and aarch64 alike.
 */
#include "bem2d_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int orc_gauss_legendre01(int32_t n, double* x, double* w); /* bem_oracle.c */

typedef struct { double re, im; } cpx;

static inline cpx cmul(cpx a, cpx b) { cpx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline cpx cscale(cpx a, double s) { cpx r = {a.re * s, a.im * s}; return r; }

/* ------------------------------------------------------------------------------------ */
/* Kernel: the prototype's green! (doubleQuadRule_2d_gpu.jl:72-78) with libm Bessel        */
/* functions: G = -(i/4) (J0 - i Y0), grad_x G = (x - y) (i k / 4) (J1 - i Y1) / R.        */
/* ------------------------------------------------------------------------------------ */
static void green2d(double k, double R, cpx* G, cpx* g1) {
  if (k == 0.0) {
    G->re = -log(R) / (2.0 * M_PI);
    G->im = 0.0;
    g1->re = -1.0 / (2.0 * M_PI * R * R);
    g1->im = 0.0;
    return;
  }
  const double z = k * R;
  G->re = -y0(z) / 4.0;
  G->im = -j0(z) / 4.0;
  g1->re = k * y1(z) / (4.0 * R);
  g1->im = k * j1(z) / (4.0 * R);
}

int orc2_green(double k, double R, double* out) {
  if (!out || !(R > 0.0) || !(k >= 0.0)) return -1;
  cpx G, g1;
  green2d(k, R, &G, &g1);
  out[0] = G.re;
  out[1] = G.im;
  out[2] = g1.re;
  out[3] = g1.im;
  return 0;
}

/* Graded rule on [0, 1] towards 0 with `levels` geometric levels (ratio 0.35): the intervals
 * [0, q^levels], [q^levels, q^(levels-1)], ..., [q, 1], n Gauss-Legendre points each, ascending. */
static int graded_levels(int n, int levels, double* x, double* w) {
  const double q = 0.35;
  double gx[16], gw[16];
  if (n < 1 || n > 16 || orc_gauss_legendre01(n, gx, gw)) return -1;
  int k = 0;
  for (int lev = levels; lev >= 0; --lev) {
    const double a = (lev == levels) ? 0.0 : pow(q, lev + 1);
    const double b = pow(q, lev);
    for (int i = 0; i < n; ++i) {
      x[k] = a + (b - a) * gx[i];
      w[k] = (b - a) * gw[i];
      ++k;
    }
  }
  return 0;
}

int orc2_graded01(int32_t n, double* x, double* w) {
  if (n < 1 || n > 16 || !x || !w) return -1;
  return graded_levels(n, 3 * n, x, w);
}

/* ------------------------------------------------------------------------------------ */
/* Geometry                                                                              */
/* ------------------------------------------------------------------------------------ */
typedef struct {
  double v[2][2];  /* v0, v1 */
  double d[2];     /* v1 - v0 */
  double len, n[2];
} seg_t;

static void load_seg(const orc2_space* s, int32_t e, seg_t* S) {
  for (int a = 0; a < 2; ++a) {
    const double* p = s->vertices + 2 * (int64_t)s->segments[2 * (int64_t)e + a];
    S->v[a][0] = p[0];
    S->v[a][1] = p[1];
  }
  S->d[0] = S->v[1][0] - S->v[0][0];
  S->d[1] = S->v[1][1] - S->v[0][1];
  S->len = sqrt(S->d[0] * S->d[0] + S->d[1] * S->d[1]);
  S->n[0] = S->d[1] / S->len;
  S->n[1] = -S->d[0] / S->len;
}

/* Class of a segment pair; *ma / *mb receive the local vertex of the first matched pair. */
static int classify_seg(const seg_t* a, const seg_t* b, double k2, int* ma, int* mb) {
  const double dtol = 2.220446049250313e-16 * 1.0e3; /* quadrule_determine.jl:1 */
  const double xtol2 = 0.2 * 0.2;                     /* quadrule_determine.jl:3 */
  int hits = 0;
  double dmin2 = DBL_MAX;
  *ma = *mb = -1;
  for (int u1 = 0; u1 < 2; ++u1)
    for (int u2 = 0; u2 < 2; ++u2) {
      double dx = a->v[u1][0] - b->v[u2][0];
      double dy = a->v[u1][1] - b->v[u2][1];
      double d2 = dx * dx + dy * dy;
      double d = sqrt(d2);
      if (d < dtol) {
        if (hits == 0) { *ma = u1; *mb = u2; }
        ++hits;
      }
      dmin2 = fmin(dmin2, d2);
    }
  if (hits > 2) return -1;
  if (hits == 2) return ORC2_CLASS_CF;
  if (hits == 1) return ORC2_CLASS_CV;
  double m = fmax(dmin2 * k2, dmin2 / (16.0 * b->len));
  return (m >= xtol2) ? ORC2_CLASS_FAR : ORC2_CLASS_NEAR;
}

int orc2_classify_block(const orc2_space* test, const orc2_space* trial, double k2, int32_t t0,
                        int32_t t1, int32_t s0, int32_t s1, int8_t* out) {
  if (!test || !trial || !out || t0 < 0 || s0 < 0 || t1 > test->ns || s1 > trial->ns || t1 < t0 || s1 < s0)
    return -1;
  int err = 0;
  int64_t nsb = s1 - s0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : err)
  for (int32_t t = t0; t < t1; ++t) {
    seg_t A, B;
    load_seg(test, t, &A);
    for (int32_t s = s0; s < s1; ++s) {
      load_seg(trial, s, &B);
      int ma, mb;
      int c = classify_seg(&A, &B, k2, &ma, &mb);
      if (c < 0) err = 1;
      out[(int64_t)(t - t0) * nsb + (s - s0)] = (int8_t)c;
    }
  }
  return err ? -2 : 0;
}

/* ------------------------------------------------------------------------------------ */
/* Integrand accumulation                                                                 */
/* ------------------------------------------------------------------------------------ */
typedef struct {
  const orc2_operator* op;
  const seg_t *A, *B;
  int nsA, nsB;      /* local shapes: 2 (C0D1) or 1 (CXD0) */
  cpx P[2][2];       /* sum of kernel * weight * f_i g_j */
  cpx M0;            /* hypersingular: sum of G * weight */
} acc_t;

static void shapes(int ns, double s, double f[2]) {
  if (ns == 1) { f[0] = 1.0; f[1] = 0.0; }
  else { f[0] = 1.0 - s; f[1] = s; }
}

/* One point pair: chart parameters s (test), t (trial), separation r = x - y, weight w
 * (product of the chart rule weights and Jacobians; segment lengths are applied here). */
static void add_point(acc_t* c, double s, double t, double rx, double ry, double w) {
  const double R = sqrt(rx * rx + ry * ry);
  cpx G, g1;
  green2d(c->op->wavenumber, R, &G, &g1);
  const double ww = w * c->A->len * c->B->len;
  cpx K;
  switch (c->op->kind) {
    case ORC2_OP_DL: K = cscale(g1, -(rx * c->B->n[0] + ry * c->B->n[1])); break;
    case ORC2_OP_DLT: K = cscale(g1, rx * c->A->n[0] + ry * c->A->n[1]); break;
    default: K = G; break;
  }
  K = cscale(K, ww);
  double f[2], g[2];
  shapes(c->nsA, s, f);
  shapes(c->nsB, t, g);
  for (int i = 0; i < c->nsA; ++i)
    for (int j = 0; j < c->nsB; ++j) {
      c->P[i][j].re += K.re * (f[i] * g[j]);
      c->P[i][j].im += K.im * (f[i] * g[j]);
    }
  if (c->op->kind == ORC2_OP_HS) {
    c->M0.re += G.re * ww;
    c->M0.im += G.im * ww;
  }
}

static void finalize(const acc_t* c, cpx L[2][2]) {
  const cpx alpha = {c->op->alpha[0], c->op->alpha[1]};
  const cpx beta = {c->op->beta[0], c->op->beta[1]};
  memset(L, 0, sizeof(cpx) * 4);
  if (c->op->kind != ORC2_OP_HS) {
    for (int i = 0; i < c->nsA; ++i)
      for (int j = 0; j < c->nsB; ++j) L[i][j] = cmul(alpha, c->P[i][j]);
    return;
  }
  const double nn = c->A->n[0] * c->B->n[0] + c->A->n[1] * c->B->n[1];
  double dA[2], dB[2];
  if (c->nsA == 2) { dA[0] = -1.0 / c->A->len; dA[1] = 1.0 / c->A->len; } else { dA[0] = dA[1] = 0.0; }
  if (c->nsB == 2) { dB[0] = -1.0 / c->B->len; dB[1] = 1.0 / c->B->len; } else { dB[0] = dB[1] = 0.0; }
  const cpx bM0 = cmul(beta, c->M0);
  for (int i = 0; i < c->nsA; ++i)
    for (int j = 0; j < c->nsB; ++j) {
      cpx a = cscale(cmul(alpha, c->P[i][j]), nn);
      cpx b = cscale(bM0, dA[i] * dB[j]);
      L[i][j].re = a.re + b.re;
      L[i][j].im = a.im + b.im;
    }
}

static int nshapes(const orc2_space* s) { return s->refspace == ORC2_REFSPACE_LAGRANGE_CXD0 ? 1 : 2; }

/* Product Gauss-Legendre rule (doubleQuadRule_2d_gpu.jl:142-181: weights womps x wimps, r =
 * x_I - y_J). */
static int double_gauss(acc_t* c, int nt, int nb) {
  double xt[32], wt[32], xb[32], wb[32];
  if (orc_gauss_legendre01(nt, xt, wt) || orc_gauss_legendre01(nb, xb, wb)) return -1;
  const seg_t *A = c->A, *B = c->B;
  for (int p = 0; p < nt; ++p) {
    const double x0 = A->v[0][0] + xt[p] * A->d[0], x1 = A->v[0][1] + xt[p] * A->d[1];
    for (int q = 0; q < nb; ++q) {
      const double y0v = B->v[0][0] + xb[q] * B->d[0], y1v = B->v[0][1] + xb[q] * B->d[1];
      add_point(c, xt[p], xb[q], x0 - y0v, x1 - y1v, wt[p] * wb[q]);
    }
  }
  return 0;
}

/* Distance between the segments p0-p1 and q0-q1 (they do not cross in a valid mesh). */
static double point_seg_dist2(const double p[2], const double a[2], const double b[2]) {
  const double dx = b[0] - a[0], dy = b[1] - a[1];
  const double L2 = dx * dx + dy * dy;
  double t = L2 > 0.0 ? ((p[0] - a[0]) * dx + (p[1] - a[1]) * dy) / L2 : 0.0;
  t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
  const double ex = a[0] + t * dx - p[0], ey = a[1] + t * dy - p[1];
  return ex * ex + ey * ey;
}

static double seg_dist(const double p0[2], const double p1[2], const double q0[2], const double q1[2]) {
  double d2 = point_seg_dist2(p0, q0, q1);
  d2 = fmin(d2, point_seg_dist2(p1, q0, q1));
  d2 = fmin(d2, point_seg_dist2(q0, p0, p1));
  d2 = fmin(d2, point_seg_dist2(q1, p0, p1));
  return sqrt(d2);
}

/* Near pairs: the chart square is bisected (the longer piece first) until each piece pair is
 * at least as far apart as its longer piece is long, or 16 bisections deep; every leaf gets the
 * near x near Gauss-Legendre product rule.  Leaves are visited depth first, the first half
 * before the second. */
static int near_rule(acc_t* c, int n) {
  double gx[32], gw[32];
  if (orc_gauss_legendre01(n, gx, gw)) return -1;
  const seg_t *A = c->A, *B = c->B;
  typedef struct { double s0, s1, t0, t1; int depth; } box_t;
  box_t stack[40];
  int top = 0;
  stack[top++] = (box_t){0.0, 1.0, 0.0, 1.0, 0};
  while (top > 0) {
    const box_t b = stack[--top];
    const double p0[2] = {A->v[0][0] + b.s0 * A->d[0], A->v[0][1] + b.s0 * A->d[1]};
    const double p1[2] = {A->v[0][0] + b.s1 * A->d[0], A->v[0][1] + b.s1 * A->d[1]};
    const double q0[2] = {B->v[0][0] + b.t0 * B->d[0], B->v[0][1] + b.t0 * B->d[1]};
    const double q1[2] = {B->v[0][0] + b.t1 * B->d[0], B->v[0][1] + b.t1 * B->d[1]};
    const double la = (b.s1 - b.s0) * A->len, lb = (b.t1 - b.t0) * B->len;
    if (b.depth < 16 && seg_dist(p0, p1, q0, q1) < fmax(la, lb)) {
      /* push the second half first so that the first half is integrated first */
      if (la >= lb) {
        const double sm = 0.5 * (b.s0 + b.s1);
        stack[top++] = (box_t){sm, b.s1, b.t0, b.t1, b.depth + 1};
        stack[top++] = (box_t){b.s0, sm, b.t0, b.t1, b.depth + 1};
      } else {
        const double tm = 0.5 * (b.t0 + b.t1);
        stack[top++] = (box_t){b.s0, b.s1, tm, b.t1, b.depth + 1};
        stack[top++] = (box_t){b.s0, b.s1, b.t0, tm, b.depth + 1};
      }
      continue;
    }
    const double hs = b.s1 - b.s0, ht = b.t1 - b.t0;
    for (int p = 0; p < n; ++p) {
      const double s = b.s0 + hs * gx[p];
      const double x0 = A->v[0][0] + s * A->d[0], x1 = A->v[0][1] + s * A->d[1];
      for (int q = 0; q < n; ++q) {
        const double t = b.t0 + ht * gx[q];
        const double y0v = B->v[0][0] + t * B->d[0], y1v = B->v[0][1] + t * B->d[1];
        add_point(c, s, t, x0 - y0v, x1 - y1v, (hs * gw[p]) * (ht * gw[q]));
      }
    }
  }
  return 0;
}

static int singular_rule(acc_t* c, int cls, int ma, int mb, int n) {
  /* coincident pairs: ln z integrands, 3n levels; common-vertex pairs carry the Jacobian z
   * (z ln z), for which 3n/2 levels reach the same accuracy */
  const int levels = cls == ORC2_CLASS_CF ? 3 * n : (3 * n) / 2;
  double gz[49 * 16], gwz[49 * 16], gx[16], gw[16];
  if (graded_levels(n, levels, gz, gwz) || orc_gauss_legendre01(n, gx, gw)) return -1;
  const int nz = (levels + 1) * n;
  const seg_t *A = c->A, *B = c->B;
  if (cls == ORC2_CLASS_CF) {
    /* same straight segment: double layers vanish (r is along the segment) */
    if (c->op->kind == ORC2_OP_DL || c->op->kind == ORC2_OP_DLT) return 0;
    const int same = (ma == mb); /* first match (0, 0): same orientation; (0, 1): reversed */
    for (int half = 0; half < 2; ++half)
      for (int a = 0; a < nz; ++a) {
        const double z = gz[a];
        for (int b = 0; b < n; ++b) {
          const double w = gx[b];
          double u, v, uv; /* uv = u - v, exactly */
          if (half == 0) { u = z + (1.0 - z) * w; v = (1.0 - z) * w; uv = z; }
          else { u = (1.0 - z) * w; v = z + (1.0 - z) * w; uv = -z; }
          const double wt = gwz[a] * gw[b] * (1.0 - z);
          const double t = same ? v : 1.0 - v;
          add_point(c, u, t, uv * A->d[0], uv * A->d[1], wt);
        }
      }
    return 0;
  }
  /* common vertex: edge vectors from the shared vertex */
  const double ax = ma == 0 ? A->d[0] : -A->d[0], ay = ma == 0 ? A->d[1] : -A->d[1];
  const double bx = mb == 0 ? B->d[0] : -B->d[0], by = mb == 0 ? B->d[1] : -B->d[1];
  for (int half = 0; half < 2; ++half)
    for (int a = 0; a < nz; ++a) {
      const double z = gz[a];
      for (int b = 0; b < n; ++b) {
        const double w = gx[b];
        double xi, eta;
        if (half == 0) { xi = z; eta = z * w; }
        else { xi = z * w; eta = z; }
        const double wt = gwz[a] * gw[b] * z;
        const double s = ma == 0 ? xi : 1.0 - xi;
        const double t = mb == 0 ? eta : 1.0 - eta;
        add_point(c, s, t, xi * ax - eta * bx, xi * ay - eta * by, wt);
      }
    }
  return 0;
}

static int valid_rules(const orc2_quadstrat* qs) {
  return qs && qs->far_test >= 1 && qs->far_test <= 32 && qs->far_trial >= 1 && qs->far_trial <= 32 &&
         qs->near >= 1 && qs->near <= 32 && qs->singular >= 1 && qs->singular <= 16;
}

static int valid_op(const orc2_operator* op) {
  return op && op->kind >= ORC2_OP_SL && op->kind <= ORC2_OP_HS && op->wavenumber >= 0.0 &&
         isfinite(op->wavenumber);
}

static int local_matrix(const orc2_operator* op, const orc2_space* test, const orc2_space* trial,
                        const orc2_quadstrat* qs, const seg_t* A, const seg_t* B, int force, cpx L[2][2],
                        int8_t* cls_out) {
  int ma, mb;
  int cls = classify_seg(A, B, op->wavenumber * op->wavenumber, &ma, &mb);
  if (cls < 0) return -1;
  if (cls_out) *cls_out = (int8_t)cls;
  const int rule = force >= 0 ? force : cls;
  /* a singular rule needs the vertices it is built around; product rules apply to any pair */
  if ((rule == ORC2_CLASS_CF || rule == ORC2_CLASS_CV) && rule != cls) return -1;
  if (rule != ORC2_CLASS_FAR && rule != ORC2_CLASS_NEAR && rule != ORC2_CLASS_CF && rule != ORC2_CLASS_CV) return -1;
  acc_t c;
  memset(&c, 0, sizeof(c));
  c.op = op;
  c.A = A;
  c.B = B;
  c.nsA = nshapes(test);
  c.nsB = nshapes(trial);
  int rc;
  if (rule == ORC2_CLASS_FAR) rc = double_gauss(&c, qs->far_test, qs->far_trial);
  else if (rule == ORC2_CLASS_NEAR) rc = near_rule(&c, qs->near);
  else rc = singular_rule(&c, rule, ma, mb, qs->singular);
  if (rc) return rc;
  finalize(&c, L);
  return 0;
}

int orc2_local_matrices(const orc2_operator* op, const orc2_space* test, const orc2_space* trial,
                        const orc2_quadstrat* qs, int64_t npairs, const int32_t* tau,
                        const int32_t* sigma, int32_t force_class, double* out, int8_t* cls) {
  if (!valid_op(op) || !valid_rules(qs) || !test || !trial || npairs < 0 || (npairs && (!tau || !sigma || !out)))
    return -1;
  int err = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : err)
  for (int64_t p = 0; p < npairs; ++p) {
    if (tau[p] < 0 || tau[p] >= test->ns || sigma[p] < 0 || sigma[p] >= trial->ns) { err = 1; continue; }
    seg_t A, B;
    load_seg(test, tau[p], &A);
    load_seg(trial, sigma[p], &B);
    cpx L[2][2];
    int8_t c = 0;
    if (local_matrix(op, test, trial, qs, &A, &B, force_class, L, &c)) { err = 1; continue; }
    if (cls) cls[p] = c;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) {
        out[p * 8 + (i * 2 + j) * 2 + 0] = L[i][j].re;
        out[p * 8 + (i * 2 + j) * 2 + 1] = L[i][j].im;
      }
  }
  return err ? -2 : 0;
}

int orc2_assemble_rows(const orc2_operator* op, const orc2_space* test, const orc2_space* trial,
                       const orc2_quadstrat* qs, int64_t nrows, const int32_t* rows, double* out,
                       int32_t nthreads) {
  if (!valid_op(op) || !valid_rules(qs) || !test || !trial || nrows < 0 || (nrows && (!rows || !out))) return -1;
  const int nsA = nshapes(test), nsB = nshapes(trial);
  const int32_t nf = test->nfun;
  /* supports of every test function, ordered by segment */
  int64_t* off = (int64_t*)calloc((size_t)nf + 2, sizeof(int64_t));
  if (!off) return -3;
  for (int64_t e = 0; e < test->ns; ++e)
    for (int i = 0; i < nsA; ++i) {
      int32_t f = test->fn_index[2 * e + i];
      if (f >= nf) { free(off); return -1; }
      if (f >= 0) off[f + 1]++;
    }
  for (int32_t f = 0; f < nf; ++f) off[f + 1] += off[f];
  int64_t nsup = off[nf];
  int32_t* se = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nsup ? nsup : 1));
  int32_t* si = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nsup ? nsup : 1));
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nf ? nf : 1));
  if (!se || !si || !fill) { free(off); free(se); free(si); free(fill); return -3; }
  for (int32_t f = 0; f < nf; ++f) fill[f] = off[f];
  for (int64_t e = 0; e < test->ns; ++e)
    for (int i = 0; i < nsA; ++i) {
      int32_t f = test->fn_index[2 * e + i];
      if (f >= 0) { se[fill[f]] = (int32_t)e; si[fill[f]] = i; fill[f]++; }
    }
  int err = 0;
  const int64_t nb = trial->nfun;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(| : err)
  for (int64_t r = 0; r < nrows; ++r) {
    double* row = out + r * nb * 2;
    memset(row, 0, sizeof(double) * 2 * (size_t)nb);
    int32_t m = rows[r];
    if (m < 0 || m >= nf) { err = 1; continue; }
    for (int64_t a = off[m]; a < off[m + 1]; ++a) {
      const int32_t tau = se[a], i = si[a];
      const double ca = test->fn_coef[2 * (int64_t)tau + i];
      seg_t A, B;
      load_seg(test, tau, &A);
      for (int32_t s = 0; s < trial->ns; ++s) {
        load_seg(trial, s, &B);
        cpx L[2][2];
        if (local_matrix(op, test, trial, qs, &A, &B, -1, L, NULL)) { err = 1; continue; }
        for (int j = 0; j < nsB; ++j) {
          const int32_t n = trial->fn_index[2 * (int64_t)s + j];
          if (n < 0) continue;
          const double cb = trial->fn_coef[2 * (int64_t)s + j];
          cpx v = cscale(cscale(L[i][j], ca), cb);
          row[2 * n] += v.re;
          row[2 * n + 1] += v.im;
        }
      }
    }
  }
  free(off); free(se); free(si); free(fill);
  return err ? -2 : 0;
}
