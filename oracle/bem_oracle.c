/*
 * FP64 CPU oracle for BEM Galerkin matrix assembly -- TEST INFRASTRUCTURE ONLY.
 * See bem_oracle.h for the scope, conventions and the parity status (unpinned against BEAST).
 *
 * Compile with -ffp-contract=off: the classification predicate must round exactly like
 * BEAST's Julia code (no fused multiply-add), on x86 and on Arm alike.
 *
 * Reference citations are paths inside the BEASTGPU repository.
 */
#include "bem_oracle.h"
#include "trirules.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cpx;

static inline cpx mk(double re, double im) { cpx r; r.re = re; r.im = im; return r; }
static inline cpx cmul(cpx a, cpx b) { return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cpx cmulr(cpx a, double s) { return mk(a.re * s, a.im * s); }
static inline cpx cdivr(cpx a, double s) { return mk(a.re / s, a.im / s); }
static inline cpx cadd(cpx a, cpx b) { return mk(a.re + b.re, a.im + b.im); }

/* exp(-R * gamma) with Julia's Complex exp: exp(re) * (cos(im), sin(im)). */
static inline cpx expmg(double R, const double g[2]) {
  double zr = -R * g[0], zi = -R * g[1];
  double er = exp(zr);
  if (zi == 0.0) return mk(er, zi);
  return mk(er * cos(zi), er * sin(zi));
}

/* 1 / (4 pi) as Julia evaluates `1 / (4pi)` (doubleQuadRuleMainCase.jl:143, Integrand_gpu.jl:4). */
static double inv4pi(void) { return 1.0 / (4.0 * M_PI); }

/* ------------------------------------------------------------------------------------ */
/* Geometry: CompScienceMeshes simplex (tangents v_i - v_3, volume |t1 x t2| / 2), as the  */
/* reference loads it in load_parameters.jl:25-46.                                          */
/* ------------------------------------------------------------------------------------ */
typedef struct {
  double v[3][3]; /* v[vertex][coord] */
  double t[2][3]; /* t[k] = v[k] - v[2] */
  double area;
} tri_t;

static void load_tri(const orc_space* s, int32_t t, tri_t* T) {
  for (int a = 0; a < 3; ++a) {
    int32_t vi = s->triangles[3 * (int64_t)t + a];
    for (int c = 0; c < 3; ++c) T->v[a][c] = s->vertices[3 * (int64_t)vi + c];
  }
  for (int k = 0; k < 2; ++k)
    for (int c = 0; c < 3; ++c) T->t[k][c] = T->v[k][c] - T->v[2][c];
  double n0 = T->t[0][1] * T->t[1][2] - T->t[0][2] * T->t[1][1];
  double n1 = T->t[0][2] * T->t[1][0] - T->t[0][0] * T->t[1][2];
  double n2 = T->t[0][0] * T->t[1][1] - T->t[0][1] * T->t[1][0];
  T->area = sqrt(n0 * n0 + n1 * n1 + n2 * n2) / 2.0;
}

double orc_triangle_area(const orc_space* s, int32_t t) {
  tri_t T;
  load_tri(s, t, &T);
  return T.area;
}

/* barytocart: r = v3; r += t1 * u; r += t2 * v  (strategy_sauterschwabints.jl:63-68). */
static inline void cart(const tri_t* T, double u, double v, double x[3]) {
  for (int c = 0; c < 3; ++c) x[c] = (T->v[2][c] + T->t[0][c] * u) + T->t[1][c] * v;
}

/* ------------------------------------------------------------------------------------ */
/* Pair classification: the faithful FP64 predicate of doubleQuadRuleMainCase.jl:187-200  */
/* (BEAST quadrule), class codes of quadrule_determine.jl:76: 0 far, 1 CV, 2 CE, 3 CF,     */
/* 4 near.  Returns -1 for degenerate input (more than three coincident vertex pairs).    */
/* ------------------------------------------------------------------------------------ */
static int classify_pair(const tri_t* a, const tri_t* b, double k2) {
  const double dtol = 2.220446049250313e-16 * 1.0e3; /* quadrule_determine.jl:1 */
  const double xtol2 = 0.2 * 0.2;                     /* quadrule_determine.jl:3 */
  int hits = 0;
  double dmin2 = DBL_MAX; /* floatmax(Float64) */
  for (int u1 = 0; u1 < 3; ++u1)
    for (int u2 = 0; u2 < 3; ++u2) {
      double dx = a->v[u1][0] - b->v[u2][0];
      double dy = a->v[u1][1] - b->v[u2][1];
      double dz = a->v[u1][2] - b->v[u2][2];
      double d2 = (dx * dx + dy * dy) + dz * dz;
      double d = sqrt(d2);
      hits += (d < dtol);
      dmin2 = fmin(dmin2, d2);
    }
  if (hits > 3) return -1;
  if (hits > 0) return hits;
  double h2 = b->area;
  double m = fmax(dmin2 * k2, dmin2 / (16.0 * h2));
  return (m >= xtol2) ? ORC_CLASS_FAR : ORC_CLASS_NEAR;
}

int orc_classify_block(const orc_space* test, const orc_space* trial, double k2, int32_t t0,
                       int32_t t1, int32_t s0, int32_t s1, int8_t* out) {
  if (!test || !trial || !out || t0 < 0 || s0 < 0 || t1 > test->nt || s1 > trial->nt || t1 < t0 || s1 < s0)
    return -1;
  int err = 0;
  int64_t ns = s1 - s0;
#pragma omp parallel for schedule(dynamic, 4) reduction(| : err)
  for (int32_t t = t0; t < t1; ++t) {
    tri_t A, B;
    load_tri(test, t, &A);
    for (int32_t s = s0; s < s1; ++s) {
      load_tri(trial, s, &B);
      int c = classify_pair(&A, &B, k2);
      if (c < 0) err = 1;
      out[(int64_t)(t - t0) * ns + (s - s0)] = (int8_t)c;
    }
  }
  return err ? -2 : 0;
}

/* ------------------------------------------------------------------------------------ */
/* Quadrature rules                                                                       */
/* ------------------------------------------------------------------------------------ */
static int trirule_index(int npoints) {
  for (int r = 0; r < ORC_TRIRULE_COUNT; ++r)
    if (orc_trirule_npoints[r] == npoints) return r;
  return -1;
}

int orc_gauss_legendre01(int32_t n, double* x, double* w) {
  if (n < 1 || n > 64) return -1;
  /* Newton iteration on the three-term Legendre recurrence; nodes ascending on [0, 1]
   * (FastGaussQuadrature order mapped as BEAST's _legendre(n, 0, 1)). */
  for (int i = 0; i < n; ++i) {
    double t = -cos(M_PI * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = t;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) { p1 = t; p0 = 1.0; }
      dp = n * (t * p1 - p0) / (t * t - 1.0);
      double dt = p1 / dp;
      t -= dt;
      if (fabs(dt) < 1e-17) break;
    }
    {
      double p0 = 1.0, p1 = t;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) { p1 = t; p0 = 1.0; }
      dp = n * (t * p1 - p0) / (t * t - 1.0);
    }
    x[i] = (t + 1.0) / 2.0;
    w[i] = (2.0 / ((1.0 - t * t) * dp * dp)) / 2.0;
  }
  return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Shape functions at a point with chart parameters (u, v)                                */
/* ------------------------------------------------------------------------------------ */
typedef struct {
  double x[3];     /* cartesian point */
  double val[3];   /* Lagrange: barycentric hats (Integrand_gpu.jl:51-55) */
  double vec[3][3];/* RT: vector values (x - v_i) / (2A) (BEAST RTRefSpace) */
  double div;      /* RT divergence 1 / A */
  double n[3];     /* unit normal (t1 x t2) / (2A) */
  double curl[3][3]; /* Lagrange: surface curl n x grad(val_i) = (v_{i+1} - v_{i+2}) / (2A) */
} shp_t;

static void eval_shapes(const tri_t* T, int32_t refspace, double u, double v, shp_t* S) {
  cart(T, u, v, S->x);
  S->val[0] = u;
  S->val[1] = v;
  S->val[2] = 1.0 - u - v;
  {
    const double inv_j = 1.0 / (T->area * 2.0);
    S->n[0] = (T->t[0][1] * T->t[1][2] - T->t[0][2] * T->t[1][1]) * inv_j;
    S->n[1] = (T->t[0][2] * T->t[1][0] - T->t[0][0] * T->t[1][2]) * inv_j;
    S->n[2] = (T->t[0][0] * T->t[1][1] - T->t[0][1] * T->t[1][0]) * inv_j;
    for (int i = 0; i < 3; ++i)
      for (int c = 0; c < 3; ++c) S->curl[i][c] = (T->v[(i + 1) % 3][c] - T->v[(i + 2) % 3][c]) * inv_j;
  }
  if (refspace == ORC_REFSPACE_RT) {
    double j = T->area * 2.0;
    double inv_j = 1.0 / j;
    for (int c = 0; c < 3; ++c) {
      double utu = u * T->t[0][c], vtv = v * T->t[1][c];
      S->vec[0][c] = ((utu - T->t[0][c]) + vtv) * inv_j;
      S->vec[1][c] = ((utu + vtv) - T->t[1][c]) * inv_j;
      S->vec[2][c] = (utu + vtv) * inv_j;
    }
    S->div = 2.0 * inv_j;
  }
}

/* Operator integrand at one point pair, weighted by `wgt` (already including Jacobians and
 * quadrature weights), accumulated into L[i][j].  Helmholtz is restated in the reference's
 * own association for the far rule (doubleQuadRuleMainCase.jl:85-103,145); the Maxwell
 * forms have no reference code and follow BEAST's MWSingleLayer3D / MWDoubleLayer3D. */
static void accumulate_far(const orc_operator* op, const shp_t* X, const shp_t* Y, double wx,
                           double wy, cpx L[3][3]) {
  double d0 = X->x[0] - Y->x[0], d1 = X->x[1] - Y->x[1], d2 = X->x[2] - Y->x[2];
  double R = sqrt((d0 * d0 + d1 * d1) + d2 * d2);
  cpx alpha = mk(op->alpha[0], op->alpha[1]);
  if (op->kind == ORC_OP_HELMHOLTZ3D_SL) {
    /* j_aG = alpha * w_I * w_J * i4pi / R * exp(-R*gamma)   (doubleQuadRuleMainCase.jl:145) */
    cpx jaG = cmul(cdivr(cmulr(cmulr(cmulr(alpha, wx), wy), inv4pi()), R), expmg(R, op->gamma));
    for (int i = 0; i < 3; ++i) {
      cpx t = cmulr(jaG, X->val[i]);
      for (int j = 0; j < 3; ++j) L[i][j] = cadd(L[i][j], cmulr(t, Y->val[j]));
    }
    return;
  }
  cpx G = cmul(mk(wx * wy * inv4pi() / R, 0.0), expmg(R, op->gamma));
  if (op->kind == ORC_OP_HELMHOLTZ3D_DL || op->kind == ORC_OP_HELMHOLTZ3D_DLT) {
    /* dG/dn_y = (gamma + 1/R) G ((x - y) . n_y) / R;  dG/dn_x = -(gamma + 1/R) G ((x - y) . n_x) / R
     * (BEAST's HH3DDoubleLayerFDBIO / HH3DDoubleLayerTransposedFDBIO, written from the kernel) */
    const double* nv = op->kind == ORC_OP_HELMHOLTZ3D_DL ? Y->n : X->n;
    double rn = (d0 * nv[0] + d1 * nv[1]) + d2 * nv[2];
    if (op->kind == ORC_OP_HELMHOLTZ3D_DLT) rn = -rn;
    cpx H = cmul(mk(op->gamma[0] + 1.0 / R, op->gamma[1]), cmulr(G, rn / R));
    H = cmul(alpha, H);
    for (int i = 0; i < 3; ++i) {
      cpx t = cmulr(H, X->val[i]);
      for (int j = 0; j < 3; ++j) L[i][j] = cadd(L[i][j], cmulr(t, Y->val[j]));
    }
    return;
  }
  if (op->kind == ORC_OP_HELMHOLTZ3D_HS) {
    /* Maue's form of the hypersingular operator (BEAST's HH3DHyperSingularFDBIO):
     * alpha (n_x . n_y) f g G + beta (curl f . curl g) G */
    const double nn = (X->n[0] * Y->n[0] + X->n[1] * Y->n[1]) + X->n[2] * Y->n[2];
    cpx a = cmulr(cmul(alpha, G), nn), b = cmul(mk(op->beta[0], op->beta[1]), G);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const double cc = (X->curl[i][0] * Y->curl[j][0] + X->curl[i][1] * Y->curl[j][1]) + X->curl[i][2] * Y->curl[j][2];
        L[i][j] = cadd(L[i][j], cadd(cmulr(a, X->val[i] * Y->val[j]), cmulr(b, cc)));
      }
    return;
  }
  if (op->kind == ORC_OP_MAXWELL3D_SL) {
    cpx beta = mk(op->beta[0], op->beta[1]);
    cpx a = cmul(alpha, G), b = cmul(beta, G);
    double dd = X->div * Y->div;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const double* f = X->vec[i];
        const double* g = Y->vec[j];
        double fg = (f[0] * g[0] + f[1] * g[1]) + f[2] * g[2];
        L[i][j] = cadd(L[i][j], cadd(cmulr(a, fg), cmulr(b, dd)));
      }
    return;
  }
  /* Maxwell double layer: f(x) . (grad_x G(x,y) x g(y)),  grad_x G = -(gamma + 1/R) G r / R. */
  cpx H = cmul(mk(-op->gamma[0] - 1.0 / R, -op->gamma[1]), cdivr(G, R));
  H = cmul(alpha, H);
  double r[3] = {d0, d1, d2};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const double* f = X->vec[i];
      const double* g = Y->vec[j];
      double c0 = r[1] * g[2] - r[2] * g[1];
      double c1 = r[2] * g[0] - r[0] * g[2];
      double c2 = r[0] * g[1] - r[1] * g[0];
      double trip = (f[0] * c0 + f[1] * c1) + f[2] * c2;
      L[i][j] = cadd(L[i][j], cmulr(H, trip));
    }
}

/* Double quadrature over a (test, trial) pair with the given triangle rules. */
static int double_quadrature(const orc_operator* op, const tri_t* A, int32_t rsA, const tri_t* B,
                             int32_t rsB, int qt, int qb, cpx L[3][3]) {
  int rt = trirule_index(qt), rb = trirule_index(qb);
  if (rt < 0 || rb < 0) return -1;
  shp_t X[16], Y[16];
  double wx[16], wy[16];
  for (int I = 0; I < qt; ++I) {
    const double* q = orc_trirule_uvw[orc_trirule_offset[rt] + I];
    eval_shapes(A, rsA, q[0], q[1], &X[I]);
    wx[I] = (q[2] / 2.0) * (A->area * 2.0); /* BEAST weight: w_ref * jacobian */
  }
  for (int J = 0; J < qb; ++J) {
    const double* q = orc_trirule_uvw[orc_trirule_offset[rb] + J];
    eval_shapes(B, rsB, q[0], q[1], &Y[J]);
    wy[J] = (q[2] / 2.0) * (B->area * 2.0);
  }
  for (int I = 0; I < qt; ++I)
    for (int J = 0; J < qb; ++J) accumulate_far(op, &X[I], &Y[J], wx[I], wy[J], L);
  return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Near pairs: singularity extraction.  BEAST integrates pairs of class 4 (close, sharing   */
/* no vertex) with WiltonSERule, the near rule of DoubleNumWiltonSauterQStrat (the rule its */
/* quadrule returns in place of the reference's near branch, doubleQuadRuleMainCase.jl:200; */
/* the reference itself drops the class, quadrule_determine.jl:76).  G = G_s + G_r with     */
/*   G_s = (1/R - gamma + gamma^2 R / 2) / (4 pi)     the first terms of the Taylor series   */
/*   G_r = (exp(-z) - 1 + z - z^2/2) / (4 pi R),  z = gamma R   (smooth)                    */
/* The inner (trial) integral of G_s times a linear shape is in closed form over the flat   */
/* trial triangle (Wilton et al., IEEE TAP 32(3) 1984; Graglia, IEEE TAP 41(10) 1993) and   */
/* the outer (test) integral is the near test rule; G_r takes the near double rule.  The    */
/* transposed double layer swaps the roles (closed form over the test triangle, outer rule  */
/* over the trial points), since its kernel is the double layer's seen from the trial side. */
/* ------------------------------------------------------------------------------------ */

/* e2 = exp(-z) - 1 + z and e3 = e2 - z^2 / 2 for complex z: the power series for |z| < 1
 * (Horner, terms to (-z)^20 / 20!), the exponential beyond. */
static void exp_tails(cpx z, cpx* e2, cpx* e3) {
  const cpx mz = mk(-z.re, -z.im);
  const cpx z2h = cmulr(cmul(z, z), 0.5);
  if (z.re * z.re + z.im * z.im < 1.0) {
    cpx sum = mk(1.0, 0.0);
    for (int n = 20; n >= 4; --n) sum = cadd(mk(1.0, 0.0), cdivr(cmul(sum, mz), (double)n));
    *e3 = cmul(cdivr(cmul(cmul(mz, mz), mz), 6.0), sum);
    *e2 = cadd(*e3, z2h);
    return;
  }
  const double er = exp(mz.re);
  const cpx ez = mk(er * cos(mz.im), er * sin(mz.im));
  *e2 = cadd(cadd(ez, mk(-1.0, 0.0)), z);
  *e3 = cadd(*e2, mk(-z2h.re, -z2h.im));
}

/* Closed-form potentials of a flat triangle T at the point x.  With n the chart normal,
 * d = n.(x - v3), rho = x - d n and R = |x - y|:
 *   Im1 = int 1/R,  I1 = int R,  Jm1 = int (y - rho)/R,  J1 = int (y - rho) R,
 *   Om = int d/R^3 (the signed solid angle, Van Oosterom & Strackee, IEEE TBME 30(2) 1983),
 *   Jm3 = int (y - rho)/R^3 = -sum_edges m ln((R+ + s+)/(R- + s-))   (x not on T).
 * Edge sums follow Wilton / Graglia: for the edge a -> b (counter-clockwise about n) with
 * unit tangent l, outward normal m = l x n, s+- = (b|a - rho).l, t0 = (a - rho).m,
 * R0^2 = t0^2 + d^2: int_e 1/R = f, int_e R = K1 = (s+R+ - s-R- + R0^2 f)/2,
 * int_e R^3 = K3 = (s+R+^3 - s-R-^3)/4 + 3 R0^2 K1 / 4, and
 * Im1 = sum t0 f - d Om,  I1 = (d^2 Im1 + sum t0 K1)/3,  Jm1 = sum m K1,  J1 = sum m K3 / 3. */
typedef struct {
  double Im1, I1, Om, d;
  double Jm1[3], J1[3], Jm3[3], rho[3], n[3];
} tripot_t;

static inline double dot3(const double a[3], const double b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
static inline void cross3(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

static void triangle_potentials(const tri_t* T, const double x[3], tripot_t* P) {
  double n[3];
  cross3(T->t[0], T->t[1], n);
  const double nn = sqrt(dot3(n, n));
  for (int c = 0; c < 3; ++c) n[c] /= nn;
  double xv[3];
  for (int c = 0; c < 3; ++c) xv[c] = x[c] - T->v[2][c];
  const double d = dot3(n, xv);
  double rho[3];
  for (int c = 0; c < 3; ++c) {
    rho[c] = x[c] - d * n[c];
    P->rho[c] = rho[c];
    P->n[c] = n[c];
    P->Jm1[c] = P->J1[c] = P->Jm3[c] = 0.0;
  }
  double sum_tf = 0.0, sum_tk1 = 0.0;
  for (int e = 0; e < 3; ++e) {
    const double* a = T->v[e];
    const double* b = T->v[(e + 1) % 3];
    double l[3], m[3], ar[3], br[3], ax[3], bx[3];
    for (int c = 0; c < 3; ++c) {
      l[c] = b[c] - a[c];
      ar[c] = a[c] - rho[c];
      br[c] = b[c] - rho[c];
      ax[c] = x[c] - a[c];
      bx[c] = x[c] - b[c];
    }
    const double ll = sqrt(dot3(l, l));
    for (int c = 0; c < 3; ++c) l[c] /= ll;
    cross3(l, n, m);
    const double sp = dot3(br, l), sm = dot3(ar, l), t0 = dot3(ar, m);
    const double Rp = sqrt(dot3(bx, bx)), Rm = sqrt(dot3(ax, ax));
    const double R02 = t0 * t0 + d * d;
    double f;
    if (sp < 0.0 && sm < 0.0) f = log((Rm - sm) / (Rp - sp)); /* beyond a: R0^2 cancels */
    else if (sm >= 0.0) f = log((Rp + sp) / (Rm + sm));        /* beyond b */
    else f = log((Rp + sp) * (Rm - sm) / R02);                 /* rho abreast of the edge */
    const double K1 = 0.5 * ((sp * Rp - sm * Rm) + R02 * f);
    const double K3 = 0.25 * (sp * Rp * Rp * Rp - sm * Rm * Rm * Rm) + 0.75 * R02 * K1;
    sum_tf += t0 * f;
    sum_tk1 += t0 * K1;
    for (int c = 0; c < 3; ++c) {
      P->Jm1[c] += m[c] * K1;
      P->J1[c] += m[c] * K3 / 3.0;
      P->Jm3[c] -= m[c] * f;
    }
  }
  double q[3][3], nq[3];
  for (int i = 0; i < 3; ++i) {
    for (int c = 0; c < 3; ++c) q[i][c] = T->v[i][c] - x[c];
    nq[i] = sqrt(dot3(q[i], q[i]));
  }
  double q12[3];
  cross3(q[1], q[2], q12);
  const double trip = dot3(q[0], q12);
  const double den = nq[0] * nq[1] * nq[2] + dot3(q[0], q[1]) * nq[2] + dot3(q[0], q[2]) * nq[1] + dot3(q[1], q[2]) * nq[0];
  P->Om = -2.0 * atan2(trip, den);
  P->d = d;
  P->Im1 = sum_tf - d * P->Om;
  P->I1 = (d * d * P->Im1 + sum_tk1) / 3.0;
}

/* Inner integrals of the singular part over T at x (factor 1/(4 pi) included):
 *   S0 = int G_s, Sv = int G_s (y - rho), Gv = int grad_x G_s,
 *   D0 = int (n.grad_y G_s) with n.grad_y G_s = (d/R^3 - gamma^2 d / (2R)) / (4 pi), Dv the same times (y - rho). */
typedef struct {
  cpx S0, D0;
  cpx Sv[3], Gv[3], Dv[3];
  double rho[3];
} singpart_t;

static void singular_part(const tri_t* T, const double x[3], const double g[2], singpart_t* S) {
  tripot_t P;
  triangle_potentials(T, x, &P);
  const double i4p = inv4pi();
  const cpx gam = mk(g[0], g[1]);
  const cpx g2h = cmulr(cmul(gam, gam), 0.5);
  double cen[3];
  for (int c = 0; c < 3; ++c) cen[c] = (T->v[0][c] + T->v[1][c] + T->v[2][c]) / 3.0;
  /* S0 = (Im1 - gamma A + gamma^2/2 I1) / (4 pi) */
  S->S0 = cmulr(cadd(cadd(mk(P.Im1, 0.0), cmulr(gam, -T->area)), cmulr(g2h, P.I1)), i4p);
  S->D0 = cmulr(cadd(mk(P.Om, 0.0), cmulr(g2h, -P.d * P.Im1)), i4p);
  for (int c = 0; c < 3; ++c) {
    S->rho[c] = P.rho[c];
    /* int (y - rho) = A (centroid - rho) */
    S->Sv[c] = cmulr(cadd(cadd(mk(P.Jm1[c], 0.0), cmulr(gam, -T->area * (cen[c] - P.rho[c]))), cmulr(g2h, P.J1[c])), i4p);
    /* int grad_x (1/R) = Jm3 - n Om; int grad_x R = d n Im1 - Jm1 */
    S->Gv[c] = cmulr(cadd(mk(P.Jm3[c] - P.n[c] * P.Om, 0.0), cmulr(g2h, P.d * P.n[c] * P.Im1 - P.Jm1[c])), i4p);
    S->Dv[c] = cmulr(cadd(mk(P.d * P.Jm3[c], 0.0), cmulr(g2h, -P.d * P.Jm1[c])), i4p);
  }
}

/* Hat j of triangle T at the in-plane point rho (affine extension) and its gradient. */
static void hat_affine(const tri_t* T, const double rho[3], double val[3], double grad[3][3]) {
  double n[3], cen[3];
  cross3(T->t[0], T->t[1], n);
  const double nn = sqrt(dot3(n, n)); /* 2A */
  for (int c = 0; c < 3; ++c) {
    n[c] /= nn;
    cen[c] = (T->v[0][c] + T->v[1][c] + T->v[2][c]) / 3.0;
  }
  for (int j = 0; j < 3; ++j) {
    double e[3], gj[3];
    for (int c = 0; c < 3; ++c) e[c] = T->v[(j + 2) % 3][c] - T->v[(j + 1) % 3][c];
    cross3(n, e, gj);
    double pr = 0.0;
    for (int c = 0; c < 3; ++c) {
      grad[j][c] = gj[c] / nn;
      pr += grad[j][c] * (rho[c] - cen[c]);
    }
    val[j] = 1.0 / 3.0 + pr;
  }
}

/* One point pair of the regular part G_r, weight w: the operator integrands of accumulate_far
 * with G_r for G and grad_x G_r = F (x - y). */
static void accumulate_regular(const orc_operator* op, const shp_t* X, const shp_t* Y, double w, cpx L[3][3]) {
  const double r[3] = {X->x[0] - Y->x[0], X->x[1] - Y->x[1], X->x[2] - Y->x[2]};
  const double R = sqrt(dot3(r, r));
  const cpx z = cmulr(mk(op->gamma[0], op->gamma[1]), R);
  cpx e2, e3;
  exp_tails(z, &e2, &e3);
  const cpx G = cmulr(e3, w * inv4pi() / R);                                       /* G_r */
  const cpx F = cmulr(cadd(cmul(z, e2), e3), -w * inv4pi() / (R * R * R));          /* G_r' / R */
  const cpx alpha = mk(op->alpha[0], op->alpha[1]);
  const cpx beta = mk(op->beta[0], op->beta[1]);
  switch (op->kind) {
    case ORC_OP_HELMHOLTZ3D_SL:
    case ORC_OP_HELMHOLTZ3D_DL:
    case ORC_OP_HELMHOLTZ3D_DLT: {
      cpx k = cmul(alpha, G);
      if (op->kind == ORC_OP_HELMHOLTZ3D_DL) k = cmul(alpha, cmulr(F, -dot3(r, Y->n))); /* n_y.grad_y G = -F r.n_y */
      if (op->kind == ORC_OP_HELMHOLTZ3D_DLT) k = cmul(alpha, cmulr(F, dot3(r, X->n))); /* n_x.grad_x G = F r.n_x */
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) L[i][j] = cadd(L[i][j], cmulr(k, X->val[i] * Y->val[j]));
      return;
    }
    case ORC_OP_HELMHOLTZ3D_HS: {
      const cpx a = cmulr(cmul(alpha, G), dot3(X->n, Y->n)), b = cmul(beta, G);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          L[i][j] = cadd(L[i][j], cadd(cmulr(a, X->val[i] * Y->val[j]), cmulr(b, dot3(X->curl[i], Y->curl[j]))));
      return;
    }
    case ORC_OP_MAXWELL3D_SL: {
      const cpx a = cmul(alpha, G), b = cmul(beta, G);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          L[i][j] = cadd(L[i][j], cadd(cmulr(a, dot3(X->vec[i], Y->vec[j])), cmulr(b, X->div * Y->div)));
      return;
    }
    default: { /* Maxwell double layer: f . (F r x g) */
      const cpx H = cmul(alpha, F);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double c[3];
          cross3(r, Y->vec[j], c);
          L[i][j] = cadd(L[i][j], cmulr(H, dot3(X->vec[i], c)));
        }
      return;
    }
  }
}

static inline cpx cdot3(const double a[3], const cpx b[3]) {
  return cadd(cadd(cmulr(b[0], a[0]), cmulr(b[1], a[1])), cmulr(b[2], a[2]));
}

static int near_extraction(const orc_operator* op, const tri_t* A, int32_t rsA, const tri_t* B, int32_t rsB, int qt,
                           int qb, cpx L[3][3]) {
  int rt = trirule_index(qt), rb = trirule_index(qb);
  if (rt < 0 || rb < 0) return -1;
  shp_t X[16], Y[16];
  double wx[16], wy[16];
  for (int I = 0; I < qt; ++I) {
    const double* q = orc_trirule_uvw[orc_trirule_offset[rt] + I];
    eval_shapes(A, rsA, q[0], q[1], &X[I]);
    wx[I] = (q[2] / 2.0) * (A->area * 2.0);
  }
  for (int J = 0; J < qb; ++J) {
    const double* q = orc_trirule_uvw[orc_trirule_offset[rb] + J];
    eval_shapes(B, rsB, q[0], q[1], &Y[J]);
    wy[J] = (q[2] / 2.0) * (B->area * 2.0);
  }
  for (int I = 0; I < qt; ++I)
    for (int J = 0; J < qb; ++J) accumulate_regular(op, &X[I], &Y[J], wx[I] * wy[J], L);
  const cpx alpha = mk(op->alpha[0], op->alpha[1]);
  const cpx beta = mk(op->beta[0], op->beta[1]);
  if (op->kind == ORC_OP_HELMHOLTZ3D_DLT) { /* outer rule over the trial points, closed form over the test triangle */
    for (int J = 0; J < qb; ++J) {
      singpart_t S;
      singular_part(A, Y[J].x, op->gamma, &S);
      double hv[3], hg[3][3];
      hat_affine(A, S.rho, hv, hg);
      for (int i = 0; i < 3; ++i) {
        const cpx in = cmul(alpha, cadd(cmulr(S.D0, hv[i]), cdot3(hg[i], S.Dv)));
        for (int j = 0; j < 3; ++j) L[i][j] = cadd(L[i][j], cmulr(in, wy[J] * Y[J].val[j]));
      }
    }
    return 0;
  }
  for (int I = 0; I < qt; ++I) {
    singpart_t S;
    singular_part(B, X[I].x, op->gamma, &S);
    const double w = wx[I];
    double hv[3], hg[3][3];
    hat_affine(B, S.rho, hv, hg);
    for (int j = 0; j < 3; ++j) {
      cpx in_j = mk(0.0, 0.0); /* the singular part's inner integral against trial shape j, times the test shapes below */
      switch (op->kind) {
        case ORC_OP_HELMHOLTZ3D_SL:
          in_j = cmul(alpha, cadd(cmulr(S.S0, hv[j]), cdot3(hg[j], S.Sv)));
          for (int i = 0; i < 3; ++i) L[i][j] = cadd(L[i][j], cmulr(in_j, w * X[I].val[i]));
          break;
        case ORC_OP_HELMHOLTZ3D_DL:
          in_j = cmul(alpha, cadd(cmulr(S.D0, hv[j]), cdot3(hg[j], S.Dv)));
          for (int i = 0; i < 3; ++i) L[i][j] = cadd(L[i][j], cmulr(in_j, w * X[I].val[i]));
          break;
        case ORC_OP_HELMHOLTZ3D_HS: {
          const cpx sl = cmul(cmulr(alpha, dot3(X[I].n, Y[0].n)), cadd(cmulr(S.S0, hv[j]), cdot3(hg[j], S.Sv)));
          const cpx cc = cmul(beta, S.S0);
          for (int i = 0; i < 3; ++i)
            L[i][j] = cadd(L[i][j], cmulr(cadd(cmulr(sl, X[I].val[i]), cmulr(cc, dot3(X[I].curl[i], Y[0].curl[j]))), w));
          break;
        }
        case ORC_OP_MAXWELL3D_SL: {
          /* int G_s g_j = (Sv + (rho - w_j) S0) / (2 A_sigma) */
          cpx gj[3];
          for (int c = 0; c < 3; ++c)
            gj[c] = cmulr(cadd(S.Sv[c], cmulr(S.S0, S.rho[c] - B->v[j][c])), 1.0 / (2.0 * B->area));
          const cpx dd = cmul(beta, cmulr(S.S0, X[I].div * Y[0].div));
          for (int i = 0; i < 3; ++i)
            L[i][j] = cadd(L[i][j], cmulr(cadd(cmul(alpha, cdot3(X[I].vec[i], gj)), dd), w));
          break;
        }
        default: { /* Maxwell double layer: int grad_x G_s x g_j = Gv x (x - w_j) / (2 A_sigma) */
          double xw[3];
          for (int c = 0; c < 3; ++c) xw[c] = (X[I].x[c] - B->v[j][c]) / (2.0 * B->area);
          cpx cr[3];
          cr[0] = cadd(cmulr(S.Gv[1], xw[2]), cmulr(S.Gv[2], -xw[1]));
          cr[1] = cadd(cmulr(S.Gv[2], xw[0]), cmulr(S.Gv[0], -xw[2]));
          cr[2] = cadd(cmulr(S.Gv[0], xw[1]), cmulr(S.Gv[1], -xw[0]));
          for (int i = 0; i < 3; ++i) L[i][j] = cadd(L[i][j], cmulr(cmul(alpha, cdot3(X[I].vec[i], cr)), w));
          break;
        }
      }
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Sauter-Schwab singular rules                                                            */
/* ------------------------------------------------------------------------------------ */

/* Vertex permutations I (test) and J (trial) that put the shared vertices in the positions
 * SauterSchwabQuadrature expects (the `reorder` step), as pulledback_integrand_gpu.jl does
 * it: CF :22-58, CE :60-102 (setdiff :111-115, circshift :104-109), CV :117-155. */
static void ss_permutation(int cls, const tri_t* A, const tri_t* B, int I[3], int J[3]) {
  const double tol = 1e3 * DBL_EPSILON; /* pulledback_integrand_gpu.jl:21 */
  I[0] = I[1] = I[2] = 0;
  J[0] = J[1] = J[2] = 0;
  int cap = (cls == ORC_CLASS_CE) ? 3 : 2;
  int e = 1;
  for (int i = 1; i <= 3; ++i)
    for (int j = 1; j <= 3; ++j) {
      double R = 0.0;
      for (int c = 0; c < 3; ++c) {
        double d = A->v[i - 1][c] - B->v[j - 1][c];
        R += d * d;
      }
      if (sqrt(R) < tol) {
        if (cls == ORC_CLASS_CF) {
          J[i - 1] = j;
        } else if (e <= cap) {
          J[e - 1] = j;
          I[e - 1] = i;
          e += 1;
        }
      }
    }
  if (cls == ORC_CLASS_CF) {
    I[0] = 1; I[1] = 2; I[2] = 3;
    return;
  }
  int* arr[2] = {J, I};
  for (int k = 0; k < 2; ++k) {
    int* a = arr[k];
    int e1 = (e == 1), e2 = (e == 2);
    a[0] = e1 ? 1 : a[0];
    a[1] = e1 ? 2 : (e2 ? (a[0] == 1 ? 2 : 1) : a[1]);
    a[2] = 6 - a[0] - a[1];
  }
  if (cls == ORC_CLASS_CE) {
    for (int k = 0; k < 2; ++k) {
      int* a = arr[k];
      int t = a[0];
      a[0] = a[1];
      a[1] = a[2];
      a[2] = t;
    }
  }
}

typedef struct {
  double cv[3][2]; /* chart vertices in the reference triangle */
  double ct[2][2]; /* chart tangents */
} chart_t;

static void make_chart(const int P[3], chart_t* C) {
  static const double V[3][2] = {{1.0, 0.0}, {0.0, 1.0}, {0.0, 0.0}}; /* SauterSchwab.jl:172 */
  for (int u = 0; u < 3; ++u) {
    C->cv[u][0] = V[P[u] - 1][0];
    C->cv[u][1] = V[P[u] - 1][1];
  }
  for (int u = 0; u < 2; ++u) { /* pulledback_integrand_gpu.jl:214-217 */
    C->ct[u][0] = C->cv[u][0] - C->cv[2][0];
    C->ct[u][1] = C->cv[u][1] - C->cv[2][1];
  }
}

typedef struct {
  const orc_operator* op;
  const tri_t *A, *B;
  int32_t rsA, rsB;
  chart_t cA, cB;
} ss_ctx;

/* One Sauter-Schwab integrand evaluation (Integrand_gpu.jl:58-132 for Helmholtz). */
static void ss_point(const ss_ctx* c, double u1, double u2, double v1, double v2, double mul,
                     cpx L[3][3]) {
  /* calc_bary (Integrand_gpu.jl:51-55) */
  double bx1 = c->cA.cv[2][0] + c->cA.ct[0][0] * u1 + c->cA.ct[1][0] * u2;
  double bx2 = c->cA.cv[2][1] + c->cA.ct[0][1] * u1 + c->cA.ct[1][1] * u2;
  double by1 = c->cB.cv[2][0] + c->cB.ct[0][0] * v1 + c->cB.ct[1][0] * v2;
  double by2 = c->cB.cv[2][1] + c->cB.ct[0][1] * v1 + c->cB.ct[1][1] * v2;
  const orc_operator* op = c->op;
  if (op->kind == ORC_OP_HELMHOLTZ3D_SL) {
    double bx[3] = {bx1, bx2, 1.0 - bx1 - bx2};
    double by[3] = {by1, by2, 1.0 - by1 - by2};
    double x[3], y[3];
    for (int k = 0; k < 3; ++k) { /* Integrand_gpu.jl:85-91 */
      x[k] = c->A->v[2][k] + c->A->t[0][k] * bx[0] + c->A->t[1][k] * bx[1];
      y[k] = c->B->v[2][k] + c->B->t[0][k] * by[0] + c->B->t[1][k] * by[1];
    }
    double dx1 = x[0] - y[0], dx2 = x[1] - y[1], dx3 = x[2] - y[2];
    double R = sqrt(dx1 * dx1 + dx2 * dx2 + dx3 * dx3);
    double green = inv4pi() / R;
    cpx green2 = expmg(R, op->gamma);
    cpx alpha = mk(op->alpha[0], op->alpha[1]);
    /* alpha * 4 * A_tau * A_sigma * green * mul  (Integrand_gpu.jl:111) */
    cpx jx = cmulr(cmulr(cmulr(cmulr(cmulr(alpha, 4.0), c->A->area), c->B->area), green), mul);
    for (int i = 0; i < 3; ++i) { /* trial local i (Integrand_gpu.jl:125-132) */
      cpx jg = cmulr(jx, by[i]);
      for (int j = 0; j < 3; ++j) { /* test local j */
        cpx t = cmulr(jg, bx[j]);
        L[j][i] = cadd(L[j][i], cmul(t, green2));
      }
    }
    return;
  }
  /* Maxwell operators on RT: same pull-back, operator integrand as in the far rule with the
   * weight 4 A_tau A_sigma mul (Jacobians 2A of both charts times the Sauter-Schwab weight). */
  shp_t X, Y;
  eval_shapes(c->A, c->rsA, bx1, bx2, &X);
  eval_shapes(c->B, c->rsB, by1, by2, &Y);
  double wgt = ((4.0 * c->A->area) * c->B->area) * mul;
  accumulate_far(op, &X, &Y, wgt, 1.0, L);
}

/* Sauter-Schwab integral of one singular pair: 4-D Gauss-Legendre over (eta1, eta2, eta3,
 * xi) with the region maps of SauterSchwab.jl:265-297 (CV 2 regions, CE 5, CF 6). */
static int sauter_schwab(const orc_operator* op, int cls, const tri_t* A, int32_t rsA, const tri_t* B,
                         int32_t rsB, int n, cpx L[3][3]) {
  if ((op->kind == ORC_OP_MAXWELL3D_DL || op->kind == ORC_OP_HELMHOLTZ3D_DL || op->kind == ORC_OP_HELMHOLTZ3D_DLT) &&
      cls == ORC_CLASS_CF)
    return 0; /* exactly zero on a flat face */
  double q[64], w[64];
  if (orc_gauss_legendre01(n, q, w)) return -1;
  int I[3], J[3];
  ss_permutation(cls, A, B, I, J);
  ss_ctx c;
  c.op = op;
  c.A = A;
  c.B = B;
  c.rsA = rsA;
  c.rsB = rsB;
  make_chart(I, &c.cA);
  make_chart(J, &c.cB);
  /* point index h*n^4 + ((i*n + j)*n + k)*n + l  (calc_index_bitshifts, SauterSchwab.jl:16-30) */
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k)
        for (int l = 0; l < n; ++l) {
          double h1 = q[i], h2 = q[j], h3 = q[k], xi = q[l];
          double wt = w[i] * w[j] * w[k] * w[l]; /* SauterSchwab.jl:251 */
          double xi3 = xi * xi * xi;
          if (cls == ORC_CLASS_CV) { /* SauterSchwab.jl:265-272 */
            double xh1 = xi * h1, xh2 = xi * h2;
            double mul = wt * xi3 * h2;
            ss_point(&c, 1 - xi, xh1, 1 - xh2, xh2 * h3, mul, L);
            ss_point(&c, 1 - xh2, xh2 * h3, 1 - xi, xh1, mul, L);
          } else if (cls == ORC_CLASS_CE) { /* SauterSchwab.jl:274-288 */
            double xh1 = xi * h1, h12 = h1 * h2, h23 = h2 * h3, h123 = h12 * h3;
            double mul = wt * xi3 * (h1 * h1) * h2;
            ss_point(&c, 1 - xi, xh1, 1 - xi * (1 - h123), xh1 * h2 * (1 - h3), mul, L);
            ss_point(&c, 1 - xi * (1 - h12), xh1 * (1 - h2), 1 - xi, xh1 * h23, mul, L);
            ss_point(&c, 1 - xi * (1 - h123), xh1 * h2 * (1 - h3), 1 - xi, xh1, mul, L);
            ss_point(&c, 1 - xi * (1 - h123), xh1 * (1 - h23), 1 - xi, xh1 * h2, mul, L);
            double mul5 = wt * xi3 * (h1 * h1);
            ss_point(&c, 1 - xi, xh1 * h3, 1 - xi * (1 - h12), xh1 * (1 - h2), mul5, L);
          } else { /* CF, SauterSchwab.jl:290-297 */
            double mul = wt * xi3 * (h1 * h1) * h2;
            double a = (xi - xi * h1) + xi * h1 * h2; /* xi - xi*eta1 + xi*eta1*eta2 */
            double b = 1 - (xi - xi * h1 * h2 * h3);
            double cc = xi - xi * h1;
            double d = xi * h1 * ((1 - h2) + h2 * h3);
            double e = 1 - (xi - xi * h1 * h2);
            double f = xi * h1 * (1 - h2);
            double g = xi * h1 * (1 - h2 * h3);
            ss_point(&c, 1 - xi, a, b, cc, mul, L);
            ss_point(&c, b, cc, 1 - xi, a, mul, L);
            ss_point(&c, 1 - xi, d, e, f, mul, L);
            ss_point(&c, e, f, 1 - xi, d, mul, L);
            ss_point(&c, b, g, 1 - xi, f, mul, L);
            ss_point(&c, 1 - xi, f, b, g, mul, L);
          }
        }
  return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Local matrices and assembly                                                            */
/* ------------------------------------------------------------------------------------ */
static double op_k2(const orc_operator* op) {
  return op->gamma[0] * op->gamma[0] + op->gamma[1] * op->gamma[1]; /* abs2(gamma) */
}

static int valid_op_space(const orc_operator* op, const orc_space* a, const orc_space* b) {
  if (!op || !a || !b) return 0;
  if (op->kind == ORC_OP_HELMHOLTZ3D_SL || op->kind == ORC_OP_HELMHOLTZ3D_DL || op->kind == ORC_OP_HELMHOLTZ3D_DLT ||
      op->kind == ORC_OP_HELMHOLTZ3D_HS)
    return a->refspace == ORC_REFSPACE_LAGRANGE_C0D1 && b->refspace == ORC_REFSPACE_LAGRANGE_C0D1;
  if (op->kind == ORC_OP_MAXWELL3D_SL || op->kind == ORC_OP_MAXWELL3D_DL)
    return a->refspace == ORC_REFSPACE_RT && b->refspace == ORC_REFSPACE_RT;
  return 0;
}

static int local_matrix(const orc_operator* op, const orc_space* test, const orc_space* trial,
                        const orc_quadstrat* qs, const tri_t* A, const tri_t* B, int force,
                        cpx L[3][3], int* cls_out) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) L[i][j] = mk(0.0, 0.0);
  int cls = force >= 0 ? force : classify_pair(A, B, op_k2(op));
  if (cls_out) *cls_out = cls;
  if (cls < 0) return -2;
  switch (cls) {
    case ORC_CLASS_FAR:
      return double_quadrature(op, A, test->refspace, B, trial->refspace, qs->far_test, qs->far_trial, L);
    case ORC_CLASS_NEAR:
      return near_extraction(op, A, test->refspace, B, trial->refspace, qs->near_test, qs->near_trial, L);
    case ORC_CLASS_CV:
      return sauter_schwab(op, cls, A, test->refspace, B, trial->refspace, qs->ss_cv, L);
    case ORC_CLASS_CE:
      return sauter_schwab(op, cls, A, test->refspace, B, trial->refspace, qs->ss_ce, L);
    case ORC_CLASS_CF:
      return sauter_schwab(op, cls, A, test->refspace, B, trial->refspace, qs->ss_cf, L);
  }
  return -2;
}

int orc_local_matrices(const orc_operator* op, const orc_space* test, const orc_space* trial,
                       const orc_quadstrat* qs, int64_t npairs, const int32_t* tau,
                       const int32_t* sigma, int32_t force_class, double* out, int8_t* cls) {
  if (!valid_op_space(op, test, trial) || !qs || npairs < 0 || (npairs && (!tau || !sigma || !out))) return -1;
  int err = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : err)
  for (int64_t p = 0; p < npairs; ++p) {
    if (tau[p] < 0 || tau[p] >= test->nt || sigma[p] < 0 || sigma[p] >= trial->nt) {
      err = 1;
      continue;
    }
    tri_t A, B;
    load_tri(test, tau[p], &A);
    load_tri(trial, sigma[p], &B);
    cpx L[3][3];
    int c = -1;
    if (local_matrix(op, test, trial, qs, &A, &B, force_class, L, &c)) err = 1;
    if (cls) cls[p] = (int8_t)c;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        out[p * 18 + (i * 3 + j) * 2 + 0] = L[i][j].re;
        out[p * 18 + (i * 3 + j) * 2 + 1] = L[i][j].im;
      }
  }
  return err ? -2 : 0;
}

int orc_assemble_rows(const orc_operator* op, const orc_space* test, const orc_space* trial,
                      const orc_quadstrat* qs, int64_t nrows, const int32_t* rows, double* out,
                      int32_t nthreads) {
  if (!valid_op_space(op, test, trial) || !qs || nrows < 0 || (nrows && (!rows || !out))) return -1;
  /* supports of every test function, ordered by triangle (the order BEAST's assemblydata
   * walks cells in) */
  int32_t nf = test->nfun;
  int64_t* off = (int64_t*)calloc((size_t)nf + 2, sizeof(int64_t));
  if (!off) return -3;
  for (int64_t t = 0; t < test->nt; ++t)
    for (int i = 0; i < 3; ++i) {
      int32_t f = test->fn_index[3 * t + i];
      if (f >= nf) { free(off); return -1; }
      if (f >= 0) off[f + 1]++;
    }
  for (int32_t f = 0; f < nf; ++f) off[f + 1] += off[f];
  int64_t nsup = off[nf];
  int32_t* st = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nsup ? nsup : 1));
  int32_t* si = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nsup ? nsup : 1));
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nf ? nf : 1));
  if (!st || !si || !fill) { free(off); free(st); free(si); free(fill); return -3; }
  for (int32_t f = 0; f < nf; ++f) fill[f] = off[f];
  for (int64_t t = 0; t < test->nt; ++t)
    for (int i = 0; i < 3; ++i) {
      int32_t f = test->fn_index[3 * t + i];
      if (f >= 0) { st[fill[f]] = (int32_t)t; si[fill[f]] = i; fill[f]++; }
    }
  int err = 0;
  int64_t nb = trial->nfun;
  if (nthreads <= 0) nthreads = orc_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(| : err)
  for (int64_t r = 0; r < nrows; ++r) {
    double* row = out + r * nb * 2;
    memset(row, 0, sizeof(double) * 2 * (size_t)nb);
    int32_t m = rows[r];
    if (m < 0 || m >= nf) { err = 1; continue; }
    for (int64_t a = off[m]; a < off[m + 1]; ++a) {
      int32_t tau = st[a], i = si[a];
      double ca = test->fn_coef[3 * (int64_t)tau + i];
      tri_t A, B;
      load_tri(test, tau, &A);
      for (int32_t s = 0; s < trial->nt; ++s) {
        load_tri(trial, s, &B);
        cpx L[3][3];
        if (local_matrix(op, test, trial, qs, &A, &B, -1, L, NULL)) { err = 1; continue; }
        for (int j = 0; j < 3; ++j) {
          int32_t n = trial->fn_index[3 * (int64_t)s + j];
          if (n < 0) continue;
          double cb = trial->fn_coef[3 * (int64_t)s + j];
          /* Z[m, n] += L[i][j] * c_m * c_n  (store_with_kernel.jl:88-97) */
          cpx v = cmulr(cmulr(L[i][j], ca), cb);
          row[2 * n] += v.re;
          row[2 * n + 1] += v.im;
        }
      }
    }
  }
  free(off); free(st); free(si); free(fill);
  return err ? -2 : 0;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
