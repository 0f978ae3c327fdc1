/*
 * FP64 CPU oracle for the 2-D (curve) Galerkin matrix fill -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference's 2-D Helmholtz prototype
 * (old_code/doubleQuadRule_2d_gpu.jl: kernel G = -(i/4) H0^(2)(kR) at :72-78, the
 * hypersingular integrand (f' g' - k^2 (n_x.n_y) f g) G at :88-97 and :162-180, the double
 * quadrature over outer (test) and inner (trial) points at :129-210 and :265-465), widened to
 * the operators of BEAST's Helmholtz2D (single layer, double layer, its transpose,
 * hypersingular) and to whole matrices.  It exists to check the CUDA library and is never
 * called by the product path.
 *
 * Differences from the prototype, on purpose: the Hankel functions are libm's Bessel
 * functions j0, y0, j1, y1 (the prototype's truncated power series, :31-64, are accurate only
 * for small kR); pairs of segments that share vertices are integrated with singular rules
 * instead of the plain double quadrature.
 *
 * Parity status: UNPINNED against BEAST itself (neither Julia nor BEAST is available, and the
 * reference holds no 2-D fixtures).  The oracle is pinned by tests/: Green functions against
 * scipy, local matrices against mpmath quadrature to ~1e-14 (tests/golden), exact identities.
 *
 * Conventions:
 *   vertices double[nv][2]; segments int32[ns][2] = (v0, v1), chart x(s) = (1-s) v0 + s v1,
 *   s in [0, 1]; length l = |v1 - v0|; normal n = (d_y, -d_x) / l with d = v1 - v0 (outward
 *   on a counter-clockwise closed curve);
 *   local shapes: LAGRANGE_C0D1: f_0 = 1 - s, f_1 = s with arc-length derivatives -1/l, +1/l;
 *                 LAGRANGE_CXD0: f_0 = 1, derivative 0 (column 1 of the tables is ignored);
 *   fn_index int32[ns][2] (-1 = none), fn_coef double[ns][2];
 *   Z[m][n] += c_m c_n L[i][j]; complex numbers are (re, im) double pairs.
 *
 * Kernel: G(R) = -(i/4) H0^(2)(kR) for k > 0, -(1/2 pi) ln R for k = 0, and
 * grad_x G = (x - y) g1(R) with g1 = (i k / 4) H1^(2)(kR) / R, resp. -1 / (2 pi R^2).
 *   SL : alpha int int G f g
 *   DL : alpha int int f (n_y . grad_y G) g
 *   DLT: alpha int int f (n_x . grad_x G) g
 *   HS : int int G [alpha (n_x . n_y) f g + beta f' g']   (the prototype: alpha = -k^2, beta = 1)
 *
 * Pair classes (the generic predicate of doubleQuadRuleMainCase.jl:187-200 over the two
 * vertices of each segment, with the trial segment's chart volume, its length, in place of
 * the triangle area): 3 coincident (two vertex pairs closer than 1e3 eps), 1 common vertex,
 * 4 near (max(dmin^2 k^2, dmin^2 / (16 l_sigma)) < 0.2^2, dmin the least vertex distance),
 * 0 far.
 *
 * Rules: far pairs Gauss-Legendre far_test x far_trial points; near pairs near x near on the
 * leaves of a bisection of the chart square (the longer piece is halved until each piece pair
 * is at least as far apart as its longer piece is long, at most 16 times, depth first);
 * coincident and common-vertex pairs the graded rules of orc2_graded01 (order `singular`)
 * after splitting the square of chart parameters along its diagonal:
 *   coincident (u, v in the test chart, singular on u = v): u = z + (1-z) w, v = (1-z) w and
 *   the mirror, weight (1 - z);  common vertex (xi, eta from the shared vertex, singular at
 *   the corner): xi = z, eta = z w and the mirror, weight z;  z graded, w Gauss-Legendre.
 *   The coincident rule grades z over 3n levels (orc2_graded01); the common-vertex rule, whose
 *   integrand carries the Jacobian z (z ln z), over 3n/2 levels (integer division).
 * Double layers vanish on coincident (straight) segments.
 */
#ifndef BEM2D_ORACLE_H
#define BEM2D_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC2_OP_SL = 0, ORC2_OP_DL = 1, ORC2_OP_DLT = 2, ORC2_OP_HS = 3 };
enum { ORC2_REFSPACE_LAGRANGE_C0D1 = 0, ORC2_REFSPACE_LAGRANGE_CXD0 = 1 };
enum { ORC2_CLASS_FAR = 0, ORC2_CLASS_CV = 1, ORC2_CLASS_CF = 3, ORC2_CLASS_NEAR = 4 };

typedef struct {
  int32_t kind;
  double wavenumber; /* k >= 0 */
  double alpha[2];
  double beta[2];    /* hypersingular only */
} orc2_operator;

typedef struct {
  int32_t refspace;
  int32_t nv, ns, nfun;
  const double* vertices;
  const int32_t* segments;
  const int32_t* fn_index;
  const double* fn_coef;
} orc2_space;

typedef struct {
  int32_t far_test, far_trial; /* Gauss-Legendre points per segment, far pairs (1..32) */
  int32_t near;                /* Gauss-Legendre points per segment, near pairs (1..32) */
  int32_t singular;            /* order n of the graded rules (1..16) */
} orc2_quadstrat;

/* G(R) and g1(R) as (re, im) pairs: out[0..1] = G, out[2..3] = g1.  R > 0, k >= 0. */
int orc2_green(double k, double R, double* out);

/* The graded rule on [0, 1] towards 0: 3n + 1 intervals [0, q^(3n)], [q^(3n), q^(3n-1)], ...,
 * [q, 1] (q = 0.35) with n Gauss-Legendre points each, ascending; (3n + 1) n points.  It
 * integrates ln z to about 1e-13 at n = 10 and 1e-15 at n = 12. */
int orc2_graded01(int32_t n, double* x, double* w);

/* Pair classes for a block of segment pairs, out[(t - t0) * (s1 - s0) + (s - s0)]. */
int orc2_classify_block(const orc2_space* test, const orc2_space* trial, double k2, int32_t t0,
                        int32_t t1, int32_t s0, int32_t s1, int8_t* out);

/* Local 2x2 complex matrices L[i][j] of a list of segment pairs, out double[npairs][2][2][2]
 * (entries of missing shapes are zero); force_class >= 0 uses that rule for every pair. */
int orc2_local_matrices(const orc2_operator* op, const orc2_space* test, const orc2_space* trial,
                        const orc2_quadstrat* qs, int64_t npairs, const int32_t* tau,
                        const int32_t* sigma, int32_t force_class, double* out, int8_t* cls);

/* Rows rows[0..nrows) of Z, out double[nrows][trial->nfun][2]; nthreads <= 0: all threads. */
int orc2_assemble_rows(const orc2_operator* op, const orc2_space* test, const orc2_space* trial,
                       const orc2_quadstrat* qs, int64_t nrows, const int32_t* rows, double* out,
                       int32_t nthreads);

#ifdef __cplusplus
}
#endif

#endif
