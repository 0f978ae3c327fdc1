/*
 * FP64 CPU oracle for BEM Galerkin matrix assembly -- TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference's assembly algorithm (BEASTGPU on top of
 * BEAST 2.6.0 / SauterSchwabQuadrature 2.4.1 / CompScienceMeshes 0.9.3).  It exists to
 * check the CUDA library and to time the CPU baseline; nothing in the product path may
 * call it.  Every function cites the reference file:line it follows.
 *
 * Parity status: UNPINNED against BEAST itself.  The reference's only golden data
 * (cashed_results/matrix_ref_*.bin, read by test/correctness.jl:25-30) is git-ignored and
 * absent, and neither Julia nor BEAST is available, so the oracle is pinned instead by
 * self-consistency tests (symmetry, quadrature exactness, Sauter-Schwab convergence,
 * independent closed-form and high-order checks) kept under tests/.
 *
 * Conventions (shared with include/beastgb.h):
 *   vertices double[nv][3]; triangles int32[nt][3] in chart order (v1, v2, v3);
 *   fn_index int32[nt][3] (-1 = none), fn_coef double[nt][3];
 *   complex values are stored as (re, im) double pairs;
 *   Z[test function m][trial function n] += c_m * c_n * L[i][j]   (store_with_kernel.jl:88-97).
 */
#ifndef BEM_ORACLE_H
#define BEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_OP_HELMHOLTZ3D_SL = 0,
  ORC_OP_MAXWELL3D_SL = 1,
  ORC_OP_MAXWELL3D_DL = 2,
  ORC_OP_HELMHOLTZ3D_DL = 3,  /* alpha int int f(x) dG/dn_y g(y) */
  ORC_OP_HELMHOLTZ3D_DLT = 4, /* alpha int int f(x) dG/dn_x g(y) */
  ORC_OP_HELMHOLTZ3D_HS = 5   /* int int G [alpha (n_x.n_y) f g + beta curl f . curl g] */
};
enum { ORC_REFSPACE_LAGRANGE_C0D1 = 0, ORC_REFSPACE_RT = 1 };
enum { ORC_CLASS_FAR = 0, ORC_CLASS_CV = 1, ORC_CLASS_CE = 2, ORC_CLASS_CF = 3, ORC_CLASS_NEAR = 4 };

typedef struct {
  int32_t kind;
  double alpha[2]; /* complex */
  double beta[2];  /* complex, Maxwell single layer only */
  double gamma[2]; /* complex, gamma = i k for wavenumber k */
} orc_operator;

typedef struct {
  int32_t refspace;
  int32_t nv, nt, nfun;
  const double* vertices;
  const int32_t* triangles;
  const int32_t* fn_index;
  const double* fn_coef;
} orc_space;

typedef struct {
  int32_t far_test, far_trial;   /* points of the far double-quadrature rules */
  int32_t near_test, near_trial; /* points of the near-pair double-quadrature rules */
  int32_t ss_cf, ss_ce, ss_cv;   /* Gauss-Legendre points per dimension, Sauter-Schwab */
} orc_quadstrat;

/* Area (BEAST chart volume) of triangle t: |(v1-v3) x (v2-v3)| / 2. */
double orc_triangle_area(const orc_space* s, int32_t t);

/* Pair class 0..4 (far, CV, CE, CF, near) for a block of pairs, out[(t-t0)*(s1-s0)+(s-s0)]. */
int orc_classify_block(const orc_space* test, const orc_space* trial, double k2,
                       int32_t t0, int32_t t1, int32_t s0, int32_t s1, int8_t* out);

/* Local 3x3 complex matrices L[i][j] (test local i, trial local j) for a list of pairs.
 * force_class < 0 classifies each pair; otherwise that rule is used for all pairs.
 * out: double[npairs][9][2]; cls (optional): int8[npairs]. */
int orc_local_matrices(const orc_operator* op, const orc_space* test, const orc_space* trial,
                       const orc_quadstrat* qs, int64_t npairs, const int32_t* tau,
                       const int32_t* sigma, int32_t force_class, double* out, int8_t* cls);

/* Rows `rows[0..nrows)` of Z, out: double[nrows][trial->nfun][2], row-major.  nthreads <= 0:
 * use all OpenMP threads. */
int orc_assemble_rows(const orc_operator* op, const orc_space* test, const orc_space* trial,
                      const orc_quadstrat* qs, int64_t nrows, const int32_t* rows, double* out,
                      int32_t nthreads);

/* Gauss-Legendre rule on [0, 1] (n <= 64). */
int orc_gauss_legendre01(int32_t n, double* x, double* w);

/* Number of OpenMP threads available. */
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif

#endif
