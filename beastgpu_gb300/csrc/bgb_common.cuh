// Shared device/host definitions of libbeastgb (GB300, sm_103a).
//
// Layout of per-triangle data in HBM (built once per space by k_prepare_*):
//   Geo64   : FP64 vertices, tangents, area -- the classification, Sauter-Schwab, near-pair
//             and plain-FP64 far kernels read these (80 B + padding per triangle).
//   Rec32   : FP32 far-pair record for the mixed kernel: double-float centroid, bounding
//             radius, quadrature-point offsets from the centroid, weights, vertex offsets.
//   Rec64   : FP64 far-pair record for the plain kernel: absolute quadrature points,
//             weights, vertices.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/beastgb.h"

#define BGB_MAXQ 13        // largest triangle rule (points)
#define BGB_MAX_SS 16      // largest Gauss-Legendre order for Sauter-Schwab

namespace bgb {

// ----------------------------------------------------------------------------------------
// Complex helpers
// ----------------------------------------------------------------------------------------
__host__ __device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__host__ __device__ inline double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// ----------------------------------------------------------------------------------------
// Double-float ("ff") primitives: error-free transformations (Knuth two-sum, Dekker/FMA
// two-product).  Written with round-to-nearest intrinsics so the compiler cannot contract
// or reassociate them.
// ----------------------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// 2 pi split for Cody-Waite reduction (three float parts; the first two have trailing
// zero bits so products with small integers are exact).
#define BGB_2PI_A 6.28125f
#define BGB_2PI_B 1.9353071795864769e-3f
#define BGB_2PI_C (6.2831853071795864769 - 6.28125 - 1.9353071795864769e-3)
#define BGB_INV_2PI 0.15915494309189535f
#define BGB_INV_4PI_D (1.0 / (4.0 * 3.141592653589793))

// ----------------------------------------------------------------------------------------
// Per-triangle records
// ----------------------------------------------------------------------------------------
struct Geo64 {          // CompScienceMeshes simplex: tangents v_i - v_3, volume |t1 x t2|/2
  double v[3][3];       // v[vertex][coord]
  double t[2][3];
  double area;
  double pad;
};

// FP32 far-pair record (mixed kernel).  Q = points of the rule on this side.
template <int Q>
struct Rec32 {
  float ch[3], cl[3];   // centroid, double-float (hi + lo)
  float rad;            // bounding radius about the centroid (rounded up) + near threshold on the trial side
  float inv2a;          // 1 / (2 A)   (RT shape scale)
  float x[Q][3];        // quadrature points minus centroid
  float w[Q];           // weights incl. Jacobian (sum = A); trial side also carries 1/(4 pi)
  float vo[3][3];       // vertices minus centroid
};

// FP64 far-pair record (plain kernel).
template <int Q>
struct Rec64 {
  double x[Q][3];       // absolute quadrature points
  double w[Q];          // weights incl. Jacobian
  double v[3][3];       // vertices
  double inv2a;         // 1 / (2 A)
};

// Operator parameters as kernels see them.
struct OpParams {
  int kind;
  double alpha[2], beta[2], gamma[2];
  double k2;            // abs2(gamma), classification
};

// Triangle rule table in constant memory: u, v, w per point for the 7 rules.
struct RuleTable {
  int npoints[7];
  int offset[7];
  double uvw[46][3];
};

// Quadrature selection for a launch.
struct QuadSel {
  int far_t, far_b, near_t, near_b;   // rule indices into RuleTable
  int ss[4];                           // GL order per class code (1 CV, 2 CE, 3 CF)
  double gl_x[4][BGB_MAX_SS];          // nodes per class
  double gl_w[4][BGB_MAX_SS];
};

// ----------------------------------------------------------------------------------------
// Shape data at a point (FP64)
// ----------------------------------------------------------------------------------------
struct Shp64 {
  double x[3];
  double val[3];
  double vec[3][3];
  double div;
};

// Cartesian point and shape values at chart parameters (u, v); BEAST's RTRefSpace form for
// RT (value_i = (u t1 + v t2 - t_i) / j, divergence 2 / j with j = 2A), barycentric hats
// for Lagrange.
__device__ inline void shapes64(const Geo64& T, int refspace, double u, double v, Shp64& S) {
#pragma unroll
  for (int c = 0; c < 3; ++c) S.x[c] = __dadd_rn(__dadd_rn(T.v[2][c], __dmul_rn(T.t[0][c], u)), __dmul_rn(T.t[1][c], v));
  S.val[0] = u;
  S.val[1] = v;
  S.val[2] = 1.0 - u - v;
  if (refspace == BGB_REFSPACE_RT) {
    double j = T.area * 2.0;
    double inv_j = 1.0 / j;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double utu = u * T.t[0][c], vtv = v * T.t[1][c];
      S.vec[0][c] = ((utu - T.t[0][c]) + vtv) * inv_j;
      S.vec[1][c] = ((utu + vtv) - T.t[1][c]) * inv_j;
      S.vec[2][c] = (utu + vtv) * inv_j;
    }
    S.div = 2.0 * inv_j;
  }
}

// exp(-R gamma) as Julia's complex exp.
__device__ inline double2 expmg(double R, const OpParams& op) {
  double zr = -R * op.gamma[0], zi = -R * op.gamma[1];
  double er = (zr == 0.0) ? 1.0 : exp(zr);
  if (zi == 0.0) return make_double2(er, zi);
  double s, c;
  sincos(zi, &s, &c);
  return make_double2(er * c, er * s);
}

// Operator integrand at one point pair with weight `wgt` (quadrature weights and Jacobians),
// accumulated into L[i][j] (test local i, trial local j).  FP64.
__device__ inline void accumulate64(const OpParams& op, const Shp64& X, const Shp64& Y, double wgt,
                                    double2 L[3][3]) {
  double d0 = X.x[0] - Y.x[0], d1 = X.x[1] - Y.x[1], d2 = X.x[2] - Y.x[2];
  double R = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
  double2 e = expmg(R, op);
  double g = wgt * BGB_INV_4PI_D / R;
  double2 G = make_double2(g * e.x, g * e.y);
  double2 alpha = make_double2(op.alpha[0], op.alpha[1]);
  if (op.kind == BGB_OP_HELMHOLTZ3D_SL) {
    double2 aG = cmul(alpha, G);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) L[i][j] = cadd(L[i][j], cscale(aG, X.val[i] * Y.val[j]));
  } else if (op.kind == BGB_OP_MAXWELL3D_SL) {
    double2 a = cmul(alpha, G), b = cmul(make_double2(op.beta[0], op.beta[1]), G);
    double dd = X.div * Y.div;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        double fg = X.vec[i][0] * Y.vec[j][0] + X.vec[i][1] * Y.vec[j][1] + X.vec[i][2] * Y.vec[j][2];
        L[i][j] = cadd(L[i][j], cadd(cscale(a, fg), cscale(b, dd)));
      }
  } else {
    // grad_x G = -(gamma + 1/R) G r / R
    double2 Gr = make_double2(G.x / R, G.y / R);
    double2 H = cmul(make_double2(-op.gamma[0] - 1.0 / R, -op.gamma[1]), Gr);
    H = cmul(alpha, H);
    double r[3] = {d0, d1, d2};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double* f = X.vec[i];
        const double* q = Y.vec[j];
        double c0 = r[1] * q[2] - r[2] * q[1];
        double c1 = r[2] * q[0] - r[0] * q[2];
        double c2 = r[0] * q[1] - r[1] * q[0];
        double trip = f[0] * c0 + f[1] * c1 + f[2] * c2;
        L[i][j] = cadd(L[i][j], cscale(H, trip));
      }
  }
}

// FP32 bounding-sphere test shared by the classifier and the far-pair kernels (identical
// rounding in both): true if the pair may be non-far.
__device__ __forceinline__ bool sphere_candidate(float4 a, float4 b) {
  const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
  const float lim = __fadd_rn(a.w, b.w);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)) <= __fmul_rn(lim, lim);
}

}  // namespace bgb

// Host helpers shared between translation units (defined in bgb_api.cu).
namespace bgb {
void set_error(const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
}  // namespace bgb

#define BGB_CUDA(call)                                         \
  do {                                                         \
    cudaError_t _e = (call);                                   \
    if (_e != cudaSuccess) return ::bgb::cuda_fail(_e, #call); \
  } while (0)
