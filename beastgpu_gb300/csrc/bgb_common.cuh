// Shared device/host definitions of libbeastgb (GB300, sm_103a).
//
// Layout of per-triangle data in HBM (built once per space by k_prepare_*):
//   Geo64   : FP64 vertices, tangents, area -- the classification, Sauter-Schwab, near-pair
//             and plain-FP64 far kernels read these (80 B + padding per triangle).
//   far records (layouts Off32 / Off64 in bgb_far_impl.cuh): FP32 record of the mixed kernel
//             (double-float centroid, radius, 1/(2A), point offsets from the centroid,
//             weights, vertex offsets) and FP64 record of the plain kernel.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/beastgb.h"

#define BGB_MAXQ 13        // largest triangle rule (points)
#define BGB_MAX_SS 16      // largest Gauss-Legendre order for Sauter-Schwab
#define BGB_TAYLOR_MAX 16  // series terms of the plain FP64 far kernel's point-pair phase

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
