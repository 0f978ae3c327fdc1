// Curve (2-D) path of libbeastgb: BEAST Helmholtz2D operators on polygonal curves.
//
//   upload curves -> k_curve_geo -> per block of output columns:
//     k_curve_classify (FP32 prefilter + exact FP64 predicate; non-far pairs into a list and a
//     bit mask) -> far pairs: k_curve_far (FP64, CUDA's Bessel functions) or k_curve_far_mixed
//     (FP32 Hankel approximations, double-float phase), one thread per pair -> coincident,
//     common-vertex and near pairs: k_curve_special (FP64) or k_curve_special_df (double-float
//     singular rules), one warp per pair -> k_curve_gather (one thread per matrix entry,
//     supports in a fixed order, no atomics)
//
// The reference's 2-D prototype (old_code/doubleQuadRule_2d_gpu.jl:129-210, :265-465) integrates
// one segment pair per host call, with one GPU thread per point pair and a reduction into the
// 2x2 result, and its Hankel functions are truncated power series (:31-64) that hold only for
// small kR.  Here one launch integrates every pair of a block of columns.
#include "bgb_host.h"
#include "besselfit.h"
#include "bgb_df.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

namespace bgb {
namespace curve {

struct SegGeo {
  double x0, y0, x1, y1;  // vertices v0, v1
  double dx, dy;          // v1 - v0
  double len, nx, ny;     // length and unit normal (dy, -dx) / len
  double cx, cy;          // midpoint
};

constexpr int kMaxGL = 32;
constexpr int kMaxSing = 16;
constexpr int kMaxGraded = (3 * kMaxSing + 1) * kMaxSing;
constexpr int kMaxGradedCv = ((3 * kMaxSing) / 2 + 1) * kMaxSing;
constexpr int kMaxDepth = 16;  // bisections of a near pair
constexpr double kInv2Pi = 0.15915494309189535;

constexpr int kSeries = 17;  // highest power of u = x^2/4 in the Bessel series (enough for x <= 4)

// Point rules of one call (copied to shared memory by the kernels that use them).
struct Rules {
  int nft, nfb, nnear, nsing, ngraded, pad;
  double ft_x[kMaxGL], ft_w[kMaxGL], fb_x[kMaxGL], fb_w[kMaxGL], nr_x[kMaxGL], nr_w[kMaxGL];
  double sg_x[kMaxSing], sg_w[kMaxSing];  // Gauss-Legendre, smooth direction of the singular rules
  double gz[kMaxGraded], gwz[kMaxGraded];  // graded rule towards 0 (coincident pairs: 3n levels)
  double lnz[kMaxGraded];                  // ln of the graded nodes
  int ngraded_cv, pad2;                    // common-vertex pairs (integrand ~ z ln z): 3n/2 levels
  double gz_cv[kMaxGradedCv], gwz_cv[kMaxGradedCv], lnz_cv[kMaxGradedCv];
  double gl2_x[2], gl2_w[2];               // 2-point Gauss-Legendre (coincident pairs, across the diagonal)
  // Power series in u = x^2/4 (Abramowitz & Stegun 9.1.10-9.1.13):
  //   J0 = sum sa_m u^m,  Y0 = (2/pi) [(ln(x/2) + gamma) J0 + u sum sb_m u^m],
  //   J1 = (x/2) sum sc_m u^m,  Y1 = (2/pi) ln(x/2) J1 - 2/(pi x) - (x/(2 pi)) sum sd_m u^m.
  double sa[kSeries + 1], sb[kSeries], sc[kSeries + 1], sd[kSeries + 1];
};

// The singular rules and series of Rules as double-floats, for the mixed path's singular kernel:
// weights pre-multiplied by the collapse Jacobians ((1 - z) coincident, z common vertex).
struct RulesDF {
  int n, nz, nzcv, pad;
  dfl gz[kMaxGraded], wcf[kMaxGraded], lnz[kMaxGraded];
  dfl gzc[kMaxGradedCv], wcv[kMaxGradedCv], lnzc[kMaxGradedCv];
  dfl sgx[kMaxSing], sgw[kMaxSing], gl2x[2], gl2w[2];
  dfl sa[kSeries + 1], sb[kSeries];
  dfl inv2pi, two_over_pi;
};

struct Op {
  int kind, nsA, nsB, LS;  // LS = nsA * nsB entries per local matrix
  double k, k2;
  double ar, ai, br, bi;
  float khi, klo;          // k as a double-float
  double lnk2;             // ln(k / 2), k > 0
  float far_, fai, fbr, fbi;
};

// FP32 copy of a segment for the mixed kernels: midpoint as double-float, direction, normal, length.
struct SegF {
  float cxh, cxl, cyh, cyl;
  float dx, dy, nx, ny;
  float len, pad0, pad1, pad2;
};

template <class LT>
__device__ __forceinline__ void store_l(LT* p, double re, double im);
template <>
__device__ __forceinline__ void store_l<double2>(double2* p, double re, double im) { *p = make_double2(re, im); }
template <>
__device__ __forceinline__ void store_l<float2>(float2* p, double re, double im) { *p = make_float2((float)re, (float)im); }

// A non-far pair: its local matrix goes to L[slot .. slot + LS).
struct Special {
  int64_t slot;
  int tau, sigma;
  int cls, match;  // match = 2 * (local vertex of tau) + (local vertex of sigma) of the first shared vertex
};

struct Acc {
  double pr[4], pi[4];  // sum of kernel x weight x f_i g_j, index 2 i + j
  double mr, mi;        // hypersingular: sum of G x weight
};

// ----------------------------------------------------------------------------------------
// Device functions
// ----------------------------------------------------------------------------------------
__global__ void k_curve_geo(const double* __restrict__ v, const int* __restrict__ seg, int ns, SegGeo* __restrict__ out,
                            SegF* __restrict__ outf) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ns) return;
  const int a = seg[2 * e], b = seg[2 * e + 1];
  SegGeo g;
  g.x0 = v[2 * a];
  g.y0 = v[2 * a + 1];
  g.x1 = v[2 * b];
  g.y1 = v[2 * b + 1];
  g.dx = __dsub_rn(g.x1, g.x0);
  g.dy = __dsub_rn(g.y1, g.y0);
  g.len = __dsqrt_rn(__dadd_rn(__dmul_rn(g.dx, g.dx), __dmul_rn(g.dy, g.dy)));
  g.nx = __ddiv_rn(g.dy, g.len);
  g.ny = __ddiv_rn(-g.dx, g.len);
  g.cx = __dadd_rn(g.x0, __dmul_rn(0.5, g.dx));
  g.cy = __dadd_rn(g.y0, __dmul_rn(0.5, g.dy));
  out[e] = g;
  SegF f;
  f.cxh = (float)g.cx;
  f.cxl = (float)(g.cx - (double)f.cxh);
  f.cyh = (float)g.cy;
  f.cyl = (float)(g.cy - (double)f.cyh);
  f.dx = (float)g.dx;
  f.dy = (float)g.dy;
  f.nx = (float)g.nx;
  f.ny = (float)g.ny;
  f.len = (float)g.len;
  f.pad0 = f.pad1 = f.pad2 = 0.f;
  outf[e] = f;
}

// Pair class with BEAST's predicate over the segments' vertices (doubleQuadRuleMainCase.jl:187-200,
// quadrule_determine.jl:1-3), the trial length standing for the chart volume; every operation
// rounded as written (no contraction), as the oracle is compiled.  -1: degenerate pair.
__device__ __forceinline__ int classify(const SegGeo& a, const SegGeo& b, double k2, int* match) {
  const double dtol = 2.220446049250313e-16 * 1.0e3;
  const double xtol2 = 0.2 * 0.2;
  const double ax[2] = {a.x0, a.x1}, ay[2] = {a.y0, a.y1};
  const double bx[2] = {b.x0, b.x1}, by[2] = {b.y0, b.y1};
  int hits = 0;
  double dmin2 = 1.7976931348623157e308;
  *match = -1;
#pragma unroll
  for (int u1 = 0; u1 < 2; ++u1)
#pragma unroll
    for (int u2 = 0; u2 < 2; ++u2) {
      const double dx = __dsub_rn(ax[u1], bx[u2]), dy = __dsub_rn(ay[u1], by[u2]);
      const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
      if (__dsqrt_rn(d2) < dtol) {
        if (hits == 0) *match = 2 * u1 + u2;
        ++hits;
      }
      dmin2 = fmin(dmin2, d2);
    }
  if (hits > 2) return -1;
  if (hits == 2) return 3;
  if (hits == 1) return 1;
  const double m = fmax(__dmul_rn(dmin2, k2), __ddiv_rn(dmin2, __dmul_rn(16.0, b.len)));
  return m >= xtol2 ? 0 : 4;
}

// True only for pairs the exact predicate classifies far: a lower bound of the least vertex
// distance (midpoint distance minus the half lengths, less a bound of its FP32 rounding) already
// passes the far thresholds with a margin of 0.25%.  All FP32: the midpoints are double-float
// (SegF), so their difference is accurate to a few units of FP32 rounding of the distance.
// Pairs it does not settle go to classify().
__device__ __forceinline__ bool certainly_far(const SegF& A, const SegF& B, float k2f) {
  const float dx = (A.cxh - B.cxh) + (A.cxl - B.cxl), dy = (A.cyh - B.cyh) + (A.cyl - B.cyl);
  const float dc = sqrtf(fmaf(dx, dx, dy * dy));
  const float hs = 0.5f * (A.len + B.len);
  const float dlb = (dc - hs) - 4e-7f * (dc + hs);
  if (!(dlb > 1e-12f)) return false;
  const float d2 = dlb * dlb;
  return d2 * k2f >= 0.0401f || d2 >= 0.0401f * 16.f * B.len;
}

// Non-far mask: bit (sl * nT + tl) set for pairs the far kernels skip.
__device__ __forceinline__ bool nonfar_bit(const unsigned* __restrict__ mask, int64_t idx) {
  return (mask[idx >> 5] >> (idx & 31)) & 1u;
}

template <int OP>
__device__ __forceinline__ void accumulate(const Op& op, const SegGeo& A, const SegGeo& B, double s, double t,
                                           double Kr, double Ki, double w, Acc& c);

// One point pair: chart parameters s (test) and t (trial), separation r = x - y, rule weight w.
template <int OP>
__device__ __forceinline__ void add_point(const Op& op, const SegGeo& A, const SegGeo& B, double s, double t,
                                          double rx, double ry, double w, Acc& c) {
  const double R = sqrt(rx * rx + ry * ry);
  double Kr, Ki;
  if (OP == BGB_OP2D_SL || OP == BGB_OP2D_HS) {
    if (op.k == 0.0) {
      Kr = -log(R) * kInv2Pi;
      Ki = 0.0;
    } else {
      const double z = op.k * R;
      Kr = -0.25 * y0(z);
      Ki = -0.25 * j0(z);
    }
  } else {
    double gr, gi;
    if (op.k == 0.0) {
      gr = -kInv2Pi / (R * R);
      gi = 0.0;
    } else {
      const double z = op.k * R, f = op.k / (4.0 * R);
      gr = f * y1(z);
      gi = f * j1(z);
    }
    const double proj = OP == BGB_OP2D_DL ? -(rx * B.nx + ry * B.ny) : rx * A.nx + ry * A.ny;
    Kr = gr * proj;
    Ki = gi * proj;
  }
  accumulate<OP>(op, A, B, s, t, Kr, Ki, w, c);
}

// Adds kernel value K (times the rule weight and the lengths) times the shape products.
template <int OP>
__device__ __forceinline__ void accumulate(const Op& op, const SegGeo& A, const SegGeo& B, double s, double t,
                                           double Kr, double Ki, double w, Acc& c) {
  const double ww = w * A.len * B.len;
  Kr *= ww;
  Ki *= ww;
  const double f[2] = {op.nsA == 1 ? 1.0 : 1.0 - s, s};
  const double g[2] = {op.nsB == 1 ? 1.0 : 1.0 - t, t};
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const double fg = f[i] * g[j];
      c.pr[2 * i + j] += Kr * fg;
      c.pi[2 * i + j] += Ki * fg;
    }
  if (OP == BGB_OP2D_HS) {
    c.mr += Kr;
    c.mi += Ki;
  }
}

template <int OP, class LT>
__device__ __forceinline__ void finalize(const Op& op, const SegGeo& A, const SegGeo& B, const Acc& c,
                                         LT* __restrict__ out) {
  const double nn = A.nx * B.nx + A.ny * B.ny;
  const double dA[2] = {op.nsA == 2 ? -1.0 / A.len : 0.0, op.nsA == 2 ? 1.0 / A.len : 0.0};
  const double dB[2] = {op.nsB == 2 ? -1.0 / B.len : 0.0, op.nsB == 2 ? 1.0 / B.len : 0.0};
  const double bmr = op.br * c.mr - op.bi * c.mi, bmi = op.br * c.mi + op.bi * c.mr;
  for (int i = 0; i < op.nsA; ++i)
    for (int j = 0; j < op.nsB; ++j) {
      const double pr = c.pr[2 * i + j], pi = c.pi[2 * i + j];
      double lr = op.ar * pr - op.ai * pi, li = op.ar * pi + op.ai * pr;
      if (OP == BGB_OP2D_HS) {
        const double d = dA[i] * dB[j];
        lr = lr * nn + bmr * d;
        li = li * nn + bmi * d;
      }
      store_l(out + i * op.nsB + j, lr, li);
    }
}

__device__ __forceinline__ void acc_zero(Acc& c) {
#pragma unroll
  for (int k = 0; k < 4; ++k) c.pr[k] = c.pi[k] = 0.0;
  c.mr = c.mi = 0.0;
}

// Far pair: Gauss-Legendre product rule, one thread (doubleQuadRule_2d_gpu.jl:142-181).
template <int OP>
__device__ __forceinline__ void far_pair(const Op& op, const double* fx, const double* fw, int nft, const double* bx,
                                         const double* bw, int nfb, const SegGeo& A, const SegGeo& B, Acc& c) {
  for (int p = 0; p < nft; ++p) {
    const double s = fx[p];
    const double x0 = A.x0 + s * A.dx, x1 = A.y0 + s * A.dy;
    for (int q = 0; q < nfb; ++q) {
      const double t = bx[q];
      const double y0v = B.x0 + t * B.dx, y1v = B.y0 + t * B.dy;
      add_point<OP>(op, A, B, s, t, x0 - y0v, x1 - y1v, fw[p] * bw[q], c);
    }
  }
}

__device__ __forceinline__ double point_seg_dist2(double px, double py, double ax, double ay, double bx, double by) {
  const double dx = __dsub_rn(bx, ax), dy = __dsub_rn(by, ay);
  const double L2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  double t = L2 > 0.0 ? __ddiv_rn(__dadd_rn(__dmul_rn(__dsub_rn(px, ax), dx), __dmul_rn(__dsub_rn(py, ay), dy)), L2) : 0.0;
  t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
  const double ex = __dsub_rn(__dadd_rn(ax, __dmul_rn(t, dx)), px), ey = __dsub_rn(__dadd_rn(ay, __dmul_rn(t, dy)), py);
  return __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey));
}

constexpr double kTwoOverPi = 0.6366197723675814, kEulerGamma = 0.5772156649015329;

// The kernel at distance R with ln R given, for the singular and near rules: power series of
// J0, Y0 (J1, Y1) up to u^M for x = k R <= 4, CUDA's Bessel functions beyond; the static kernel
// for k = 0.  The logarithm comes from the caller (for the graded rules it is a sum of tabulated
// logarithms), so most points need no transcendental function.
template <int OP>
__device__ __forceinline__ void kernel_series(const Op& op, const Rules& Rl, double R, double lnR, int M, double rx,
                                              double ry, const SegGeo& A, const SegGeo& B, double& Kr, double& Ki) {
  if (OP == BGB_OP2D_SL || OP == BGB_OP2D_HS) {
    if (op.k == 0.0) {
      Kr = -kInv2Pi * lnR;
      Ki = 0.0;
      return;
    }
    const double x = op.k * R;
    if (x <= 4.0) {
      const double u = 0.25 * x * x;
      double j0 = Rl.sa[M];
      for (int m = M - 1; m >= 0; --m) j0 = fma(j0, u, Rl.sa[m]);
      double s0 = Rl.sb[M - 1];
      for (int m = M - 2; m >= 0; --m) s0 = fma(s0, u, Rl.sb[m]);
      const double y0v = kTwoOverPi * fma(lnR + op.lnk2 + kEulerGamma, j0, s0 * u);
      Kr = -0.25 * y0v;
      Ki = -0.25 * j0;
    } else {
      Kr = -0.25 * y0(x);
      Ki = -0.25 * j0(x);
    }
    return;
  }
  double gr, gi;
  if (op.k == 0.0) {
    gr = -kInv2Pi / (R * R);
    gi = 0.0;
  } else {
    const double x = op.k * R;
    double j1v, y1v;
    if (x <= 4.0) {
      const double u = 0.25 * x * x;
      double c1 = Rl.sc[M], d1 = Rl.sd[M];
      for (int m = M - 1; m >= 0; --m) {
        c1 = fma(c1, u, Rl.sc[m]);
        d1 = fma(d1, u, Rl.sd[m]);
      }
      j1v = 0.5 * x * c1;
      y1v = kTwoOverPi * (lnR + op.lnk2) * j1v - kTwoOverPi / x - x * kInv2Pi * d1;
    } else {
      j1v = j1(x);
      y1v = y1(x);
    }
    const double f = op.k / (4.0 * R);
    gr = f * y1v;
    gi = f * j1v;
  }
  const double proj = OP == BGB_OP2D_DL ? -(rx * B.nx + ry * B.ny) : rx * A.nx + ry * A.ny;
  Kr = gr * proj;
  Ki = gi * proj;
}

// Series order for a pair whose points are at most Rmax apart: the smallest M with
// u^M / (M!)^2 < 1e-18 at u = (k Rmax / 2)^2 (all of kSeries when k Rmax > 4).
__device__ __forceinline__ int series_order(double k, double Rmax) {
  const double u = 0.25 * (k * Rmax) * (k * Rmax);
  if (u >= 4.0) return kSeries;
  double term = 1.0;
  int M = 1;
  for (; M < kSeries; ++M) {
    term *= u / ((double)M * M);
    if (term < 1e-18) break;
  }
  return M;
}

__device__ __forceinline__ double max_vertex_distance(const SegGeo& A, const SegGeo& B) {
  const double ax[2] = {A.x0, A.x1}, ay[2] = {A.y0, A.y1}, bx[2] = {B.x0, B.x1}, by[2] = {B.y0, B.y1};
  double m = 0.0;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) m = fmax(m, (ax[i] - bx[j]) * (ax[i] - bx[j]) + (ay[i] - by[j]) * (ay[i] - by[j]));
  return sqrt(m);
}

// Warp-cooperative rules: every lane runs the same control flow and integrates the points
// k = lane, lane + 32, ... of each rule; the partial sums are reduced by the caller.
template <int OP>
__device__ void near_rule_warp(const Op& op, const Rules& R, const SegGeo& A, const SegGeo& B, int lane, Acc& c) {
  struct Box {
    double s0, s1, t0, t1;
    int depth;
  };
  Box stack[2 * kMaxDepth + 4];
  int top = 0;
  stack[top++] = Box{0.0, 1.0, 0.0, 1.0, 0};
  const int n = R.nnear;
  const int M = series_order(op.k, max_vertex_distance(A, B));
  while (top > 0) {
    const Box b = stack[--top];
    const double p0x = __dadd_rn(A.x0, __dmul_rn(b.s0, A.dx)), p0y = __dadd_rn(A.y0, __dmul_rn(b.s0, A.dy));
    const double p1x = __dadd_rn(A.x0, __dmul_rn(b.s1, A.dx)), p1y = __dadd_rn(A.y0, __dmul_rn(b.s1, A.dy));
    const double q0x = __dadd_rn(B.x0, __dmul_rn(b.t0, B.dx)), q0y = __dadd_rn(B.y0, __dmul_rn(b.t0, B.dy));
    const double q1x = __dadd_rn(B.x0, __dmul_rn(b.t1, B.dx)), q1y = __dadd_rn(B.y0, __dmul_rn(b.t1, B.dy));
    const double la = __dmul_rn(__dsub_rn(b.s1, b.s0), A.len), lb = __dmul_rn(__dsub_rn(b.t1, b.t0), B.len);
    double d2 = point_seg_dist2(p0x, p0y, q0x, q0y, q1x, q1y);
    d2 = fmin(d2, point_seg_dist2(p1x, p1y, q0x, q0y, q1x, q1y));
    d2 = fmin(d2, point_seg_dist2(q0x, q0y, p0x, p0y, p1x, p1y));
    d2 = fmin(d2, point_seg_dist2(q1x, q1y, p0x, p0y, p1x, p1y));
    if (b.depth < kMaxDepth && __dsqrt_rn(d2) < fmax(la, lb)) {
      if (la >= lb) {
        const double sm = 0.5 * (b.s0 + b.s1);
        stack[top++] = Box{sm, b.s1, b.t0, b.t1, b.depth + 1};
        stack[top++] = Box{b.s0, sm, b.t0, b.t1, b.depth + 1};
      } else {
        const double tm = 0.5 * (b.t0 + b.t1);
        stack[top++] = Box{b.s0, b.s1, tm, b.t1, b.depth + 1};
        stack[top++] = Box{b.s0, b.s1, b.t0, tm, b.depth + 1};
      }
      continue;
    }
    const double hs = b.s1 - b.s0, ht = b.t1 - b.t0;
    for (int k = lane; k < n * n; k += 32) {
      const int p = k / n, q = k - p * n;
      const double s = b.s0 + hs * R.nr_x[p], t = b.t0 + ht * R.nr_x[q];
      const double rx = (A.x0 + s * A.dx) - (B.x0 + t * B.dx), ry = (A.y0 + s * A.dy) - (B.y0 + t * B.dy);
      const double Rd = sqrt(rx * rx + ry * ry);
      double Kr, Ki;
      kernel_series<OP>(op, R, Rd, log(Rd), M, rx, ry, A, B, Kr, Ki);
      accumulate<OP>(op, A, B, s, t, Kr, Ki, (hs * R.nr_w[p]) * (ht * R.nr_w[q]), c);
    }
  }
}

// Coincident (match 0: same orientation, 1: reversed) and common-vertex rules: the chart square
// split along its diagonal, graded coordinate z towards the singularity, Gauss coordinate w.
template <int OP>
__device__ void singular_rule_warp(const Op& op, const Rules& R, const SegGeo& A, const SegGeo& B, int cls,
                                   int match, int lane, double* __restrict__ wtab, Acc& c) {
  const int n = R.nsing, nz = R.ngraded;
  const int M = series_order(op.k, max_vertex_distance(A, B));
  if (cls == 3) {
    if (OP == BGB_OP2D_DL || OP == BGB_OP2D_DLT) return;  // r lies along the segment
    const bool same = match == 0;
    const double lnl = log(A.len);  // R = z l
    // R depends on z only: across the diagonal the integrand is the product of two shapes linear
    // in w, which the 2-point Gauss rule integrates exactly
    const int ch = nz * 2;
    for (int k = lane; k < 2 * ch; k += 32) {
      const int half = k >= ch;
      const int rem = k - half * ch, a = rem >> 1, b = rem & 1;
      const double z = R.gz[a], w = R.gl2_x[b];
      double u, v, uv;
      if (!half) { u = z + (1.0 - z) * w; v = (1.0 - z) * w; uv = z; }
      else { u = (1.0 - z) * w; v = z + (1.0 - z) * w; uv = -z; }
      const double wt = R.gwz[a] * R.gl2_w[b] * (1.0 - z);
      double Kr, Ki;
      kernel_series<OP>(op, R, z * A.len, R.lnz[a] + lnl, M, uv * A.dx, uv * A.dy, A, B, Kr, Ki);
      accumulate<OP>(op, A, B, u, same ? v : 1.0 - v, Kr, Ki, wt, c);
    }
    return;
  }
  const int ma = match >> 1, mb = match & 1;
  const double ax = ma == 0 ? A.dx : -A.dx, ay = ma == 0 ? A.dy : -A.dy;
  const double bx = mb == 0 ? B.dx : -B.dx, by = mb == 0 ? B.dy : -B.dy;
  // R = z |a - w b| (first half) or z |w a - b| (second half): the lengths and their logarithms per
  // Gauss node w, one lane each, in this warp's table
  if (lane < n) {
    const double w = R.sg_x[lane];
    const double l0 = sqrt((ax - w * bx) * (ax - w * bx) + (ay - w * by) * (ay - w * by));
    const double l1 = sqrt((w * ax - bx) * (w * ax - bx) + (w * ay - by) * (w * ay - by));
    wtab[lane] = l0;
    wtab[kMaxSing + lane] = log(l0);
    wtab[2 * kMaxSing + lane] = l1;
    wtab[3 * kMaxSing + lane] = log(l1);
  }
  __syncwarp();
  const int per_half_cv = R.ngraded_cv * n;  // ngraded_cv z nodes times n Gauss nodes
  for (int k = lane; k < 2 * per_half_cv; k += 32) {
    const int half = k >= per_half_cv;
    const int rem = k - half * per_half_cv, a = rem / n, b = rem - a * n;
    const double z = R.gz_cv[a], w = R.sg_x[b];
    double xi, eta;
    if (!half) { xi = z; eta = z * w; }
    else { xi = z * w; eta = z; }
    const double wt = R.gwz_cv[a] * R.sg_w[b] * z;
    const double* tb = wtab + 2 * kMaxSing * half;
    double Kr, Ki;
    kernel_series<OP>(op, R, z * tb[b], R.lnz_cv[a] + tb[kMaxSing + b], M, xi * ax - eta * bx, xi * ay - eta * by, A,
                      B, Kr, Ki);
    accumulate<OP>(op, A, B, ma == 0 ? xi : 1.0 - xi, mb == 0 ? eta : 1.0 - eta, Kr, Ki, wt, c);
  }
  __syncwarp();
}

// ---- Mixed precision: FP32 point pairs, the phase k R carried in FP64 per pair --------------
// Polynomial approximations of H0^(2) and H1^(2) (besselfit.h: the forms of Abramowitz & Stegun
// 9.4.1-9.4.6, coefficients fitted against scipy.special to 5e-9): x < 3 power series in
// u = (x/3)^2 with the logarithmic part of Y explicit; x >= 3 modulus / phase in t = 3/x.
__constant__ float c_P0[BGB_BESSEL_P0_N] = BGB_BESSEL_P0;
__constant__ float c_Q0[BGB_BESSEL_Q0_N] = BGB_BESSEL_Q0;
__constant__ float c_P1[BGB_BESSEL_P1_N] = BGB_BESSEL_P1;
__constant__ float c_Q1[BGB_BESSEL_Q1_N] = BGB_BESSEL_Q1;
__constant__ float c_F0[BGB_BESSEL_F0_N] = BGB_BESSEL_F0;
__constant__ float c_G0[BGB_BESSEL_G0_N] = BGB_BESSEL_G0;
__constant__ float c_F1[BGB_BESSEL_F1_N] = BGB_BESSEL_F1;
__constant__ float c_G1[BGB_BESSEL_G1_N] = BGB_BESSEL_G1;

template <int N>
__device__ __forceinline__ float horner(const float (&c)[N], float u) {
  float v = c[N - 1];
#pragma unroll
  for (int i = N - 2; i >= 0; --i) v = fmaf(v, u, c[i]);
  return v;
}

constexpr float kTwoOverPiF = 0.636619772f, kInv2PiF = 0.159154943f, kTwoPiF = 6.28318531f;

// sin / cos of an angle within a few multiples of pi, reduced to [-pi, pi] first.
__device__ __forceinline__ void sincos_reduced(float th, float* s, float* c) {
  th = fmaf(-kTwoPiF, rintf(th * kInv2PiF), th);
  __sincosf(th, s, c);
}

// G = -(i/4) H0^(2)(x) with x = k R; phi equals x modulo 2 pi (carried in FP64 by the caller).
__device__ __forceinline__ void hankel0_mixed(float x, float phi, float& Gr, float& Gi) {
  if (x < 3.f) {
    const float u = x * x * (1.f / 9.f);
    const float j0 = horner(c_P0, u);
    const float y0 = fmaf(kTwoOverPiF * __logf(0.5f * x), j0, horner(c_Q0, u));
    Gr = -0.25f * y0;
    Gi = -0.25f * j0;
  } else {
    const float t = __fdividef(3.f, x);
    const float amp = horner(c_F0, t) * rsqrtf(x);
    float sn, cs;
    sincos_reduced(phi - 0.785398163f + horner(c_G0, t), &sn, &cs);
    Gr = -0.25f * amp * sn;
    Gi = -0.25f * amp * cs;
  }
}

// g1 = (i k / 4) H1^(2)(x) / R = (k / 4R) (Y1 + i J1); phi as for hankel0_mixed.
__device__ __forceinline__ void hankel1_mixed(float x, float phi, float k_over_4R, float& gr, float& gi) {
  if (x < 3.f) {
    const float u = x * x * (1.f / 9.f);
    const float j1 = x * horner(c_P1, u);
    const float y1 = __fdividef(fmaf(kTwoOverPiF * x * __logf(0.5f * x), j1, horner(c_Q1, u)), x);
    gr = k_over_4R * y1;
    gi = k_over_4R * j1;
  } else {
    const float t = __fdividef(3.f, x);
    const float amp = horner(c_F1, t) * rsqrtf(x) * k_over_4R;
    float sn, cs;
    sincos_reduced(phi - 2.35619449f + horner(c_G1, t), &sn, &cs);
    gr = amp * sn;
    gi = amp * cs;
  }
}

// Far pair in mixed precision.  Per pair in FP64: midpoint separation D, R0 = |D| and the phase
// k R0 reduced modulo 2 pi.  Per point pair in FP32: w = (point offsets from the midpoints),
// R = |D + w|, delta = R - R0 = (2 D.w + w.w) / (R + R0) without cancellation, x = k R and
// phase phi0 + k delta.  The trial sums of each test point are formed first (moments S_j), then spread
// over the test shapes.
struct FAcc {
  float pr[4], pi[4], mr, mi;
};

// k R0 modulo 2 pi for a double-float k R0 (Cody-Waite: 2 pi = P1 + P2 + P3, P1 = 6.28125 with 8
// significant bits, so n P1 is exact for |n| < 2^16, i.e. k R0 < 4e5).
__device__ __forceinline__ float reduce_2pi(dfl K) {
  const float n = rintf(__fmul_rn(K.hi, 0.159154937f));
  const float a = __fmaf_rn(-n, 6.28125f, K.hi);  // exact
  const float q2 = __fmul_rn(n, 1.935307169e-03f);
  const float q2e = __fmaf_rn(n, 1.935307169e-03f, -q2);
  dfl t = df_add(dfl{a, K.lo}, dfl{-q2, -q2e});
  return __fadd_rn(t.hi, __fsub_rn(t.lo, __fmul_rn(n, 1.025337627e-11f)));
}

// Far pair in mixed precision, all on the FP32 pipes.  Per pair in double-float: midpoint
// separation D, R0 = |D| and the phase k R0 reduced modulo 2 pi.  Per point pair in FP32:
// w = point offsets from the midpoints, R = |D + w|, delta = R - R0 = (2 D.w + w.w) / (R + R0)
// without cancellation, x = k R and phase phi0 + k delta.  The trial sums of each test point are
// formed first (moments S_j), then spread over the test shapes.
template <int OP>
__device__ __forceinline__ void far_pair_mixed(const Op& op, const float* fx, const float* fw, int nft,
                                               const float* bx, const float* bw, int nfb, const SegF& A,
                                               const SegF& B, FAcc& c) {
  const dfl Dx = df_sub(dfl{A.cxh, A.cxl}, dfl{B.cxh, B.cxl});
  const dfl Dy = df_sub(dfl{A.cyh, A.cyl}, dfl{B.cyh, B.cyl});
  const float dfx = Dx.hi + Dx.lo, dfy = Dy.hi + Dy.lo;
  float r0 = 0.f, phi0 = 0.f;
  const float kf = op.khi;
  if (kf != 0.f) {
    const dfl R0sq = df_add(df_mul(Dx, Dx), df_mul(Dy, Dy));
    const dfl R0 = df_mul(R0sq, df_rsqrt(R0sq));
    r0 = R0.hi + R0.lo;
    phi0 = reduce_2pi(df_mul(R0, dfl{op.khi, op.klo}));
  }
  float pr[4] = {0.f, 0.f, 0.f, 0.f}, pi[4] = {0.f, 0.f, 0.f, 0.f}, mr = 0.f, mi = 0.f;
  for (int p = 0; p < nft; ++p) {
    const float sp = fx[p];
    const float ox = (sp - 0.5f) * A.dx, oy = (sp - 0.5f) * A.dy;
    float s0r = 0.f, s0i = 0.f, s1r = 0.f, s1i = 0.f;
    for (int q = 0; q < nfb; ++q) {
      const float tq = bx[q];
      const float wx = ox - (tq - 0.5f) * B.dx, wy = oy - (tq - 0.5f) * B.dy;
      // R from r = D + w itself (no cancellation against R0^2 for close, parallel segments); the
      // phase increment delta from q = 2 D.w + w.w, accurate in absolute terms
      const float rx = dfx + wx, ry = dfy + wy;
      const float R2 = fmaf(rx, rx, ry * ry);
      const float invR = rsqrtf(R2);
      const float R = R2 * invR;
      float Kr, Ki;
      if (OP == BGB_OP2D_SL || OP == BGB_OP2D_HS) {
        if (kf == 0.f) {
          Kr = -kInv2PiF * __logf(R);
          Ki = 0.f;
        } else {
          const float qv = fmaf(2.f * dfx + wx, wx, (2.f * dfy + wy) * wy);
          const float delta = __fdividef(qv, R + r0);
          hankel0_mixed(kf * R, fmaf(kf, delta, phi0), Kr, Ki);
        }
      } else {
        float gr, gi;
        if (kf == 0.f) {
          gr = -kInv2PiF * invR * invR;
          gi = 0.f;
        } else {
          const float qv = fmaf(2.f * dfx + wx, wx, (2.f * dfy + wy) * wy);
          const float delta = __fdividef(qv, R + r0);
          hankel1_mixed(kf * R, fmaf(kf, delta, phi0), 0.25f * kf * invR, gr, gi);
        }
        const float proj = OP == BGB_OP2D_DL ? -(rx * B.nx + ry * B.ny) : rx * A.nx + ry * A.ny;
        Kr = gr * proj;
        Ki = gi * proj;
      }
      const float wq = bw[q] * B.len;
      const float g0 = op.nsB == 1 ? wq : wq * (1.f - tq), g1 = wq * tq;
      s0r = fmaf(Kr, g0, s0r);
      s0i = fmaf(Ki, g0, s0i);
      s1r = fmaf(Kr, g1, s1r);
      s1i = fmaf(Ki, g1, s1i);
    }
    const float wp = fw[p] * A.len;
    const float f0 = op.nsA == 1 ? wp : wp * (1.f - sp), f1 = wp * sp;
    pr[0] = fmaf(f0, s0r, pr[0]);
    pi[0] = fmaf(f0, s0i, pi[0]);
    pr[1] = fmaf(f0, s1r, pr[1]);
    pi[1] = fmaf(f0, s1i, pi[1]);
    pr[2] = fmaf(f1, s0r, pr[2]);
    pi[2] = fmaf(f1, s0i, pi[2]);
    pr[3] = fmaf(f1, s1r, pr[3]);
    pi[3] = fmaf(f1, s1i, pi[3]);
    if (OP == BGB_OP2D_HS) {
      const float sr = op.nsB == 1 ? s0r : s0r + s1r, si = op.nsB == 1 ? s0i : s0i + s1i;
      mr = fmaf(wp, sr, mr);
      mi = fmaf(wp, si, mi);
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    c.pr[k] = pr[k];
    c.pi[k] = pi[k];
  }
  c.mr = mr;
  c.mi = mi;
}

// The local matrix of a mixed far pair, in FP32.
template <int OP, class LT>
__device__ __forceinline__ void finalize_mixed(const Op& op, const SegF& A, const SegF& B, const FAcc& c,
                                               LT* __restrict__ out) {
  const float nn = A.nx * B.nx + A.ny * B.ny;
  const float ia = 1.f / A.len, ib = 1.f / B.len;
  const float dA[2] = {op.nsA == 2 ? -ia : 0.f, op.nsA == 2 ? ia : 0.f};
  const float dB[2] = {op.nsB == 2 ? -ib : 0.f, op.nsB == 2 ? ib : 0.f};
  const float bmr = op.fbr * c.mr - op.fbi * c.mi, bmi = op.fbr * c.mi + op.fbi * c.mr;
  for (int i = 0; i < op.nsA; ++i)
    for (int j = 0; j < op.nsB; ++j) {
      const float pr = c.pr[2 * i + j], pi = c.pi[2 * i + j];
      float lr = op.far_ * pr - op.fai * pi, li = op.far_ * pi + op.fai * pr;
      if (OP == BGB_OP2D_HS) {
        const float d = dA[i] * dB[j];
        lr = fmaf(lr, nn, bmr * d);
        li = fmaf(li, nn, bmi * d);
      }
      out[i * op.nsB + j] = LT{lr, li};
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// ----------------------------------------------------------------------------------------
// Kernels
// ----------------------------------------------------------------------------------------
// counts[0]: list length, [1]: degenerate-pair flag, [2 + class]: non-far pairs of owned columns;
// mask: bit (sl * nT + tl) set for every non-far pair.
__global__ void __launch_bounds__(256) k_curve_classify(const SegGeo* __restrict__ gT, const SegGeo* __restrict__ gB,
                                                        const SegF* __restrict__ gTf, const SegF* __restrict__ gBf,
                                                        const int* __restrict__ T, int nT, const int* __restrict__ S,
                                                        int nS, const unsigned char* __restrict__ own, double k2,
                                                        int LS, Special* __restrict__ list, int cap,
                                                        int* __restrict__ counts, unsigned* __restrict__ mask) {
  const int tl = blockIdx.x * blockDim.x + threadIdx.x;
  if (tl >= nT) return;
  const SegF Af = gTf[T[tl]];
  const float k2f = (float)k2;
  for (int sl = blockIdx.y; sl < nS; sl += gridDim.y) {
    if (certainly_far(Af, gBf[S[sl]], k2f)) continue;
    const SegGeo A = gT[T[tl]], B = gB[S[sl]];
    int match;
    const int cls = classify(A, B, k2, &match);
    if (cls == 0) continue;
    const int64_t bit = (int64_t)sl * nT + tl;
    atomicOr(&mask[bit >> 5], 1u << (bit & 31));
    if (cls < 0) {
      atomicOr(&counts[1], 1);
      continue;
    }
    const int idx = atomicAdd(&counts[0], 1);
    if (idx < cap) {
      Special sp;
      sp.slot = ((int64_t)sl * nT + tl) * LS;
      sp.tau = T[tl];
      sp.sigma = S[sl];
      sp.cls = cls;
      sp.match = match;
      list[idx] = sp;
    }
    if (own[sl]) atomicAdd(&counts[2 + cls], 1);
  }
}

template <int OP>
__global__ void __launch_bounds__(128) k_curve_far(Op op, const Rules* __restrict__ rules, const SegGeo* __restrict__ gT,
                                                   const SegGeo* __restrict__ gB, const int* __restrict__ T, int nT,
                                                   const int* __restrict__ S, int nS, const unsigned* __restrict__ mask,
                                                   double2* __restrict__ L) {
  __shared__ double fx[kMaxGL], fw[kMaxGL], bx[kMaxGL], bw[kMaxGL];
  const int nft = rules->nft, nfb = rules->nfb;
  for (int i = threadIdx.x; i < kMaxGL; i += blockDim.x) {
    fx[i] = rules->ft_x[i];
    fw[i] = rules->ft_w[i];
    bx[i] = rules->fb_x[i];
    bw[i] = rules->fb_w[i];
  }
  __syncthreads();
  const int tl = blockIdx.x * blockDim.x + threadIdx.x;
  if (tl >= nT) return;
  const SegGeo A = gT[T[tl]];
  for (int sl = blockIdx.y; sl < nS; sl += gridDim.y) {
    if (nonfar_bit(mask, (int64_t)sl * nT + tl)) continue;
    const SegGeo B = gB[S[sl]];
    Acc c;
    acc_zero(c);
    far_pair<OP>(op, fx, fw, nft, bx, bw, nfb, A, B, c);
    finalize<OP>(op, A, B, c, L + ((int64_t)sl * nT + tl) * op.LS);
  }
}

template <int OP>
__global__ void __launch_bounds__(128) k_curve_far_mixed(Op op, const Rules* __restrict__ rules,
                                                         const SegF* __restrict__ gT, const SegF* __restrict__ gB,
                                                         const int* __restrict__ T, int nT, const int* __restrict__ S,
                                                         int nS, const unsigned* __restrict__ mask,
                                                         float2* __restrict__ L) {
  __shared__ float fx[kMaxGL], fw[kMaxGL], bx[kMaxGL], bw[kMaxGL];
  const int nft = rules->nft, nfb = rules->nfb;
  for (int i = threadIdx.x; i < kMaxGL; i += blockDim.x) {
    fx[i] = (float)rules->ft_x[i];
    fw[i] = (float)rules->ft_w[i];
    bx[i] = (float)rules->fb_x[i];
    bw[i] = (float)rules->fb_w[i];
  }
  __syncthreads();
  const int tl = blockIdx.x * blockDim.x + threadIdx.x;
  if (tl >= nT) return;
  const SegF A = gT[T[tl]];
  for (int sl = blockIdx.y; sl < nS; sl += gridDim.y) {
    if (nonfar_bit(mask, (int64_t)sl * nT + tl)) continue;
    const SegF B = gB[S[sl]];
    FAcc c;
    far_pair_mixed<OP>(op, fx, fw, nft, bx, bw, nfb, A, B, c);
    finalize_mixed<OP>(op, A, B, c, L + ((int64_t)sl * nT + tl) * op.LS);
  }
}

template <int OP, class LT>
__global__ void __launch_bounds__(256) k_curve_special(Op op, const Rules* __restrict__ rules,
                                                       const SegGeo* __restrict__ gT, const SegGeo* __restrict__ gB,
                                                       const Special* __restrict__ list, int n, LT* __restrict__ L) {
  __shared__ Rules sR;
  __shared__ double wtabs[8][4 * kMaxSing];  // per warp: common-vertex lengths and logarithms
  {
    const int* src = (const int*)rules;
    int* dst = (int*)&sR;
    for (int i = threadIdx.x; i < (int)(sizeof(Rules) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  double* wtab = wtabs[threadIdx.x >> 5];
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n; e += nwarps) {
    const Special sp = list[e];
    const SegGeo A = gT[sp.tau], B = gB[sp.sigma];
    Acc c;
    acc_zero(c);
    if (sp.cls == 4) near_rule_warp<OP>(op, sR, A, B, lane, c);
    else singular_rule_warp<OP>(op, sR, A, B, sp.cls, sp.match, lane, wtab, c);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      c.pr[k] = warp_sum(c.pr[k]);
      c.pi[k] = warp_sum(c.pi[k]);
    }
    c.mr = warp_sum(c.mr);
    c.mi = warp_sum(c.mi);
    if (lane == 0) finalize<OP>(op, A, B, c, L + sp.slot);
  }
}

// ---- Mixed path: coincident and common-vertex pairs in double-float ---------------------------
// The FP64 rules and series of singular_rule_warp / kernel_series evaluated with double-float
// arithmetic on the FP32 pipes (about 48 bits), single and hypersingular kernels (the double layers
// keep the FP64 kernel).  Each lane sums the kernel times the weight into four moments
// (1, s, t, s t), from which the shape products follow.
struct DfMom {
  dfl r[4], i[4];  // sum of K w, K w s, K w t, K w s t
};

__device__ __forceinline__ dfl df_scale(dfl a, float f) { return dfl{a.hi * f, a.lo * f}; }  // f a power of 2

template <int OP>
__device__ __forceinline__ void df_point(const Op& op, const RulesDF& R, dfl Rd, dfl lnR, int M, dfl lnk2g, dfl wl,
                                         dfl s, dfl t, DfMom& mo) {
  dfl Kr, Ki;
  if (op.khi == 0.f) {
    Kr = df_neg(df_mul(R.inv2pi, lnR));
    Ki = dfl{0.f, 0.f};
  } else {
    const dfl x = df_mul(Rd, dfl{op.khi, op.klo});
    if (x.hi <= 4.f) {
      const dfl u = df_scale(df_mul(x, x), 0.25f);
      dfl j0 = R.sa[M];
      for (int m = M - 1; m >= 0; --m) j0 = df_add(df_mul(j0, u), R.sa[m]);
      dfl s0 = R.sb[M - 1];
      for (int m = M - 2; m >= 0; --m) s0 = df_add(df_mul(s0, u), R.sb[m]);
      const dfl y0v = df_mul(R.two_over_pi, df_add(df_mul(df_add(lnR, lnk2g), j0), df_mul(s0, u)));
      Kr = df_scale(y0v, -0.25f);
      Ki = df_scale(j0, -0.25f);
    } else {
      const double xd = df_to_double(x);
      const double yr = -0.25 * y0(xd), yi = -0.25 * j0(xd);
      Kr.hi = (float)yr;
      Kr.lo = (float)(yr - (double)Kr.hi);
      Ki.hi = (float)yi;
      Ki.lo = (float)(yi - (double)Ki.hi);
    }
  }
  const dfl kwr = df_mul(Kr, wl), kwi = df_mul(Ki, wl);
  const dfl st = df_mul(s, t);
  mo.r[0] = df_add(mo.r[0], kwr);
  mo.i[0] = df_add(mo.i[0], kwi);
  mo.r[1] = df_add(mo.r[1], df_mul(kwr, s));
  mo.i[1] = df_add(mo.i[1], df_mul(kwi, s));
  mo.r[2] = df_add(mo.r[2], df_mul(kwr, t));
  mo.i[2] = df_add(mo.i[2], df_mul(kwi, t));
  mo.r[3] = df_add(mo.r[3], df_mul(kwr, st));
  mo.i[3] = df_add(mo.i[3], df_mul(kwi, st));
}

__device__ __forceinline__ dfl df_from_double(double v) {
  const float h = (float)v;
  return dfl{h, (float)(v - (double)h)};
}

template <int OP>
__device__ void singular_rule_warp_df(const Op& op, const RulesDF& R, const SegGeo& A, const SegGeo& B, int cls,
                                      int match, int lane, dfl* __restrict__ wtab, DfMom& mo) {
  const int n = R.n;
  const int M = series_order(op.k, max_vertex_distance(A, B));
  const dfl lnk2g = df_from_double(op.lnk2 + kEulerGamma);
  const dfl ll = df_from_double(A.len * B.len);
  const dfl one{1.f, 0.f};
  if (cls == 3) {
    const bool same = match == 0;
    const dfl lA = df_from_double(A.len), lnl = df_from_double(log(A.len));
    const int ch = R.nz * 2;
    for (int k = lane; k < 2 * ch; k += 32) {
      const int half = k >= ch;
      const int rem = k - half * ch, a = rem >> 1, b = rem & 1;
      const dfl z = R.gz[a], w = R.gl2x[b];
      const dfl t1 = df_mul(df_sub(one, z), w);  // (1 - z) w
      const dfl u = half ? t1 : df_add(z, t1), v = half ? df_add(z, t1) : t1;
      const dfl wl = df_mul(df_mul(R.wcf[a], R.gl2w[b]), ll);
      df_point<OP>(op, R, df_mul(z, lA), df_add(R.lnz[a], lnl), M, lnk2g, wl, u, same ? v : df_sub(one, v), mo);
    }
    return;
  }
  const int ma = match >> 1, mb = match & 1;
  const double ax = ma == 0 ? A.dx : -A.dx, ay = ma == 0 ? A.dy : -A.dy;
  const double bx = mb == 0 ? B.dx : -B.dx, by = mb == 0 ? B.dy : -B.dy;
  if (lane < n) {
    const double w = (double)R.sgx[lane].hi + (double)R.sgx[lane].lo;
    const double l0 = sqrt((ax - w * bx) * (ax - w * bx) + (ay - w * by) * (ay - w * by));
    const double l1 = sqrt((w * ax - bx) * (w * ax - bx) + (w * ay - by) * (w * ay - by));
    wtab[lane] = df_from_double(l0);
    wtab[kMaxSing + lane] = df_from_double(log(l0));
    wtab[2 * kMaxSing + lane] = df_from_double(l1);
    wtab[3 * kMaxSing + lane] = df_from_double(log(l1));
  }
  __syncwarp();
  const int per_half = R.nzcv * n;
  for (int k = lane; k < 2 * per_half; k += 32) {
    const int half = k >= per_half;
    const int rem = k - half * per_half, a = rem / n, b = rem - a * n;
    const dfl z = R.gzc[a], zw = df_mul(z, R.sgx[b]);
    const dfl xi = half ? zw : z, eta = half ? z : zw;
    const dfl* tb = wtab + 2 * kMaxSing * half;
    const dfl wl = df_mul(df_mul(R.wcv[a], R.sgw[b]), ll);
    df_point<OP>(op, R, df_mul(z, tb[b]), df_add(R.lnzc[a], tb[kMaxSing + b]), M, lnk2g, wl,
                 ma == 0 ? xi : df_sub(one, xi), mb == 0 ? eta : df_sub(one, eta), mo);
  }
  __syncwarp();
}

__device__ __forceinline__ dfl warp_sum_df(dfl v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const dfl o{__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off)};
    v = df_add(v, o);
  }
  return v;
}

// Mixed path, single layer and hypersingular: coincident and common-vertex pairs in double-float,
// near pairs by the FP64 rule (rules read from global memory).
template <int OP, class LT>
__global__ void __launch_bounds__(256) k_curve_special_df(Op op, const Rules* __restrict__ rules,
                                                          const RulesDF* __restrict__ rdf,
                                                          const SegGeo* __restrict__ gT, const SegGeo* __restrict__ gB,
                                                          const Special* __restrict__ list, int n, LT* __restrict__ L) {
  __shared__ RulesDF sR;
  __shared__ dfl wtabs[8][4 * kMaxSing];
  {
    const int* src = (const int*)rdf;
    int* dst = (int*)&sR;
    for (int i = threadIdx.x; i < (int)(sizeof(RulesDF) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  dfl* wtab = wtabs[threadIdx.x >> 5];
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n; e += nwarps) {
    const Special sp = list[e];
    const SegGeo A = gT[sp.tau], B = gB[sp.sigma];
    Acc c;
    acc_zero(c);
    if (sp.cls == 4) {
      near_rule_warp<OP>(op, *rules, A, B, lane, c);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        c.pr[k] = warp_sum(c.pr[k]);
        c.pi[k] = warp_sum(c.pi[k]);
      }
      c.mr = warp_sum(c.mr);
      c.mi = warp_sum(c.mi);
    } else {
      DfMom mo;
#pragma unroll
      for (int k = 0; k < 4; ++k) mo.r[k] = mo.i[k] = dfl{0.f, 0.f};
      singular_rule_warp_df<OP>(op, sR, A, B, sp.cls, sp.match, lane, wtab, mo);
      double mr[4], mi[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        mr[k] = df_to_double(warp_sum_df(mo.r[k]));
        mi[k] = df_to_double(warp_sum_df(mo.i[k]));
      }
      // shape products from the moments: f = (1 - s, s) or 1, g = (1 - t, t) or 1
      const bool hA = op.nsA == 2, hB = op.nsB == 2;
      c.pr[0] = mr[0] - (hA ? mr[1] : 0.0) - (hB ? mr[2] : 0.0) + (hA && hB ? mr[3] : 0.0);
      c.pi[0] = mi[0] - (hA ? mi[1] : 0.0) - (hB ? mi[2] : 0.0) + (hA && hB ? mi[3] : 0.0);
      c.pr[1] = mr[2] - (hA ? mr[3] : 0.0);
      c.pi[1] = mi[2] - (hA ? mi[3] : 0.0);
      c.pr[2] = mr[1] - (hB ? mr[3] : 0.0);
      c.pi[2] = mi[1] - (hB ? mi[3] : 0.0);
      c.pr[3] = mr[3];
      c.pi[3] = mi[3];
      c.mr = mr[0];
      c.mi = mi[0];
    }
    if (lane == 0) finalize<OP>(op, A, B, c, L + sp.slot);
  }
}

// Explicit pairs (bgb_local_matrices_curve): far pairs by the far-kernel code, the others listed
// for k_curve_special.  err[0]: list length, err[1]: invalid pair / rule.
template <int OP>
__global__ void __launch_bounds__(128) k_curve_pairs(Op op, const Rules* __restrict__ rules, const SegGeo* __restrict__ gT,
                                                     const SegGeo* __restrict__ gB, const SegF* __restrict__ gTf,
                                                     const SegF* __restrict__ gBf, const int2* __restrict__ pairs,
                                                     int64_t npairs, int force, int mixed, double2* __restrict__ L,
                                                     signed char* __restrict__ cls_out, Special* __restrict__ list,
                                                     int* __restrict__ err) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npairs) return;
  const SegGeo A = gT[pairs[p].x], B = gB[pairs[p].y];
  int match;
  const int cls = classify(A, B, op.k2, &match);
  cls_out[p] = (signed char)cls;
  const int rule = force >= 0 ? force : cls;
  if (cls < 0 || ((rule == 1 || rule == 3) && rule != cls)) {
    atomicOr(&err[1], 1);
    return;
  }
  if (rule == 0) {
    if (mixed) {
      float fx[kMaxGL], fw[kMaxGL], bx[kMaxGL], bw[kMaxGL];
      for (int i = 0; i < rules->nft; ++i) {
        fx[i] = (float)rules->ft_x[i];
        fw[i] = (float)rules->ft_w[i];
      }
      for (int i = 0; i < rules->nfb; ++i) {
        bx[i] = (float)rules->fb_x[i];
        bw[i] = (float)rules->fb_w[i];
      }
      FAcc c;
      const SegF Af = gTf[pairs[p].x], Bf = gBf[pairs[p].y];
      far_pair_mixed<OP>(op, fx, fw, rules->nft, bx, bw, rules->nfb, Af, Bf, c);
      finalize_mixed<OP>(op, Af, Bf, c, L + p * 4);
    } else {
      Acc c;
      acc_zero(c);
      far_pair<OP>(op, rules->ft_x, rules->ft_w, rules->nft, rules->fb_x, rules->fb_w, rules->nfb, A, B, c);
      finalize<OP>(op, A, B, c, L + p * 4);
    }
    return;
  }
  const int idx = atomicAdd(&err[0], 1);
  Special sp;
  sp.slot = p * 4;
  sp.tau = pairs[p].x;
  sp.sigma = pairs[p].y;
  sp.cls = rule;
  sp.match = match;
  list[idx] = sp;
}

// Z[m, n] = sum over supports (test outer, trial inner, both by segment) of c_m c_n L.
// Local matrices, coefficients and sums in FP64 (double2) or FP32 (float2, the mixed path).
template <typename OutT, typename LT>
__global__ void __launch_bounds__(256) k_curve_gather(const LT* __restrict__ L, int nT, int LS, int nsB,
                                                      int nrows, int ncols, const int64_t* __restrict__ toff,
                                                      const int* __restrict__ tcode,
                                                      const decltype(LT::x)* __restrict__ tcoef,
                                                      const int64_t* __restrict__ boff, const int* __restrict__ bcode,
                                                      const decltype(LT::x)* __restrict__ bcoef, OutT* __restrict__ out,
                                                      int64_t ld) {
  typedef decltype(LT::x) R;
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nrows) return;
  const int64_t a0 = toff[m], a1 = toff[m + 1];
  for (int n = blockIdx.y; n < ncols; n += gridDim.y) {
    R zr = 0, zi = 0;
    const int64_t b0 = boff[n], b1 = boff[n + 1];
    for (int64_t a = a0; a < a1; ++a) {
      const int ta = tcode[a];
      const R ca = tcoef[a];
      for (int64_t b = b0; b < b1; ++b) {
        const int tb = bcode[b];
        const LT v = L[((int64_t)(tb >> 1) * nT + (ta >> 1)) * LS + (ta & 1) * nsB + (tb & 1)];
        const R cb = bcoef[b];
        zr += (v.x * ca) * cb;
        zi += (v.y * ca) * cb;
      }
    }
    OutT o;
    o.x = zr;
    o.y = zi;
    out[m + (int64_t)n * ld] = o;
  }
}

// ----------------------------------------------------------------------------------------
// Host side
// ----------------------------------------------------------------------------------------
static int validate_curve(const bgb_curve_space* s, const char* name) {
  if (!s) { set_error("%s curve space is NULL", name); return BGB_ERR_INVALID; }
  if (s->refspace != BGB_REFSPACE2D_LAGRANGE_C0D1 && s->refspace != BGB_REFSPACE2D_LAGRANGE_CXD0) {
    set_error("%s curve space: unknown refspace %d", name, s->refspace);
    return BGB_ERR_INVALID;
  }
  if (s->nv < 0 || s->ns < 0 || s->nfun < 0) { set_error("%s curve space: negative sizes", name); return BGB_ERR_INVALID; }
  if (s->ns > 0 && (!s->vertices || !s->segments || !s->fn_index || !s->fn_coef)) {
    set_error("%s curve space: NULL table", name);
    return BGB_ERR_INVALID;
  }
  for (int64_t i = 0; i < 2 * (int64_t)s->nv; ++i)
    if (!std::isfinite(s->vertices[i])) { set_error("%s curve space: non-finite vertex coordinate at %lld", name, (long long)i); return BGB_ERR_INVALID; }
  const int nsh = s->refspace == BGB_REFSPACE2D_LAGRANGE_CXD0 ? 1 : 2;
  for (int64_t e = 0; e < s->ns; ++e) {
    const int a = s->segments[2 * e], b = s->segments[2 * e + 1];
    if (a < 0 || a >= s->nv || b < 0 || b >= s->nv) { set_error("%s curve space: segment %lld has a vertex index out of range", name, (long long)e); return BGB_ERR_INVALID; }
    const double dx = s->vertices[2 * b] - s->vertices[2 * a], dy = s->vertices[2 * b + 1] - s->vertices[2 * a + 1];
    if (a == b || !(dx * dx + dy * dy > 0.0)) { set_error("%s curve space: segment %lld is degenerate", name, (long long)e); return BGB_ERR_INVALID; }
    for (int i = 0; i < nsh; ++i) {
      const int f = s->fn_index[2 * e + i];
      if (f < -1 || f >= s->nfun) { set_error("%s curve space: segment %lld local %d has function index %d out of range", name, (long long)e, i, f); return BGB_ERR_INVALID; }
      if (f >= 0 && !std::isfinite(s->fn_coef[2 * e + i])) { set_error("%s curve space: non-finite coefficient", name); return BGB_ERR_INVALID; }
    }
    if (nsh == 2 && s->fn_index[2 * e] >= 0 && s->fn_index[2 * e] == s->fn_index[2 * e + 1]) {
      set_error("%s curve space: segment %lld maps both local shapes to one function", name, (long long)e);
      return BGB_ERR_INVALID;
    }
  }
  return 0;
}

static int make_op(const bgb_operator2d* op, const bgb_curve_space* a, const bgb_curve_space* b, Op* out) {
  if (!op) { set_error("operator is NULL"); return BGB_ERR_INVALID; }
  if (op->kind < BGB_OP2D_SL || op->kind > BGB_OP2D_HS) { set_error("unknown 2-D operator kind %d", op->kind); return BGB_ERR_INVALID; }
  if (!std::isfinite(op->wavenumber) || op->wavenumber < 0.0) { set_error("wave number must be finite and >= 0"); return BGB_ERR_INVALID; }
  for (int c = 0; c < 2; ++c)
    if (!std::isfinite(op->alpha[c]) || !std::isfinite(op->beta[c])) { set_error("operator has non-finite parameters"); return BGB_ERR_INVALID; }
  Op o{};
  o.kind = op->kind;
  o.nsA = a->refspace == BGB_REFSPACE2D_LAGRANGE_CXD0 ? 1 : 2;
  o.nsB = b->refspace == BGB_REFSPACE2D_LAGRANGE_CXD0 ? 1 : 2;
  o.LS = o.nsA * o.nsB;
  o.k = op->wavenumber;
  o.k2 = op->wavenumber * op->wavenumber;
  o.ar = op->alpha[0];
  o.ai = op->alpha[1];
  o.br = op->beta[0];
  o.bi = op->beta[1];
  o.lnk2 = o.k > 0.0 ? std::log(0.5 * o.k) : 0.0;
  o.khi = (float)o.k;
  o.klo = (float)(o.k - (double)o.khi);
  o.far_ = (float)o.ar;
  o.fai = (float)o.ai;
  o.fbr = (float)o.br;
  o.fbi = (float)o.bi;
  *out = o;
  return 0;
}

static int make_rules(const bgb_quadstrat2d* qs, Rules* R) {
  if (!qs) { set_error("quadstrat is NULL"); return BGB_ERR_INVALID; }
  if (qs->far_test < 1 || qs->far_test > kMaxGL || qs->far_trial < 1 || qs->far_trial > kMaxGL || qs->near < 1 ||
      qs->near > kMaxGL || qs->singular < 1 || qs->singular > kMaxSing) {
    set_error("curve quadstrat: Gauss points must be 1..%d and the singular order 1..%d (got %d %d %d %d)", kMaxGL,
              kMaxSing, qs->far_test, qs->far_trial, qs->near, qs->singular);
    return BGB_ERR_INVALID;
  }
  std::memset(R, 0, sizeof(Rules));
  R->nft = qs->far_test;
  R->nfb = qs->far_trial;
  R->nnear = qs->near;
  R->nsing = qs->singular;
  gauss_legendre01(R->nft, R->ft_x, R->ft_w);
  gauss_legendre01(R->nfb, R->fb_x, R->fb_w);
  gauss_legendre01(R->nnear, R->nr_x, R->nr_w);
  const int n = R->nsing;
  gauss_legendre01(n, R->sg_x, R->sg_w);
  // graded rules: [0, q^L] then [q^(lev+1), q^lev] for lev = L - 1 .. 0, n Gauss points each;
  // L = 3n for coincident pairs (ln z), 3n/2 for common-vertex pairs (z ln z)
  const double q = 0.35;
  auto graded = [&](int levels, double* gz, double* gwz, double* lnz) {
    int k = 0;
    for (int lev = levels; lev >= 0; --lev) {
      const double a = lev == levels ? 0.0 : std::pow(q, lev + 1), b = std::pow(q, lev);
      for (int i = 0; i < n; ++i) {
        gz[k] = a + (b - a) * R->sg_x[i];
        gwz[k] = (b - a) * R->sg_w[i];
        lnz[k] = std::log(gz[k]);
        ++k;
      }
    }
    return k / n;
  };
  R->ngraded = graded(3 * n, R->gz, R->gwz, R->lnz) * n;
  R->ngraded_cv = graded((3 * n) / 2, R->gz_cv, R->gwz_cv, R->lnz_cv) * n;
  gauss_legendre01(2, R->gl2_x, R->gl2_w);
  // series coefficients (A&S 9.1.10-9.1.13): factorials and harmonic numbers in FP64
  double fact = 1.0, H = 0.0;  // m!, H_m
  for (int m = 0; m <= kSeries; ++m) {
    if (m > 0) {
      fact *= m;
      H += 1.0 / m;
    }
    const double sign = (m % 2) ? -1.0 : 1.0;
    const double H1 = H + 1.0 / (m + 1);
    R->sa[m] = sign / (fact * fact);
    R->sc[m] = sign / (fact * fact * (m + 1));
    R->sd[m] = sign * (H + H1 - 2.0 * 0.5772156649015329) / (fact * fact * (m + 1));
    if (m < kSeries) {
      const double f1 = fact * (m + 1);  // (m+1)!
      R->sb[m] = sign * H1 / (f1 * f1);  // coefficient of u^(m+1): (-1)^m H_{m+1} / ((m+1)!)^2
    }
  }
  return 0;
}

static int upload_curve(cudaStream_t st, const bgb_curve_space* s, DevBuf& verts, DevBuf& segs, DevBuf& geo,
                        DevBuf& geof) {
  int rc;
  if ((rc = verts.ensure(sizeof(double) * 2 * (size_t)std::max(1, s->nv))) ||
      (rc = segs.ensure(sizeof(int) * 2 * (size_t)std::max(1, s->ns))) ||
      (rc = geo.ensure(sizeof(SegGeo) * (size_t)std::max(1, s->ns))) ||
      (rc = geof.ensure(sizeof(SegF) * (size_t)std::max(1, s->ns))))
    return rc;
  if (s->nv) BGB_CUDA(cudaMemcpyAsync(verts.p, s->vertices, sizeof(double) * 2 * (size_t)s->nv, cudaMemcpyHostToDevice, st));
  if (s->ns) {
    BGB_CUDA(cudaMemcpyAsync(segs.p, s->segments, sizeof(int) * 2 * (size_t)s->ns, cudaMemcpyHostToDevice, st));
    k_curve_geo<<<(s->ns + 255) / 256, 256, 0, st>>>(verts.as<double>(), segs.as<int>(), s->ns, geo.as<SegGeo>(),
                                                     geof.as<SegF>());
    BGB_CUDA(cudaGetLastError());
  }
  return 0;
}

template <class T>
static int put(cudaStream_t st, DevBuf& buf, const std::vector<T>& v) {
  int rc;
  if ((rc = buf.ensure(sizeof(T) * std::max<size_t>(1, v.size())))) return rc;
  if (!v.empty()) BGB_CUDA(cudaMemcpyAsync(buf.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st));
  return 0;
}

template <int OP>
static void launch_far(const Op& op, const Rules* rules, const SegGeo* gT, const SegGeo* gB, const int* T, int nT,
                       const int* S, int nS, const unsigned* mask, double2* L, cudaStream_t st) {
  dim3 grid((nT + 127) / 128, std::min(nS, 65535));
  k_curve_far<OP><<<grid, 128, 0, st>>>(op, rules, gT, gB, T, nT, S, nS, mask, L);
}

template <int OP>
static void launch_far_mixed(const Op& op, const Rules* rules, const SegF* gT, const SegF* gB, const int* T, int nT,
                             const int* S, int nS, const unsigned* mask, float2* L, cudaStream_t st) {
  dim3 grid((nT + 127) / 128, std::min(nS, 65535));
  k_curve_far_mixed<OP><<<grid, 128, 0, st>>>(op, rules, gT, gB, T, nT, S, nS, mask, L);
}

template <int OP, class LT>
static void launch_special_t(const Op& op, const Rules* rules, const SegGeo* gT, const SegGeo* gB, const Special* list,
                             int n, LT* L, int num_sms, cudaStream_t st) {
  if (n <= 0) return;
  const int blocks = std::max(1, std::min((n + 7) / 8, num_sms * 8));
  k_curve_special<OP, LT><<<blocks, 256, 0, st>>>(op, rules, gT, gB, list, n, L);
}

template <int OP>
static void launch_special(const Op& op, const Rules* rules, const RulesDF* rdf, const SegGeo* gT, const SegGeo* gB,
                           const Special* list, int n, void* L, bool fp32_l, int num_sms, cudaStream_t st) {
  if (n <= 0) return;
  const int blocks = std::max(1, std::min((n + 7) / 8, num_sms * 8));
  if (rdf && (OP == BGB_OP2D_SL || OP == BGB_OP2D_HS)) {
    if (fp32_l) k_curve_special_df<OP, float2><<<blocks, 256, 0, st>>>(op, rules, rdf, gT, gB, list, n, (float2*)L);
    else k_curve_special_df<OP, double2><<<blocks, 256, 0, st>>>(op, rules, rdf, gT, gB, list, n, (double2*)L);
    return;
  }
  if (fp32_l) launch_special_t<OP, float2>(op, rules, gT, gB, list, n, (float2*)L, num_sms, st);
  else launch_special_t<OP, double2>(op, rules, gT, gB, list, n, (double2*)L, num_sms, st);
}

static void make_rules_df(const Rules& R, RulesDF* D) {
  std::memset(D, 0, sizeof(RulesDF));
  auto df = [](double v) {
    const float h = (float)v;
    return dfl{h, (float)(v - (double)h)};
  };
  D->n = R.nsing;
  D->nz = R.ngraded;
  D->nzcv = R.ngraded_cv;
  for (int a = 0; a < R.ngraded; ++a) {
    D->gz[a] = df(R.gz[a]);
    D->wcf[a] = df(R.gwz[a] * (1.0 - R.gz[a]));
    D->lnz[a] = df(R.lnz[a]);
  }
  for (int a = 0; a < R.ngraded_cv; ++a) {
    D->gzc[a] = df(R.gz_cv[a]);
    D->wcv[a] = df(R.gwz_cv[a] * R.gz_cv[a]);
    D->lnzc[a] = df(R.lnz_cv[a]);
  }
  for (int b = 0; b < R.nsing; ++b) {
    D->sgx[b] = df(R.sg_x[b]);
    D->sgw[b] = df(R.sg_w[b]);
  }
  for (int b = 0; b < 2; ++b) {
    D->gl2x[b] = df(R.gl2_x[b]);
    D->gl2w[b] = df(R.gl2_w[b]);
  }
  for (int m = 0; m <= kSeries; ++m) D->sa[m] = df(R.sa[m]);
  for (int m = 0; m < kSeries; ++m) D->sb[m] = df(R.sb[m]);
  D->inv2pi = df(0.15915494309189535);
  D->two_over_pi = df(0.6366197723675814);
}

template <int OP>
static void launch_pairs(const Op& op, const Rules* rules, const SegGeo* gT, const SegGeo* gB, const SegF* gTf,
                         const SegF* gBf, const int2* pairs, int64_t np, int force, int mixed, double2* L,
                         signed char* cls, Special* list, int* err, cudaStream_t st) {
  k_curve_pairs<OP><<<(unsigned)((np + 127) / 128), 128, 0, st>>>(op, rules, gT, gB, gTf, gBf, pairs, np, force, mixed,
                                                                  L, cls, list, err);
}

#define BGB_CURVE_DISPATCH(kind, fn, ...)                              \
  switch (kind) {                                                      \
    case BGB_OP2D_SL: fn<BGB_OP2D_SL>(__VA_ARGS__); break;             \
    case BGB_OP2D_DL: fn<BGB_OP2D_DL>(__VA_ARGS__); break;             \
    case BGB_OP2D_DLT: fn<BGB_OP2D_DLT>(__VA_ARGS__); break;           \
    default: fn<BGB_OP2D_HS>(__VA_ARGS__); break;                      \
  }

// Supports of functions [f0, f1) as (segment, local, coef), sorted by function then segment.
struct CurveSupports {
  std::vector<int64_t> off;
  std::vector<int> seg, loc;
  std::vector<double> coef;
};

static CurveSupports curve_supports(const bgb_curve_space* s, int64_t f0, int64_t f1) {
  const int nsh = s->refspace == BGB_REFSPACE2D_LAGRANGE_CXD0 ? 1 : 2;
  CurveSupports C;
  C.off.assign((size_t)(f1 - f0) + 1, 0);
  for (int64_t e = 0; e < s->ns; ++e)
    for (int i = 0; i < nsh; ++i) {
      const int f = s->fn_index[2 * e + i];
      if (f >= f0 && f < f1) C.off[(size_t)(f - f0) + 1]++;
    }
  for (size_t k = 1; k < C.off.size(); ++k) C.off[k] += C.off[k - 1];
  const size_t tot = (size_t)C.off.back();
  C.seg.resize(tot);
  C.loc.resize(tot);
  C.coef.resize(tot);
  std::vector<int64_t> fill(C.off.begin(), C.off.end() - 1);
  for (int64_t e = 0; e < s->ns; ++e)  // ascending segments: each function's list comes out sorted
    for (int i = 0; i < nsh; ++i) {
      const int f = s->fn_index[2 * e + i];
      if (f >= f0 && f < f1) {
        const int64_t k = fill[(size_t)(f - f0)]++;
        C.seg[(size_t)k] = (int)e;
        C.loc[(size_t)k] = i;
        C.coef[(size_t)k] = s->fn_coef[2 * e + i];
      }
    }
  return C;
}

// Local segment indices: sorted distinct segments of the supports; code = 2 * local + shape.
static void localise(const CurveSupports& C, std::vector<int>& segs, std::vector<int>& code, std::vector<int>& map_scratch) {
  segs.assign(C.seg.begin(), C.seg.end());
  std::sort(segs.begin(), segs.end());
  segs.erase(std::unique(segs.begin(), segs.end()), segs.end());
  for (size_t k = 0; k < segs.size(); ++k) map_scratch[(size_t)segs[k]] = (int)k;
  code.resize(C.seg.size());
  for (size_t k = 0; k < C.seg.size(); ++k) code[k] = 2 * map_scratch[(size_t)C.seg[k]] + C.loc[k];
}

// The mixed far kernels reduce k R0 modulo 2 pi with 2 pi split in three floats, exact for
// k R0 < 4e5 (2^16 turns): reject problems whose k times the diameter of the two curves exceeds 3e5.
static int check_mixed_range(const bgb_operator2d* op, const bgb_curve_space* a, const bgb_curve_space* b) {
  double lo[2] = {1e300, 1e300}, hi[2] = {-1e300, -1e300};
  for (const bgb_curve_space* sp : {a, b})
    for (int64_t v = 0; v < sp->nv; ++v)
      for (int c = 0; c < 2; ++c) {
        lo[c] = std::min(lo[c], sp->vertices[2 * v + c]);
        hi[c] = std::max(hi[c], sp->vertices[2 * v + c]);
      }
  const double diam = std::hypot(hi[0] - lo[0], hi[1] - lo[1]);
  if (op->wavenumber * diam > 3e5) {
    set_error("mixed precision covers k times the curves' diameter up to 3e5 (got %.3g); use BGB_PREC_FP64",
              op->wavenumber * diam);
    return BGB_ERR_NOT_SUPPORTED;
  }
  return 0;
}

}  // namespace curve
}  // namespace bgb

using namespace bgb;
using namespace bgb::curve;

extern "C" {

int bgb_assemble_curve(bgb_handle* h, const bgb_operator2d* op, const bgb_curve_space* test,
                       const bgb_curve_space* trial, const bgb_quadstrat2d* qs, int32_t precision, void* out,
                       int32_t out_kind, int64_t ld, int64_t row0, int64_t nrows, void* stream, bgb_stats* stats) {
  const auto t_start = std::chrono::steady_clock::now();
  if (!h) { set_error("handle is NULL"); return BGB_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(h->mu);
  int rc;
  if ((rc = validate_curve(test, "test")) || (rc = validate_curve(trial, "trial"))) return rc;
  Op o;
  Rules R;
  if ((rc = make_op(op, test, trial, &o)) || (rc = make_rules(qs, &R))) return rc;
  if (precision != BGB_PREC_FP64 && precision != BGB_PREC_MIXED) { set_error("bad precision %d", precision); return BGB_ERR_INVALID; }
  if (precision == BGB_PREC_MIXED && (rc = check_mixed_range(op, test, trial))) return rc;
  if (out_kind < BGB_OUT_HOST_C64 || out_kind > BGB_OUT_DEVICE_C32) { set_error("bad out_kind %d", out_kind); return BGB_ERR_INVALID; }
  if (nrows < 0) nrows = (int64_t)test->nfun - row0;
  if (row0 < 0 || row0 + nrows > test->nfun) { set_error("row window [%lld, %lld) outside [0, %d)", (long long)row0, (long long)(row0 + nrows), test->nfun); return BGB_ERR_INVALID; }
  if (ld < std::max<int64_t>(1, nrows)) { set_error("ld %lld < nrows %lld", (long long)ld, (long long)nrows); return BGB_ERR_INVALID; }
  if (!out && nrows > 0 && trial->nfun > 0) { set_error("out is NULL"); return BGB_ERR_INVALID; }
  *h->abort_host = 0;
  bgb_stats st{};
  if (nrows == 0 || trial->nfun == 0) {
    if (stats) *stats = st;
    return 0;
  }
  cudaSetDevice(h->device);
  cudaStream_t s = h->stream;
  cudaStream_t user = stream ? (cudaStream_t)stream : h->stream;
  const bool host_out = out_kind == BGB_OUT_HOST_C64 || out_kind == BGB_OUT_HOST_C32;
  const bool c64 = out_kind == BGB_OUT_HOST_C64 || out_kind == BGB_OUT_DEVICE_C64;
  const size_t esz = c64 ? 16 : 8;
  if (!host_out && user != s) {
    BGB_CUDA(cudaEventRecord(h->ev[7], user));
    BGB_CUDA(cudaStreamWaitEvent(s, h->ev[7], 0));
  }
  CurveBufs& B = h->curve;
  if ((rc = upload_curve(s, test, B.verts_t, B.segs_t, B.geo_t, B.geof_t)) ||
      (rc = upload_curve(s, trial, B.verts_b, B.segs_b, B.geo_b, B.geof_b)))
    return rc;
  if ((rc = B.rules.ensure(sizeof(Rules)))) return rc;
  BGB_CUDA(cudaMemcpyAsync(B.rules.p, &R, sizeof(Rules), cudaMemcpyHostToDevice, s));
  RulesDF RD;
  make_rules_df(R, &RD);
  if ((rc = B.rulesdf.ensure(sizeof(RulesDF)))) return rc;
  BGB_CUDA(cudaMemcpyAsync(B.rulesdf.p, &RD, sizeof(RulesDF), cudaMemcpyHostToDevice, s));
  BGB_CUDA(cudaStreamSynchronize(s));  // RD lives on this stack frame
  int launches = test->ns > 0 ? 1 : 0;
  launches += trial->ns > 0 ? 1 : 0;

  // test side: supports of the rows, local test segments
  std::vector<int> scratch((size_t)std::max(test->ns, trial->ns) + 1, -1);
  CurveSupports TS = curve_supports(test, row0, row0 + nrows);
  std::vector<int> T, tcode;
  localise(TS, T, tcode, scratch);
  const int nT = (int)T.size();
  const bool fp32_l = precision == BGB_PREC_MIXED;  // mixed: local matrices, coefficients, gather in FP32
  const size_t lsz = fp32_l ? sizeof(float2) : sizeof(double2);
  std::vector<float> tcoef_f(TS.coef.begin(), TS.coef.end());
  if ((rc = put(s, B.T, T)) || (rc = put(s, B.tsup_off, TS.off)) || (rc = put(s, B.tsup_i, tcode)) ||
      (rc = (fp32_l ? put(s, B.tsup_c, tcoef_f) : put(s, B.tsup_c, TS.coef))))
    return rc;

  // column blocks sized to the HBM budget: local matrices of nT x |S_b| pairs (|S_b| <= 2 per column)
  size_t freeb = 0, totalb = 0;
  cudaMemGetInfo(&freeb, &totalb);
  const int64_t budget = h->cfg.hbm_budget_bytes > 0 ? h->cfg.hbm_budget_bytes : (int64_t)(0.9 * (double)freeb);
  const int64_t ncols = trial->nfun;
  const int64_t per_col = 2 * (int64_t)std::max(1, nT) * o.LS * (int64_t)lsz + (host_out ? nrows * (int64_t)esz : 0);
  int64_t cols_per_block = std::max<int64_t>(1, std::min<int64_t>(ncols, budget / 2 / std::max<int64_t>(1, per_col)));
  if (host_out) {
    // host outputs: about 8 blocks (of at least 32 MiB), each copied on the copy stream while the
    // next block is computed; two staging slots
    const int64_t min_cols = ((int64_t)32 << 20) / std::max<int64_t>(1, nrows * (int64_t)esz);
    cols_per_block = std::min(cols_per_block, std::max<int64_t>((ncols + 7) / 8, std::max<int64_t>(1, min_cols)));
  }
  // Block boundaries.  With host outputs the last block is cut to about a quarter: its copy is
  // the one not hidden behind the next block's kernels.
  std::vector<int64_t> col_start;
  for (int64_t c = 0; c < ncols; c += cols_per_block) col_start.push_back(c);
  if (host_out && col_start.size() >= 4) {
    const int64_t last = std::max<int64_t>(1, ncols - std::max<int64_t>(1, (cols_per_block + 3) / 4));
    if (last > col_start.back()) col_start.push_back(last);
  }
  col_start.push_back(ncols);
  double ms_cls = 0, ms_far = 0, ms_sp = 0, ms_copy_acc = 0;
  int pending[2] = {0, 0};  // staging slot holds a copy in flight
  auto finish_copy = [&](int slot) -> int {
    if (!pending[slot]) return 0;
    BGB_CUDA(cudaEventSynchronize(h->ev2[4 * slot + 2]));
    ms_copy_acc += event_ms(h->ev2[4 * slot + 1], h->ev2[4 * slot + 2]);
    pending[slot] = 0;
    return 0;
  };
  std::vector<unsigned char> seen((size_t)trial->ns, 0);
  int64_t computed = 0, nonfar[5] = {0, 0, 0, 0, 0};
  int nblocks = 0;
  int cap = std::max(1 << 16, 8 * nT);
  // the block loop; on any early return the copies still in flight are drained below
  auto run_blocks = [&]() -> int {
  for (size_t bi = 0; bi + 1 < col_start.size(); ++bi) {
    if (h->abort_host && *h->abort_host) { set_error("aborted by bgb_abort"); return BGB_ERR_ABORTED; }
    const int64_t c0 = col_start[bi], c1 = col_start[bi + 1];
    ++nblocks;
    CurveSupports BS = curve_supports(trial, c0, c1);
    std::vector<int> S, bcode;
    localise(BS, S, bcode, scratch);
    const int nS = (int)S.size();
    std::vector<unsigned char> own((size_t)std::max(1, nS));
    for (int k = 0; k < nS; ++k) {
      own[(size_t)k] = !seen[(size_t)S[(size_t)k]];
      seen[(size_t)S[(size_t)k]] = 1;
    }
    std::vector<float> bcoef_f(BS.coef.begin(), BS.coef.end());
    if ((rc = put(s, B.S, S)) || (rc = put(s, B.own, own)) || (rc = put(s, B.bsup_off, BS.off)) ||
        (rc = put(s, B.bsup_i, bcode)) || (rc = (fp32_l ? put(s, B.bsup_c, bcoef_f) : put(s, B.bsup_c, BS.coef))))
      return rc;
    const int64_t npairs = (int64_t)nT * nS;
    computed += npairs;
    if ((rc = B.L.ensure(lsz * (size_t)std::max<int64_t>(1, npairs * o.LS)))) return rc;
    if ((rc = B.counts.ensure(sizeof(int) * 8))) return rc;
    const size_t mask_bytes = sizeof(unsigned) * (size_t)((npairs + 31) / 32);
    if ((rc = B.mask.ensure(std::max<size_t>(4, mask_bytes)))) return rc;
    int counts[8] = {0};
    if (nT > 0 && nS > 0) {
      for (int attempt = 0; attempt < 2; ++attempt) {
        if ((rc = B.list.ensure(sizeof(Special) * (size_t)cap))) return rc;
        BGB_CUDA(cudaMemsetAsync(B.counts.p, 0, sizeof(int) * 8, s));
        BGB_CUDA(cudaMemsetAsync(B.mask.p, 0, mask_bytes, s));
        BGB_CUDA(cudaEventRecord(h->ev[0], s));
        dim3 grid((nT + 255) / 256, std::min(nS, 65535));
        k_curve_classify<<<grid, 256, 0, s>>>(B.geo_t.as<SegGeo>(), B.geo_b.as<SegGeo>(), B.geof_t.as<SegF>(),
                                              B.geof_b.as<SegF>(), B.T.as<int>(), nT, B.S.as<int>(),
                                              nS, B.own.as<unsigned char>(), o.k2, o.LS, B.list.as<Special>(), cap,
                                              B.counts.as<int>(), B.mask.as<unsigned>());
        BGB_CUDA(cudaGetLastError());
        BGB_CUDA(cudaEventRecord(h->ev[1], s));
        // through the mapped mailbox: a copy would wait behind the previous block's output copy
        launch_publish(B.counts.as<int>(), 8, h->mbox_dev, s);
        BGB_CUDA(cudaGetLastError());
        BGB_CUDA(cudaStreamSynchronize(s));
        for (int c = 0; c < 8; ++c) counts[c] = h->mbox_host[c];
        ms_cls += event_ms(h->ev[0], h->ev[1]);
        ++launches;
        if (counts[1]) { set_error("degenerate geometry: a segment pair shares more than two vertices"); return BGB_ERR_INVALID; }
        if (counts[0] <= cap) break;
        cap = counts[0];
      }
      if (counts[0] > cap) { set_error("non-far pair list overflow"); return BGB_ERR_CAPACITY; }
      for (int c = 1; c < 5; ++c) nonfar[c] += counts[2 + c];
      BGB_CUDA(cudaEventRecord(h->ev[2], s));
      if (precision == BGB_PREC_MIXED) {
        BGB_CURVE_DISPATCH(o.kind, launch_far_mixed, o, B.rules.as<Rules>(), B.geof_t.as<SegF>(), B.geof_b.as<SegF>(),
                           B.T.as<int>(), nT, B.S.as<int>(), nS, B.mask.as<unsigned>(), B.L.as<float2>(), s);
      } else {
        BGB_CURVE_DISPATCH(o.kind, launch_far, o, B.rules.as<Rules>(), B.geo_t.as<SegGeo>(), B.geo_b.as<SegGeo>(),
                           B.T.as<int>(), nT, B.S.as<int>(), nS, B.mask.as<unsigned>(), B.L.as<double2>(), s);
      }
      BGB_CUDA(cudaGetLastError());
      BGB_CUDA(cudaEventRecord(h->ev[3], s));
      BGB_CURVE_DISPATCH(o.kind, launch_special, o, B.rules.as<Rules>(), fp32_l ? B.rulesdf.as<RulesDF>() : nullptr,
                         B.geo_t.as<SegGeo>(), B.geo_b.as<SegGeo>(), B.list.as<Special>(), counts[0], B.L.p, fp32_l,
                         h->num_sms, s);
      BGB_CUDA(cudaGetLastError());
      BGB_CUDA(cudaEventRecord(h->ev[4], s));
      launches += 1 + (counts[0] > 0);
    } else {
      BGB_CUDA(cudaEventRecord(h->ev[2], s));
      BGB_CUDA(cudaEventRecord(h->ev[3], s));
      BGB_CUDA(cudaEventRecord(h->ev[4], s));
    }
    // gather into the output (device) or the staging buffer (host)
    const int64_t bc = c1 - c0;
    const int slot = (nblocks - 1) & 1;
    DevBuf& stage = slot ? B.stage2 : B.stage;
    void* dst;
    int64_t dld;
    if (host_out) {
      if ((rc = finish_copy(slot))) return rc;  // the copy of block b - 2 left this slot
      if ((rc = stage.ensure(esz * (size_t)nrows * (size_t)cols_per_block))) return rc;
      dst = stage.p;
      dld = nrows;
    } else {
      dst = (char*)out + esz * (size_t)c0 * (size_t)ld;
      dld = ld;
    }
    dim3 gg((unsigned)((nrows + 255) / 256), (unsigned)std::min<int64_t>(bc, 65535));
#define BGB_CURVE_GATHER(OutT, LT)                                                                                 \
  k_curve_gather<OutT, LT><<<gg, 256, 0, s>>>(B.L.as<LT>(), nT, o.LS, o.nsB, (int)nrows, (int)bc,                       \
                                              B.tsup_off.as<int64_t>(), B.tsup_i.as<int>(),                             \
                                              B.tsup_c.as<decltype(LT::x)>(), B.bsup_off.as<int64_t>(),                 \
                                              B.bsup_i.as<int>(), B.bsup_c.as<decltype(LT::x)>(), (OutT*)dst, dld)
    if (c64 && !fp32_l) BGB_CURVE_GATHER(double2, double2);
    else if (c64) BGB_CURVE_GATHER(double2, float2);
    else if (!fp32_l) BGB_CURVE_GATHER(float2, double2);
    else BGB_CURVE_GATHER(float2, float2);
#undef BGB_CURVE_GATHER
    BGB_CUDA(cudaGetLastError());
    ++launches;
    BGB_CUDA(cudaEventRecord(h->ev[5], s));
    if (host_out) {
      // copy on the copy stream: the next block's classification and far pairs run meanwhile
      BGB_CUDA(cudaEventRecord(h->ev2[4 * slot], s));
      BGB_CUDA(cudaStreamWaitEvent(h->copy_stream, h->ev2[4 * slot], 0));
      BGB_CUDA(cudaEventRecord(h->ev2[4 * slot + 1], h->copy_stream));
      BGB_CUDA(cudaMemcpy2DAsync((char*)out + esz * (size_t)c0 * (size_t)ld, esz * (size_t)ld, stage.p,
                                 esz * (size_t)nrows, esz * (size_t)nrows, (size_t)bc, cudaMemcpyDeviceToHost,
                                 h->copy_stream));
      BGB_CUDA(cudaEventRecord(h->ev2[4 * slot + 2], h->copy_stream));
      pending[slot] = 1;
    }
    BGB_CUDA(cudaStreamSynchronize(s));
    ms_far += event_ms(h->ev[2], h->ev[3]) + event_ms(h->ev[4], h->ev[5]);
    ms_sp += event_ms(h->ev[3], h->ev[4]);
  }
  for (int k = 0; k < 2; ++k)
    if ((rc = finish_copy(k))) return rc;
  return 0;
  };
  rc = run_blocks();
  if (host_out) cudaStreamSynchronize(h->copy_stream);
  if (rc) return rc;
  if (!host_out && user != s) {
    BGB_CUDA(cudaEventRecord(h->ev[7], s));
    BGB_CUDA(cudaStreamWaitEvent(user, h->ev[7], 0));
  }
  st.pairs_total = (int64_t)nT * trial->ns;
  int64_t nf = 0;
  for (int c = 1; c < 5; ++c) {
    st.pairs_class[c] = nonfar[c];
    nf += nonfar[c];
  }
  st.pairs_class[0] = st.pairs_total - nf;
  st.pairs_computed = computed;
  st.ms_classify = ms_cls;
  st.ms_far = ms_far;
  st.ms_singular = ms_sp;
  st.ms_copy = ms_copy_acc;
  st.out_blocks = nblocks;
  st.tile_config = -1;
  st.kernel_launches = launches;
  st.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  st.ms_pipeline = st.ms_total;
  if (stats) *stats = st;
  return 0;
}

int bgb_local_matrices_curve(bgb_handle* h, const bgb_operator2d* op, const bgb_curve_space* test,
                             const bgb_curve_space* trial, const bgb_quadstrat2d* qs, int32_t precision,
                             int64_t npairs, const int32_t* tau, const int32_t* sigma, int32_t force_class,
                             double* out, int8_t* cls_out) {
  if (!h) { set_error("handle is NULL"); return BGB_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(h->mu);
  int rc;
  if ((rc = validate_curve(test, "test")) || (rc = validate_curve(trial, "trial"))) return rc;
  Op o;
  Rules R;
  if ((rc = make_op(op, test, trial, &o)) || (rc = make_rules(qs, &R))) return rc;
  if (precision != BGB_PREC_FP64 && precision != BGB_PREC_MIXED) { set_error("bad precision %d", precision); return BGB_ERR_INVALID; }
  if (precision == BGB_PREC_MIXED && (rc = check_mixed_range(op, test, trial))) return rc;
  if (npairs < 0 || (npairs > 0 && (!tau || !sigma || !out))) { set_error("invalid pair list"); return BGB_ERR_INVALID; }
  if (force_class != -1 && force_class != 0 && force_class != 1 && force_class != 3 && force_class != 4) {
    set_error("force_class %d is not a curve pair class", force_class);
    return BGB_ERR_INVALID;
  }
  if (npairs > (int64_t)1 << 28) { set_error("at most 2^28 pairs per call"); return BGB_ERR_INVALID; }
  std::vector<int2> pairs((size_t)npairs);
  for (int64_t p = 0; p < npairs; ++p) {
    if (tau[p] < 0 || tau[p] >= test->ns || sigma[p] < 0 || sigma[p] >= trial->ns) {
      set_error("pair %lld: segment index out of range", (long long)p);
      return BGB_ERR_INVALID;
    }
    pairs[(size_t)p] = make_int2(tau[p], sigma[p]);
  }
  if (npairs == 0) return 0;
  cudaSetDevice(h->device);
  cudaStream_t s = h->stream;
  CurveBufs& B = h->curve;
  if ((rc = upload_curve(s, test, B.verts_t, B.segs_t, B.geo_t, B.geof_t)) ||
      (rc = upload_curve(s, trial, B.verts_b, B.segs_b, B.geo_b, B.geof_b)))
    return rc;
  if ((rc = B.rules.ensure(sizeof(Rules)))) return rc;
  BGB_CUDA(cudaMemcpyAsync(B.rules.p, &R, sizeof(Rules), cudaMemcpyHostToDevice, s));
  RulesDF RD;
  make_rules_df(R, &RD);
  if ((rc = B.rulesdf.ensure(sizeof(RulesDF)))) return rc;
  BGB_CUDA(cudaMemcpyAsync(B.rulesdf.p, &RD, sizeof(RulesDF), cudaMemcpyHostToDevice, s));
  BGB_CUDA(cudaStreamSynchronize(s));  // RD lives on this stack frame
  if ((rc = put(s, B.pairs, pairs)) || (rc = B.out.ensure(sizeof(double2) * 4 * (size_t)npairs)) ||
      (rc = B.own.ensure((size_t)npairs)) || (rc = B.list.ensure(sizeof(Special) * (size_t)npairs)) ||
      (rc = B.counts.ensure(sizeof(int) * 8)))
    return rc;
  BGB_CUDA(cudaMemsetAsync(B.out.p, 0, sizeof(double2) * 4 * (size_t)npairs, s));
  BGB_CUDA(cudaMemsetAsync(B.counts.p, 0, sizeof(int) * 8, s));
  BGB_CURVE_DISPATCH(o.kind, launch_pairs, o, B.rules.as<Rules>(), B.geo_t.as<SegGeo>(), B.geo_b.as<SegGeo>(),
                     B.geof_t.as<SegF>(), B.geof_b.as<SegF>(), B.pairs.as<int2>(), npairs, force_class, precision == BGB_PREC_MIXED ? 1 : 0,
                     B.out.as<double2>(), (signed char*)B.own.p,
                     B.list.as<Special>(), B.counts.as<int>(), s);
  BGB_CUDA(cudaGetLastError());
  int counts[8] = {0};
  BGB_CUDA(cudaMemcpyAsync(counts, B.counts.p, sizeof(int) * 8, cudaMemcpyDeviceToHost, s));
  BGB_CUDA(cudaStreamSynchronize(s));
  if (counts[1]) {
    set_error("a pair is degenerate or its forced rule does not match its class");
    return BGB_ERR_INVALID;
  }
  BGB_CURVE_DISPATCH(o.kind, launch_special, o, B.rules.as<Rules>(),
                     precision == BGB_PREC_MIXED ? B.rulesdf.as<RulesDF>() : nullptr, B.geo_t.as<SegGeo>(),
                     B.geo_b.as<SegGeo>(), B.list.as<Special>(), counts[0], B.out.p, false, h->num_sms, s);
  BGB_CUDA(cudaGetLastError());
  std::vector<double2> L((size_t)npairs * 4);
  std::vector<signed char> cls((size_t)npairs);
  BGB_CUDA(cudaMemcpyAsync(L.data(), B.out.p, sizeof(double2) * L.size(), cudaMemcpyDeviceToHost, s));
  BGB_CUDA(cudaMemcpyAsync(cls.data(), B.own.p, (size_t)npairs, cudaMemcpyDeviceToHost, s));
  BGB_CUDA(cudaStreamSynchronize(s));
  for (int64_t p = 0; p < npairs; ++p) {
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) {
        double2 v = make_double2(0.0, 0.0);
        if (i < o.nsA && j < o.nsB) v = L[(size_t)p * 4 + i * o.nsB + j];
        out[p * 8 + (i * 2 + j) * 2] = v.x;
        out[p * 8 + (i * 2 + j) * 2 + 1] = v.y;
      }
    if (cls_out) cls_out[p] = cls[(size_t)p];
  }
  return 0;
}

}  // extern "C"
