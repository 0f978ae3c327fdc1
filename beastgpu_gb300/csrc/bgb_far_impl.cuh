// Far-pair tile kernels (plain FP64 and mixed FP32) with the deterministic gather write.
//
// A CTA owns one output tile: a block of test functions (rows) x a block of trial
// functions (columns), each a compact patch of a recursive coordinate bisection of the functions.
// It stages the triangles supporting those functions ("halo" included) in shared memory,
// sweeps the trial triangles in chunks, computes the 3x3 local matrix of every (test
// triangle, trial triangle) pair of the chunk into shared memory, and then lets each thread
// add the chunk's contributions to the output entries it owns.  Every entry Z[m, n]
// therefore accumulates its contributions in one fixed order -- trial triangle ascending,
// then test triangle ascending -- no matter how the tiles are shaped: results are
// bit-identical across tile configurations and runs, with no atomics.  Each output entry is
// written exactly once.  Non-far pairs (singular or near, found by the classifier) are
// taken from the FP64 singular-pair buffer instead of the far rule.
//
// Roofline: compute-bound on FP32 issue (mixed) or FP64 issue (plain), plus MUFU
// (rsqrt, rcp, sin, cos).  Per point pair the mixed kernel spends ~23 FP32 ops + 4 MUFU on
// the kernel value and 13 (Helmholtz / EFIE) or ~26 (MFIE) on accumulation.
//
// Mixed precision (FP32) keeps the phase k R accurate without FP64: per pair, the centroid
// distance D = c_tau - c_sigma is formed in double-float, R0 is any FP32 number close to |D|,
// and phi0 = k R0 mod 2 pi is reduced exactly (Dekker product + Cody-Waite); per point pair
// only delta = R - R0 = q / (R + R0) with q = |D_hi + s|^2 - R0^2 computed cancellation-free
// in FP32 enters the phase (psi = phi0 + k delta), so the absolute phase error stays ~1e-7
// rad regardless of k R.  Shape functions use coordinates relative to each triangle's
// centroid, so the EFIE/MFIE bilinear forms carry no cancellation either.
// Far-pair kernel templates; instantiated per precision and operator in bgb_far_*_op*.cu.
#pragma once
#include "bgb_kernels.cuh"

#include <algorithm>

namespace bgb {
namespace farimpl {

constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr float kPiA = 6.28125f;
constexpr float kPiB = (float)(kTwoPi - 6.28125);
constexpr float kPiC = (float)(kTwoPi - 6.28125 - (double)(float)(kTwoPi - 6.28125));
constexpr float kInv2Pi = (float)(1.0 / kTwoPi);
constexpr int kThreads = 256;

// Hardware approximations (PTX .approx with flush-to-zero).  Their arguments in the FP32 pair loop
// are normal numbers (squared distances, sums of distances, phases within a few pi), so the
// denormal handling that the non-flushing forms add to each call is dead weight there.
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_ftz(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ void sincos_ftz(float x, float* s, float* c) {
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(*s) : "f"(x));
  asm("cos.approx.ftz.f32 %0, %1;" : "=f"(*c) : "f"(x));
}
// e^x = 2^(x log2 e)
__device__ __forceinline__ float exp_ftz(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x * 1.4426950408889634f));
  return y;
}

// Operators on Lagrange hats: Helmholtz single layer, double layer, transposed double layer,
// hypersingular.  They share the hat accumulation of the single layer.
__host__ __device__ constexpr bool is_lagrange_op(int op) {
  return op == BGB_OP_HELMHOLTZ3D_SL || op == BGB_OP_HELMHOLTZ3D_DL || op == BGB_OP_HELMHOLTZ3D_DLT ||
         op == BGB_OP_HELMHOLTZ3D_HS;
}
// Unit normal (v0 - v2) x (v1 - v2) / (2A) from the centroid-relative vertices vo[3][3].
template <class T>
__device__ __forceinline__ void tri_normal(const T* vo, T inv2a, T n[3]) {
  const T a0 = vo[0] - vo[6], a1 = vo[1] - vo[7], a2 = vo[2] - vo[8];
  const T b0 = vo[3] - vo[6], b1 = vo[4] - vo[7], b2 = vo[5] - vo[8];
  n[0] = (a1 * b2 - a2 * b1) * inv2a;
  n[1] = (a2 * b0 - a0 * b2) * inv2a;
  n[2] = (a0 * b1 - a1 * b0) * inv2a;
}
// Surface curls of the hats, n x grad(lambda_i) = (v_{i+1} - v_{i+2}) / (2A).
template <class T>
__device__ __forceinline__ void tri_curls(const T* vo, T inv2a, T c[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) c[i][k] = (vo[3 * ((i + 1) % 3) + k] - vo[3 * ((i + 2) % 3) + k]) * inv2a;
}

// FP32 record of a triangle, in 16-byte groups read with 128-bit shared-memory loads:
// [CH.xyz CL.x] [CL.yz - -] [x y z w] per quadrature point [VO (9) INV2A - -]; the stride is an odd
// number of groups, so the records of different triangles start in different bank groups.
template <int Q>
struct Off32 {
  static constexpr int CH = 0, CL = 3, X = 8, PS = 4, VO = 8 + 4 * Q, INV2A = VO + 9, SIZE = 4 * ((5 + Q) | 1);
  static constexpr int px(int I) { return X + PS * I; }      // point I: x, y, z
  static constexpr int pw(int I) { return X + PS * I + 3; }  // point I: weight
};
__host__ __device__ constexpr int off32_size(int Q) { return 4 * ((5 + Q) | 1); }
template <int Q>
struct Off64 {
  static constexpr int C = 0, X = 3, W = 3 + 3 * Q, VO = 3 + 4 * Q, INV2A = 12 + 4 * Q, SIZE = 13 + 4 * Q;
};

struct PMixed {
  using R = float;
  using C = float2;
  static constexpr int kMinBlocks = 3;  // 3 CTAs of 256 threads per SM (<= 85 registers)
  template <int Q>
  static constexpr int rec() { return Off32<Q>::SIZE; }
  static __device__ __forceinline__ C mk(double a, double b) { return make_float2((float)a, (float)b); }
};
struct PFp64 {
  using R = double;
  using C = double2;
  static constexpr int kMinBlocks = 1;
  template <int Q>
  static constexpr int rec() { return Off64<Q>::SIZE; }
  static __device__ __forceinline__ C mk(double a, double b) { return make_double2(a, b); }
};

// ----------------------------------------------------------------------------------------
// Mixed FP32 far pair
// ----------------------------------------------------------------------------------------
// the 9 vertex offsets of an FP32 record (three 16-byte groups)
__device__ __forceinline__ void load_vo(const float4* __restrict__ g, float V[3][3]) {
  const float4 v0 = g[0], v1 = g[1], v2 = g[2];
  V[0][0] = v0.x; V[0][1] = v0.y; V[0][2] = v0.z;
  V[1][0] = v0.w; V[1][1] = v1.x; V[1][2] = v1.y;
  V[2][0] = v1.z; V[2][1] = v1.w; V[2][2] = v2.x;
}

template <int OP, int QT, int QB>
__device__ __forceinline__ void far_pair_mixed(const FarScalars& K, const float (*__restrict__ shpT)[3],
                                               const float (*__restrict__ shpB)[3], const float* __restrict__ a,
                                               const float* __restrict__ b, float2 L[9]) {
  using OA = Off32<QT>;
  using OB = Off32<QB>;
  const float4* __restrict__ a4 = reinterpret_cast<const float4*>(a);
  const float4* __restrict__ b4 = reinterpret_cast<const float4*>(b);
  float Dh[3], Dl[3];
  {
    const float4 a0 = a4[0], a1 = a4[1], b0 = b4[0], b1 = b4[1];
    const float ach[3] = {a0.x, a0.y, a0.z}, acl[3] = {a0.w, a1.x, a1.y};
    const float bch[3] = {b0.x, b0.y, b0.z}, bcl[3] = {b0.w, b1.x, b1.y};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float s, e;
      two_sum(ach[c], -bch[c], s, e);
      e = __fadd_rn(e, __fsub_rn(acl[c], bcl[c]));
      fast_two_sum(s, e, Dh[c], Dl[c]);
    }
  }
  const float n2 = fmaf(Dh[0], Dh[0], fmaf(Dh[1], Dh[1], Dh[2] * Dh[2]));
  const float R0 = n2 * rsqrt_ftz(n2);
  // c0 = |D_hi|^2 - R0^2, exact to double-float accuracy
  float p0, e0, p1, e1, p2, e2, s1, f1, s2, f2, r2h, r2l;
  two_prod(Dh[0], Dh[0], p0, e0);
  two_prod(Dh[1], Dh[1], p1, e1);
  two_prod(Dh[2], Dh[2], p2, e2);
  two_sum(p0, p1, s1, f1);
  two_sum(s1, p2, s2, f2);
  const float lo = __fadd_rn(__fadd_rn(__fadd_rn(f1, f2), __fadd_rn(e0, e1)), e2);
  two_prod(R0, R0, r2h, r2l);
  const float c0 = __fadd_rn(__fsub_rn(s2, r2h), __fsub_rn(lo, r2l));
  // phi0 = k R0 mod 2 pi
  float ph, pl;
  two_prod(K.k_hi, R0, ph, pl);
  pl = fmaf(K.k_lo, R0, pl);
  const float nq = rintf(ph * kInv2Pi);
  float phi0 = fmaf(-nq, kPiA, ph);
  phi0 = fmaf(-nq, kPiB, phi0);
  phi0 = fmaf(-nq, kPiC, phi0);
  phi0 = __fadd_rn(phi0, pl);
  const float R0sq = R0 * R0;
  const float D2x = 2.f * Dh[0], D2y = 2.f * Dh[1], D2z = 2.f * Dh[2];
  const float kh = K.k_hi;
  const float amp0 = K.lossy ? exp_ftz(-K.gre * R0) : 1.f;
  constexpr bool kHH = is_lagrange_op(OP);
  float nA[3] = {0.f, 0.f, 0.f}, nB[3] = {0.f, 0.f, 0.f};
  if (OP == BGB_OP_HELMHOLTZ3D_DLT || OP == BGB_OP_HELMHOLTZ3D_HS) tri_normal(a + OA::VO, a[OA::INV2A], nA);
  if (OP == BGB_OP_HELMHOLTZ3D_DL || OP == BGB_OP_HELMHOLTZ3D_HS) tri_normal(b + OB::VO, b[OB::INV2A], nB);
  const int qt = QT < BGB_MAXQ ? QT : K.qt;
  const int qb = QB < BGB_MAXQ ? QB : K.qb;

  // accumulators
  float2 S = make_float2(0.f, 0.f), P0 = make_float2(0.f, 0.f);
  float2 Px[3], Py[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) Px[c] = Py[c] = make_float2(0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 9; ++k) L[k] = make_float2(0.f, 0.f);

  if constexpr (OP != BGB_OP_MAXWELL3D_DL) {
    // Helmholtz / EFIE: q = s.(2 D_hi + s) with s = a_I - y_J, a_I = D_lo + x_I, split as
    //   q = [c0 + a_I.(a_I + 2 D_hi)] + [y_J.(y_J - 2 D_hi)] - 2 a_I.y_J
    // (per test point, per trial point, per point pair): 5 operations per point pair.
    // trial points of the pair in registers when the rule is small (shared-memory loads otherwise)
    constexpr int QY = QB <= 4 ? QB : 1;
    float MJ[QY];
    if constexpr (QB <= 4) {
#pragma unroll
      for (int J = 0; J < QB; ++J) {
        if (J >= qb) break;
        const float4 y = b4[OB::px(J) / 4];
        MJ[J] = fmaf(y.x, y.x - D2x, fmaf(y.y, y.y - D2y, y.z * (y.z - D2z)));
      }
    }
#pragma unroll
    for (int I = 0; I < QT; ++I) {
      if (I >= qt) break;
      const float4 XI = a4[OA::px(I) / 4];
      const float Xx = XI.x, Xy = XI.y, Xz = XI.z;
      const float ax = Dl[0] + Xx, ay = Dl[1] + Xy, az = Dl[2] + Xz;
      const float KI = fmaf(ax, ax + D2x, fmaf(ay, ay + D2y, fmaf(az, az + D2z, c0)));
      const float wI = XI.w;
      // double layer: (x - y) . n_y = (D + X_I) . n_y, constant over the trial points
      const float cI = OP == BGB_OP_HELMHOLTZ3D_DL
                           ? fmaf(Dh[0] + ax, nB[0], fmaf(Dh[1] + ay, nB[1], (Dh[2] + az) * nB[2]))
                           : 1.f;
      float2 TI = make_float2(0.f, 0.f);
      float2 UI[3], M[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) UI[c] = M[c] = make_float2(0.f, 0.f);
#pragma unroll
      for (int J = 0; J < QB; ++J) {
        if (J >= qb) break;
        const float4 YJ = b4[OB::px(J) / 4];
        const float yx = YJ.x, yy = YJ.y, yz = YJ.z;
        float mj;
        if constexpr (QB <= 4) mj = MJ[J];
        else mj = fmaf(yx, yx - D2x, fmaf(yy, yy - D2y, yz * (yz - D2z)));
        const float dot = fmaf(ax, yx, fmaf(ay, yy, az * yz));
        const float q = fmaf(-2.f, dot, KI + mj);
        const float R2 = R0sq + q;
        const float rs = rsqrt_ftz(R2);
        const float delta = q * rcp_ftz(fmaf(R2, rs, R0));
        float psi = fmaf(kh, delta, phi0);
        if (!K.phase_direct) {  // |psi| may exceed 2 pi: reduce again
          const float nn = rintf(psi * kInv2Pi);
          psi = fmaf(-nn, kPiA, psi);
          psi = fmaf(-nn, kPiB, psi);
        }
        float sn, cs;
        sincos_ftz(psi, &sn, &cs);
        float amp = (wI * YJ.w) * rs;
        if (K.lossy) amp *= amp0 * exp_ftz(-K.gre * delta);
        const float gr = amp * cs, gi = -amp * sn;
        if (kHH) {
          float hr = gr, hi = gi;
          if (OP == BGB_OP_HELMHOLTZ3D_DL || OP == BGB_OP_HELMHOLTZ3D_DLT) {
            // (gamma + 1/R) G / R, times -(x - y) . n_x = -(D - y_J) . n_x for the transposed layer
            const float t = (K.gre + rs) * rs, u = kh * rs;
            hr = t * gr - u * gi;
            hi = t * gi + u * gr;
            if (OP == BGB_OP_HELMHOLTZ3D_DLT) {
              const float e = -fmaf(Dh[0] + (Dl[0] - yx), nA[0], fmaf(Dh[1] + (Dl[1] - yy), nA[1], (Dh[2] + (Dl[2] - yz)) * nA[2]));
              hr *= e;
              hi *= e;
            }
          }
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const float g = shpB[J][j];
            M[j].x = fmaf(hr, g, M[j].x);
            M[j].y = fmaf(hi, g, M[j].y);
          }
        } else {
          TI.x += gr;
          TI.y += gi;
          UI[0].x = fmaf(gr, yx, UI[0].x); UI[0].y = fmaf(gi, yx, UI[0].y);
          UI[1].x = fmaf(gr, yy, UI[1].x); UI[1].y = fmaf(gi, yy, UI[1].y);
          UI[2].x = fmaf(gr, yz, UI[2].x); UI[2].y = fmaf(gi, yz, UI[2].y);
        }
      }
      if (kHH) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const float f = shpT[I][i] * cI;
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            L[i * 3 + j].x = fmaf(f, M[j].x, L[i * 3 + j].x);
            L[i * 3 + j].y = fmaf(f, M[j].y, L[i * 3 + j].y);
          }
        }
      } else {
        S.x = fmaf(Xx, UI[0].x, fmaf(Xy, UI[1].x, fmaf(Xz, UI[2].x, S.x)));
        S.y = fmaf(Xx, UI[0].y, fmaf(Xy, UI[1].y, fmaf(Xz, UI[2].y, S.y)));
        Px[0].x = fmaf(Xx, TI.x, Px[0].x); Px[0].y = fmaf(Xx, TI.y, Px[0].y);
        Px[1].x = fmaf(Xy, TI.x, Px[1].x); Px[1].y = fmaf(Xy, TI.y, Px[1].y);
        Px[2].x = fmaf(Xz, TI.x, Px[2].x); Px[2].y = fmaf(Xz, TI.y, Px[2].y);
#pragma unroll
        for (int c = 0; c < 3; ++c) { Py[c].x += UI[c].x; Py[c].y += UI[c].y; }
        P0.x += TI.x;
        P0.y += TI.y;
      }
    }
  } else {
#pragma unroll
  for (int I = 0; I < QT; ++I) {
    if (I >= qt) break;
    const float4 XI = a4[OA::px(I) / 4];
    const float Xx = XI.x, Xy = XI.y, Xz = XI.z;
    const float ax = Dl[0] + Xx, ay = Dl[1] + Xy, az = Dl[2] + Xz;
    const float wI = XI.w;
    float2 TI = make_float2(0.f, 0.f);
    float2 UI[3], EI[3], BI[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) UI[c] = EI[c] = BI[c] = make_float2(0.f, 0.f);
    float2 M[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) M[c] = make_float2(0.f, 0.f);
#pragma unroll
    for (int J = 0; J < QB; ++J) {
      if (J >= qb) break;
      const float4 YJ = b4[OB::px(J) / 4];
      const float Yx = YJ.x, Yy = YJ.y, Yz = YJ.z;
      const float sx = ax - Yx, sy = ay - Yy, sz = az - Yz;
      const float q = fmaf(sx, D2x + sx, fmaf(sy, D2y + sy, fmaf(sz, D2z + sz, c0)));
      const float R2 = R0sq + q;
      const float rs = rsqrt_ftz(R2);
      const float Rr = R2 * rs;
      const float delta = q * rcp_ftz(Rr + R0);
      float psi = fmaf(kh, delta, phi0);
      const float nn = rintf(psi * kInv2Pi);
      psi = fmaf(-nn, kPiA, psi);
      psi = fmaf(-nn, kPiB, psi);
      float sn, cs;
      sincos_ftz(psi, &sn, &cs);
      float amp = wI * YJ.w * rs;
      if (K.lossy) amp *= amp0 * exp_ftz(-K.gre * delta);
      const float gr = amp * cs, gi = -amp * sn;
      if (OP == BGB_OP_HELMHOLTZ3D_SL) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float g = shpB[J][j];
          M[j].x = fmaf(gr, g, M[j].x);
          M[j].y = fmaf(gi, g, M[j].y);
        }
      } else if (OP == BGB_OP_MAXWELL3D_SL) {
        TI.x += gr;
        TI.y += gi;
        UI[0].x = fmaf(gr, Yx, UI[0].x); UI[0].y = fmaf(gi, Yx, UI[0].y);
        UI[1].x = fmaf(gr, Yy, UI[1].x); UI[1].y = fmaf(gi, Yy, UI[1].y);
        UI[2].x = fmaf(gr, Yz, UI[2].x); UI[2].y = fmaf(gi, Yz, UI[2].y);
      } else {
        // H = -(gamma + 1/R) G / R ; d = x - y
        const float g2r = gr * rs, g2i = gi * rs;
        const float re = K.gre + rs;
        const float Hx = -(re * g2r - kh * g2i), Hy = -(re * g2i + kh * g2r);
        const float dx = Dh[0] + sx, dy = Dh[1] + sy, dz = Dh[2] + sz;
        EI[0].x = fmaf(Hx, dx, EI[0].x); EI[0].y = fmaf(Hy, dx, EI[0].y);
        EI[1].x = fmaf(Hx, dy, EI[1].x); EI[1].y = fmaf(Hy, dy, EI[1].y);
        EI[2].x = fmaf(Hx, dz, EI[2].x); EI[2].y = fmaf(Hy, dz, EI[2].y);
        const float c0x = dy * Yz - dz * Yy, c0y = dz * Yx - dx * Yz, c0z = dx * Yy - dy * Yx;
        BI[0].x = fmaf(Hx, c0x, BI[0].x); BI[0].y = fmaf(Hy, c0x, BI[0].y);
        BI[1].x = fmaf(Hx, c0y, BI[1].x); BI[1].y = fmaf(Hy, c0y, BI[1].y);
        BI[2].x = fmaf(Hx, c0z, BI[2].x); BI[2].y = fmaf(Hy, c0z, BI[2].y);
      }
    }
    if (OP == BGB_OP_HELMHOLTZ3D_SL) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float f = shpT[I][i];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          L[i * 3 + j].x = fmaf(f, M[j].x, L[i * 3 + j].x);
          L[i * 3 + j].y = fmaf(f, M[j].y, L[i * 3 + j].y);
        }
      }
    } else if (OP == BGB_OP_MAXWELL3D_SL) {
      S.x = fmaf(Xx, UI[0].x, fmaf(Xy, UI[1].x, fmaf(Xz, UI[2].x, S.x)));
      S.y = fmaf(Xx, UI[0].y, fmaf(Xy, UI[1].y, fmaf(Xz, UI[2].y, S.y)));
      Px[0].x = fmaf(Xx, TI.x, Px[0].x); Px[0].y = fmaf(Xx, TI.y, Px[0].y);
      Px[1].x = fmaf(Xy, TI.x, Px[1].x); Px[1].y = fmaf(Xy, TI.y, Px[1].y);
      Px[2].x = fmaf(Xz, TI.x, Px[2].x); Px[2].y = fmaf(Xz, TI.y, Px[2].y);
#pragma unroll
      for (int c = 0; c < 3; ++c) { Py[c].x += UI[c].x; Py[c].y += UI[c].y; }
      P0.x += TI.x;
      P0.y += TI.y;
    } else {
      // C += X x E_I (stored in Px), A1 += X . B_I (stored in S), B += B_I (Py), E += E_I (stored via L[0..2])
      Px[0].x += Xy * EI[2].x - Xz * EI[1].x; Px[0].y += Xy * EI[2].y - Xz * EI[1].y;
      Px[1].x += Xz * EI[0].x - Xx * EI[2].x; Px[1].y += Xz * EI[0].y - Xx * EI[2].y;
      Px[2].x += Xx * EI[1].x - Xy * EI[0].x; Px[2].y += Xx * EI[1].y - Xy * EI[0].y;
      S.x = fmaf(Xx, BI[0].x, fmaf(Xy, BI[1].x, fmaf(Xz, BI[2].x, S.x)));
      S.y = fmaf(Xx, BI[0].y, fmaf(Xy, BI[1].y, fmaf(Xz, BI[2].y, S.y)));
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        Py[c].x += BI[c].x; Py[c].y += BI[c].y;
        L[c].x += EI[c].x; L[c].y += EI[c].y;
      }
    }
  }

  }
  const float2 alpha = make_float2(K.alpha32[0], K.alpha32[1]);
  if (OP == BGB_OP_HELMHOLTZ3D_HS) {
    // alpha (n_x . n_y) int int f g G + beta (curl f . curl g) int int G, int int G = sum of L
    float2 P = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 9; ++k) { P.x += L[k].x; P.y += L[k].y; }
    const float nn = fmaf(nA[0], nB[0], fmaf(nA[1], nB[1], nA[2] * nB[2]));
    const float2 an = make_float2(alpha.x * nn, alpha.y * nn);
    const float2 bP = cmulf(make_float2(K.beta32[0], K.beta32[1]), P);
    float cA[3][3], cB[3][3];
    tri_curls(a + OA::VO, a[OA::INV2A], cA);
    tri_curls(b + OB::VO, b[OB::INV2A], cB);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float cc = fmaf(cA[i][0], cB[j][0], fmaf(cA[i][1], cB[j][1], cA[i][2] * cB[j][2]));
        const float2 t = cmulf(an, L[i * 3 + j]);
        L[i * 3 + j] = make_float2(fmaf(cc, bP.x, t.x), fmaf(cc, bP.y, t.y));
      }
    return;
  }
  if (kHH) {
#pragma unroll
    for (int k = 0; k < 9; ++k) L[k] = cmulf(alpha, L[k]);
    return;
  }
  const float inv4AA = a[OA::INV2A] * b[OB::INV2A];
  const float2 ca = make_float2(alpha.x * inv4AA, alpha.y * inv4AA);
  if (OP == BGB_OP_MAXWELL3D_SL) {
    // L_ij = alpha/(4 A A) (S - V_i.Py - W_j.Px + (V_i.W_j) P0) + beta/(A A) P0
    const float invAA = 4.f * inv4AA;
    const float2 cb = make_float2(K.beta32[0] * invAA, K.beta32[1] * invAA);
    const float2 tb = cmulf(cb, P0);
    float V[3][3], W[3][3];
    load_vo(a4 + OA::VO / 4, V);
    load_vo(b4 + OB::VO / 4, W);
    float2 Ai[3], Bj[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      Ai[i].x = S.x - fmaf(V[i][0], Py[0].x, fmaf(V[i][1], Py[1].x, V[i][2] * Py[2].x));
      Ai[i].y = S.y - fmaf(V[i][0], Py[0].y, fmaf(V[i][1], Py[1].y, V[i][2] * Py[2].y));
      Bj[i].x = fmaf(W[i][0], Px[0].x, fmaf(W[i][1], Px[1].x, W[i][2] * Px[2].x));
      Bj[i].y = fmaf(W[i][0], Px[0].y, fmaf(W[i][1], Px[1].y, W[i][2] * Px[2].y));
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float vw = fmaf(V[i][0], W[j][0], fmaf(V[i][1], W[j][1], V[i][2] * W[j][2]));
        const float tx = fmaf(vw, P0.x, Ai[i].x - Bj[j].x);
        const float ty = fmaf(vw, P0.y, Ai[i].y - Bj[j].y);
        L[i * 3 + j] = make_float2(fmaf(ca.x, tx, fmaf(-ca.y, ty, tb.x)), fmaf(ca.x, ty, fmaf(ca.y, tx, tb.y)));
      }
    return;
  }
  // MFIE: L = alpha/(4AA) (A1 - W_j . C - V_i . B + V_i . (E x W_j))
  const float2 E0 = L[0], E1 = L[1], E2 = L[2];
  float2 vb[3], wc[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float vx = a[OA::VO + 3 * i], vy = a[OA::VO + 3 * i + 1], vz = a[OA::VO + 3 * i + 2];
    vb[i].x = vx * Py[0].x + vy * Py[1].x + vz * Py[2].x;
    vb[i].y = vx * Py[0].y + vy * Py[1].y + vz * Py[2].y;
    const float wx = b[OB::VO + 3 * i], wy = b[OB::VO + 3 * i + 1], wz = b[OB::VO + 3 * i + 2];
    wc[i].x = wx * Px[0].x + wy * Px[1].x + wz * Px[2].x;
    wc[i].y = wx * Px[0].y + wy * Px[1].y + wz * Px[2].y;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float wx = b[OB::VO + 3 * j], wy = b[OB::VO + 3 * j + 1], wz = b[OB::VO + 3 * j + 2];
    // E x W_j
    const float2 x0 = make_float2(E1.x * wz - E2.x * wy, E1.y * wz - E2.y * wy);
    const float2 x1 = make_float2(E2.x * wx - E0.x * wz, E2.y * wx - E0.y * wz);
    const float2 x2 = make_float2(E0.x * wy - E1.x * wx, E0.y * wy - E1.y * wx);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float vx = a[OA::VO + 3 * i], vy = a[OA::VO + 3 * i + 1], vz = a[OA::VO + 3 * i + 2];
      float2 t;
      t.x = S.x - wc[j].x - vb[i].x + (vx * x0.x + vy * x1.x + vz * x2.x);
      t.y = S.y - wc[j].y - vb[i].y + (vx * x0.y + vy * x1.y + vz * x2.y);
      L[i * 3 + j] = cmulf(ca, t);
    }
  }
}

// ----------------------------------------------------------------------------------------
// Plain FP64 far pair (same accumulation structure, FP64 throughout, CUDA sincos / exp)
// ----------------------------------------------------------------------------------------
template <int OP, int QT, int QB>
__device__ __forceinline__ void far_pair_fp64(const FarScalars& K, const double (*__restrict__ shpT)[3],
                                              const double (*__restrict__ shpB)[3], const double* __restrict__ tay_s,
                                              const double* __restrict__ tay_c, const double* __restrict__ a,
                                              const double* __restrict__ b, double2 L[9]) {
  using OA = Off64<QT>;
  using OB = Off64<QB>;
  constexpr bool kHH = is_lagrange_op(OP);
  const double Dx = a[OA::C] - b[OB::C], Dy = a[OA::C + 1] - b[OB::C + 1], Dz = a[OA::C + 2] - b[OB::C + 2];
  const double gre = K.gamma[0], gim = K.gamma[1];
  // Phase k R = k R0 + k (R - R0) with R0 the centroid distance: sin / cos of k R0 once per pair, and
  // of the small k (R - R0) (|.| <= 2) from K.tay_n series terms per point pair (sincos otherwise).
  const int tn = gim != 0.0 ? K.tay_n : 0;
  double R0 = 0.0, s0 = 0.0, c0 = 1.0;
  if (tn > 0) {
    R0 = sqrt(Dx * Dx + Dy * Dy + Dz * Dz);
    sincos(gim * R0, &s0, &c0);
  }
  double nA[3] = {0, 0, 0}, nB[3] = {0, 0, 0};
  if (OP == BGB_OP_HELMHOLTZ3D_DLT || OP == BGB_OP_HELMHOLTZ3D_HS) tri_normal(a + OA::VO, a[OA::INV2A], nA);
  if (OP == BGB_OP_HELMHOLTZ3D_DL || OP == BGB_OP_HELMHOLTZ3D_HS) tri_normal(b + OB::VO, b[OB::INV2A], nB);
  const int qt = QT < BGB_MAXQ ? QT : K.qt;
  const int qb = QB < BGB_MAXQ ? QB : K.qb;
  double2 S = make_double2(0, 0), P0 = make_double2(0, 0);
  double2 Px[3], Py[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) Px[c] = Py[c] = make_double2(0, 0);
#pragma unroll
  for (int k = 0; k < 9; ++k) L[k] = make_double2(0, 0);
#pragma unroll
  for (int I = 0; I < QT; ++I) {
    if (I >= qt) break;
    const double Xx = a[OA::X + 3 * I], Xy = a[OA::X + 3 * I + 1], Xz = a[OA::X + 3 * I + 2];
    const double ax = Dx + Xx, ay = Dy + Xy, az = Dz + Xz;
    const double wI = a[OA::W + I];
    // double layer: (x - y) . n_y = (D + X_I) . n_y, constant over the trial points
    const double cI = OP == BGB_OP_HELMHOLTZ3D_DL ? ax * nB[0] + ay * nB[1] + az * nB[2] : 1.0;
    double2 TI = make_double2(0, 0);
    double2 UI[3], EI[3], BI[3], M[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) UI[c] = EI[c] = BI[c] = M[c] = make_double2(0, 0);
#pragma unroll
    for (int J = 0; J < QB; ++J) {
      if (J >= qb) break;
      const double Yx = b[OB::X + 3 * J], Yy = b[OB::X + 3 * J + 1], Yz = b[OB::X + 3 * J + 2];
      const double dx = ax - Yx, dy = ay - Yy, dz = az - Yz;
      const double R2 = dx * dx + dy * dy + dz * dz;
      const double rinv = rsqrt(R2);
      const double R = R2 * rinv;
      double sn = 0.0, cs = 1.0;
      if (tn > 0) {
        const double x = gim * (R - R0), x2 = x * x;
        double ps = tay_s[tn - 1], pc = tay_c[tn - 1];
        for (int j = tn - 2; j >= 0; --j) {
          ps = fma(ps, x2, tay_s[j]);
          pc = fma(pc, x2, tay_c[j]);
        }
        const double s1 = x * ps;
        sn = fma(s0, pc, c0 * s1);  // sin(k R0 + x)
        cs = fma(c0, pc, -s0 * s1); // cos(k R0 + x)
      } else if (gim != 0.0) {
        sincos(gim * R, &sn, &cs);
      }
      double amp = wI * b[OB::W + J] * rinv;
      if (gre != 0.0) amp *= exp(-gre * R);
      const double gr = amp * cs, gi = -amp * sn;
      if (kHH) {
        double hr = gr, hi = gi;
        if (OP == BGB_OP_HELMHOLTZ3D_DL || OP == BGB_OP_HELMHOLTZ3D_DLT) {
          // (gamma + 1/R) G / R, times -(x - y) . n_x for the transposed double layer
          const double t = (gre + rinv) * rinv, u = gim * rinv;
          hr = t * gr - u * gi;
          hi = t * gi + u * gr;
          if (OP == BGB_OP_HELMHOLTZ3D_DLT) {
            const double e = -(dx * nA[0] + dy * nA[1] + dz * nA[2]);
            hr *= e;
            hi *= e;
          }
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const double g = shpB[J][j];
          M[j].x = fma(hr, g, M[j].x);
          M[j].y = fma(hi, g, M[j].y);
        }
      } else if (OP == BGB_OP_MAXWELL3D_SL) {
        TI.x += gr;
        TI.y += gi;
        UI[0].x = fma(gr, Yx, UI[0].x); UI[0].y = fma(gi, Yx, UI[0].y);
        UI[1].x = fma(gr, Yy, UI[1].x); UI[1].y = fma(gi, Yy, UI[1].y);
        UI[2].x = fma(gr, Yz, UI[2].x); UI[2].y = fma(gi, Yz, UI[2].y);
      } else {
        const double g2r = gr * rinv, g2i = gi * rinv;
        const double re = gre + rinv;
        const double Hx = -(re * g2r - gim * g2i), Hy = -(re * g2i + gim * g2r);
        EI[0].x = fma(Hx, dx, EI[0].x); EI[0].y = fma(Hy, dx, EI[0].y);
        EI[1].x = fma(Hx, dy, EI[1].x); EI[1].y = fma(Hy, dy, EI[1].y);
        EI[2].x = fma(Hx, dz, EI[2].x); EI[2].y = fma(Hy, dz, EI[2].y);
        const double c0x = dy * Yz - dz * Yy, c0y = dz * Yx - dx * Yz, c0z = dx * Yy - dy * Yx;
        BI[0].x = fma(Hx, c0x, BI[0].x); BI[0].y = fma(Hy, c0x, BI[0].y);
        BI[1].x = fma(Hx, c0y, BI[1].x); BI[1].y = fma(Hy, c0y, BI[1].y);
        BI[2].x = fma(Hx, c0z, BI[2].x); BI[2].y = fma(Hy, c0z, BI[2].y);
      }
    }
    if (kHH) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const double f = shpT[I][i] * cI;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          L[i * 3 + j].x = fma(f, M[j].x, L[i * 3 + j].x);
          L[i * 3 + j].y = fma(f, M[j].y, L[i * 3 + j].y);
        }
      }
    } else if (OP == BGB_OP_MAXWELL3D_SL) {
      S.x = fma(Xx, UI[0].x, fma(Xy, UI[1].x, fma(Xz, UI[2].x, S.x)));
      S.y = fma(Xx, UI[0].y, fma(Xy, UI[1].y, fma(Xz, UI[2].y, S.y)));
      Px[0].x = fma(Xx, TI.x, Px[0].x); Px[0].y = fma(Xx, TI.y, Px[0].y);
      Px[1].x = fma(Xy, TI.x, Px[1].x); Px[1].y = fma(Xy, TI.y, Px[1].y);
      Px[2].x = fma(Xz, TI.x, Px[2].x); Px[2].y = fma(Xz, TI.y, Px[2].y);
#pragma unroll
      for (int c = 0; c < 3; ++c) { Py[c].x += UI[c].x; Py[c].y += UI[c].y; }
      P0.x += TI.x;
      P0.y += TI.y;
    } else {
      Px[0].x += Xy * EI[2].x - Xz * EI[1].x; Px[0].y += Xy * EI[2].y - Xz * EI[1].y;
      Px[1].x += Xz * EI[0].x - Xx * EI[2].x; Px[1].y += Xz * EI[0].y - Xx * EI[2].y;
      Px[2].x += Xx * EI[1].x - Xy * EI[0].x; Px[2].y += Xx * EI[1].y - Xy * EI[0].y;
      S.x = fma(Xx, BI[0].x, fma(Xy, BI[1].x, fma(Xz, BI[2].x, S.x)));
      S.y = fma(Xx, BI[0].y, fma(Xy, BI[1].y, fma(Xz, BI[2].y, S.y)));
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        Py[c].x += BI[c].x; Py[c].y += BI[c].y;
        L[c].x += EI[c].x; L[c].y += EI[c].y;
      }
    }
  }
  const double2 alpha = make_double2(K.alpha[0], K.alpha[1]);
  if (OP == BGB_OP_HELMHOLTZ3D_HS) {
    // alpha (n_x . n_y) int int f g G + beta (curl f . curl g) int int G, int int G = sum of L
    double2 P = make_double2(0, 0);
#pragma unroll
    for (int k = 0; k < 9; ++k) { P.x += L[k].x; P.y += L[k].y; }
    const double nn = nA[0] * nB[0] + nA[1] * nB[1] + nA[2] * nB[2];
    const double2 an = make_double2(alpha.x * nn, alpha.y * nn);
    const double2 bP = cmul(make_double2(K.beta[0], K.beta[1]), P);
    double cA[3][3], cB[3][3];
    tri_curls(a + OA::VO, a[OA::INV2A], cA);
    tri_curls(b + OB::VO, b[OB::INV2A], cB);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double cc = cA[i][0] * cB[j][0] + cA[i][1] * cB[j][1] + cA[i][2] * cB[j][2];
        const double2 t = cmul(an, L[i * 3 + j]);
        L[i * 3 + j] = make_double2(fma(cc, bP.x, t.x), fma(cc, bP.y, t.y));
      }
    return;
  }
  if (kHH) {
#pragma unroll
    for (int k = 0; k < 9; ++k) L[k] = cmul(alpha, L[k]);
    return;
  }
  const double inv4AA = a[OA::INV2A] * b[OB::INV2A];
  const double2 ca = make_double2(alpha.x * inv4AA, alpha.y * inv4AA);
  if (OP == BGB_OP_MAXWELL3D_SL) {
    const double invAA = 4.0 * inv4AA;
    const double2 cb = make_double2(K.beta[0] * invAA, K.beta[1] * invAA);
    const double2 tb = cmul(cb, P0);
    double2 av[3], bv[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double vx = a[OA::VO + 3 * i], vy = a[OA::VO + 3 * i + 1], vz = a[OA::VO + 3 * i + 2];
      av[i].x = vx * Py[0].x + vy * Py[1].x + vz * Py[2].x;
      av[i].y = vx * Py[0].y + vy * Py[1].y + vz * Py[2].y;
      const double wx = b[OB::VO + 3 * i], wy = b[OB::VO + 3 * i + 1], wz = b[OB::VO + 3 * i + 2];
      bv[i].x = wx * Px[0].x + wy * Px[1].x + wz * Px[2].x;
      bv[i].y = wx * Px[0].y + wy * Px[1].y + wz * Px[2].y;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double vw = a[OA::VO + 3 * i] * b[OB::VO + 3 * j] + a[OA::VO + 3 * i + 1] * b[OB::VO + 3 * j + 1] +
                          a[OA::VO + 3 * i + 2] * b[OB::VO + 3 * j + 2];
        double2 t;
        t.x = S.x - av[i].x - bv[j].x + vw * P0.x;
        t.y = S.y - av[i].y - bv[j].y + vw * P0.y;
        const double2 r = cmul(ca, t);
        L[i * 3 + j] = make_double2(r.x + tb.x, r.y + tb.y);
      }
    return;
  }
  const double2 E0 = L[0], E1 = L[1], E2 = L[2];
  double2 vb[3], wc[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double vx = a[OA::VO + 3 * i], vy = a[OA::VO + 3 * i + 1], vz = a[OA::VO + 3 * i + 2];
    vb[i].x = vx * Py[0].x + vy * Py[1].x + vz * Py[2].x;
    vb[i].y = vx * Py[0].y + vy * Py[1].y + vz * Py[2].y;
    const double wx = b[OB::VO + 3 * i], wy = b[OB::VO + 3 * i + 1], wz = b[OB::VO + 3 * i + 2];
    wc[i].x = wx * Px[0].x + wy * Px[1].x + wz * Px[2].x;
    wc[i].y = wx * Px[0].y + wy * Px[1].y + wz * Px[2].y;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const double wx = b[OB::VO + 3 * j], wy = b[OB::VO + 3 * j + 1], wz = b[OB::VO + 3 * j + 2];
    const double2 x0 = make_double2(E1.x * wz - E2.x * wy, E1.y * wz - E2.y * wy);
    const double2 x1 = make_double2(E2.x * wx - E0.x * wz, E2.y * wx - E0.y * wz);
    const double2 x2 = make_double2(E0.x * wy - E1.x * wx, E0.y * wy - E1.y * wx);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double vx = a[OA::VO + 3 * i], vy = a[OA::VO + 3 * i + 1], vz = a[OA::VO + 3 * i + 2];
      double2 t;
      t.x = S.x - wc[j].x - vb[i].x + (vx * x0.x + vy * x1.x + vz * x2.x);
      t.y = S.y - wc[j].y - vb[i].y + (vx * x0.y + vy * x1.y + vz * x2.y);
      L[i * 3 + j] = cmul(ca, t);
    }
  }
}

__device__ __forceinline__ FarScalars far_scalars(const FarConst& K) {
  FarScalars S;
  S.qt = K.qt;
  S.qb = K.qb;
  S.lossy = K.lossy;
  S.phase_direct = K.phase_direct;
  S.tay_n = K.tay_n;
  S.k_hi = K.k_hi;
  S.k_lo = K.k_lo;
  S.gre = K.gre;
  for (int c = 0; c < 2; ++c) {
    S.alpha32[c] = K.alpha32[c];
    S.beta32[c] = K.beta32[c];
    S.alpha[c] = K.alpha[c];
    S.beta[c] = K.beta[c];
    S.gamma[c] = K.gamma[c];
  }
  return S;
}

template <class P, int OP, int QT, int QB>
__device__ __forceinline__ void far_pair(const FarScalars& S, const FarConst& K, const typename P::R* a,
                                         const typename P::R* b, typename P::C L[9]) {
  if constexpr (sizeof(typename P::R) == 4)
    far_pair_mixed<OP, QT, QB>(S, K.shpT, K.shpB, a, b, L);
  else
    far_pair_fp64<OP, QT, QB>(S, K.shpT64, K.shpB64, K.tay_s, K.tay_c, a, b, L);
}

__device__ __forceinline__ int64_t find_sigma(const int64_t* __restrict__ off, const int* __restrict__ sig, int tau,
                                              int sigma) {
  int64_t lo = off[tau], hi = off[tau + 1];
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    int v = sig[mid];
    if (v == sigma) return mid;
    if (v < sigma) lo = mid + 1;
    else hi = mid;
  }
  return -1;
}

// ----------------------------------------------------------------------------------------
// Tile kernel
// ----------------------------------------------------------------------------------------
template <class P>
struct Smem {
  float4* bndT;
  float4* bndB;
  int* triT;
  int* triB;
  typename P::R* recT;
  typename P::R* recB;
  int* fcnt;
  int* fcode;
  typename P::R* fcoef;
  typename P::C* Lbuf;
  typename P::C* Zs;
  int* grpFn;      // per group of the trial block: local function
  int* grpOff;     // per group: first support (block-relative), plus one end marker per chunk
  int* chGrp;      // per chunk: first group (block-relative)
  int* gsCode;
  typename P::R* gsCoef;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Trial records staged per chunk (two chunk buffers, the next copied in while the current one is
// computed) instead of per tile: for the FP32 Lagrange kernels, whose ~6-support hats make wide
// trial blocks, the freed shared memory keeps more test triangles per tile (the d = 40 cube: 3%
// faster); the RWG kernels keep per-tile staging (3% faster there: no copy per chunk, no spills).
template <class P, int OP>
__host__ __device__ constexpr bool chunk_trial_records() {
  return sizeof(typename P::R) == 4 && is_lagrange_op(OP);
}

template <class P>
__host__ __device__ inline size_t carve(unsigned char* base, int tmax, int nmax, int rt, int rb, int FM, int FN,
                                        int MAXS, int SC, int gmax, int gsmax, bool chunk_recb, Smem<P>* s) {
  using R = typename P::R;
  using C = typename P::C;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align16(off + bytes);
    return base ? base + o : nullptr;
  };
  unsigned char* p;
  p = take(sizeof(float4) * tmax); if (s) s->bndT = (float4*)p;
  p = take(sizeof(float4) * nmax); if (s) s->bndB = (float4*)p;
  p = take(sizeof(int) * tmax); if (s) s->triT = (int*)p;
  p = take(sizeof(int) * nmax); if (s) s->triB = (int*)p;
  p = take(sizeof(R) * (size_t)tmax * rt); if (s) s->recT = (R*)p;
  p = take(sizeof(R) * (size_t)(chunk_recb ? 2 * SC : nmax) * rb); if (s) s->recB = (R*)p;
  p = take(sizeof(int) * FM); if (s) s->fcnt = (int*)p;
  p = take(sizeof(int) * (size_t)FM * MAXS); if (s) s->fcode = (int*)p;
  p = take(sizeof(R) * (size_t)FM * MAXS); if (s) s->fcoef = (R*)p;
  p = take(sizeof(C) * 9 * (size_t)tmax * SC); if (s) s->Lbuf = (C*)p;
  p = take(sizeof(C) * (size_t)FM * FN); if (s) s->Zs = (C*)p;
  const int nch = (nmax + SC - 1) / SC;
  p = take(sizeof(int) * (size_t)gmax); if (s) s->grpFn = (int*)p;
  p = take(sizeof(int) * (size_t)(gmax + 1)); if (s) s->grpOff = (int*)p;
  p = take(sizeof(int) * (size_t)(nch + 1)); if (s) s->chGrp = (int*)p;
  p = take(sizeof(int) * (size_t)gsmax); if (s) s->gsCode = (int*)p;
  p = take(sizeof(R) * (size_t)gsmax); if (s) s->gsCoef = (R*)p;
  return off;
}

// 16-byte asynchronous global -> shared copies (completion awaited by the issuing thread).
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// One output tile (test-function block bm x trial-function block bn).
template <class P, int OP, int QT, int QB>
__device__ __forceinline__ void tile_body(const FarConst& K, const TilePlan& p, int bm, int bn, unsigned char* smem,
                                          int* s_nonfar) {
  using R = typename P::R;
  using C = typename P::C;
  constexpr int RT = P::template rec<QT>();
  constexpr int RB = P::template rec<QB>();
  const int tid = threadIdx.x;
  const FarScalars S = far_scalars(K);  // registers, not shared-memory loads in the pair loop
  const int SC = p.SC, MAXS = p.MAXS;
  Smem<P> s;
  constexpr bool kChunkB = chunk_trial_records<P, OP>();
  carve<P>(smem, p.tmax, p.nmax, RT, RB, p.FM, p.FN, MAXS, SC, p.gmax, p.gsmax, kChunkB, &s);

  const int t0 = p.tb_off[bm], tm = p.tb_off[bm + 1] - t0;
  const int b0 = p.bb_off[bn], nbk = p.bb_off[bn + 1] - b0;
  const int f0 = p.tb_fn_off[bm], fm = p.tb_fn_off[bm + 1] - f0;
  const int g0 = p.bb_fn_off[bn], fn = p.bb_fn_off[bn + 1] - g0;
  const R* __restrict__ gRT = (const R*)p.rec_t;
  const R* __restrict__ gRB = (const R*)p.rec_b;

  for (int i = tid; i < tm; i += kThreads) {
    const int t = p.tb_tris[t0 + i];
    s.triT[i] = t;
    s.bndT[i] = p.bnd_t[t];
  }
  for (int i = tid; i < nbk; i += kThreads) {
    const int t = p.bb_tris[b0 + i];
    s.triB[i] = t;
    s.bndB[i] = p.bnd_b[t];
  }
  if constexpr (sizeof(R) == 4) {  // FP32 records: whole 16-byte groups
    constexpr int RT4 = RT / 4, RB4 = RB / 4;
    const float4* __restrict__ gT4 = reinterpret_cast<const float4*>(gRT);
    const float4* __restrict__ gB4 = reinterpret_cast<const float4*>(gRB);
    for (int i = tid; i < tm * RT4; i += kThreads) {
      const int r = i / RT4, c = i - r * RT4;
      reinterpret_cast<float4*>(s.recT)[i] = gT4[(int64_t)p.tb_tris[t0 + r] * RT4 + c];
    }
    for (int i = tid; i < (kChunkB ? min(SC, nbk) : nbk) * RB4; i += kThreads) {  // kChunkB: the first chunk's
      const int r = i / RB4, c = i - r * RB4;
      reinterpret_cast<float4*>(s.recB)[i] = gB4[(int64_t)p.bb_tris[b0 + r] * RB4 + c];
    }
  } else {
    for (int i = tid; i < tm * RT; i += kThreads) {
      const int r = i / RT, c = i - r * RT;
      s.recT[i] = gRT[(int64_t)p.tb_tris[t0 + r] * RT + c];
    }
    for (int i = tid; i < nbk * RB; i += kThreads) {
      const int r = i / RB, c = i - r * RB;
      s.recB[i] = gRB[(int64_t)p.bb_tris[b0 + r] * RB + c];
    }
  }
  const bool f32 = sizeof(R) == 4;
  // local matrices of a chunk: entry (i, j) of pair (ti, si) at Lbuf[(i * 3 + j) * LS + ti * SC + si];
  // supports are staged as their offsets in it (test: (i * 3) * LS + ti * SC, trial: j * LS + slot)
  const int LS = p.tmax * SC;
  for (int m = tid; m < fm; m += kThreads) {
    const int a0 = p.fs_off[f0 + m], a1 = p.fs_off[f0 + m + 1];
    const int cnt = min(a1 - a0, MAXS);
    s.fcnt[m] = cnt;
    for (int k = 0; k < cnt; ++k) {
      const int fc = p.fs_code[a0 + k];  // test triangle << 2 | local
      s.fcode[m * MAXS + k] = (fc & 3) * 3 * LS + (fc >> 2) * SC;
      s.fcoef[m * MAXS + k] = f32 ? (R)p.fs_coef32[a0 + k] : (R)p.fs_coef[a0 + k];
    }
  }
  // the trial block's gather groups (all chunks), block-relative
  const int c0 = p.bb_chunk_off[bn], c1 = p.bb_chunk_off[bn + 1];
  const int gb0 = p.ch_grp_off[c0], gb1 = p.ch_grp_off[c1];
  const int sb0 = p.grp_sup_off[gb0], sb1 = p.grp_sup_off[gb1];
  for (int i = tid; i < gb1 - gb0; i += kThreads) {
    s.grpFn[i] = p.grp_fn[gb0 + i];
    s.grpOff[i] = p.grp_sup_off[gb0 + i] - sb0;
  }
  if (tid == 0) s.grpOff[gb1 - gb0] = sb1 - sb0;
  for (int i = tid; i <= c1 - c0; i += kThreads) s.chGrp[i] = p.ch_grp_off[c0 + i] - gb0;
  for (int i = tid; i < sb1 - sb0; i += kThreads) {
    const int code = p.gs_code[sb0 + i];  // trial slot << 2 | local
    s.gsCode[i] = (code & 3) * LS + (code >> 2);
    s.gsCoef[i] = f32 ? (R)p.gs_coef32[sb0 + i] : (R)p.gs_coef[sb0 + i];
  }
  for (int i = tid; i < fm * fn; i += kThreads) s.Zs[i] = P::mk(0.0, 0.0);
  if (tid == 0) *s_nonfar = 0;
  __syncthreads();
  // Does the tile hold any non-far pair?  Most tiles do not, and skip the per-pair test.  First a
  // sphere around each block's triangle spheres (warp 0: test block, warp 1: trial block): blocks
  // whose spheres are clearly apart hold no pair that passes the per-pair sphere test, so no
  // non-far pair; only the other tiles scan their test triangles' lists of non-far pairs.
  __shared__ float4 s_blk[2];
  if (tid < 64) {
    const int w = tid >> 5, lane = tid & 31;
    const float4* __restrict__ bl = w ? s.bndB : s.bndT;
    const int nb = w ? nbk : tm;
    float cx = 0.f, cy = 0.f, cz = 0.f;
    for (int i = lane; i < nb; i += 32) {
      cx += bl[i].x;
      cy += bl[i].y;
      cz += bl[i].z;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      cx += __shfl_xor_sync(0xffffffffu, cx, o);
      cy += __shfl_xor_sync(0xffffffffu, cy, o);
      cz += __shfl_xor_sync(0xffffffffu, cz, o);
    }
    const float inv = 1.f / (float)max(nb, 1);
    cx *= inv;
    cy *= inv;
    cz *= inv;
    float r = 0.f;
    for (int i = lane; i < nb; i += 32) {
      const float dx = bl[i].x - cx, dy = bl[i].y - cy, dz = bl[i].z - cz;
      r = fmaxf(r, sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) + bl[i].w);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, o));
    if (lane == 0) s_blk[w] = make_float4(cx, cy, cz, r);
  }
  __syncthreads();
  bool blocks_apart;
  {
    const float4 A = s_blk[0], B = s_blk[1];
    const float dx = A.x - B.x, dy = A.y - B.y, dz = A.z - B.z;
    // margin over the FP32 rounding of the block spheres (sums of ~64 centres: relative to the
    // coordinates' size) and of the per-pair test
    const float mag = fmaxf(fmaxf(fabsf(A.x), fabsf(A.y)), fmaxf(fabsf(A.z), fmaxf(fmaxf(fabsf(B.x), fabsf(B.y)), fabsf(B.z))));
    const float lim = 1.001f * (A.w + B.w) + 1e-5f * mag + 1e-30f;
    blocks_apart = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) > lim * lim;  // false for NaN: scan
  }
  for (int i = tid; i < (blocks_apart ? 0 : tm); i += kThreads) {
    const int T = s.triT[i];
    for (int64_t e = p.sing_off[T], e1 = p.sing_off[T + 1]; e < e1; ++e) {
      const int sg = p.sing_sigma[e];
      int lo = 0, hi = nbk;  // triB is sorted ascending
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s.triB[mid] < sg) lo = mid + 1;
        else hi = mid;
      }
      if (lo < nbk && s.triB[lo] == sg) {
        *s_nonfar = 1;
        break;
      }
    }
  }
  // fixed roles of this thread: pair (ti0 + k * tstep, si) of a chunk; gather row m, groups gq + k * gstep
  const int tstep = kThreads / SC, ti0 = tid / SC, si = tid - ti0 * SC;
  // gather rows in whole warps (one group stream per warp) when that keeps the groups in flight
  const int FM32 = (p.FM + 31) & ~31;
  const int FMb = kThreads / FM32 == kThreads / p.FM ? FM32 : p.FM;
  const int gstep = kThreads / FMb, gq = tid / FMb, m = tid - gq * FMb;
  const bool gather_on = m < fm && gq < gstep;
  __syncthreads();
  const bool check = *s_nonfar != 0;

  for (int c = c0; c < c1; ++c) {
    const int sbase = (c - c0) * SC;
    const int scn = min(SC, nbk - sbase);
    const R* __restrict__ recb = s.recB;  // this chunk's trial records (kChunkB: one of two buffers)
    if constexpr (kChunkB) {
      constexpr int RB4 = RB / 4;
      recb = s.recB + ((c - c0) & 1) * SC * RB;
      const int nn = c + 1 < c1 ? min(SC, nbk - sbase - SC) : 0;  // the next chunk's records
      if (tid < nn * RB4) {
        const int r = tid / RB4, k = tid - r * RB4;
        cp_async16(s.recB + ((((c + 1 - c0) & 1) * SC + r) * RB + 4 * k),
                   (const float4*)gRB + (int64_t)s.triB[sbase + SC + r] * RB4 + k);
      }
      cp_async_commit();
    }
    if (si < scn) {
      const int sb = sbase + si;
      for (int ti = ti0; ti < tm; ti += tstep) {
        C L[9];
        bool done = false;
        if (check && sphere_candidate(s.bndT[ti], s.bndB[sb])) {
          const int64_t e = find_sigma(p.sing_off, p.sing_sigma, s.triT[ti], s.triB[sb]);
          if (e >= 0) {
#pragma unroll
            for (int k = 0; k < 9; ++k) {
              const double2 v = p.sing_L[e * 9 + k];
              L[k] = P::mk(v.x, v.y);
            }
            done = true;
          }
        }
        if (!done)
          far_pair<P, OP, QT, QB>(S, K, s.recT + ti * RT, kChunkB ? recb + si * RB : s.recB + sb * RB, L);
        const int li = ti * SC + si;
#pragma unroll
        for (int k = 0; k < 9; ++k) s.Lbuf[k * LS + li] = L[k];
      }
    }
    if constexpr (kChunkB) cp_async_wait_all();  // the next chunk's records, before the barrier
    __syncthreads();
    if (gather_on) {
      const int gg0 = s.chGrp[c - c0], ng = s.chGrp[c - c0 + 1] - gg0;
      // this row's test supports (two for RWG) in registers for the chunk
      const int cnt = s.fcnt[m];
      int fcA = 0, fcB = 0;
      R fwA = 0, fwB = 0;
      if (MAXS <= 2) {
        fcA = s.fcode[m * MAXS];
        fwA = s.fcoef[m * MAXS];
        if (cnt > 1) {
          fcB = s.fcode[m * MAXS + 1];
          fwB = s.fcoef[m * MAXS + 1];
        }
      }
      for (int g = gq; g < ng; g += gstep) {
        const int gi = gg0 + g;
        const int n = s.grpFn[gi];
        C acc = s.Zs[n * fm + m];
        const int q0 = s.grpOff[gi], q1 = s.grpOff[gi + 1];
        for (int bsup = q0; bsup < q1; ++bsup) {
          const int col = s.gsCode[bsup] - sbase;
          const R cb = s.gsCoef[bsup];
          if (MAXS <= 2) {
            {
              const R w = fwA * cb;
              const C l = s.Lbuf[fcA + col];
              acc.x = fma(w, l.x, acc.x);
              acc.y = fma(w, l.y, acc.y);
            }
            if (cnt > 1) {
              const R w = fwB * cb;
              const C l = s.Lbuf[fcB + col];
              acc.x = fma(w, l.x, acc.x);
              acc.y = fma(w, l.y, acc.y);
            }
          } else {
            for (int a = 0; a < cnt; ++a) {
              const R w = s.fcoef[m * MAXS + a] * cb;
              const C l = s.Lbuf[s.fcode[m * MAXS + a] + col];
              acc.x = fma(w, l.x, acc.x);
              acc.y = fma(w, l.y, acc.y);
            }
          }
        }
        s.Zs[n * fm + m] = acc;
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < fm * fn; i += kThreads) {
    const int n = i / fm, m = i - n * fm;
    const int64_t idx = p.rows[f0 + m] + p.cols[g0 + n] * p.ld;
    const C v = s.Zs[i];
    if (p.out_c64) ((double2*)p.out)[idx] = make_double2(v.x, v.y);
    else ((float2*)p.out)[idx] = make_float2((float)v.x, (float)v.y);
  }
}

// The far kernel: persistent CTAs pull tiles (problem, bm, bn) from a work queue (an atomic
// counter; no CTA ever waits on another): items[t], or without a list the tiles of plans[0] with
// the row block fastest.  A single assembly is a one-problem queue.  Each
// problem has its own constants (wave number, alpha, beta) and plan; the tile shape and rules
// are common to the launch.  The problem's constants and plan are copied to shared memory
// when a CTA's tile belongs to another problem than its previous one; each CTA claims its next
// tile when it starts a tile.
template <class P, int OP, int QT, int QB>
__global__ void __launch_bounds__(kThreads, P::kMinBlocks) k_far_persistent(const FarConst* __restrict__ Ks,
                                                             const TilePlan* __restrict__ plans,
                                                             const int4* __restrict__ items, int nitems,
                                                             int* __restrict__ counter,
                                                             const volatile int* abort_flag) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int next, nonfar;
  __shared__ FarConst sK;
  __shared__ TilePlan sP;
  if (threadIdx.x == 0) next = (abort_flag && *abort_flag) ? nitems : atomicAdd(counter, 1);
  __syncthreads();
  int cur = -1;  // the problem whose constants and plan are in shared memory (the same in all threads)
  for (;;) {
    const int t = next;
    if (t >= nitems) return;
    // an item list (batches), or tile t = bn * n_tblocks + bm of the single plan
    int4 it;
    if (items) {
      it = items[t];
    } else {
      const int ntb = plans[0].n_tblocks;
      it = make_int4(0, t % ntb, t / ntb, 0);
    }
    if (it.x != cur) {
      for (int i = threadIdx.x; i < (int)(sizeof(FarConst) / 4); i += kThreads)
        ((int*)&sK)[i] = ((const int*)&Ks[it.x])[i];
      for (int i = threadIdx.x; i < (int)(sizeof(TilePlan) / 4); i += kThreads)
        ((int*)&sP)[i] = ((const int*)&plans[it.x])[i];
      cur = it.x;
    }
    __syncthreads();
    // claim the next tile now: the atomic completes while this one is computed
    int claimed = 0;
    if (threadIdx.x == 0) claimed = (abort_flag && *abort_flag) ? nitems : atomicAdd(counter, 1);
    tile_body<P, OP, QT, QB>(sK, sP, it.y, it.z, smem, &nonfar);
    if (threadIdx.x == 0) next = claimed;
    __syncthreads();
  }
}

// ----------------------------------------------------------------------------------------
// Records
// ----------------------------------------------------------------------------------------
template <int Q>
__global__ void k_prepare_rec32(const Geo64* __restrict__ g, int nt, const __grid_constant__ RuleTable rules, int rule,
                                double wscale, float* __restrict__ out) {
  using O = Off32<Q>;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const Geo64& T = g[t];
  float* r = out + (int64_t)t * O::SIZE;
  double c[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) c[k] = (T.v[0][k] + T.v[1][k] + T.v[2][k]) / 3.0;
  for (int k = 0; k < O::SIZE; ++k) r[k] = 0.f;  // spare slots
  for (int k = 0; k < 3; ++k) {
    const float hi = (float)c[k];
    r[O::CH + k] = hi;
    r[O::CL + k] = (float)(c[k] - (double)hi);
  }
  r[O::INV2A] = (float)(1.0 / (2.0 * T.area));
  const int q = rules.npoints[rule];
  for (int I = 0; I < Q; ++I) {
    double u = 0, v = 0, w = 0;
    if (I < q) {
      u = rules.uvw[rules.offset[rule] + I][0];
      v = rules.uvw[rules.offset[rule] + I][1];
      w = rules.uvw[rules.offset[rule] + I][2];
    }
    for (int k = 0; k < 3; ++k) {
      const double x = (T.v[2][k] + T.t[0][k] * u) + T.t[1][k] * v;
      r[O::px(I) + k] = (float)(x - c[k]);
    }
    r[O::pw(I)] = (float)((w / 2.0) * (2.0 * T.area) * wscale);
  }
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) r[O::VO + 3 * i + k] = (float)(T.v[i][k] - c[k]);
}

template <int Q>
__global__ void k_prepare_rec64(const Geo64* __restrict__ g, int nt, const __grid_constant__ RuleTable rules, int rule,
                                double wscale, double* __restrict__ out) {
  using O = Off64<Q>;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const Geo64& T = g[t];
  double* r = out + (int64_t)t * O::SIZE;
  double c[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) c[k] = (T.v[0][k] + T.v[1][k] + T.v[2][k]) / 3.0;
  for (int k = 0; k < 3; ++k) r[O::C + k] = c[k];
  const int q = rules.npoints[rule];
  for (int I = 0; I < Q; ++I) {
    double u = 0, v = 0, w = 0;
    if (I < q) {
      u = rules.uvw[rules.offset[rule] + I][0];
      v = rules.uvw[rules.offset[rule] + I][1];
      w = rules.uvw[rules.offset[rule] + I][2];
    }
    for (int k = 0; k < 3; ++k) {
      const double x = (T.v[2][k] + T.t[0][k] * u) + T.t[1][k] * v;
      r[O::X + 3 * I + k] = x - c[k];
    }
    r[O::W + I] = (w / 2.0) * (2.0 * T.area) * wscale;
  }
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) r[O::VO + 3 * i + k] = T.v[i][k] - c[k];
  r[O::INV2A] = 1.0 / (2.0 * T.area);
}

// Diagnostic kernel: far rule of explicit pairs, one thread per pair, records from HBM.
template <class P, int OP, int QT, int QB>
__global__ void k_far_pairs_diag(const __grid_constant__ FarConst K, const typename P::R* __restrict__ rt,
                                 const typename P::R* __restrict__ rb, const int* __restrict__ tau,
                                 const int* __restrict__ sigma, int64_t n, double2* __restrict__ out) {
  constexpr int RT = P::template rec<QT>();
  constexpr int RB = P::template rec<QB>();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    typename P::C L[9];
    far_pair<P, OP, QT, QB>(far_scalars(K), K, rt + (int64_t)tau[e] * RT, rb + (int64_t)sigma[e] * RB, L);
#pragma unroll
    for (int k = 0; k < 9; ++k) out[e * 9 + k] = make_double2(L[k].x, L[k].y);
  }
}

// The dynamic shared-memory limit of a kernel is set to the device maximum less its static
// shared memory (not to one launch's size), so that concurrent callers never lower it under
// each other's launches.
template <class K>
inline int max_dynamic_smem(K kern) {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) return v;
  return v - (int)fa.sharedSizeBytes;
}

template <class P, int OP, int QT, int QB>
int launch_persistent_t(const FarConst* Ks, const TilePlan* plans, const int4* items, int nitems, int* counter,
                        size_t smem_bytes, int ctas, const volatile int* abort_flag, cudaStream_t st) {
  auto kern = k_far_persistent<P, OP, QT, QB>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem(kern));
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(far persistent)");
  if (nitems <= 0) return 0;
  kern<<<ctas, kThreads, smem_bytes, st>>>(Ks, plans, items, nitems, counter, abort_flag);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "k_far_persistent launch");
}

template <class P, int OP, int QT, int QB>
int occupancy_t(size_t smem_bytes, int* per_sm) {
  cudaError_t e = cudaFuncSetAttribute(k_far_persistent<P, OP, QT, QB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       max_dynamic_smem(k_far_persistent<P, OP, QT, QB>));
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(far persistent)");
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_far_persistent<P, OP, QT, QB>, kThreads, smem_bytes);
  return e == cudaSuccess ? 0 : cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
}

template <class P, int OP, int QT, int QB>
size_t smem_t(const TilePlan& p) {
  return carve<P>(nullptr, p.tmax, p.nmax, P::template rec<QT>(), P::template rec<QB>(), p.FM, p.FN, p.MAXS, p.SC,
                  p.gmax, p.gsmax, chunk_trial_records<P, OP>(), nullptr);
}

template <class P, int OP, int QT, int QB>
int launch_diag_t(const FarConst& K, const void* rt, const void* rb, const int* tau, const int* sigma, int64_t n,
                  double2* out, cudaStream_t st) {
  if (n <= 0) return 0;
  const int blocks = (int)std::min<int64_t>((n + 127) / 128, 65535);
  using R = typename P::R;
  k_far_pairs_diag<P, OP, QT, QB><<<blocks, 128, 0, st>>>(K, (const R*)rt, (const R*)rb, tau, sigma, n, out);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "k_far_pairs_diag launch");
}

// Instances live in bgb_far_{mixed,fp64}_op{0,1,2}.cu.
#define BGB_FAR_EXTERN(P, OP)                                                                                   \
  extern template int launch_diag_t<P, OP, 3, 4>(const FarConst&, const void*, const void*, const int*,        \
                                                 const int*, int64_t, double2*, cudaStream_t);                \
  extern template int launch_diag_t<P, OP, BGB_MAXQ, BGB_MAXQ>(const FarConst&, const void*, const void*,      \
                                                               const int*, const int*, int64_t, double2*,     \
                                                               cudaStream_t);                                 \
  extern template int launch_persistent_t<P, OP, 3, 4>(const FarConst*, const TilePlan*, const int4*, int, int*, \
                                                       size_t, int, const volatile int*, cudaStream_t);        \
  extern template int launch_persistent_t<P, OP, BGB_MAXQ, BGB_MAXQ>(const FarConst*, const TilePlan*,       \
                                                                     const int4*, int, int*, size_t, int,      \
                                                                     const volatile int*, cudaStream_t);       \
  extern template int occupancy_t<P, OP, 3, 4>(size_t, int*);                                                 \
  extern template int occupancy_t<P, OP, BGB_MAXQ, BGB_MAXQ>(size_t, int*);

}  // namespace farimpl
}  // namespace bgb
