// Geometry preparation, pair classification and the FP64 singular / near-pair kernels.
//
//  k_prepare_geo64    FP64 simplex data per triangle (CompScienceMeshes rounding).
//  k_prepare_bounds   FP32 bounding spheres used to skip obviously-far pairs.
//  k_classify<FILL>   one warp per test triangle sweeps all trial triangles: an FP32 sphere
//                     test rejects far pairs, the exact FP64 predicate (BEAST quadrule,
//                     doubleQuadRuleMainCase.jl:324-339) decides the rest; non-far pairs are
//                     compacted in trial order (ballot/popc), so the list is deterministic.
//  k_singular         one warp per non-far pair: Sauter-Schwab CF/CE/CV (SauterSchwab.jl:212-297)
//                     or the near-pair double quadrature, FP64, warp-shuffle reduction, one
//                     3x3 complex local matrix per pair (no atomics).
//  k_classify_dense   diagnostic: exact class of every pair of a block.
#include "bgb_kernels.cuh"

namespace bgb {

__global__ void k_prepare_geo64(const double* __restrict__ verts, const int32_t* __restrict__ tris, int nt,
                                Geo64* __restrict__ out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  Geo64 g;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int vi = tris[3 * t + a];
#pragma unroll
    for (int c = 0; c < 3; ++c) g.v[a][c] = verts[3 * (int64_t)vi + c];
  }
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) g.t[k][c] = __dsub_rn(g.v[k][c], g.v[2][c]);
  // normal = t1 x t2, volume = norm / 2, evaluated without contraction (bit-identical to the oracle)
  double n0 = __dsub_rn(__dmul_rn(g.t[0][1], g.t[1][2]), __dmul_rn(g.t[0][2], g.t[1][1]));
  double n1 = __dsub_rn(__dmul_rn(g.t[0][2], g.t[1][0]), __dmul_rn(g.t[0][0], g.t[1][2]));
  double n2 = __dsub_rn(__dmul_rn(g.t[0][0], g.t[1][1]), __dmul_rn(g.t[0][1], g.t[1][0]));
  double s = __dadd_rn(__dadd_rn(__dmul_rn(n0, n0), __dmul_rn(n1, n1)), __dmul_rn(n2, n2));
  g.area = __ddiv_rn(__dsqrt_rn(s), 2.0);
  g.pad = 0.0;
  out[t] = g;
}

// Bounding sphere (centroid, radius) in FP32, rounded so that an FP32 distance test never
// rejects a pair the FP64 predicate would call non-far.  On the trial side the radius also
// carries the near-pair distance threshold sqrt(min(0.04 / k2, 0.64 A)).
__global__ void k_prepare_bounds(const Geo64* __restrict__ g, int nt, double k2, int trial_side,
                                 float4* __restrict__ out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const Geo64& T = g[t];
  double c[3], r = 0.0, cn = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) c[k] = (T.v[0][k] + T.v[1][k] + T.v[2][k]) / 3.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double d0 = T.v[a][0] - c[0], d1 = T.v[a][1] - c[1], d2 = T.v[a][2] - c[2];
    r = fmax(r, sqrt(d0 * d0 + d1 * d1 + d2 * d2));
  }
  cn = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  if (trial_side) {
    double lim = 0.64 * T.area;  // 16 * xtol2 * A
    if (k2 > 0.0) lim = fmin(lim, 0.04 / k2);
    r += sqrt(lim);
  }
  r = r * (1.0 + 1e-6) + 4e-7 * (cn + 1.0) + 1e-30;
  out[t] = make_float4((float)c[0], (float)c[1], (float)c[2], (float)r);
}

// ----------------------------------------------------------------------------------------
// Exact FP64 predicate (doubleQuadRuleMainCase.jl:324-339; codes quadrule_determine.jl:76).
// Rounded like the Julia code: no contraction, IEEE sqrt and division.
// ----------------------------------------------------------------------------------------
__device__ int classify_exact(const Geo64& a, const Geo64& b, double k2) {
  const double dtol = 2.220446049250313e-16 * 1.0e3;
  const double xtol2 = 0.2 * 0.2;
  int hits = 0;
  double dmin2 = 1.7976931348623157e308;  // floatmax(Float64)
#pragma unroll
  for (int u1 = 0; u1 < 3; ++u1)
#pragma unroll
    for (int u2 = 0; u2 < 3; ++u2) {
      double dx = __dsub_rn(a.v[u1][0], b.v[u2][0]);
      double dy = __dsub_rn(a.v[u1][1], b.v[u2][1]);
      double dz = __dsub_rn(a.v[u1][2], b.v[u2][2]);
      double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
      hits += (__dsqrt_rn(d2) < dtol);
      dmin2 = fmin(dmin2, d2);
    }
  if (hits > 3) return -1;
  if (hits > 0) return hits;
  double m = fmax(__dmul_rn(dmin2, k2), __ddiv_rn(dmin2, __dmul_rn(16.0, b.area)));
  return (m >= xtol2) ? BGB_CLASS_FAR : BGB_CLASS_NEAR;
}

template <bool FILL>
__global__ void __launch_bounds__(256) k_classify(const float4* __restrict__ tb, const float4* __restrict__ bb,
                                                  const Geo64* __restrict__ tg, const Geo64* __restrict__ bg,
                                                  int nt, int nb, double k2, int* __restrict__ count,
                                                  const int64_t* __restrict__ offset, int* __restrict__ out_tau,
                                                  int* __restrict__ out_sigma, int8_t* __restrict__ out_cls,
                                                  int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int tau = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; tau < nt; tau += warps) {
    float4 a = tb[tau];
    int64_t base = FILL ? offset[tau] : 0;
    int n = 0;
    for (int s0 = 0; s0 < nb; s0 += 32) {
      int s = s0 + lane;
      int cls = 0;
      if (s < nb) {
        if (sphere_candidate(a, bb[s])) {
          cls = classify_exact(tg[tau], bg[s], k2);
          if (cls < 0) {
            atomicOr(err, 1);
            cls = 0;
          }
        }
      }
      unsigned bal = __ballot_sync(0xffffffffu, cls != 0);
      if (FILL && cls != 0) {
        int64_t pos = base + n + __popc(bal & ((1u << lane) - 1u));
        out_tau[pos] = tau;
        out_sigma[pos] = s;
        out_cls[pos] = (int8_t)cls;
      }
      n += __popc(bal);
    }
    if (!FILL && lane == 0) count[tau] = n;
  }
}

// Exclusive scan of counts[0..n) into offsets[0..n] (one block; n up to a few million).
__global__ void k_scan_counts(const int* __restrict__ counts, int n, int64_t* __restrict__ offsets) {
  __shared__ int64_t part[1024];
  const int T = blockDim.x;
  int per = (n + T - 1) / T;
  int b = threadIdx.x * per, e = min(n, b + per);
  int64_t s = 0;
  for (int i = b; i < e; ++i) s += counts[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {
    int64_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int64_t run = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (int i = b; i < e; ++i) {
    offsets[i] = run;
    run += counts[i];
  }
  if (threadIdx.x == T - 1) offsets[n] = part[T - 1];
}

__global__ void k_classify_dense(const Geo64* __restrict__ tg, const Geo64* __restrict__ bg, int t0, int t1,
                                 int s0, int s1, double k2, int8_t* __restrict__ out, int* __restrict__ err) {
  int64_t ns = s1 - s0;
  int64_t total = (int64_t)(t1 - t0) * ns;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    int t = t0 + (int)(p / ns), s = s0 + (int)(p % ns);
    int c = classify_exact(tg[t], bg[s], k2);
    if (c < 0) atomicOr(err, 1);
    out[p] = (int8_t)c;
  }
}

// ----------------------------------------------------------------------------------------
// Sauter-Schwab
// ----------------------------------------------------------------------------------------
struct Chart {
  double cv[3][2];
  double ct[2][2];
};

// Shared-vertex permutation of pulledback_integrand_gpu.jl (CF :22-58, CE :60-102, CV :117-155).
__device__ inline void ss_permutation(int cls, const Geo64& A, const Geo64& B, int I[3], int J[3]) {
  const double tol = 1e3 * 2.220446049250313e-16;
  I[0] = I[1] = I[2] = 0;
  J[0] = J[1] = J[2] = 0;
  int cap = (cls == BGB_CLASS_CE) ? 3 : 2;
  int e = 1;
  for (int i = 1; i <= 3; ++i)
    for (int j = 1; j <= 3; ++j) {
      double R = 0.0;
      for (int c = 0; c < 3; ++c) {
        double d = __dsub_rn(A.v[i - 1][c], B.v[j - 1][c]);
        R = __dadd_rn(R, __dmul_rn(d, d));
      }
      if (__dsqrt_rn(R) < tol) {
        if (cls == BGB_CLASS_CF) {
          J[i - 1] = j;
        } else if (e <= cap) {
          J[e - 1] = j;
          I[e - 1] = i;
          e += 1;
        }
      }
    }
  if (cls == BGB_CLASS_CF) {
    I[0] = 1;
    I[1] = 2;
    I[2] = 3;
    return;
  }
  for (int k = 0; k < 2; ++k) {
    int* a = k ? I : J;
    bool e1 = (e == 1), e2 = (e == 2);
    a[0] = e1 ? 1 : a[0];
    a[1] = e1 ? 2 : (e2 ? (a[0] == 1 ? 2 : 1) : a[1]);
    a[2] = 6 - a[0] - a[1];
    if (cls == BGB_CLASS_CE) {
      int t = a[0];
      a[0] = a[1];
      a[1] = a[2];
      a[2] = t;
    }
  }
}

__device__ inline void make_chart(const int P[3], Chart& C) {
  const double V[3][2] = {{1.0, 0.0}, {0.0, 1.0}, {0.0, 0.0}};
  for (int u = 0; u < 3; ++u) {
    int p = P[u] - 1;
    p = p < 0 ? 0 : (p > 2 ? 2 : p);
    C.cv[u][0] = V[p][0];
    C.cv[u][1] = V[p][1];
  }
  for (int u = 0; u < 2; ++u) {
    C.ct[u][0] = C.cv[u][0] - C.cv[2][0];
    C.ct[u][1] = C.cv[u][1] - C.cv[2][1];
  }
}

__device__ inline void ss_point(const OpParams& op, const Geo64& A, const Geo64& B, int rsA, int rsB,
                                const Chart& cA, const Chart& cB, double u1, double u2, double v1, double v2,
                                double mul, double2 L[3][3]) {
  double bx1 = cA.cv[2][0] + cA.ct[0][0] * u1 + cA.ct[1][0] * u2;
  double bx2 = cA.cv[2][1] + cA.ct[0][1] * u1 + cA.ct[1][1] * u2;
  double by1 = cB.cv[2][0] + cB.ct[0][0] * v1 + cB.ct[1][0] * v2;
  double by2 = cB.cv[2][1] + cB.ct[0][1] * v1 + cB.ct[1][1] * v2;
  Shp64 X, Y;
  shapes64(A, rsA, bx1, bx2, X);
  shapes64(B, rsB, by1, by2, Y);
  double wgt = ((4.0 * A.area) * B.area) * mul;  // Jacobians 2A * 2A times the SS weight
  accumulate64(op, X, Y, wgt, L);
}

// All regions of one 4-D Gauss-Legendre point (SauterSchwab.jl:265-297).
__device__ inline void ss_gl_point(const OpParams& op, int cls, const Geo64& A, const Geo64& B, int rsA, int rsB,
                                   const Chart& cA, const Chart& cB, double h1, double h2, double h3, double xi,
                                   double wt, double2 L[3][3]) {
  double xi3 = xi * xi * xi;
  if (cls == BGB_CLASS_CV) {
    double xh1 = xi * h1, xh2 = xi * h2;
    double mul = wt * xi3 * h2;
    ss_point(op, A, B, rsA, rsB, cA, cB, 1 - xi, xh1, 1 - xh2, xh2 * h3, mul, L);
    ss_point(op, A, B, rsA, rsB, cA, cB, 1 - xh2, xh2 * h3, 1 - xi, xh1, mul, L);
  } else if (cls == BGB_CLASS_CE) {
    double xh1 = xi * h1, h12 = h1 * h2, h23 = h2 * h3, h123 = h12 * h3;
    double mul = wt * xi3 * (h1 * h1) * h2;
    ss_point(op, A, B, rsA, rsB, cA, cB, 1 - xi, xh1, 1 - xi * (1 - h123), xh1 * h2 * (1 - h3), mul, L);
    ss_point(op, A, B, rsA, rsB, cA, cB, 1 - xi * (1 - h12), xh1 * (1 - h2), 1 - xi, xh1 * h23, mul, L);
    ss_point(op, A, B, rsA, rsB, cA, cB, 1 - xi * (1 - h123), xh1 * h2 * (1 - h3), 1 - xi, xh1, mul, L);
    ss_point(op, A, B, rsA, rsB, cA, cB, 1 - xi * (1 - h123), xh1 * (1 - h23), 1 - xi, xh1 * h2, mul, L);
    double mul5 = wt * xi3 * (h1 * h1);
    ss_point(op, A, B, rsA, rsB, cA, cB, 1 - xi, xh1 * h3, 1 - xi * (1 - h12), xh1 * (1 - h2), mul5, L);
  } else {
    double mul = wt * xi3 * (h1 * h1) * h2;
    double a = (xi - xi * h1) + xi * h1 * h2;
    double b = 1 - (xi - xi * h1 * h2 * h3);
    double c = xi - xi * h1;
    double d = xi * h1 * ((1 - h2) + h2 * h3);
    double e = 1 - (xi - xi * h1 * h2);
    double f = xi * h1 * (1 - h2);
    double g = xi * h1 * (1 - h2 * h3);
    ss_point(op, A, B, rsA, rsB, cA, cB, 1 - xi, a, b, c, mul, L);
    ss_point(op, A, B, rsA, rsB, cA, cB, b, c, 1 - xi, a, mul, L);
    ss_point(op, A, B, rsA, rsB, cA, cB, 1 - xi, d, e, f, mul, L);
    ss_point(op, A, B, rsA, rsB, cA, cB, e, f, 1 - xi, d, mul, L);
    ss_point(op, A, B, rsA, rsB, cA, cB, b, g, 1 - xi, f, mul, L);
    ss_point(op, A, B, rsA, rsB, cA, cB, 1 - xi, f, b, g, mul, L);
  }
}

__device__ inline void warp_reduce_L(double2 L[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        L[i][j].x += __shfl_xor_sync(0xffffffffu, L[i][j].x, off);
        L[i][j].y += __shfl_xor_sync(0xffffffffu, L[i][j].y, off);
      }
}

// Integral of one non-far pair by a warp; every lane returns the full (reduced) matrix.
__device__ void pair_integral64(const OpParams& op, const QuadSel& qs, const RuleTable& rules, int cls,
                                const Geo64& A, const Geo64& B, int rsA, int rsB, double2 L[3][3]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) L[i][j] = make_double2(0.0, 0.0);
  if (cls == BGB_CLASS_NEAR || cls == BGB_CLASS_FAR) {
    int rt = cls == BGB_CLASS_NEAR ? qs.near_t : qs.far_t;
    int rb = cls == BGB_CLASS_NEAR ? qs.near_b : qs.far_b;
    int qt = rules.npoints[rt], qb = rules.npoints[rb];
    for (int idx = lane; idx < qt * qb; idx += 32) {
      int I = idx / qb, J = idx % qb;
      const double* p = rules.uvw[rules.offset[rt] + I];
      const double* q = rules.uvw[rules.offset[rb] + J];
      Shp64 X, Y;
      shapes64(A, rsA, p[0], p[1], X);
      shapes64(B, rsB, q[0], q[1], Y);
      double wx = (p[2] / 2.0) * (A.area * 2.0), wy = (q[2] / 2.0) * (B.area * 2.0);
      accumulate64(op, X, Y, wx * wy, L);
    }
  } else if (!(op.kind == BGB_OP_MAXWELL3D_DL && cls == BGB_CLASS_CF)) {  // DL on a flat face is 0
    int I[3], J[3];
    ss_permutation(cls, A, B, I, J);
    Chart cA, cB;
    make_chart(I, cA);
    make_chart(J, cB);
    const int n = qs.ss[cls];
    const int n2 = n * n, n3 = n2 * n, n4 = n3 * n;
    const double* gx = qs.gl_x[cls];
    const double* gw = qs.gl_w[cls];
    for (int idx = lane; idx < n4; idx += 32) {
      int i = idx / n3, j = (idx / n2) % n, k = (idx / n) % n, l = idx % n;
      double wt = gw[i] * gw[j] * gw[k] * gw[l];
      ss_gl_point(op, cls, A, B, rsA, rsB, cA, cB, gx[i], gx[j], gx[k], gx[l], wt, L);
    }
  }
  warp_reduce_L(L);
}

__global__ void __launch_bounds__(256) k_singular(OpParams op, const __grid_constant__ QuadSel qs,
                                                  const __grid_constant__ RuleTable rules, int rsA, int rsB,
                                                  const Geo64* __restrict__ tg, const Geo64* __restrict__ bg,
                                                  const int* __restrict__ ent_tau, const int* __restrict__ ent_sigma,
                                                  const int8_t* __restrict__ ent_cls, int64_t n,
                                                  double2* __restrict__ out, const volatile int* abort_flag) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n; e += warps) {
    if (abort_flag && *abort_flag) return;
    Geo64 A = tg[ent_tau[e]], B = bg[ent_sigma[e]];
    double2 L[3][3];
    pair_integral64(op, qs, rules, ent_cls[e], A, B, rsA, rsB, L);
    if (lane < 9) {
      double2 v = L[0][0];
#pragma unroll
      for (int q = 1; q < 9; ++q)
        if (lane == q) v = L[q / 3][q % 3];
      out[e * 9 + lane] = v;
    }
  }
}

// Diagnostic: local matrices of a list of pairs (classified exactly or forced), FP64.
__global__ void __launch_bounds__(256) k_local_diag64(OpParams op, const __grid_constant__ QuadSel qs,
                                                      const __grid_constant__ RuleTable rules, int rsA, int rsB,
                                                      const Geo64* __restrict__ tg, const Geo64* __restrict__ bg,
                                                      const int* __restrict__ tau, const int* __restrict__ sigma,
                                                      int64_t n, int force, double2* __restrict__ out,
                                                      int8_t* __restrict__ cls_out, int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n; e += warps) {
    Geo64 A = tg[tau[e]], B = bg[sigma[e]];
    int cls = force >= 0 ? force : classify_exact(A, B, op.k2);
    if (cls < 0) {
      if (lane == 0) atomicOr(err, 1);
      cls = BGB_CLASS_FAR;
    }
    double2 L[3][3];
    pair_integral64(op, qs, rules, cls, A, B, rsA, rsB, L);
    if (lane < 9) {
      double2 v = L[0][0];
#pragma unroll
      for (int q = 1; q < 9; ++q)
        if (lane == q) v = L[q / 3][q % 3];
      out[e * 9 + lane] = v;
    }
    if (lane == 0 && cls_out) cls_out[e] = (int8_t)cls;
  }
}

// ----------------------------------------------------------------------------------------
// Host launchers
// ----------------------------------------------------------------------------------------
void launch_prepare_geo64(const double* verts, const int32_t* tris, int nt, Geo64* out, cudaStream_t st) {
  if (nt > 0) k_prepare_geo64<<<(nt + 255) / 256, 256, 0, st>>>(verts, tris, nt, out);
}
void launch_prepare_bounds(const Geo64* g, int nt, double k2, int trial_side, float4* out, cudaStream_t st) {
  if (nt > 0) k_prepare_bounds<<<(nt + 255) / 256, 256, 0, st>>>(g, nt, k2, trial_side, out);
}
void launch_classify(bool fill, const float4* tb, const float4* bb, const Geo64* tg, const Geo64* bg, int nt, int nb,
                     double k2, int* count, const int64_t* offset, int* out_tau, int* out_sigma, int8_t* out_cls,
                     int* err, int num_sms, cudaStream_t st) {
  if (nt <= 0) return;
  int blocks = (nt + 7) / 8;
  blocks = blocks < num_sms * 16 ? blocks : num_sms * 16;
  if (fill)
    k_classify<true><<<blocks, 256, 0, st>>>(tb, bb, tg, bg, nt, nb, k2, count, offset, out_tau, out_sigma, out_cls, err);
  else
    k_classify<false><<<blocks, 256, 0, st>>>(tb, bb, tg, bg, nt, nb, k2, count, offset, out_tau, out_sigma, out_cls, err);
}
void launch_scan(const int* counts, int n, int64_t* offsets, cudaStream_t st) {
  k_scan_counts<<<1, 1024, 0, st>>>(counts, n, offsets);
}
void launch_classify_dense(const Geo64* tg, const Geo64* bg, int t0, int t1, int s0, int s1, double k2, int8_t* out,
                           int* err, cudaStream_t st) {
  int64_t total = (int64_t)(t1 - t0) * (s1 - s0);
  if (total <= 0) return;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 65535) blocks = 65535;
  k_classify_dense<<<(int)blocks, 256, 0, st>>>(tg, bg, t0, t1, s0, s1, k2, out, err);
}
void launch_singular(const OpParams& op, const QuadSel& qs, const RuleTable& rules, int rsA, int rsB, const Geo64* tg,
                     const Geo64* bg, const int* et, const int* es, const int8_t* ec, int64_t n, double2* out,
                     const volatile int* abort_flag, int num_sms, cudaStream_t st) {
  if (n <= 0) return;
  int64_t blocks = (n + 7) / 8;
  if (blocks > (int64_t)num_sms * 32) blocks = (int64_t)num_sms * 32;
  k_singular<<<(int)blocks, 256, 0, st>>>(op, qs, rules, rsA, rsB, tg, bg, et, es, ec, n, out, abort_flag);
}
void launch_local_diag64(const OpParams& op, const QuadSel& qs, const RuleTable& rules, int rsA, int rsB,
                         const Geo64* tg, const Geo64* bg, const int* tau, const int* sigma, int64_t n, int force,
                         double2* out, int8_t* cls, int* err, int num_sms, cudaStream_t st) {
  if (n <= 0) return;
  int64_t blocks = (n + 7) / 8;
  if (blocks > (int64_t)num_sms * 32) blocks = (int64_t)num_sms * 32;
  k_local_diag64<<<(int)blocks, 256, 0, st>>>(op, qs, rules, rsA, rsB, tg, bg, tau, sigma, n, force, out, cls, err);
}

}  // namespace bgb
