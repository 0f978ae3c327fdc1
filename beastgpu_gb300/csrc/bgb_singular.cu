// Geometry preparation, pair classification and the FP64 singular / near-pair kernels.
//
//  k_prepare_geo64    FP64 simplex data per triangle (CompScienceMeshes rounding).
//  k_prepare_bounds   FP32 bounding spheres used to skip obviously-far pairs.
//  k_classify<FILL>   one warp per test triangle sweeps all trial triangles: an FP32 sphere
//                     test rejects far pairs, the exact FP64 predicate (BEAST quadrule,
//                     doubleQuadRuleMainCase.jl:187-200) decides the rest; non-far pairs are
//                     compacted in trial order (ballot/popc), so the list is deterministic.
//  k_singular<OP>     one warp per non-far pair: Sauter-Schwab CF/CE/CV (SauterSchwab.jl:212-297)
//                     or the near-pair rule with singularity extraction (BEAST's WiltonSERule:
//                     closed-form inner integrals of 1/R - gamma + gamma^2 R / 2, the smooth rest
//                     by the near double rule), FP64.  Each point adds a few operator moments
//                     (8-10 complex), reduced by warp shuffles; the 3x3 complex local matrix is
//                     formed once per pair (no atomics).
//  k_classify_dense   diagnostic: exact class of every pair of a block.
#include "bgb_kernels.cuh"
#include "bgb_ss.cuh"

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

// One sphere around the spheres of 32 consecutive trial triangles (chunk c = [32 c, 32 c + 32)),
// inflated so that the FP32 sphere test against it is true whenever it is true for a member:
// the classifier skips a whole chunk with one test.  Tight when consecutive triangles are
// spatially close (structured and hierarchical meshes); still correct when they are not.
__global__ void k_chunk_bounds(const float4* __restrict__ b, int nb, float4* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int s0 = 32 * c, s1 = min(nb, s0 + 32);
  if (s0 >= nb) return;
  double m[3] = {0.0, 0.0, 0.0};
  for (int s = s0; s < s1; ++s) {
    m[0] += b[s].x;
    m[1] += b[s].y;
    m[2] += b[s].z;
  }
  for (int k = 0; k < 3; ++k) m[k] /= (double)(s1 - s0);
  const float cx = (float)m[0], cy = (float)m[1], cz = (float)m[2];
  double R = 0.0;
  for (int s = s0; s < s1; ++s) {
    const double d0 = (double)b[s].x - cx, d1 = (double)b[s].y - cy, d2 = (double)b[s].z - cz;
    R = fmax(R, sqrt(d0 * d0 + d1 * d1 + d2 * d2) + (double)b[s].w);
  }
  const double cn = sqrt((double)cx * cx + (double)cy * cy + (double)cz * cz);
  R = R * (1.0 + 1e-5) + 1e-6 * (cn + R) + 1e-30;
  out[c] = make_float4(cx, cy, cz, __double2float_ru(R));
}

// ----------------------------------------------------------------------------------------
// Exact FP64 predicate (doubleQuadRuleMainCase.jl:187-200; codes quadrule_determine.jl:76).
// Rounded like the Julia code: no contraction, IEEE sqrt and division.  *mask (optional)
// receives the coincident vertex pairs, bit u1 * 3 + u2 (the same test as the reference's
// vertex matching, pulledback_integrand_gpu.jl:41-51).
// ----------------------------------------------------------------------------------------
__device__ int classify_exact(const Geo64& a, const Geo64& b, double k2, int* mask = nullptr) {
  const double dtol = 2.220446049250313e-16 * 1.0e3;
  const double xtol2 = 0.2 * 0.2;
  int hits = 0, m = 0;
  double dmin2 = 1.7976931348623157e308;  // floatmax(Float64)
#pragma unroll
  for (int u1 = 0; u1 < 3; ++u1)
#pragma unroll
    for (int u2 = 0; u2 < 3; ++u2) {
      double dx = __dsub_rn(a.v[u1][0], b.v[u2][0]);
      double dy = __dsub_rn(a.v[u1][1], b.v[u2][1]);
      double dz = __dsub_rn(a.v[u1][2], b.v[u2][2]);
      double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
      const bool hit = __dsqrt_rn(d2) < dtol;
      hits += hit;
      m |= (int)hit << (u1 * 3 + u2);
      dmin2 = fmin(dmin2, d2);
    }
  if (mask) *mask = m;
  if (hits > 3) return -1;
  if (hits > 0) return hits;
  const double mx = fmax(__dmul_rn(dmin2, k2), __ddiv_rn(dmin2, __dmul_rn(16.0, b.area)));
  return (mx >= xtol2) ? BGB_CLASS_FAR : BGB_CLASS_NEAR;
}

// One warp classifies test triangle tau against trial triangles [s_begin, s_end).  The FP32
// sphere test sweeps 32 trial triangles per step; its candidates are queued (ascending) in a
// per-warp shared-memory list, and the exact FP64 predicate runs on 32 queued candidates at a
// time, one per lane, instead of on whichever lanes happen to hold a candidate (a divergent
// FP64 warp pays the full warp cost for one lane).  The output order stays trial-ascending.
template <bool FILL>
__device__ __forceinline__ void classify_sweep(int tau, float4 a, const Geo64& A, int s_begin, int s_end,
                                               const float4* __restrict__ bb, const float4* __restrict__ cb,
                                               const Geo64* __restrict__ bg,
                                               double k2, int* __restrict__ queue, int* __restrict__ count,
                                               const int64_t* __restrict__ offset, int* __restrict__ out_tau,
                                               int* __restrict__ out_sigma, int8_t* __restrict__ out_cls,
                                               int16_t* __restrict__ out_mask, int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int64_t base = FILL ? offset[tau] : 0;
  int n = 0, queued = 0;
  auto drain = [&](int k) {  // classify queue[0..k) (k <= 32), one candidate per lane
    int cls = 0, mask = 0, s = 0;
    if (lane < k) {
      s = queue[lane];
      cls = classify_exact(A, bg[s], k2, &mask);
      if (cls < 0) {
        atomicOr(err, 1);
        cls = 0;
      }
    }
    const unsigned bal = __ballot_sync(0xffffffffu, cls != 0);
    if (FILL && cls != 0) {
      const int64_t pos = base + n + __popc(bal & ((1u << lane) - 1u));
      out_tau[pos] = tau;
      out_sigma[pos] = s;
      out_cls[pos] = (int8_t)cls;
      if (out_mask) out_mask[pos] = (int16_t)mask;
    }
    n += __popc(bal);
  };
  for (int c = s_begin >> 5; 32 * c < s_end; ++c) {
    if (cb && !sphere_candidate(a, cb[c])) continue;  // no member of the chunk can be near (warp-uniform)
    const int s = 32 * c + lane;
    const bool cand = s >= s_begin && s < s_end && sphere_candidate(a, bb[s]);
    const unsigned bal = __ballot_sync(0xffffffffu, cand);
    if (cand) queue[queued + __popc(bal & ((1u << lane) - 1u))] = s;  // queued < 32: room for 32 more
    queued += __popc(bal);
    __syncwarp();
    if (queued >= 32) {
      drain(32);
      __syncwarp();
      const int rest = queued - 32;
      const int moved = lane < rest ? queue[32 + lane] : 0;
      __syncwarp();
      if (lane < rest) queue[lane] = moved;
      __syncwarp();
      queued = rest;
    }
  }
  if (queued > 0) drain(queued);
  __syncwarp();
  if (!FILL && lane == 0) count[tau] = n;
}

template <bool FILL>
__global__ void __launch_bounds__(256) k_classify(const float4* __restrict__ tb, const float4* __restrict__ bb,
                                                  const float4* __restrict__ cb,
                                                  const Geo64* __restrict__ tg, const Geo64* __restrict__ bg,
                                                  int nt, int nb, double k2, int* __restrict__ count,
                                                  const int64_t* __restrict__ offset, int* __restrict__ out_tau,
                                                  int* __restrict__ out_sigma, int8_t* __restrict__ out_cls,
                                                  int16_t* __restrict__ out_mask, int* __restrict__ err) {
  __shared__ int queues[8][64];
  int* queue = queues[threadIdx.x >> 5];
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int tau = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; tau < nt; tau += warps) {
    const Geo64 A = tg[tau];
    classify_sweep<FILL>(tau, tb[tau], A, 0, nb, bb, cb, bg, k2, queue, count, offset, out_tau, out_sigma, out_cls,
                         out_mask, err);
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

// Entries per class (0..4) of the non-far list, warp-aggregated, into hist[5] (zeroed by the caller).
__global__ void k_class_hist(const int8_t* __restrict__ cls, int64_t n, unsigned long long* __restrict__ hist) {
  const int lane = threadIdx.x & 31;
  for (int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~(int64_t)31; b < n;
       b += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = b + lane;
    const int c = e < n ? (int)cls[e] : -1;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const unsigned m = __ballot_sync(0xffffffffu, c == k);
      if (lane == 0 && m) atomicAdd(&hist[k], (unsigned long long)__popc(m));
    }
  }
}

// Singular entries in groups: entry e belongs to group tri_group[ent_sigma[e]] (clamped to
// [0, ngroups)).  Count per group (a shared histogram when the groups fit), scan, then place each
// entry at the next free position of its group.  The order inside a group depends on the atomics;
// each entry writes only its own local matrix, so the results do not.
constexpr int kGroupHist = 2048;
__device__ __forceinline__ int entry_group(const int* __restrict__ sigma, const int* __restrict__ tri_group, int64_t e,
                                           int ngroups) {
  const int g = tri_group[sigma[e]];
  return (g < 0 || g >= ngroups) ? ngroups - 1 : g;
}
__global__ void k_group_count(const int* __restrict__ sigma, int64_t n, const int* __restrict__ tri_group, int ngroups,
                              int* __restrict__ counts) {
  __shared__ int hist[kGroupHist];
  const bool sh = ngroups <= kGroupHist;
  if (sh)
    for (int i = threadIdx.x; i < ngroups; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int g = entry_group(sigma, tri_group, e, ngroups);
    if (sh) atomicAdd(&hist[g], 1);
    else atomicAdd(&counts[g], 1);
  }
  __syncthreads();
  if (sh)
    for (int i = threadIdx.x; i < ngroups; i += blockDim.x)
      if (hist[i]) atomicAdd(&counts[i], hist[i]);
}
__global__ void k_group_fill(const int* __restrict__ sigma, int64_t n, const int* __restrict__ tri_group, int ngroups,
                             const int64_t* __restrict__ off, int* __restrict__ cursor, int* __restrict__ perm) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int g = entry_group(sigma, tri_group, e, ngroups);
    perm[off[g] + atomicAdd(&cursor[g], 1)] = (int)e;
  }
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
// ----------------------------------------------------------------------------------------
// Integrand moments.  Each evaluation point adds a handful of operator-specific moments
// (instead of 9 shape-function products); the 3x3 local matrix is formed once per pair.
//   Helmholtz SL: m[a][b] = sum G p_a q_b,  p = (1, bx1, bx2), q = (1, by1, by2) (chart
//                 coordinates), f = (bx1, bx2, 1-bx1-bx2).
//   Maxwell SL:   S = sum G X.Y, Px = sum G X, Py = sum G Y, P0 = sum G  (X, Y relative to the
//                 centroids), f_i.g_j = (X - V_i).(Y - W_j) / (4 A_tau A_sigma).
//   Maxwell DL:   A1 = sum H X.(d x Y), B = sum H d x Y, C = sum H X x d, E = sum H d with
//                 grad_x G = H d, d = x - y.
// ----------------------------------------------------------------------------------------
template <int OP>
struct NAcc { static constexpr int N = OP == BGB_OP_MAXWELL3D_SL ? 8 : (OP == BGB_OP_MAXWELL3D_DL ? 10 : 9); };

// The Helmholtz operators on Lagrange hats share the 9 hat moments.
__host__ __device__ constexpr bool hat_op(int op) {
  return op == BGB_OP_HELMHOLTZ3D_SL || op == BGB_OP_HELMHOLTZ3D_DL || op == BGB_OP_HELMHOLTZ3D_DLT ||
         op == BGB_OP_HELMHOLTZ3D_HS;
}
// Double layers vanish on a flat common face ((x - y) . n = 0).
__host__ __device__ constexpr bool flat_face_zero(int op) {
  return op == BGB_OP_MAXWELL3D_DL || op == BGB_OP_HELMHOLTZ3D_DL || op == BGB_OP_HELMHOLTZ3D_DLT;
}
__device__ inline void unit_normal(const Geo64& T, double n[3]) {
  const double inv = 1.0 / (2.0 * T.area);
  n[0] = (T.t[0][1] * T.t[1][2] - T.t[0][2] * T.t[1][1]) * inv;
  n[1] = (T.t[0][2] * T.t[1][0] - T.t[0][0] * T.t[1][2]) * inv;
  n[2] = (T.t[0][0] * T.t[1][1] - T.t[0][1] * T.t[1][0]) * inv;
}

struct PairGeo {
  double xa[3][3];   // x = xa[0] + xa[1] u1 + xa[2] u2   (test point from SS chart params)
  double xb[3][3];
  double ba[3][2];   // (bx1, bx2) = ba[0] + ba[1] u1 + ba[2] u2
  double bb[3][2];
  double cA[3], cB[3];
};

__device__ inline void make_pair_geo(const Geo64& A, const Geo64& B, const Chart& cA, const Chart& cB, PairGeo& P) {
  // chart (u1, u2) -> barycentric (b1, b2) -> cartesian, composed into one affine map per side
  const Geo64* T[2] = {&A, &B};
  const Chart* C[2] = {&cA, &cB};
  for (int side = 0; side < 2; ++side) {
    double(*ba)[2] = side ? P.bb : P.ba;
    double(*xa)[3] = side ? P.xb : P.xa;
    const Chart& ch = *C[side];
    const Geo64& G = *T[side];
    ba[0][0] = ch.cv[2][0]; ba[0][1] = ch.cv[2][1];
    ba[1][0] = ch.ct[0][0]; ba[1][1] = ch.ct[0][1];
    ba[2][0] = ch.ct[1][0]; ba[2][1] = ch.ct[1][1];
    for (int c = 0; c < 3; ++c) {
      xa[0][c] = G.v[2][c] + G.t[0][c] * ba[0][0] + G.t[1][c] * ba[0][1];
      xa[1][c] = G.t[0][c] * ba[1][0] + G.t[1][c] * ba[1][1];
      xa[2][c] = G.t[0][c] * ba[2][0] + G.t[1][c] * ba[2][1];
    }
  }
  for (int c = 0; c < 3; ++c) {
    P.cA[c] = (A.v[0][c] + A.v[1][c] + A.v[2][c]) / 3.0;
    P.cB[c] = (B.v[0][c] + B.v[1][c] + B.v[2][c]) / 3.0;
  }
}

// e2 = exp(-z) - 1 + z and e3 = e2 - z^2 / 2 for complex z = (zr, zi): the power series for
// |z| < 1 (Horner, terms to (-z)^20 / 20!), the exponential beyond.
__device__ inline void exp_tails(double zr, double zi, double2& e2, double2& e3) {
  const double2 mz = make_double2(-zr, -zi);
  const double2 z2h = make_double2(0.5 * (zr * zr - zi * zi), zr * zi);
  if (zr * zr + zi * zi < 1.0) {
    double2 s = make_double2(1.0, 0.0);
    for (int n = 20; n >= 4; --n) {
      const double2 t = cmul(s, mz);
      s = make_double2(1.0 + t.x / n, t.y / n);
    }
    const double2 m3 = cmul(cmul(mz, mz), mz);
    e3 = cmul(make_double2(m3.x / 6.0, m3.y / 6.0), s);
    e2 = cadd(e3, z2h);
    return;
  }
  const double er = exp(-zr);
  double sn, cs;
  sincos(-zi, &sn, &cs);
  e2 = make_double2(er * cs - 1.0 + zr, er * sn + zi);
  e3 = make_double2(e2.x - z2h.x, e2.y - z2h.y);
}

// Add one point pair with weight w (quadrature weights and Jacobians included).  REG: the
// regular part of the kernel of a near pair, G_r = (exp(-z) - 1 + z - z^2/2) / (4 pi R), z = gamma R,
// with grad_x G_r = F (x - y), F = -(z e2 + e3) / (4 pi R^3).
template <int OP, bool REG = false>
__device__ __forceinline__ void add_point(const OpParams& op, const double x[3], const double y[3], double bx1,
                                          double bx2, double by1, double by2, const double cA[3],
                                          const double cB[3], const double nA[3], const double nB[3], double w,
                                          double2* acc) {
  const double d0 = x[0] - y[0], d1 = x[1] - y[1], d2 = x[2] - y[2];
  const double R2 = d0 * d0 + d1 * d1 + d2 * d2;
  const double rinv = rsqrt(R2);
  const double R = R2 * rinv;
  double gr, gi, Fr = 0.0, Fi = 0.0;
  if (REG) {
    const double zr = op.gamma[0] * R, zi = op.gamma[1] * R;
    double2 e2, e3;
    exp_tails(zr, zi, e2, e3);
    const double a = w * BGB_INV_4PI_D * rinv;
    gr = a * e3.x;
    gi = a * e3.y;
    const double2 c = cadd(cmul(make_double2(zr, zi), e2), e3);
    const double b = -a * rinv * rinv;
    Fr = b * c.x;
    Fi = b * c.y;
  } else {
    double sn = 0.0, cs = 1.0;
    if (op.gamma[1] != 0.0) sincos(op.gamma[1] * R, &sn, &cs);
    double amp = w * BGB_INV_4PI_D * rinv;
    if (op.gamma[0] != 0.0) amp *= exp(-op.gamma[0] * R);
    gr = amp * cs;
    gi = -amp * sn;
  }
  if (hat_op(OP)) {
    double hr = gr, hi = gi;
    if (OP == BGB_OP_HELMHOLTZ3D_DL || OP == BGB_OP_HELMHOLTZ3D_DLT) {
      // dG/dn_y = (gamma + 1/R) G ((x - y) . n_y) / R; dG/dn_x = -(gamma + 1/R) G ((x - y) . n_x) / R
      const double* nv = OP == BGB_OP_HELMHOLTZ3D_DL ? nB : nA;
      double rn = (d0 * nv[0] + d1 * nv[1] + d2 * nv[2]) * rinv;
      if (OP == BGB_OP_HELMHOLTZ3D_DLT) rn = -rn;
      if (REG) {  // n_y.grad_y G_r = -F (x - y).n_y, n_x.grad_x G_r = F (x - y).n_x: both -F rn R
        hr = -Fr * rn * R;
        hi = -Fi * rn * R;
      } else {
        const double t = (op.gamma[0] + rinv) * rn, u = op.gamma[1] * rn;
        hr = t * gr - u * gi;
        hi = t * gi + u * gr;
      }
    }
    const double p[3] = {1.0, bx1, bx2}, q[3] = {1.0, by1, by2};
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const double pq = p[a] * q[b];
        acc[a * 3 + b].x = fma(hr, pq, acc[a * 3 + b].x);
        acc[a * 3 + b].y = fma(hi, pq, acc[a * 3 + b].y);
      }
  } else if (OP == BGB_OP_MAXWELL3D_SL) {
    const double X0 = x[0] - cA[0], X1 = x[1] - cA[1], X2 = x[2] - cA[2];
    const double Y0 = y[0] - cB[0], Y1 = y[1] - cB[1], Y2 = y[2] - cB[2];
    const double xy = X0 * Y0 + X1 * Y1 + X2 * Y2;
    acc[0].x = fma(gr, xy, acc[0].x); acc[0].y = fma(gi, xy, acc[0].y);
    acc[1].x = fma(gr, X0, acc[1].x); acc[1].y = fma(gi, X0, acc[1].y);
    acc[2].x = fma(gr, X1, acc[2].x); acc[2].y = fma(gi, X1, acc[2].y);
    acc[3].x = fma(gr, X2, acc[3].x); acc[3].y = fma(gi, X2, acc[3].y);
    acc[4].x = fma(gr, Y0, acc[4].x); acc[4].y = fma(gi, Y0, acc[4].y);
    acc[5].x = fma(gr, Y1, acc[5].x); acc[5].y = fma(gi, Y1, acc[5].y);
    acc[6].x = fma(gr, Y2, acc[6].x); acc[6].y = fma(gi, Y2, acc[6].y);
    acc[7].x += gr; acc[7].y += gi;
  } else {
    // H = -(gamma + 1/R) G / R (F for the regular part)
    const double g2r = gr * rinv, g2i = gi * rinv;
    const double re = op.gamma[0] + rinv;
    const double Hx = REG ? Fr : -(re * g2r - op.gamma[1] * g2i), Hy = REG ? Fi : -(re * g2i + op.gamma[1] * g2r);
    const double X0 = x[0] - cA[0], X1 = x[1] - cA[1], X2 = x[2] - cA[2];
    const double Y0 = y[0] - cB[0], Y1 = y[1] - cB[1], Y2 = y[2] - cB[2];
    const double e0 = d1 * Y2 - d2 * Y1, e1 = d2 * Y0 - d0 * Y2, e2 = d0 * Y1 - d1 * Y0;  // d x Y
    const double f0 = X1 * d2 - X2 * d1, f1 = X2 * d0 - X0 * d2, f2 = X0 * d1 - X1 * d0;  // X x d
    const double a1 = X0 * e0 + X1 * e1 + X2 * e2;
    const double v[10] = {a1, e0, e1, e2, f0, f1, f2, d0, d1, d2};
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      acc[k].x = fma(Hx, v[k], acc[k].x);
      acc[k].y = fma(Hy, v[k], acc[k].y);
    }
  }
}

// ----------------------------------------------------------------------------------------
// Near pairs: the singular part G_s = (1/R - gamma + gamma^2 R / 2) / (4 pi) integrated in closed
// form over a flat triangle T at the point x (Wilton et al. 1984; Graglia 1993).  With n the chart
// normal, d = n.(x - v3), rho = x - d n: Im1 = int 1/R, I1 = int R, Jm1 = int (y - rho)/R,
// J1 = int (y - rho) R, Om = int d/R^3 (signed solid angle, Van Oosterom & Strackee 1983),
// Jm3 = int (y - rho)/R^3, from edge sums over a -> b (counter-clockwise about n), unit tangent l,
// outward normal m = l x n, s+- = (b|a - rho).l, t0 = (a - rho).m, R0^2 = t0^2 + d^2,
// f = int_e 1/R, K1 = int_e R, K3 = int_e R^3.
// ----------------------------------------------------------------------------------------
struct SingPart {
  double2 S0, D0;    // int G_s, int n.grad_y G_s  (n.grad_y G_s = (d/R^3 - gamma^2 d / (2R)) / (4 pi))
  double2 Sv[3];     // int G_s (y - rho)
  double2 Gv[3];     // int grad_x G_s
  double2 Dv[3];     // int n.grad_y G_s (y - rho)
  double rho[3];
};

__device__ inline double dot3d(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ inline void cross3d(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

__device__ void singular_part(const Geo64& T, const double x[3], const double gam[2], SingPart& S) {
  double n[3];
  cross3d(T.t[0], T.t[1], n);
  const double inn = 1.0 / sqrt(dot3d(n, n));
  for (int c = 0; c < 3; ++c) n[c] *= inn;
  double rho[3];
  const double d = n[0] * (x[0] - T.v[2][0]) + n[1] * (x[1] - T.v[2][1]) + n[2] * (x[2] - T.v[2][2]);
  for (int c = 0; c < 3; ++c) rho[c] = x[c] - d * n[c];
  double Jm1[3] = {0, 0, 0}, J1[3] = {0, 0, 0}, Jm3[3] = {0, 0, 0};
  double sum_tf = 0.0, sum_tk1 = 0.0;
#pragma unroll 1
  for (int e = 0; e < 3; ++e) {
    const double* a = T.v[e];
    const double* b = T.v[e == 2 ? 0 : e + 1];
    double l[3], m[3], ar[3], br[3], ax[3], bx[3];
    for (int c = 0; c < 3; ++c) {
      l[c] = b[c] - a[c];
      ar[c] = a[c] - rho[c];
      br[c] = b[c] - rho[c];
      ax[c] = x[c] - a[c];
      bx[c] = x[c] - b[c];
    }
    const double il = 1.0 / sqrt(dot3d(l, l));
    for (int c = 0; c < 3; ++c) l[c] *= il;
    cross3d(l, n, m);
    const double sp = dot3d(br, l), sm = dot3d(ar, l), t0 = dot3d(ar, m);
    const double Rp = sqrt(dot3d(bx, bx)), Rm = sqrt(dot3d(ax, ax));
    const double R02 = t0 * t0 + d * d;
    double f;
    if (sp < 0.0 && sm < 0.0) f = log((Rm - sm) / (Rp - sp));  // beyond a: R0^2 cancels
    else if (sm >= 0.0) f = log((Rp + sp) / (Rm + sm));         // beyond b
    else f = log((Rp + sp) * (Rm - sm) / R02);                  // rho abreast of the edge
    const double K1 = 0.5 * ((sp * Rp - sm * Rm) + R02 * f);
    const double K3 = 0.25 * (sp * Rp * Rp * Rp - sm * Rm * Rm * Rm) + 0.75 * R02 * K1;
    sum_tf += t0 * f;
    sum_tk1 += t0 * K1;
    for (int c = 0; c < 3; ++c) {
      Jm1[c] += m[c] * K1;
      J1[c] += m[c] * K3 / 3.0;
      Jm3[c] -= m[c] * f;
    }
  }
  double q[3][3], nq[3];
  for (int i = 0; i < 3; ++i) {
    for (int c = 0; c < 3; ++c) q[i][c] = T.v[i][c] - x[c];
    nq[i] = sqrt(dot3d(q[i], q[i]));
  }
  double q12[3];
  cross3d(q[1], q[2], q12);
  const double trip = dot3d(q[0], q12);
  const double den = nq[0] * nq[1] * nq[2] + dot3d(q[0], q[1]) * nq[2] + dot3d(q[0], q[2]) * nq[1] + dot3d(q[1], q[2]) * nq[0];
  const double Om = -2.0 * atan2(trip, den);
  const double Im1 = sum_tf - d * Om;
  const double I1 = (d * d * Im1 + sum_tk1) / 3.0;
  const double i4p = BGB_INV_4PI_D;
  const double g2hr = 0.5 * (gam[0] * gam[0] - gam[1] * gam[1]), g2hi = gam[0] * gam[1];  // gamma^2 / 2
  S.S0 = make_double2((Im1 - gam[0] * T.area + g2hr * I1) * i4p, (-gam[1] * T.area + g2hi * I1) * i4p);
  S.D0 = make_double2((Om - g2hr * d * Im1) * i4p, (-g2hi * d * Im1) * i4p);
  for (int c = 0; c < 3; ++c) {
    S.rho[c] = rho[c];
    const double cen = (T.v[0][c] + T.v[1][c] + T.v[2][c]) / 3.0;
    const double a0 = T.area * (cen - rho[c]);  // int (y - rho)
    S.Sv[c] = make_double2((Jm1[c] - gam[0] * a0 + g2hr * J1[c]) * i4p, (-gam[1] * a0 + g2hi * J1[c]) * i4p);
    const double gR = d * n[c] * Im1 - Jm1[c];  // int grad_x R
    S.Gv[c] = make_double2((Jm3[c] - n[c] * Om + g2hr * gR) * i4p, (g2hi * gR) * i4p);
    S.Dv[c] = make_double2((d * Jm3[c] - g2hr * d * Jm1[c]) * i4p, (-g2hi * d * Jm1[c]) * i4p);
  }
}

// Hats of T at the in-plane point rho (affine extension) and their gradients.
__device__ inline void hat_affine(const Geo64& T, const double rho[3], double val[3], double grad[3][3]) {
  double n[3];
  cross3d(T.t[0], T.t[1], n);
  const double inn = 1.0 / sqrt(dot3d(n, n));  // 1 / (2A)
  for (int c = 0; c < 3; ++c) n[c] *= inn;
  for (int j = 0; j < 3; ++j) {
    const int j1 = j == 2 ? 0 : j + 1, j2 = j == 0 ? 2 : j - 1;
    double e[3], g[3];
    for (int c = 0; c < 3; ++c) e[c] = T.v[j2][c] - T.v[j1][c];
    cross3d(n, e, g);
    double pr = 0.0;
    for (int c = 0; c < 3; ++c) {
      grad[j][c] = g[c] * inn;
      pr += grad[j][c] * (rho[c] - (T.v[0][c] + T.v[1][c] + T.v[2][c]) / 3.0);
    }
    val[j] = 1.0 / 3.0 + pr;
  }
}

// Moments of the singular part of a near pair at one outer point (weight w): the outer point x
// lies on the test triangle with chart coordinates (u, v) and T is the trial triangle, except for
// the transposed double layer, whose outer point lies on the trial triangle and T is the test one.
template <int OP>
__device__ void add_singular_part(const OpParams& op, const Geo64& T, const double x[3], double u, double v, double w,
                                  const double cA[3], const double cB[3], double2* acc) {
  SingPart S;
  singular_part(T, x, op.gamma, S);
  if (hat_op(OP)) {
    const bool dl = OP == BGB_OP_HELMHOLTZ3D_DL || OP == BGB_OP_HELMHOLTZ3D_DLT;
    double hv[3], hg[3][3];
    hat_affine(T, S.rho, hv, hg);
    const double2 K0 = dl ? S.D0 : S.S0;
    const double2* Kv = dl ? S.Dv : S.Sv;
    double2 M[3];  // inner moments against (1, hat 0, hat 1) of T
    M[0] = K0;
    for (int h = 0; h < 2; ++h) {
      double2 t = cscale(K0, hv[h]);
      for (int c = 0; c < 3; ++c) t = cadd(t, cscale(Kv[c], hg[h][c]));
      M[h + 1] = t;
    }
    const double o[3] = {w, w * u, w * v};  // outer (1, u, v) times the weight
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        // acc[a*3+b]: test moment a, trial moment b; the transposed layer's outer point is on the trial side
        const double2 m = OP == BGB_OP_HELMHOLTZ3D_DLT ? cscale(M[a], o[b]) : cscale(M[b], o[a]);
        acc[a * 3 + b] = cadd(acc[a * 3 + b], m);
      }
  } else if (OP == BGB_OP_MAXWELL3D_SL) {
    const double X[3] = {x[0] - cA[0], x[1] - cA[1], x[2] - cA[2]};
    double2 V[3];
    for (int c = 0; c < 3; ++c) V[c] = cadd(S.Sv[c], cscale(S.S0, S.rho[c] - cB[c]));  // int G_s (y - cB)
    double2 xv = make_double2(0.0, 0.0);
    for (int c = 0; c < 3; ++c) xv = cadd(xv, cscale(V[c], X[c]));
    acc[0] = cadd(acc[0], cscale(xv, w));
    for (int c = 0; c < 3; ++c) {
      acc[1 + c] = cadd(acc[1 + c], cscale(S.S0, w * X[c]));
      acc[4 + c] = cadd(acc[4 + c], cscale(V[c], w));
    }
    acc[7] = cadd(acc[7], cscale(S.S0, w));
  } else {
    // Maxwell double layer: int grad_x G_s x (y - cB) = Gv x (x - cB) (grad_x G is parallel to x - y)
    const double X[3] = {x[0] - cA[0], x[1] - cA[1], x[2] - cA[2]};
    const double xc[3] = {x[0] - cB[0], x[1] - cB[1], x[2] - cB[2]};
    const double2* G = S.Gv;
    const double2 Bv[3] = {cadd(cscale(G[1], xc[2]), cscale(G[2], -xc[1])), cadd(cscale(G[2], xc[0]), cscale(G[0], -xc[2])),
                           cadd(cscale(G[0], xc[1]), cscale(G[1], -xc[0]))};
    const double2 Cv[3] = {cadd(cscale(G[2], X[1]), cscale(G[1], -X[2])), cadd(cscale(G[0], X[2]), cscale(G[2], -X[0])),
                           cadd(cscale(G[1], X[0]), cscale(G[0], -X[1]))};
    double2 a1 = make_double2(0.0, 0.0);
    for (int c = 0; c < 3; ++c) a1 = cadd(a1, cscale(Bv[c], X[c]));
    acc[0] = cadd(acc[0], cscale(a1, w));
    for (int c = 0; c < 3; ++c) {
      acc[1 + c] = cadd(acc[1 + c], cscale(Bv[c], w));
      acc[4 + c] = cadd(acc[4 + c], cscale(Cv[c], w));
      acc[7 + c] = cadd(acc[7 + c], cscale(G[c], w));
    }
  }
}

// Local matrix L[i][j] from the moments.
template <int OP>
__device__ inline void finalize(const OpParams& op, const Geo64& A, const Geo64& B, const double cA[3],
                                const double cB[3], const double2* acc, double2 L[3][3]) {
  const double2 alpha = make_double2(op.alpha[0], op.alpha[1]);
  if (hat_op(OP)) {
    // f = T p with T = [[0,1,0],[0,0,1],[1,-1,-1]]
    const double T[3][3] = {{0, 1, 0}, {0, 0, 1}, {1, -1, -1}};
    double2 a = alpha, bP = make_double2(0, 0);
    double cA3[3][3], cB3[3][3];
    if (OP == BGB_OP_HELMHOLTZ3D_HS) {
      // alpha (n_x . n_y) int int f g G + beta (curl f . curl g) int int G, int int G = acc[0]
      double nA[3], nB[3];
      unit_normal(A, nA);
      unit_normal(B, nB);
      const double nn = nA[0] * nB[0] + nA[1] * nB[1] + nA[2] * nB[2];
      a = make_double2(alpha.x * nn, alpha.y * nn);
      bP = cmul(make_double2(op.beta[0], op.beta[1]), acc[0]);
      const double ia = 1.0 / (2.0 * A.area), ib = 1.0 / (2.0 * B.area);
      for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) {  // curl of hat i: (v_{i+1} - v_{i+2}) / (2A)
          cA3[i][c] = (A.v[(i + 1) % 3][c] - A.v[(i + 2) % 3][c]) * ia;
          cB3[i][c] = (B.v[(i + 1) % 3][c] - B.v[(i + 2) % 3][c]) * ib;
        }
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double2 s = make_double2(0, 0);
        for (int p = 0; p < 3; ++p)
          for (int q = 0; q < 3; ++q) {
            const double t = T[i][p] * T[j][q];
            s.x += t * acc[p * 3 + q].x;
            s.y += t * acc[p * 3 + q].y;
          }
        L[i][j] = cmul(a, s);
        if (OP == BGB_OP_HELMHOLTZ3D_HS) {
          const double cc = cA3[i][0] * cB3[j][0] + cA3[i][1] * cB3[j][1] + cA3[i][2] * cB3[j][2];
          L[i][j].x += cc * bP.x;
          L[i][j].y += cc * bP.y;
        }
      }
    return;
  }
  const double inv4AA = 1.0 / (4.0 * A.area * B.area);
  double V[3][3], W[3][3];
  for (int i = 0; i < 3; ++i)
    for (int c = 0; c < 3; ++c) {
      V[i][c] = A.v[i][c] - cA[c];
      W[i][c] = B.v[i][c] - cB[c];
    }
  const double2 ca = cscale(alpha, inv4AA);
  if (OP == BGB_OP_MAXWELL3D_SL) {
    const double2 S = acc[0], P0 = acc[7];
    const double2 tb = cmul(cscale(make_double2(op.beta[0], op.beta[1]), 4.0 * inv4AA), P0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double2 t = S;
        for (int c = 0; c < 3; ++c) {
          t.x -= V[i][c] * acc[4 + c].x + W[j][c] * acc[1 + c].x;
          t.y -= V[i][c] * acc[4 + c].y + W[j][c] * acc[1 + c].y;
        }
        const double vw = V[i][0] * W[j][0] + V[i][1] * W[j][1] + V[i][2] * W[j][2];
        t.x += vw * P0.x;
        t.y += vw * P0.y;
        L[i][j] = cadd(cmul(ca, t), tb);
      }
    return;
  }
  // MFIE: alpha/(4AA) (A1 - W_j.C - V_i.B + V_i.(E x W_j)); B = acc[1..3], C = acc[4..6], E = acc[7..9]
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double2 t = acc[0];
      const double* w = W[j];
      const double* v = V[i];
      for (int c = 0; c < 3; ++c) {
        t.x -= w[c] * acc[4 + c].x + v[c] * acc[1 + c].x;
        t.y -= w[c] * acc[4 + c].y + v[c] * acc[1 + c].y;
      }
      const double2 x0 = make_double2(acc[8].x * w[2] - acc[9].x * w[1], acc[8].y * w[2] - acc[9].y * w[1]);
      const double2 x1 = make_double2(acc[9].x * w[0] - acc[7].x * w[2], acc[9].y * w[0] - acc[7].y * w[2]);
      const double2 x2 = make_double2(acc[7].x * w[1] - acc[8].x * w[0], acc[7].y * w[1] - acc[8].y * w[0]);
      t.x += v[0] * x0.x + v[1] * x1.x + v[2] * x2.x;
      t.y += v[0] * x0.y + v[1] * x1.y + v[2] * x2.y;
      L[i][j] = cmul(ca, t);
    }
}

// Integral of one non-far pair by a warp; every lane returns the full (reduced) matrix.  NEAR:
// near pairs only (the other branches are not compiled: fewer registers, more warps per SM).
template <int OP, bool NEAR = false>
__device__ void pair_integral64(const OpParams& op, const QuadSel& qs, const RuleTable& rules, int cls,
                                const Geo64& A, const Geo64& B, double2 L[3][3]) {
  if (NEAR) cls = BGB_CLASS_NEAR;
  constexpr int NA = NAcc<OP>::N;
  const int lane = threadIdx.x & 31;
  double2 acc[NA];
#pragma unroll
  for (int k = 0; k < NA; ++k) acc[k] = make_double2(0.0, 0.0);
  double cA[3], cB[3], nA[3] = {0, 0, 0}, nB[3] = {0, 0, 0};
  for (int c = 0; c < 3; ++c) {
    cA[c] = (A.v[0][c] + A.v[1][c] + A.v[2][c]) / 3.0;
    cB[c] = (B.v[0][c] + B.v[1][c] + B.v[2][c]) / 3.0;
  }
  if (OP == BGB_OP_HELMHOLTZ3D_DLT) unit_normal(A, nA);
  if (OP == BGB_OP_HELMHOLTZ3D_DL) unit_normal(B, nB);
  if (cls == BGB_CLASS_NEAR || cls == BGB_CLASS_FAR) {
    const int rt = cls == BGB_CLASS_NEAR ? qs.near_t : qs.far_t;
    const int rb = cls == BGB_CLASS_NEAR ? qs.near_b : qs.far_b;
    const int qt = rules.npoints[rt], qb = rules.npoints[rb];
    for (int idx = lane; idx < qt * qb; idx += 32) {
      const int I = idx / qb, J = idx - I * qb;
      const double* p = rules.uvw[rules.offset[rt] + I];
      const double* q = rules.uvw[rules.offset[rb] + J];
      double x[3], y[3];
      for (int c = 0; c < 3; ++c) {
        x[c] = __dadd_rn(__dadd_rn(A.v[2][c], __dmul_rn(A.t[0][c], p[0])), __dmul_rn(A.t[1][c], p[1]));
        y[c] = __dadd_rn(__dadd_rn(B.v[2][c], __dmul_rn(B.t[0][c], q[0])), __dmul_rn(B.t[1][c], q[1]));
      }
      const double w = ((p[2] / 2.0) * (A.area * 2.0)) * ((q[2] / 2.0) * (B.area * 2.0));
      if (cls == BGB_CLASS_NEAR) add_point<OP, true>(op, x, y, p[0], p[1], q[0], q[1], cA, cB, nA, nB, w, acc);
      else add_point<OP>(op, x, y, p[0], p[1], q[0], q[1], cA, cB, nA, nB, w, acc);
    }
    if (cls == BGB_CLASS_NEAR) {  // the singular part: closed form inside, one outer point per lane
      constexpr bool swap = OP == BGB_OP_HELMHOLTZ3D_DLT;
      const Geo64& O = swap ? B : A;
      const int ro = swap ? rb : rt;
      for (int I = lane; I < rules.npoints[ro]; I += 32) {
        const double* p = rules.uvw[rules.offset[ro] + I];
        double x[3];
        for (int c = 0; c < 3; ++c)
          x[c] = __dadd_rn(__dadd_rn(O.v[2][c], __dmul_rn(O.t[0][c], p[0])), __dmul_rn(O.t[1][c], p[1]));
        add_singular_part<OP>(op, swap ? A : B, x, p[0], p[1], (p[2] / 2.0) * (O.area * 2.0), cA, cB, acc);
      }
    }
  } else if (!(flat_face_zero(OP) && cls == BGB_CLASS_CF)) {  // double layers on a flat face are 0
    int I[3], J[3];
    ss_permutation(cls, A, B, I, J);
    Chart chA, chB;
    make_chart(I, chA);
    make_chart(J, chB);
    PairGeo P;
    make_pair_geo(A, B, chA, chB, P);
    const double jac = (4.0 * A.area) * B.area;  // Jacobians 2A * 2A
    const int n = qs.ss[cls];
    const int n2 = n * n, n3 = n2 * n, n4 = n3 * n;
    const int nreg = cls == BGB_CLASS_CV ? 2 : (cls == BGB_CLASS_CE ? 5 : 6);
    const double* gx = qs.gl_x[cls];
    const double* gw = qs.gl_w[cls];
    for (int idx = lane; idx < n4; idx += 32) {
      const int i = idx / n3, j = (idx / n2) % n, k = (idx / n) % n, l = idx % n;
      const double wt = gw[i] * gw[j] * gw[k] * gw[l];
#pragma unroll 1
      for (int r = 0; r < nreg; ++r) {
        double u1, u2, v1, v2, mul;
        ss_region(cls, r, gx[i], gx[j], gx[k], gx[l], wt, u1, u2, v1, v2, mul);
        double x[3], y[3];
        for (int c = 0; c < 3; ++c) {
          x[c] = P.xa[0][c] + P.xa[1][c] * u1 + P.xa[2][c] * u2;
          y[c] = P.xb[0][c] + P.xb[1][c] * v1 + P.xb[2][c] * v2;
        }
        double bx1 = 0, bx2 = 0, by1 = 0, by2 = 0;
        if (hat_op(OP)) {
          bx1 = P.ba[0][0] + P.ba[1][0] * u1 + P.ba[2][0] * u2;
          bx2 = P.ba[0][1] + P.ba[1][1] * u1 + P.ba[2][1] * u2;
          by1 = P.bb[0][0] + P.bb[1][0] * v1 + P.bb[2][0] * v2;
          by2 = P.bb[0][1] + P.bb[1][1] * v1 + P.bb[2][1] * v2;
        }
        add_point<OP>(op, x, y, bx1, bx2, by1, by2, cA, cB, nA, nB, jac * mul, acc);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < NA; ++k)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      acc[k].x += __shfl_xor_sync(0xffffffffu, acc[k].x, off);
      acc[k].y += __shfl_xor_sync(0xffffffffu, acc[k].y, off);
    }
  finalize<OP>(op, A, B, cA, cB, acc, L);
}

// Singular / near pairs, one warp per entry.  BATCH: the operator constants of the test
// triangle's problem (ops[tri_problem[tau]]) instead of op1.  Single and batched assemblies
// share this code, so their values are bit-identical.
template <int OP, bool BATCH, bool NEAR = false>
__global__ void __launch_bounds__(256, NEAR ? 2 : 1) k_singular(OpParams op1, const OpParams* __restrict__ ops,
                                                  const int* __restrict__ tri_problem,
                                                  const __grid_constant__ QuadSel qs,
                                                  const __grid_constant__ RuleTable rules,
                                                  const Geo64* __restrict__ tg, const Geo64* __restrict__ bg,
                                                  const int* __restrict__ ent_tau, const int* __restrict__ ent_sigma,
                                                  const int8_t* __restrict__ ent_cls, int64_t n,
                                                  double2* __restrict__ out, const volatile int* abort_flag,
                                                  int near_only, const int* __restrict__ perm,
                                                  const int64_t* __restrict__ range) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  // perm: the entries perm[range[0] .. range[1]) (one output block's group); otherwise 0 .. n
  const int64_t i0 = perm ? range[0] : 0, i1 = perm ? range[1] : n;
  auto ent_at = [&](int64_t i) -> int64_t { return perm ? (int64_t)perm[i] : i; };
  auto entry = [&](int64_t e) {
    const int tau = ent_tau[e];
    const OpParams op = BATCH ? ops[tri_problem[tau]] : op1;
    const Geo64 A = tg[tau], B = bg[ent_sigma[e]];
    double2 L[3][3];
    pair_integral64<OP, NEAR>(op, qs, rules, ent_cls[e], A, B, L);
    if (lane < 9) {
      double2 v = L[0][0];
#pragma unroll
      for (int q = 1; q < 9; ++q)
        if (lane == q) v = L[q / 3][q % 3];
      out[e * 9 + lane] = v;
    }
  };
  if (NEAR) {
    // near pairs only (the others come from the double-float kernel): a warp reads the classes of
    // 32 entries at once and integrates the near ones among them
    for (int64_t b = i0 + warp0 * 32; b < i1; b += warps * 32) {
      if (abort_flag && *abort_flag) return;
      const int64_t i = b + lane;
      unsigned near = __ballot_sync(0xffffffffu, i < i1 && ent_cls[ent_at(i)] == BGB_CLASS_NEAR);
      while (near) {
        const int l = __ffs(near) - 1;
        near &= near - 1;
        entry(ent_at(b + l));
      }
    }
    return;
  }
  for (int64_t i = i0 + warp0; i < i1; i += warps) {
    if (abort_flag && *abort_flag) return;
    entry(ent_at(i));
  }
}

// Diagnostic: local matrices of a list of pairs (classified exactly or forced), FP64.
template <int OP>
__global__ void __launch_bounds__(256) k_local_diag64(OpParams op, const __grid_constant__ QuadSel qs,
                                                      const __grid_constant__ RuleTable rules,
                                                      const Geo64* __restrict__ tg, const Geo64* __restrict__ bg,
                                                      const int* __restrict__ tau, const int* __restrict__ sigma,
                                                      int64_t n, int force, double2* __restrict__ out,
                                                      int8_t* __restrict__ cls_out, int16_t* __restrict__ mask_out,
                                                      int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n; e += warps) {
    const Geo64 A = tg[tau[e]], B = bg[sigma[e]];
    int mask = 0;
    const int exact = classify_exact(A, B, op.k2, &mask);
    int cls = force >= 0 ? force : exact;
    if (lane == 0 && mask_out) mask_out[e] = (int16_t)mask;
    if (cls < 0) {
      if (lane == 0) atomicOr(err, 1);
      cls = BGB_CLASS_FAR;
    }
    double2 L[3][3];
    pair_integral64<OP>(op, qs, rules, cls, A, B, L);
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
// Batched variants: the triangles of all problems are concatenated; tri_problem[t] names the
// problem of test triangle t, prob_trial[p] its trial-triangle range and prob_k2[p] its k^2.
// Pairs never cross problems.
// ----------------------------------------------------------------------------------------
__global__ void k_prepare_bounds_batched(const Geo64* __restrict__ g, int nt, const int* __restrict__ tri_problem,
                                         const double* __restrict__ prob_k2, int trial_side, float4* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const Geo64& T = g[t];
  const double k2 = prob_k2[tri_problem[t]];
  double c[3], r = 0.0;
  for (int k = 0; k < 3; ++k) c[k] = (T.v[0][k] + T.v[1][k] + T.v[2][k]) / 3.0;
  for (int a = 0; a < 3; ++a) {
    const double d0 = T.v[a][0] - c[0], d1 = T.v[a][1] - c[1], d2 = T.v[a][2] - c[2];
    r = fmax(r, sqrt(d0 * d0 + d1 * d1 + d2 * d2));
  }
  const double cn = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  if (trial_side) {
    double lim = 0.64 * T.area;
    if (k2 > 0.0) lim = fmin(lim, 0.04 / k2);
    r += sqrt(lim);
  }
  r = r * (1.0 + 1e-6) + 4e-7 * (cn + 1.0) + 1e-30;
  out[t] = make_float4((float)c[0], (float)c[1], (float)c[2], (float)r);
}

template <bool FILL>
__global__ void __launch_bounds__(256) k_classify_batched(const float4* __restrict__ tb, const float4* __restrict__ bb,
                                                          const float4* __restrict__ cb,
                                                          const Geo64* __restrict__ tg, const Geo64* __restrict__ bg,
                                                          int nt, const int* __restrict__ tri_problem,
                                                          const int2* __restrict__ prob_trial,
                                                          const double* __restrict__ prob_k2, int* __restrict__ count,
                                                          const int64_t* __restrict__ offset, int* __restrict__ out_tau,
                                                          int* __restrict__ out_sigma, int8_t* __restrict__ out_cls,
                                                          int16_t* __restrict__ out_mask, int* __restrict__ err) {
  __shared__ int queues[8][64];
  int* queue = queues[threadIdx.x >> 5];
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int tau = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; tau < nt; tau += warps) {
    const int pr = tri_problem[tau];
    const int2 rg = prob_trial[pr];
    const Geo64 A = tg[tau];
    classify_sweep<FILL>(tau, tb[tau], A, rg.x, rg.y, bb, cb, bg, prob_k2[pr], queue, count, offset, out_tau,
                         out_sigma, out_cls, out_mask, err);
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
void launch_chunk_bounds(const float4* b, int nb, float4* out, cudaStream_t st) {
  const int nc = (nb + 31) / 32;
  if (nc > 0) k_chunk_bounds<<<(nc + 127) / 128, 128, 0, st>>>(b, nb, out);
}
void launch_classify(bool fill, const float4* tb, const float4* bb, const Geo64* tg, const Geo64* bg, int nt, int nb,
                     double k2, int* count, const int64_t* offset, int* out_tau, int* out_sigma, int8_t* out_cls,
                     int* err, int num_sms, cudaStream_t st, int16_t* out_mask, const float4* cb) {
  if (nt <= 0) return;
  int blocks = (nt + 7) / 8;
  blocks = blocks < num_sms * 16 ? blocks : num_sms * 16;
  if (fill)
    k_classify<true><<<blocks, 256, 0, st>>>(tb, bb, cb, tg, bg, nt, nb, k2, count, offset, out_tau, out_sigma,
                                              out_cls, out_mask, err);
  else
    k_classify<false><<<blocks, 256, 0, st>>>(tb, bb, cb, tg, bg, nt, nb, k2, count, offset, out_tau, out_sigma,
                                               out_cls, nullptr, err);
}
void launch_scan(const int* counts, int n, int64_t* offsets, cudaStream_t st) {
  k_scan_counts<<<1, 1024, 0, st>>>(counts, n, offsets);
}
void launch_class_hist(const int8_t* cls, int64_t n, unsigned long long* hist, int num_sms, cudaStream_t st) {
  cudaMemsetAsync(hist, 0, sizeof(unsigned long long) * 5, st);
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)num_sms * 4));
  if (n > 0) k_class_hist<<<blocks, 256, 0, st>>>(cls, n, hist);
}
void launch_group_entries(const int* sigma, int64_t n, const int* tri_group, int ngroups, int* counts, int64_t* off,
                          int* perm, int num_sms, cudaStream_t st) {
  cudaMemsetAsync(counts, 0, sizeof(int) * (size_t)ngroups, st);
  int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)num_sms * 4);
  if (blocks < 1) blocks = 1;
  if (n > 0) k_group_count<<<blocks, 256, 0, st>>>(sigma, n, tri_group, ngroups, counts);
  k_scan_counts<<<1, 1024, 0, st>>>(counts, ngroups, off);
  cudaMemsetAsync(counts, 0, sizeof(int) * (size_t)ngroups, st);
  if (n > 0) k_group_fill<<<blocks, 256, 0, st>>>(sigma, n, tri_group, ngroups, off, counts, perm);
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
                     const volatile int* abort_flag, int num_sms, cudaStream_t st, bool near_only, const int* perm,
                     const int64_t* range) {
  (void)rsA;
  (void)rsB;
  if (n <= 0) return;
  int64_t blocks = (n + 7) / 8;
  const int64_t cap = (int64_t)num_sms * (perm ? 2 : 32);  // a group: about one wave beside a far kernel
  if (blocks > cap) blocks = cap;
#define BGB_LAUNCH_SING(OPK)                                                                                   \
  if (near_only)                                                                                                 \
    k_singular<OPK, false, true><<<(int)blocks, 256, 0, st>>>(op, nullptr, nullptr, qs, rules, tg, bg, et, es, ec, n, \
                                                              out, abort_flag, 1, perm, range);                    \
  else                                                                                                           \
    k_singular<OPK, false><<<(int)blocks, 256, 0, st>>>(op, nullptr, nullptr, qs, rules, tg, bg, et, es, ec, n, out, \
                                                        abort_flag, 0, perm, range)
  switch (op.kind) {
    case BGB_OP_HELMHOLTZ3D_SL: BGB_LAUNCH_SING(BGB_OP_HELMHOLTZ3D_SL); break;
    case BGB_OP_MAXWELL3D_SL: BGB_LAUNCH_SING(BGB_OP_MAXWELL3D_SL); break;
    case BGB_OP_MAXWELL3D_DL: BGB_LAUNCH_SING(BGB_OP_MAXWELL3D_DL); break;
    case BGB_OP_HELMHOLTZ3D_DL: BGB_LAUNCH_SING(BGB_OP_HELMHOLTZ3D_DL); break;
    case BGB_OP_HELMHOLTZ3D_DLT: BGB_LAUNCH_SING(BGB_OP_HELMHOLTZ3D_DLT); break;
    case BGB_OP_HELMHOLTZ3D_HS: BGB_LAUNCH_SING(BGB_OP_HELMHOLTZ3D_HS); break;
  }
#undef BGB_LAUNCH_SING
}
void launch_local_diag64(const OpParams& op, const QuadSel& qs, const RuleTable& rules, int rsA, int rsB,
                         const Geo64* tg, const Geo64* bg, const int* tau, const int* sigma, int64_t n, int force,
                         double2* out, int8_t* cls, int* err, int num_sms, cudaStream_t st, int16_t* mask) {
  (void)rsA;
  (void)rsB;
  if (n <= 0) return;
  int64_t blocks = (n + 7) / 8;
  if (blocks > (int64_t)num_sms * 32) blocks = (int64_t)num_sms * 32;
  switch (op.kind) {
    case BGB_OP_HELMHOLTZ3D_SL: k_local_diag64<BGB_OP_HELMHOLTZ3D_SL><<<(int)blocks, 256, 0, st>>>(op, qs, rules, tg, bg, tau, sigma, n, force, out, cls, mask, err); break;
    case BGB_OP_MAXWELL3D_SL: k_local_diag64<BGB_OP_MAXWELL3D_SL><<<(int)blocks, 256, 0, st>>>(op, qs, rules, tg, bg, tau, sigma, n, force, out, cls, mask, err); break;
    case BGB_OP_MAXWELL3D_DL: k_local_diag64<BGB_OP_MAXWELL3D_DL><<<(int)blocks, 256, 0, st>>>(op, qs, rules, tg, bg, tau, sigma, n, force, out, cls, mask, err); break;
    case BGB_OP_HELMHOLTZ3D_DL: k_local_diag64<BGB_OP_HELMHOLTZ3D_DL><<<(int)blocks, 256, 0, st>>>(op, qs, rules, tg, bg, tau, sigma, n, force, out, cls, mask, err); break;
    case BGB_OP_HELMHOLTZ3D_DLT: k_local_diag64<BGB_OP_HELMHOLTZ3D_DLT><<<(int)blocks, 256, 0, st>>>(op, qs, rules, tg, bg, tau, sigma, n, force, out, cls, mask, err); break;
    case BGB_OP_HELMHOLTZ3D_HS: k_local_diag64<BGB_OP_HELMHOLTZ3D_HS><<<(int)blocks, 256, 0, st>>>(op, qs, rules, tg, bg, tau, sigma, n, force, out, cls, mask, err); break;
  }
}

void launch_prepare_bounds_batched(const Geo64* g, int nt, const int* tri_problem, const double* prob_k2, int trial_side,
                                   float4* out, cudaStream_t st) {
  if (nt > 0) k_prepare_bounds_batched<<<(nt + 255) / 256, 256, 0, st>>>(g, nt, tri_problem, prob_k2, trial_side, out);
}
void launch_classify_batched(bool fill, const float4* tb, const float4* bb, const Geo64* tg, const Geo64* bg, int nt,
                             const int* tri_problem, const int2* prob_trial, const double* prob_k2, int* count,
                             const int64_t* offset, int* out_tau, int* out_sigma, int8_t* out_cls, int* err,
                             int num_sms, cudaStream_t st, int16_t* out_mask, const float4* cb) {
  if (nt <= 0) return;
  int blocks = (nt + 7) / 8;
  blocks = blocks < num_sms * 16 ? blocks : num_sms * 16;
  if (fill)
    k_classify_batched<true><<<blocks, 256, 0, st>>>(tb, bb, cb, tg, bg, nt, tri_problem, prob_trial, prob_k2, count, offset,
                                                     out_tau, out_sigma, out_cls, out_mask, err);
  else
    k_classify_batched<false><<<blocks, 256, 0, st>>>(tb, bb, cb, tg, bg, nt, tri_problem, prob_trial, prob_k2, count,
                                                      offset, out_tau, out_sigma, out_cls, nullptr, err);
}
void launch_singular_batched(int op_kind, const OpParams* ops, const QuadSel& qs, const RuleTable& rules,
                             const Geo64* tg, const Geo64* bg, const int* tri_problem, const int* et, const int* es,
                             const int8_t* ec, int64_t n, double2* out, const volatile int* abort_flag, int num_sms,
                             cudaStream_t st, bool near_only) {
  if (n <= 0) return;
  int64_t blocks = (n + 7) / 8;
  if (blocks > (int64_t)num_sms * 32) blocks = (int64_t)num_sms * 32;
#define BGB_LAUNCH_SING(OPK)                                                                                  \
  if (near_only)                                                                                                \
    k_singular<OPK, true, true><<<(int)blocks, 256, 0, st>>>(OpParams{}, ops, tri_problem, qs, rules, tg, bg, et, es, \
                                                             ec, n, out, abort_flag, 1, nullptr, nullptr);          \
  else                                                                                                          \
    k_singular<OPK, true><<<(int)blocks, 256, 0, st>>>(OpParams{}, ops, tri_problem, qs, rules, tg, bg, et, es, ec, n, \
                                                       out, abort_flag, 0, nullptr, nullptr)
  switch (op_kind) {
    case BGB_OP_HELMHOLTZ3D_SL: BGB_LAUNCH_SING(BGB_OP_HELMHOLTZ3D_SL); break;
    case BGB_OP_MAXWELL3D_SL: BGB_LAUNCH_SING(BGB_OP_MAXWELL3D_SL); break;
    case BGB_OP_MAXWELL3D_DL: BGB_LAUNCH_SING(BGB_OP_MAXWELL3D_DL); break;
    case BGB_OP_HELMHOLTZ3D_DL: BGB_LAUNCH_SING(BGB_OP_HELMHOLTZ3D_DL); break;
    case BGB_OP_HELMHOLTZ3D_DLT: BGB_LAUNCH_SING(BGB_OP_HELMHOLTZ3D_DLT); break;
    case BGB_OP_HELMHOLTZ3D_HS: BGB_LAUNCH_SING(BGB_OP_HELMHOLTZ3D_HS); break;
  }
#undef BGB_LAUNCH_SING
}

}  // namespace bgb
