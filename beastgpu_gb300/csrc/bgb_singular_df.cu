// Singular and near-pair integrals in double-float arithmetic (mixed-precision path).
//
// Same rules as k_singular<OP> (Sauter-Schwab CF/CE/CV regions, SauterSchwab.jl:265-297, and
// the near-pair double quadrature), evaluated with df = float + float values on the FP32
// pipes instead of native FP64, which runs at 1/62 of the FP32 rate on GB300.  The region
// points and weights are tabulated on the host in FP64 (the same formulas as ss_region) and
// stored as df pairs; each point costs ~800 FP32-pipe operations against ~95 FP64 operations
// (~5900 FP32-equivalents) in k_singular.  Accuracy: ~48-bit operations; local matrices
// agree with the FP64 kernels and the oracle to ~1e-14 relative.  Operators with a lossy
// wave number (Re gamma != 0) and angles k R >= 400 use the FP64 kernel.
//
// Points are written relative to the charts' origin vertex: x = o_a + e_a1 u1 + e_a2 u2 and
// d = x - y = (o_a - o_b) + X - Y, so the difference near the singularity is formed from
// small terms (o_a = o_b for common faces and edges).  The operator moments are those of
// k_singular (taken about the chart origins); the per-lane df sums are converted to FP64 for
// the warp reduction and the 3x3 local matrix.
#include <cmath>
#include <vector>

#include "bgb_df.cuh"
#include "bgb_kernels.cuh"
#include "bgb_ss.cuh"

namespace bgb {

namespace {

constexpr int kSsEntryFloats = 10;   // u1, u2, v1, v2, w (df each)
constexpr int kNearEntryFloats = 6;  // u, v, w (df each)

__device__ __forceinline__ dfl ldf(const float* p) { return dfl{p[0], p[1]}; }

template <int OP>
struct DfAcc {
  static constexpr int N = OP == BGB_OP_HELMHOLTZ3D_SL ? 9 : (OP == BGB_OP_MAXWELL3D_SL ? 8 : 10);
  dfl re[N], im[N];
};

// One point pair: X, Y are the points relative to the chart origins, d = x - y, (bx, by) the
// barycentric chart coordinates (Helmholtz), w the weight (quadrature weights x Jacobians).
template <int OP>
__device__ __forceinline__ void df_point(const dfl X[3], const dfl Y[3], const dfl d[3], dfl bx1, dfl bx2, dfl by1,
                                         dfl by2, dfl w, dfl kd, bool oscill, const float4* __restrict__ tab,
                                         const DfTrig& T, DfAcc<OP>& acc) {
  const dfl R2 = df_add(df_add(df_mul(d[0], d[0]), df_mul(d[1], d[1])), df_mul(d[2], d[2]));
  const dfl rinv = df_rsqrt(R2);
  const dfl amp = df_mul(df_mul(w, rinv), T.inv4pi);
  dfl gr = amp, gi = dfl{0.f, 0.f};
  if (oscill) {
    const dfl R = df_mul(R2, rinv);
    dfl sn, cs;
    df_sincos(df_mul(kd, R), tab, T, sn, cs);
    gr = df_mul(amp, cs);
    gi = df_neg(df_mul(amp, sn));
  }
  if (OP == BGB_OP_HELMHOLTZ3D_SL) {
    const dfl one{1.f, 0.f};
    const dfl p[3] = {one, bx1, bx2}, q[3] = {one, by1, by2};
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const dfl pq = (a == 0) ? q[b] : (b == 0 ? p[a] : df_mul(p[a], q[b]));
        acc.re[a * 3 + b] = df_add(acc.re[a * 3 + b], df_mul(gr, pq));
        acc.im[a * 3 + b] = df_add(acc.im[a * 3 + b], df_mul(gi, pq));
      }
  } else if (OP == BGB_OP_MAXWELL3D_SL) {
    const dfl xy = df_add(df_add(df_mul(X[0], Y[0]), df_mul(X[1], Y[1])), df_mul(X[2], Y[2]));
    const dfl v[8] = {xy, X[0], X[1], X[2], Y[0], Y[1], Y[2], dfl{1.f, 0.f}};
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      acc.re[k] = df_add(acc.re[k], df_mul(gr, v[k]));
      acc.im[k] = df_add(acc.im[k], df_mul(gi, v[k]));
    }
    acc.re[7] = df_add(acc.re[7], gr);
    acc.im[7] = df_add(acc.im[7], gi);
  } else {
    // H = -(gamma + 1/R) G / R with gamma = i k:  H = -(rinv + i k) (G rinv)
    const dfl g2r = df_mul(gr, rinv), g2i = df_mul(gi, rinv);
    const dfl Hr = df_neg(df_sub(df_mul(rinv, g2r), df_mul(kd, g2i)));
    const dfl Hi = df_neg(df_add(df_mul(rinv, g2i), df_mul(kd, g2r)));
    const dfl e0 = df_sub(df_mul(d[1], Y[2]), df_mul(d[2], Y[1]));
    const dfl e1 = df_sub(df_mul(d[2], Y[0]), df_mul(d[0], Y[2]));
    const dfl e2 = df_sub(df_mul(d[0], Y[1]), df_mul(d[1], Y[0]));
    const dfl f0 = df_sub(df_mul(X[1], d[2]), df_mul(X[2], d[1]));
    const dfl f1 = df_sub(df_mul(X[2], d[0]), df_mul(X[0], d[2]));
    const dfl f2 = df_sub(df_mul(X[0], d[1]), df_mul(X[1], d[0]));
    const dfl a1 = df_add(df_add(df_mul(X[0], e0), df_mul(X[1], e1)), df_mul(X[2], e2));
    const dfl v[10] = {a1, e0, e1, e2, f0, f1, f2, d[0], d[1], d[2]};
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      acc.re[k] = df_add(acc.re[k], df_mul(Hr, v[k]));
      acc.im[k] = df_add(acc.im[k], df_mul(Hi, v[k]));
    }
  }
}

__device__ __forceinline__ dfl gdf(const float* p) { return dfl{p[0], p[1]}; }

// Local matrix entry (i, j) from the reduced moments, in df (moments about the chart origins).
template <int OP>
__device__ __forceinline__ double2 df_entry(const OpDf& op, const GeoDf& A, const GeoDf& B, const dfl oa[3],
                                            const dfl ob[3], const dfl* mr, const dfl* mi, int i, int j) {
  const dfl ar = gdf(op.alpha[0]), ai = gdf(op.alpha[1]);
  dfl tr, ti;
  if (OP == BGB_OP_HELMHOLTZ3D_SL) {
    // f = T p with T = [[0,1,0],[0,0,1],[1,-1,-1]]
    const int Tm[3][3] = {{0, 1, 0}, {0, 0, 1}, {1, -1, -1}};
    tr = ti = dfl{0.f, 0.f};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        const int t = Tm[i][a] * Tm[j][b];
        if (t > 0) {
          tr = df_add(tr, mr[a * 3 + b]);
          ti = df_add(ti, mi[a * 3 + b]);
        } else if (t < 0) {
          tr = df_sub(tr, mr[a * 3 + b]);
          ti = df_sub(ti, mi[a * 3 + b]);
        }
      }
    const dfl Lr = df_sub(df_mul(ar, tr), df_mul(ai, ti)), Li = df_add(df_mul(ar, ti), df_mul(ai, tr));
    return make_double2(df_to_double(Lr), df_to_double(Li));
  }
  dfl V[3], W[3];
  for (int c = 0; c < 3; ++c) {
    V[c] = df_sub(gdf(A.v[i][c]), oa[c]);
    W[c] = df_sub(gdf(B.v[j][c]), ob[c]);
  }
  const dfl inv4AA = df_mulf(df_mul(gdf(A.inv_area), gdf(B.inv_area)), 0.25f);
  if (OP == BGB_OP_MAXWELL3D_SL) {
    tr = mr[0];
    ti = mi[0];
    for (int c = 0; c < 3; ++c) {
      tr = df_sub(tr, df_add(df_mul(V[c], mr[4 + c]), df_mul(W[c], mr[1 + c])));
      ti = df_sub(ti, df_add(df_mul(V[c], mi[4 + c]), df_mul(W[c], mi[1 + c])));
    }
    const dfl vw = df_add(df_add(df_mul(V[0], W[0]), df_mul(V[1], W[1])), df_mul(V[2], W[2]));
    tr = df_add(tr, df_mul(vw, mr[7]));
    ti = df_add(ti, df_mul(vw, mi[7]));
    const dfl car = df_mul(ar, inv4AA), cai = df_mul(ai, inv4AA);
    const dfl invAA = df_mulf(inv4AA, 4.f);
    const dfl cbr = df_mul(gdf(op.beta[0]), invAA), cbi = df_mul(gdf(op.beta[1]), invAA);
    dfl Lr = df_sub(df_mul(car, tr), df_mul(cai, ti));
    dfl Li = df_add(df_mul(car, ti), df_mul(cai, tr));
    Lr = df_add(Lr, df_sub(df_mul(cbr, mr[7]), df_mul(cbi, mi[7])));
    Li = df_add(Li, df_add(df_mul(cbr, mi[7]), df_mul(cbi, mr[7])));
    return make_double2(df_to_double(Lr), df_to_double(Li));
  }
  // MFIE: A1 - W.C - V.B + V.(E x W)
  tr = mr[0];
  ti = mi[0];
  for (int c = 0; c < 3; ++c) {
    tr = df_sub(tr, df_add(df_mul(W[c], mr[4 + c]), df_mul(V[c], mr[1 + c])));
    ti = df_sub(ti, df_add(df_mul(W[c], mi[4 + c]), df_mul(V[c], mi[1 + c])));
  }
  const dfl* Er = mr + 7;
  const dfl* Ei = mi + 7;
  const dfl xr[3] = {df_sub(df_mul(Er[1], W[2]), df_mul(Er[2], W[1])), df_sub(df_mul(Er[2], W[0]), df_mul(Er[0], W[2])),
                     df_sub(df_mul(Er[0], W[1]), df_mul(Er[1], W[0]))};
  const dfl xi[3] = {df_sub(df_mul(Ei[1], W[2]), df_mul(Ei[2], W[1])), df_sub(df_mul(Ei[2], W[0]), df_mul(Ei[0], W[2])),
                     df_sub(df_mul(Ei[0], W[1]), df_mul(Ei[1], W[0]))};
  for (int c = 0; c < 3; ++c) {
    tr = df_add(tr, df_mul(V[c], xr[c]));
    ti = df_add(ti, df_mul(V[c], xi[c]));
  }
  const dfl car = df_mul(ar, inv4AA), cai = df_mul(ai, inv4AA);
  const dfl Lr = df_sub(df_mul(car, tr), df_mul(cai, ti)), Li = df_add(df_mul(car, ti), df_mul(cai, tr));
  return make_double2(df_to_double(Lr), df_to_double(Li));
}

template <int OP, bool BATCH>
__global__ void __launch_bounds__(256) k_singular_df(OpDf op1, const OpDf* __restrict__ ops,
                                                     const int* __restrict__ tri_problem, const __grid_constant__ DfTables M,
                                                     const float* __restrict__ tab, const GeoDf* __restrict__ tg,
                                                     const GeoDf* __restrict__ bg, const int* __restrict__ ent_tau,
                                                     const int* __restrict__ ent_sigma, const int8_t* __restrict__ ent_cls,
                                                     const int16_t* __restrict__ ent_mask, int64_t n,
                                                     double2* __restrict__ out, const volatile int* abort_flag,
                                                     const int* __restrict__ perm, const int64_t* __restrict__ range) {
  __shared__ float4 trig[128];
  for (int i = threadIdx.x; i < 128; i += blockDim.x) trig[i] = ((const float4*)(tab + M.trig_off))[i];
  __syncthreads();
  constexpr int NA = DfAcc<OP>::N;
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  // perm: the entries perm[range[0] .. range[1]) (one output block's group); otherwise 0 .. n
  const int64_t i0 = perm ? range[0] : 0, i1 = perm ? range[1] : n;
  for (int64_t i = i0 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < i1; i += warps) {
    if (abort_flag && *abort_flag) return;
    const int64_t e = perm ? (int64_t)perm[i] : i;
    const int cls = ent_cls[e];
    if (cls == BGB_CLASS_NEAR) continue;  // near pairs stay FP64 (k_singular with near_only)
    const int tau = ent_tau[e];
    const OpDf op = BATCH ? ops[tri_problem[tau]] : op1;
    const GeoDf A = tg[tau], B = bg[ent_sigma[e]];
    DfAcc<OP> acc;
#pragma unroll
    for (int k = 0; k < NA; ++k) acc.re[k] = acc.im[k] = dfl{0.f, 0.f};
    const dfl kd = gdf(op.k);
    const bool oscill = op.oscill != 0;
    dfl oa[3], ob[3];
    if (cls == BGB_CLASS_NEAR) {
      dfl ea[2][3], eb[2][3], D0[3];
      for (int c = 0; c < 3; ++c) {
        oa[c] = gdf(A.v[2][c]);
        ob[c] = gdf(B.v[2][c]);
        ea[0][c] = df_sub(gdf(A.v[0][c]), oa[c]);
        ea[1][c] = df_sub(gdf(A.v[1][c]), oa[c]);
        eb[0][c] = df_sub(gdf(B.v[0][c]), ob[c]);
        eb[1][c] = df_sub(gdf(B.v[1][c]), ob[c]);
        D0[c] = df_sub(oa[c], ob[c]);
      }
      const dfl AB = df_mul(gdf(A.area), gdf(B.area));
      const float* tt = tab + M.near_t_off;
      const float* tb = tab + M.near_b_off;
      for (int idx = lane; idx < M.near_qt * M.near_qb; idx += 32) {
        const int I = idx / M.near_qb, J = idx - I * M.near_qb;
        const float* p = tt + I * kNearEntryFloats;
        const float* q = tb + J * kNearEntryFloats;
        const dfl u = ldf(p), v = ldf(p + 2), wI = ldf(p + 4);
        const dfl s = ldf(q), t = ldf(q + 2), wJ = ldf(q + 4);
        dfl X[3], Y[3], d[3];
        for (int c = 0; c < 3; ++c) {
          X[c] = df_add(df_mul(ea[0][c], u), df_mul(ea[1][c], v));
          Y[c] = df_add(df_mul(eb[0][c], s), df_mul(eb[1][c], t));
          d[c] = df_sub(df_add(D0[c], X[c]), Y[c]);
        }
        df_point<OP>(X, Y, d, u, v, s, t, df_mul(df_mul(wI, wJ), AB), kd, oscill, trig, M.trig, acc);
      }
    } else if (!(OP == BGB_OP_MAXWELL3D_DL && cls == BGB_CLASS_CF)) {
      int I[3], J[3];
      ss_permutation_mask(cls, ent_mask[e], I, J);
      for (int k = 0; k < 3; ++k) {  // guard against an inconsistent mask
        I[k] = I[k] < 1 ? 1 : (I[k] > 3 ? 3 : I[k]);
        J[k] = J[k] < 1 ? 1 : (J[k] > 3 ? 3 : J[k]);
      }
      const int ia0 = I[2] - 1, ia1 = I[0] - 1, ia2 = I[1] - 1;
      const int ib0 = J[2] - 1, ib1 = J[0] - 1, ib2 = J[1] - 1;
      dfl ea[2][3], eb[2][3], D0[3];
      for (int c = 0; c < 3; ++c) {
        oa[c] = gdf(A.v[ia0][c]);
        ob[c] = gdf(B.v[ib0][c]);
        ea[0][c] = df_sub(gdf(A.v[ia1][c]), oa[c]);
        ea[1][c] = df_sub(gdf(A.v[ia2][c]), oa[c]);
        eb[0][c] = df_sub(gdf(B.v[ib1][c]), ob[c]);
        eb[1][c] = df_sub(gdf(B.v[ib2][c]), ob[c]);
        D0[c] = df_sub(oa[c], ob[c]);
      }
      // barycentric chart coordinates b = cv3 + (cv1 - cv3) u1 + (cv2 - cv3) u2 with the
      // reference-triangle vertices (1,0), (0,1), (0,0) (integer coefficients)
      const float VX[3] = {1.f, 0.f, 0.f}, VY[3] = {0.f, 1.f, 0.f};
      const float ba0 = VX[ia0], ba1 = VY[ia0], bb0 = VX[ib0], bb1 = VY[ib0];
      const float cax1 = VX[ia1] - ba0, cax2 = VX[ia2] - ba0, cay1 = VY[ia1] - ba1, cay2 = VY[ia2] - ba1;
      const float cbx1 = VX[ib1] - bb0, cbx2 = VX[ib2] - bb0, cby1 = VY[ib1] - bb1, cby2 = VY[ib2] - bb1;
      const dfl jac = df_mulf(df_mul(gdf(A.area), gdf(B.area)), 4.f);
      const float* tbl = tab + M.ss_off[cls];
      const int cnt = M.ss_cnt[cls];
      for (int idx = lane; idx < cnt; idx += 32) {
        const float* p = tbl + idx * kSsEntryFloats;
        const dfl u1 = ldf(p), u2 = ldf(p + 2), v1 = ldf(p + 4), v2 = ldf(p + 6), mul = ldf(p + 8);
        dfl X[3], Y[3], d[3];
        for (int c = 0; c < 3; ++c) {
          X[c] = df_add(df_mul(ea[0][c], u1), df_mul(ea[1][c], u2));
          Y[c] = df_add(df_mul(eb[0][c], v1), df_mul(eb[1][c], v2));
          d[c] = df_sub(df_add(D0[c], X[c]), Y[c]);
        }
        dfl bx1{0.f, 0.f}, bx2{0.f, 0.f}, by1{0.f, 0.f}, by2{0.f, 0.f};
        if (OP == BGB_OP_HELMHOLTZ3D_SL) {
          bx1 = df_addf(df_add(df_mulf(u1, cax1), df_mulf(u2, cax2)), ba0);
          bx2 = df_addf(df_add(df_mulf(u1, cay1), df_mulf(u2, cay2)), ba1);
          by1 = df_addf(df_add(df_mulf(v1, cbx1), df_mulf(v2, cbx2)), bb0);
          by2 = df_addf(df_add(df_mulf(v1, cby1), df_mulf(v2, cby2)), bb1);
        }
        df_point<OP>(X, Y, d, bx1, bx2, by1, by2, df_mul(jac, mul), kd, oscill, trig, M.trig, acc);
      }
    } else {
      for (int c = 0; c < 3; ++c) oa[c] = ob[c] = dfl{0.f, 0.f};
    }
    // warp reduction in df
#pragma unroll
    for (int k = 0; k < NA; ++k)
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const dfl orr{__shfl_xor_sync(0xffffffffu, acc.re[k].hi, off), __shfl_xor_sync(0xffffffffu, acc.re[k].lo, off)};
        const dfl oii{__shfl_xor_sync(0xffffffffu, acc.im[k].hi, off), __shfl_xor_sync(0xffffffffu, acc.im[k].lo, off)};
        acc.re[k] = df_add(acc.re[k], orr);
        acc.im[k] = df_add(acc.im[k], oii);
      }
    if (lane < 9) out[e * 9 + lane] = df_entry<OP>(op, A, B, oa, ob, acc.re, acc.im, lane / 3, lane % 3);
  }
}

__global__ void k_prepare_geodf(const Geo64* __restrict__ g, int nt, GeoDf* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  GeoDf r;
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) {
      const double x = g[t].v[a][c];
      r.v[a][c][0] = (float)x;
      r.v[a][c][1] = (float)(x - (double)r.v[a][c][0]);
    }
  const double A = g[t].area, iA = 1.0 / A;
  r.area[0] = (float)A;
  r.area[1] = (float)(A - (double)r.area[0]);
  r.inv_area[0] = (float)iA;
  r.inv_area[1] = (float)(iA - (double)r.inv_area[0]);
  out[t] = r;
}

void split(double x, float* out) {
  const float hi = (float)x;
  out[0] = hi;
  out[1] = (float)(x - (double)hi);
}

void split_ld(long double x, float* out) {
  const float hi = (float)x;
  out[0] = hi;
  out[1] = (float)(x - (long double)hi);
}

}  // namespace

void build_df_tables(const QuadSel& qs, const RuleTable& R, std::vector<float>& buf, DfTables& M) {
  buf.clear();
  M = DfTables{};
  auto align4 = [&]() {
    while (buf.size() % 4) buf.push_back(0.f);
  };
  for (int cls = 1; cls <= 3; ++cls) {
    align4();
    M.ss_off[cls] = (int)buf.size();
    const int n = qs.ss[cls];
    const int nreg = cls == BGB_CLASS_CV ? 2 : (cls == BGB_CLASS_CE ? 5 : 6);
    const double* gx = qs.gl_x[cls];
    const double* gw = qs.gl_w[cls];
    int cnt = 0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k)
          for (int l = 0; l < n; ++l) {
            const double wt = gw[i] * gw[j] * gw[k] * gw[l];
            for (int r = 0; r < nreg; ++r) {
              double u1, u2, v1, v2, mul;
              ss_region(cls, r, gx[i], gx[j], gx[k], gx[l], wt, u1, u2, v1, v2, mul);
              float e[10];
              split(u1, e);
              split(u2, e + 2);
              split(v1, e + 4);
              split(v2, e + 6);
              split(mul, e + 8);
              buf.insert(buf.end(), e, e + 10);
              ++cnt;
            }
          }
    M.ss_cnt[cls] = cnt;
  }
  for (int side = 0; side < 2; ++side) {
    align4();
    const int rule = side ? qs.near_b : qs.near_t;
    if (side) M.near_b_off = (int)buf.size();
    else M.near_t_off = (int)buf.size();
    const int q = R.npoints[rule];
    if (side) M.near_qb = q;
    else M.near_qt = q;
    for (int I = 0; I < q; ++I) {
      const double* p = R.uvw[R.offset[rule] + I];
      float e[6];
      split(p[0], e);
      split(p[1], e + 2);
      split(p[2], e + 4);  // normalised weight (sum 1); the areas are applied per pair
      buf.insert(buf.end(), e, e + 6);
    }
  }
  align4();
  M.trig_off = (int)buf.size();
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int j = 0; j < 128; ++j) {
    float e[4];
    split_ld(sinl(pi * j / 64.0L), e);
    split_ld(cosl(pi * j / 64.0L), e + 2);
    buf.insert(buf.end(), e, e + 4);
  }
  const long double step = pi / 64.0L;
  int ex;
  const double mant = frexp((double)step, &ex);
  const float p1 = (float)ldexp(floor(mant * 2048.0) / 2048.0, ex);
  const float p2 = (float)(step - (long double)p1);
  const float p3 = (float)(step - (long double)p1 - (long double)p2);
  M.trig.inv_step = (float)(64.0L / pi);
  M.trig.p1 = p1;
  M.trig.p2 = p2;
  M.trig.p3 = p3;
  float t[2];
  split(-1.0 / 6.0, t);
  M.trig.s3 = dfl{t[0], t[1]};
  split(1.0 / 120.0, t);
  M.trig.s5 = dfl{t[0], t[1]};
  M.trig.s7 = (float)(-1.0 / 5040.0);
  M.trig.c4 = (float)(1.0 / 24.0);
  M.trig.c6 = (float)(-1.0 / 720.0);
  split_ld(1.0L / (4.0L * pi), t);
  M.trig.inv4pi = dfl{t[0], t[1]};
  M.total_floats = (int)buf.size();
}

void launch_prepare_geodf(const Geo64* g, int nt, GeoDf* out, cudaStream_t st) {
  if (nt > 0) k_prepare_geodf<<<(nt + 255) / 256, 256, 0, st>>>(g, nt, out);
}

OpDf make_opdf(const OpParams& op) {
  OpDf r{};
  for (int c = 0; c < 2; ++c) {
    split(op.alpha[c], r.alpha[c]);
    split(op.beta[c], r.beta[c]);
  }
  split(op.gamma[1], r.k);
  r.kind = op.kind;
  r.oscill = op.gamma[1] != 0.0;
  return r;
}

void launch_singular_df(int op_kind, const OpDf& op, const OpDf* opdf_array, const int* tri_problem,
                        const DfTables& M, const float* dtab, const GeoDf* tg, const GeoDf* bg, const int* et,
                        const int* es, const int8_t* ec, const int16_t* emask, int64_t n, double2* out,
                        const volatile int* abort_flag, int num_sms, cudaStream_t st, const int* perm,
                        const int64_t* range) {
  if (n <= 0) return;
  int64_t blocks = (n + 7) / 8;
  const int64_t cap = (int64_t)num_sms * (perm ? 2 : 32);  // a group: about one wave beside a far kernel
  if (blocks > cap) blocks = cap;
  const bool batch = opdf_array != nullptr;
#define BGB_LAUNCH_DF(OPK)                                                                                        \
  if (batch)                                                                                                      \
    k_singular_df<OPK, true><<<(int)blocks, 256, 0, st>>>(op, opdf_array, tri_problem, M, dtab, tg, bg, et, es, ec, \
                                                          emask, n, out, abort_flag, perm, range);               \
  else                                                                                                            \
    k_singular_df<OPK, false><<<(int)blocks, 256, 0, st>>>(op, opdf_array, tri_problem, M, dtab, tg, bg, et, es, ec, \
                                                           emask, n, out, abort_flag, perm, range);
  if (op_kind == BGB_OP_HELMHOLTZ3D_SL) {
    BGB_LAUNCH_DF(BGB_OP_HELMHOLTZ3D_SL)
  } else if (op_kind == BGB_OP_MAXWELL3D_SL) {
    BGB_LAUNCH_DF(BGB_OP_MAXWELL3D_SL)
  } else if (op_kind == BGB_OP_MAXWELL3D_DL) {
    BGB_LAUNCH_DF(BGB_OP_MAXWELL3D_DL)
  }  // other operators take the FP64 singular kernel (df_singular_ok)
#undef BGB_LAUNCH_DF
}

}  // namespace bgb
