// C ABI of libbeastgb: handles, validation, host-side tile planning and the assembly pipeline
//
//   upload spaces -> k_prepare_geo64 -> k_prepare_bounds -> k_classify (count, scan, fill)
//   -> k_singular (FP64 Sauter-Schwab / near pairs) -> k_prepare_rec -> k_far_persistent
//   (FP64 or mixed) -> output on the device, or row blocks copied to the host.
//
// The pipeline mirrors assemble_gpu (assamble_gpu.jl:25-137) and assemblechunk_body_gpu!
// (assamble_chunk_gpu.jl:104-196): classify, singular pairs, far pairs, write-back.  Unlike the
// reference, the write-back is a deterministic gather inside the far kernel (no FP64 atomics
// into a 2 x N x N buffer, no make_complex pass) and non-far pairs of class "near" are integrated
// (the reference drops them, quadrule_determine.jl:76 with doubleQuadRuleMainCase.jl:154).
#include "bgb_host.h"
#include "trirules.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

namespace bgb {

static thread_local std::string g_err;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}

int cuda_fail(cudaError_t e, const char* what) {
  set_error("CUDA error in %s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? BGB_ERR_OOM : BGB_ERR_CUDA;
}

}  // namespace bgb

namespace bgb {

// ----------------------------------------------------------------------------------------
// Validation
// ----------------------------------------------------------------------------------------
int validate_space(const bgb_space* s, const char* name) {
  if (!s) { set_error("%s space is NULL", name); return BGB_ERR_INVALID; }
  if (s->refspace != BGB_REFSPACE_LAGRANGE_C0D1 && s->refspace != BGB_REFSPACE_RT) {
    set_error("%s space: unknown refspace %d", name, s->refspace);
    return BGB_ERR_INVALID;
  }
  if (s->nv < 0 || s->nt < 0 || s->nfun < 0) { set_error("%s space: negative sizes", name); return BGB_ERR_INVALID; }
  if (s->nt > 0 && (!s->vertices || !s->triangles || !s->fn_index || !s->fn_coef)) {
    set_error("%s space: NULL table", name);
    return BGB_ERR_INVALID;
  }
  for (int64_t i = 0; i < 3 * (int64_t)s->nv; ++i)
    if (!std::isfinite(s->vertices[i])) { set_error("%s space: non-finite vertex coordinate at %lld", name, (long long)i); return BGB_ERR_INVALID; }
  for (int64_t t = 0; t < s->nt; ++t) {
    for (int a = 0; a < 3; ++a) {
      int v = s->triangles[3 * t + a];
      if (v < 0 || v >= s->nv) { set_error("%s space: triangle %lld has vertex index %d out of range", name, (long long)t, v); return BGB_ERR_INVALID; }
      int f = s->fn_index[3 * t + a];
      if (f < -1 || f >= s->nfun) { set_error("%s space: triangle %lld local %d has function index %d out of range", name, (long long)t, a, f); return BGB_ERR_INVALID; }
      if (f >= 0 && !std::isfinite(s->fn_coef[3 * t + a])) { set_error("%s space: non-finite coefficient", name); return BGB_ERR_INVALID; }
    }
    int f0 = s->fn_index[3 * t], f1 = s->fn_index[3 * t + 1], f2 = s->fn_index[3 * t + 2];
    if ((f0 >= 0 && (f0 == f1 || f0 == f2)) || (f1 >= 0 && f1 == f2)) {
      set_error("%s space: triangle %lld maps two local shapes to one function", name, (long long)t);
      return BGB_ERR_INVALID;
    }
    int v0 = s->triangles[3 * t], v1 = s->triangles[3 * t + 1], v2 = s->triangles[3 * t + 2];
    if (v0 == v1 || v0 == v2 || v1 == v2) { set_error("%s space: triangle %lld is degenerate", name, (long long)t); return BGB_ERR_INVALID; }
  }
  return 0;
}

static int rule_index(int npoints) {
  for (int r = 0; r < BGB_TRIRULE_COUNT; ++r)
    if (bgb_trirule_npoints[r] == npoints) return r;
  return -1;
}

RuleTable make_rules() {
  RuleTable R{};
  for (int r = 0; r < BGB_TRIRULE_COUNT; ++r) {
    R.npoints[r] = bgb_trirule_npoints[r];
    R.offset[r] = bgb_trirule_offset[r];
  }
  for (int i = 0; i < 46; ++i)
    for (int k = 0; k < 3; ++k) R.uvw[i][k] = bgb_trirule_uvw[i][k];
  return R;
}

// Gauss-Legendre on [0, 1], ascending (Newton on the Legendre recurrence).
static void gauss_legendre01(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double t = -std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
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
      if (std::fabs(dt) < 1e-17) break;
    }
    double p0 = 1.0, p1 = t;
    for (int k = 2; k <= n; ++k) {
      double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    if (n == 1) { p1 = t; p0 = 1.0; }
    dp = n * (t * p1 - p0) / (t * t - 1.0);
    x[i] = (t + 1.0) / 2.0;
    w[i] = (2.0 / ((1.0 - t * t) * dp * dp)) / 2.0;
  }
}

int make_quadsel(const bgb_quadstrat* qs, QuadSel* out) {
  QuadSel q{};
  q.far_t = rule_index(qs->far_test);
  q.far_b = rule_index(qs->far_trial);
  q.near_t = rule_index(qs->near_test);
  q.near_b = rule_index(qs->near_trial);
  if (q.far_t < 0 || q.far_b < 0 || q.near_t < 0 || q.near_b < 0) {
    set_error("quadstrat: triangle rules must have 1, 3, 4, 6, 7, 12 or 13 points (got %d %d %d %d)", qs->far_test,
              qs->far_trial, qs->near_test, qs->near_trial);
    return BGB_ERR_NOT_SUPPORTED;
  }
  int orders[4] = {0, qs->ss_cv, qs->ss_ce, qs->ss_cf};
  for (int c = 1; c <= 3; ++c) {
    if (orders[c] < 1 || orders[c] > BGB_MAX_SS) {
      set_error("quadstrat: Sauter-Schwab order %d out of range 1..%d", orders[c], BGB_MAX_SS);
      return BGB_ERR_NOT_SUPPORTED;
    }
    q.ss[c] = orders[c];
    gauss_legendre01(orders[c], q.gl_x[c], q.gl_w[c]);
  }
  *out = q;
  return 0;
}

int make_opparams(const bgb_operator* op, const bgb_space* a, const bgb_space* b, OpParams* out) {
  if (!op) { set_error("operator is NULL"); return BGB_ERR_INVALID; }
  if (op->kind == BGB_OP_HELMHOLTZ3D_SL) {
    if (a->refspace != BGB_REFSPACE_LAGRANGE_C0D1 || b->refspace != BGB_REFSPACE_LAGRANGE_C0D1) {
      set_error("Helmholtz3D single layer is implemented on lagrangec0d1 spaces");
      return BGB_ERR_NOT_SUPPORTED;
    }
  } else if (op->kind == BGB_OP_MAXWELL3D_SL || op->kind == BGB_OP_MAXWELL3D_DL) {
    if (a->refspace != BGB_REFSPACE_RT || b->refspace != BGB_REFSPACE_RT) {
      set_error("Maxwell3D operators are implemented on Raviart-Thomas (RWG) spaces");
      return BGB_ERR_NOT_SUPPORTED;
    }
  } else {
    set_error("unknown operator kind %d", op->kind);
    return BGB_ERR_INVALID;
  }
  for (int k = 0; k < 2; ++k)
    if (!std::isfinite(op->alpha[k]) || !std::isfinite(op->beta[k]) || !std::isfinite(op->gamma[k])) {
      set_error("operator has non-finite parameters");
      return BGB_ERR_INVALID;
    }
  OpParams p{};
  p.kind = op->kind;
  for (int k = 0; k < 2; ++k) {
    p.alpha[k] = op->alpha[k];
    p.beta[k] = op->beta[k];
    p.gamma[k] = op->gamma[k];
  }
  p.k2 = op->gamma[0] * op->gamma[0] + op->gamma[1] * op->gamma[1];  // abs2(gamma)
  *out = p;
  return 0;
}

FarConst make_farconst(const OpParams& op, const RuleTable& R, const QuadSel& qs) {
  FarConst k{};
  k.op_kind = op.kind;
  k.qt = R.npoints[qs.far_t];
  k.qb = R.npoints[qs.far_b];
  k.lossy = op.gamma[0] != 0.0;
  for (int c = 0; c < 2; ++c) {
    k.alpha[c] = op.alpha[c];
    k.beta[c] = op.beta[c];
    k.gamma[c] = op.gamma[c];
  }
  for (int c = 0; c < 2; ++c) {
    k.alpha32[c] = (float)op.alpha[c];
    k.beta32[c] = (float)op.beta[c];
  }
  k.k_hi = (float)op.gamma[1];
  k.k_lo = (float)(op.gamma[1] - (double)k.k_hi);
  k.gre = (float)op.gamma[0];
  for (int I = 0; I < k.qt; ++I) {
    const double* p = R.uvw[R.offset[qs.far_t] + I];
    double h[3] = {p[0], p[1], 1.0 - p[0] - p[1]};
    for (int i = 0; i < 3; ++i) { k.shpT64[I][i] = h[i]; k.shpT[I][i] = (float)h[i]; }
  }
  for (int J = 0; J < k.qb; ++J) {
    const double* p = R.uvw[R.offset[qs.far_b] + J];
    double h[3] = {p[0], p[1], 1.0 - p[0] - p[1]};
    for (int i = 0; i < 3; ++i) { k.shpB64[J][i] = h[i]; k.shpB[J][i] = (float)h[i]; }
  }
  return k;
}

// ----------------------------------------------------------------------------------------
// Host planning: Morton-ordered function blocks and their triangle sets
// ----------------------------------------------------------------------------------------
static inline uint64_t spread3(uint64_t x) {
  x &= 0x1fffff;
  x = (x | x << 32) & 0x1f00000000ffffULL;
  x = (x | x << 16) & 0x1f0000ff0000ffULL;
  x = (x | x << 8) & 0x100f00f00f00f00fULL;
  x = (x | x << 4) & 0x10c30c30c30c30c3ULL;
  x = (x | x << 2) & 0x1249249249249249ULL;
  return x;
}

// Morton position of every triangle (rank in the order of 3-D Morton codes of centroids).
std::vector<int> morton_rank(const bgb_space* s) {
  const int nt = s->nt;
  std::vector<double> c(3 * (size_t)nt);
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int t = 0; t < nt; ++t)
    for (int k = 0; k < 3; ++k) {
      double v = 0;
      for (int a = 0; a < 3; ++a) v += s->vertices[3 * (int64_t)s->triangles[3 * (int64_t)t + a] + k];
      v /= 3.0;
      c[3 * (size_t)t + k] = v;
      lo[k] = std::min(lo[k], v);
      hi[k] = std::max(hi[k], v);
    }
  double span = std::max({hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2], 1e-300});
  std::vector<std::pair<uint64_t, int>> key(nt);
  for (int t = 0; t < nt; ++t) {
    uint64_t code = 0;
    for (int k = 0; k < 3; ++k) {
      double f = (c[3 * (size_t)t + k] - lo[k]) / span;
      uint64_t q = (uint64_t)std::min(std::max(f, 0.0) * 2097151.0, 2097151.0);
      code |= spread3(q) << k;
    }
    key[t] = {code, t};
  }
  std::sort(key.begin(), key.end());
  std::vector<int> rank(nt);
  for (int i = 0; i < nt; ++i) rank[key[i].second] = i;
  return rank;
}

Supports build_supports(const bgb_space* s) {
  Supports S;
  S.off.assign((size_t)s->nfun + 1, 0);
  for (int64_t t = 0; t < s->nt; ++t)
    for (int i = 0; i < 3; ++i) {
      int f = s->fn_index[3 * t + i];
      if (f >= 0) S.off[f + 1]++;
    }
  for (int f = 0; f < s->nfun; ++f) S.off[f + 1] += S.off[f];
  S.tri.resize(S.off[s->nfun]);
  S.loc.resize(S.off[s->nfun]);
  S.coef.resize(S.off[s->nfun]);
  std::vector<int64_t> fill(S.off.begin(), S.off.end() - 1);
  for (int64_t t = 0; t < s->nt; ++t)  // triangles ascending -> supports sorted by triangle
    for (int i = 0; i < 3; ++i) {
      int f = s->fn_index[3 * t + i];
      if (f < 0) continue;
      int64_t k = fill[f]++;
      S.tri[k] = (int)t;
      S.loc[k] = i;
      S.coef[k] = s->fn_coef[3 * t + i];
    }
  return S;
}

// Functions [f_begin, f_end) ordered by the Morton rank of their first support.
std::vector<int> order_functions(const Supports& S, const std::vector<int>& rank, int f_begin, int f_end) {
  std::vector<std::pair<int64_t, int>> key;
  key.reserve(f_end - f_begin);
  for (int f = f_begin; f < f_end; ++f) {
    int64_t first = INT64_MAX;
    for (int64_t k = S.off[f]; k < S.off[f + 1]; ++k) first = std::min<int64_t>(first, rank[S.tri[k]]);
    key.push_back({first, f});
  }
  std::sort(key.begin(), key.end());
  std::vector<int> out(key.size());
  for (size_t i = 0; i < key.size(); ++i) out[i] = key[i].second;
  return out;
}

void plan_test_side(const Supports& S, const std::vector<int>& order, int FM, int64_t row0, HostPlan& P) {
  P.tb_off.push_back(0);
  P.tb_fn_off.push_back(0);
  P.fs_off.push_back(0);
  std::vector<int> tris;
  for (size_t b0 = 0; b0 < order.size(); b0 += FM) {
    size_t b1 = std::min(order.size(), b0 + FM);
    tris.clear();
    for (size_t i = b0; i < b1; ++i) {
      int f = order[i];
      for (int64_t k = S.off[f]; k < S.off[f + 1]; ++k) tris.push_back(S.tri[k]);
    }
    std::sort(tris.begin(), tris.end());
    tris.erase(std::unique(tris.begin(), tris.end()), tris.end());
    for (size_t i = b0; i < b1; ++i) {
      int f = order[i];
      int cnt = 0;
      for (int64_t k = S.off[f]; k < S.off[f + 1]; ++k) {
        int slot = (int)(std::lower_bound(tris.begin(), tris.end(), S.tri[k]) - tris.begin());
        P.fs_code.push_back(slot << 2 | S.loc[k]);
        P.fs_coef.push_back(S.coef[k]);
        ++cnt;
      }
      P.MAXS = std::max(P.MAXS, cnt);
      P.fs_off.push_back((int)P.fs_code.size());
      P.rows.push_back((int64_t)f - row0);
    }
    P.tb_tris.insert(P.tb_tris.end(), tris.begin(), tris.end());
    P.tb_off.push_back((int)P.tb_tris.size());
    P.tb_fn_off.push_back((int)b1);
    P.tmax = std::max(P.tmax, (int)tris.size());
  }
}

void plan_trial_side(const Supports& S, const std::vector<int>& order, int FN, int SC, HostPlan& P) {
  P.bb_off.push_back(0);
  P.bb_fn_off.push_back(0);
  P.bb_chunk_off.push_back(0);
  P.ch_grp_off.push_back(0);
  P.grp_sup_off.push_back(0);
  std::vector<int> tris;
  struct Ent { int chunk, nl, slot, loc; double coef; };
  std::vector<Ent> ents;
  for (size_t b0 = 0; b0 < order.size(); b0 += FN) {
    size_t b1 = std::min(order.size(), b0 + FN);
    tris.clear();
    for (size_t i = b0; i < b1; ++i) {
      int f = order[i];
      for (int64_t k = S.off[f]; k < S.off[f + 1]; ++k) tris.push_back(S.tri[k]);
    }
    std::sort(tris.begin(), tris.end());
    tris.erase(std::unique(tris.begin(), tris.end()), tris.end());
    ents.clear();
    for (size_t i = b0; i < b1; ++i) {
      int f = order[i];
      for (int64_t k = S.off[f]; k < S.off[f + 1]; ++k) {
        int slot = (int)(std::lower_bound(tris.begin(), tris.end(), S.tri[k]) - tris.begin());
        ents.push_back({slot / SC, (int)(i - b0), slot, S.loc[k], S.coef[k]});
      }
    }
    // groups: per chunk, per local function, supports by slot (= trial triangle) ascending
    std::sort(ents.begin(), ents.end(), [](const Ent& a, const Ent& b) {
      if (a.chunk != b.chunk) return a.chunk < b.chunk;
      if (a.nl != b.nl) return a.nl < b.nl;
      return a.slot < b.slot;
    });
    int nchunks = ((int)tris.size() + SC - 1) / SC;
    size_t e = 0;
    for (int c = 0; c < nchunks; ++c) {
      while (e < ents.size() && ents[e].chunk == c) {
        int nl = ents[e].nl;
        P.grp_fn.push_back(nl);
        while (e < ents.size() && ents[e].chunk == c && ents[e].nl == nl) {
          P.gs_code.push_back(ents[e].slot << 2 | ents[e].loc);
          P.gs_coef.push_back(ents[e].coef);
          ++e;
        }
        P.grp_sup_off.push_back((int)P.gs_code.size());
      }
      P.ch_grp_off.push_back((int)P.grp_fn.size());
    }
    for (size_t i = b0; i < b1; ++i) P.cols.push_back(order[i]);
    const int g_lo = P.ch_grp_off[P.ch_grp_off.size() - 1 - nchunks];
    const int g_hi = P.ch_grp_off.back();
    P.gmax = std::max(P.gmax, g_hi - g_lo);
    P.gsmax = std::max(P.gsmax, P.grp_sup_off[g_hi] - P.grp_sup_off[g_lo]);
    P.bb_tris.insert(P.bb_tris.end(), tris.begin(), tris.end());
    P.bb_off.push_back((int)P.bb_tris.size());
    P.bb_fn_off.push_back((int)b1);
    P.bb_chunk_off.push_back(P.bb_chunk_off.back() + nchunks);
    P.nmax = std::max(P.nmax, (int)tris.size());
  }
}

// Tile configurations: (FM, FN, SC) per precision.
const TileCfg kTileCfgs[] = {
    {64, 64, 16},   // 0: mixed, RWG
    {64, 64, 8},    // 1
    {128, 64, 8},   // 2
    {96, 96, 8},    // 3
    {64, 64, 4},    // 4: FP64, RWG
    {32, 32, 8},    // 5
    {32, 32, 4},    // 6: FP64, Lagrange
    {16, 16, 4},    // 7
    {48, 48, 8},    // 8: mixed, RWG
    {48, 48, 4},    // 9
    {40, 40, 8},    // 10
    {48, 48, 16},   // 11
    {56, 56, 8},    // 12
};
// Preference order when the caller does not pin a tile: the first whose shared memory fits.
const int kPrefMixed[] = {4, 8, 1, 5, 6, 7};
const int kNumPrefMixed = sizeof(kPrefMixed) / sizeof(int);
const int kPrefFp64[] = {4, 8, 5, 6, 7};
const int kNumPrefFp64 = sizeof(kPrefFp64) / sizeof(int);
const int kNumTileCfgs = sizeof(kTileCfgs) / sizeof(kTileCfgs[0]);

// ----------------------------------------------------------------------------------------
// Upload helpers
// ----------------------------------------------------------------------------------------
template <class T>
static int upload(bgb_handle* h, DevBuf& buf, const std::vector<T>& v, size_t offset_bytes) {
  if (v.empty()) return 0;
  BGB_CUDA(cudaMemcpyAsync((char*)buf.p + offset_bytes, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice,
                           h->stream));
  return 0;
}

static int upload_space(bgb_handle* h, const bgb_space* s, DevBuf& verts, DevBuf& tris, DevBuf& geo) {
  int rc;
  if ((rc = verts.ensure(sizeof(double) * 3 * (size_t)std::max(1, s->nv)))) return rc;
  if ((rc = tris.ensure(sizeof(int32_t) * 3 * (size_t)std::max(1, s->nt)))) return rc;
  if ((rc = geo.ensure(sizeof(Geo64) * (size_t)std::max(1, s->nt)))) return rc;
  if (s->nv) BGB_CUDA(cudaMemcpyAsync(verts.p, s->vertices, sizeof(double) * 3 * (size_t)s->nv, cudaMemcpyHostToDevice, h->stream));
  if (s->nt) BGB_CUDA(cudaMemcpyAsync(tris.p, s->triangles, sizeof(int32_t) * 3 * (size_t)s->nt, cudaMemcpyHostToDevice, h->stream));
  launch_prepare_geo64(verts.as<double>(), tris.as<int32_t>(), s->nt, geo.as<Geo64>(), h->stream);
  return 0;
}

bool same_space(const bgb_space* a, const bgb_space* b) {
  return a == b || (a->vertices == b->vertices && a->triangles == b->triangles && a->nv == b->nv && a->nt == b->nt);
}

double max_edge(const bgb_space* s) {
  double m = 0.0;
  for (int64_t t = 0; t < s->nt; ++t)
    for (int a = 0; a < 3; ++a) {
      const double* p = s->vertices + 3 * (int64_t)s->triangles[3 * t + a];
      const double* q = s->vertices + 3 * (int64_t)s->triangles[3 * t + (a + 1) % 3];
      const double d = std::sqrt((p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) + (p[2] - q[2]) * (p[2] - q[2]));
      m = std::max(m, d);
    }
  return m;
}

bool df_singular_ok(const OpParams& op, double edge_t, double edge_b) {
  // singular / near pairs have R <= (edge_t + edge_b) * 2 at most; df_sincos covers |k R| < 400
  return op.gamma[0] == 0.0 && std::fabs(op.gamma[1]) * 2.0 * (edge_t + edge_b) < 350.0;
}

static int check_abort(bgb_handle* h) {
  if (h->abort_host && *h->abort_host) {
    set_error("aborted by bgb_abort");
    return BGB_ERR_ABORTED;
  }
  return 0;
}

// Classification of all (test, trial) triangle pairs into the non-far CSR; returns the count.
static int classify_all(bgb_handle* h, const bgb_space* test, const bgb_space* trial, const Geo64* gt,
                        const Geo64* gb, double k2, int64_t* total) {
  int rc;
  const int nt = test->nt, nb = trial->nt;
  if ((rc = h->bnd_t.ensure(sizeof(float4) * std::max(1, nt)))) return rc;
  if ((rc = h->bnd_b.ensure(sizeof(float4) * std::max(1, nb)))) return rc;
  if ((rc = h->cls_count.ensure(sizeof(int) * (size_t)(nt + 1)))) return rc;
  if ((rc = h->cls_off.ensure(sizeof(int64_t) * (size_t)(nt + 1)))) return rc;
  if ((rc = h->err.ensure(sizeof(int) * 4))) return rc;
  BGB_CUDA(cudaMemsetAsync(h->err.p, 0, sizeof(int) * 4, h->stream));
  launch_prepare_bounds(gt, nt, k2, 0, h->bnd_t.as<float4>(), h->stream);
  launch_prepare_bounds(gb, nb, k2, 1, h->bnd_b.as<float4>(), h->stream);
  launch_classify(false, h->bnd_t.as<float4>(), h->bnd_b.as<float4>(), gt, gb, nt, nb, k2, h->cls_count.as<int>(),
                  nullptr, nullptr, nullptr, nullptr, h->err.as<int>(), h->num_sms, h->stream);
  launch_scan(h->cls_count.as<int>(), nt, h->cls_off.as<int64_t>(), h->stream);
  int64_t tot = 0;
  int herr = 0;
  BGB_CUDA(cudaMemcpyAsync(&tot, h->cls_off.as<int64_t>() + nt, sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream));
  BGB_CUDA(cudaMemcpyAsync(&herr, h->err.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  BGB_CUDA(cudaStreamSynchronize(h->stream));
  if (herr) {
    set_error("degenerate geometry: a triangle pair shares more than three vertices");
    return BGB_ERR_INVALID;
  }
  if ((rc = h->ent_tau.ensure(sizeof(int) * (size_t)std::max<int64_t>(1, tot)))) return rc;
  if ((rc = h->ent_sigma.ensure(sizeof(int) * (size_t)std::max<int64_t>(1, tot)))) return rc;
  if ((rc = h->ent_cls.ensure((size_t)std::max<int64_t>(1, tot)))) return rc;
  if ((rc = h->ent_mask.ensure(sizeof(int16_t) * (size_t)std::max<int64_t>(1, tot)))) return rc;
  launch_classify(true, h->bnd_t.as<float4>(), h->bnd_b.as<float4>(), gt, gb, nt, nb, k2, h->cls_count.as<int>(),
                  h->cls_off.as<int64_t>(), h->ent_tau.as<int>(), h->ent_sigma.as<int>(), h->ent_cls.as<int8_t>(),
                  h->err.as<int>(), h->num_sms, h->stream, h->ent_mask.as<int16_t>());
  BGB_CUDA(cudaGetLastError());
  *total = tot;
  return 0;
}

double event_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

}  // namespace bgb

using namespace bgb;

// ========================================================================================
// C ABI
// ========================================================================================
extern "C" {

int bgb_abi_version(void) { return BGB_ABI_VERSION; }

const char* bgb_last_error(void) { return g_err.c_str(); }

int bgb_create(bgb_handle** out, const bgb_config* cfg) {
  if (!out) { set_error("out is NULL"); return BGB_ERR_INVALID; }
  *out = nullptr;
  bgb_config c{};
  if (cfg) c = *cfg;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    set_error("no CUDA device available (%s)", cudaGetErrorString(e));
    return BGB_ERR_CUDA;
  }
  if (c.device < 0 || c.device >= ndev) { set_error("device %d out of range", c.device); return BGB_ERR_INVALID; }
  BGB_CUDA(cudaSetDevice(c.device));
  bgb_handle* h = new bgb_handle();
  h->device = c.device;
  h->cfg = c;
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, c.device);
  int rc = 0;
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking)) != cudaSuccess) {
    rc = cuda_fail(e, "cudaStreamCreate");
  }
  for (int i = 0; i < 8 && !rc; ++i)
    if ((e = cudaEventCreate(&h->ev[i])) != cudaSuccess) rc = cuda_fail(e, "cudaEventCreate");
  if (!rc) {
    int* p = nullptr;
    if ((e = cudaHostAlloc((void**)&p, sizeof(int), cudaHostAllocMapped)) != cudaSuccess) rc = cuda_fail(e, "cudaHostAlloc");
    else {
      *p = 0;
      h->abort_host = p;
      if ((e = cudaHostGetDevicePointer((void**)&h->abort_dev, p, 0)) != cudaSuccess) rc = cuda_fail(e, "cudaHostGetDevicePointer");
    }
  }
  if (rc) {
    bgb_destroy(h);
    return rc;
  }
  *out = h;
  return 0;
}

int bgb_destroy(bgb_handle* h) {
  if (!h) return 0;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
  DevBuf* bufs[] = {&h->verts_t, &h->tris_t, &h->verts_b, &h->tris_b, &h->geo_t, &h->geo_b, &h->bnd_t, &h->bnd_b,
                    &h->rec_t, &h->rec_b, &h->cls_count, &h->cls_off, &h->ent_tau, &h->ent_sigma, &h->ent_cls, &h->ent_mask, &h->geodf_t, &h->geodf_b,
                    &h->sing_L, &h->err, &h->plan_i, &h->plan_l, &h->plan_d, &h->plan_f, &h->far_items, &h->far_const, &h->df_tab, &h->stage[0], &h->stage[1],
                    &h->diag_a, &h->diag_b, &h->diag_c, &h->diag_d};
  for (DevBuf* b : bufs) b->release();
  for (int i = 0; i < 8; ++i)
    if (h->ev[i]) cudaEventDestroy(h->ev[i]);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  if (h->abort_host) cudaFreeHost((void*)h->abort_host);
  delete h;
  return 0;
}

int bgb_abort(bgb_handle* h) {
  if (!h || !h->abort_host) { set_error("invalid handle"); return BGB_ERR_INVALID; }
  *h->abort_host = 1;
  return 0;
}

int bgb_tile_info(int32_t* ids, int32_t cap) {
  for (int i = 0; i < kNumTileCfgs && i < cap; ++i)
    if (ids) ids[i] = i;
  return kNumTileCfgs;
}

int bgb_measure_issue_peaks(bgb_handle* h, double* fp32, double* fp64, double* mufu) {
  if (!h || !fp32 || !fp64 || !mufu) { set_error("invalid argument"); return BGB_ERR_INVALID; }
  cudaSetDevice(h->device);
  return measure_issue_peaks(h->num_sms, fp32, fp64, mufu);
}

int bgb_classify_block(bgb_handle* h, const bgb_space* test, const bgb_space* trial, double k2, int32_t t0,
                       int32_t t1, int32_t s0, int32_t s1, int8_t* out) {
  if (!h) { set_error("invalid handle"); return BGB_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(h->mu);
  int rc;
  if ((rc = validate_space(test, "test")) || (rc = validate_space(trial, "trial"))) return rc;
  if (!out || t0 < 0 || s0 < 0 || t1 > test->nt || s1 > trial->nt || t1 < t0 || s1 < s0 || !std::isfinite(k2)) {
    set_error("bgb_classify_block: bad block or output");
    return BGB_ERR_INVALID;
  }
  cudaSetDevice(h->device);
  if ((rc = upload_space(h, test, h->verts_t, h->tris_t, h->geo_t))) return rc;
  if ((rc = upload_space(h, trial, h->verts_b, h->tris_b, h->geo_b))) return rc;
  size_t n = (size_t)(t1 - t0) * (s1 - s0);
  if ((rc = h->diag_a.ensure(std::max<size_t>(n, 1)))) return rc;
  if ((rc = h->err.ensure(sizeof(int) * 4))) return rc;
  BGB_CUDA(cudaMemsetAsync(h->err.p, 0, sizeof(int), h->stream));
  launch_classify_dense(h->geo_t.as<Geo64>(), h->geo_b.as<Geo64>(), t0, t1, s0, s1, k2, h->diag_a.as<int8_t>(),
                        h->err.as<int>(), h->stream);
  int herr = 0;
  if (n) BGB_CUDA(cudaMemcpyAsync(out, h->diag_a.p, n, cudaMemcpyDeviceToHost, h->stream));
  BGB_CUDA(cudaMemcpyAsync(&herr, h->err.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  BGB_CUDA(cudaStreamSynchronize(h->stream));
  if (herr) { set_error("degenerate geometry: a triangle pair shares more than three vertices"); return BGB_ERR_INVALID; }
  return 0;
}

int bgb_local_matrices(bgb_handle* h, const bgb_operator* op, const bgb_space* test, const bgb_space* trial,
                       const bgb_quadstrat* qs, int32_t precision, int64_t npairs, const int32_t* tau,
                       const int32_t* sigma, int32_t force_class, double* out, int8_t* cls_out) {
  if (!h) { set_error("invalid handle"); return BGB_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(h->mu);
  int rc;
  if ((rc = validate_space(test, "test")) || (rc = validate_space(trial, "trial"))) return rc;
  OpParams opp;
  QuadSel qsel;
  if ((rc = make_opparams(op, test, trial, &opp))) return rc;
  if (!qs) { set_error("quadstrat is NULL"); return BGB_ERR_INVALID; }
  if ((rc = make_quadsel(qs, &qsel))) return rc;
  if (precision != BGB_PREC_FP64 && precision != BGB_PREC_MIXED) { set_error("bad precision"); return BGB_ERR_INVALID; }
  if (npairs < 0 || (npairs && (!tau || !sigma || !out)) || force_class > 4) { set_error("bad pair list"); return BGB_ERR_INVALID; }
  for (int64_t p = 0; p < npairs; ++p)
    if (tau[p] < 0 || tau[p] >= test->nt || sigma[p] < 0 || sigma[p] >= trial->nt) {
      set_error("pair %lld out of range", (long long)p);
      return BGB_ERR_INVALID;
    }
  if (npairs == 0) return 0;
  cudaSetDevice(h->device);
  if ((rc = upload_space(h, test, h->verts_t, h->tris_t, h->geo_t))) return rc;
  if ((rc = upload_space(h, trial, h->verts_b, h->tris_b, h->geo_b))) return rc;
  RuleTable R = make_rules();
  if ((rc = h->diag_a.ensure(sizeof(int) * npairs)) || (rc = h->diag_b.ensure(sizeof(int) * npairs)) ||
      (rc = h->diag_c.ensure(sizeof(double2) * 9 * npairs)) || (rc = h->diag_d.ensure(sizeof(double2) * 9 * npairs + npairs)) ||
      (rc = h->ent_mask.ensure(sizeof(int16_t) * npairs)) || (rc = h->err.ensure(sizeof(int) * 4)))
    return rc;
  BGB_CUDA(cudaMemcpyAsync(h->diag_a.p, tau, sizeof(int) * npairs, cudaMemcpyHostToDevice, h->stream));
  BGB_CUDA(cudaMemcpyAsync(h->diag_b.p, sigma, sizeof(int) * npairs, cudaMemcpyHostToDevice, h->stream));
  BGB_CUDA(cudaMemsetAsync(h->err.p, 0, sizeof(int), h->stream));
  int8_t* dcls = (int8_t*)((char*)h->diag_d.p + sizeof(double2) * 9 * npairs);
  launch_local_diag64(opp, qsel, R, test->refspace, trial->refspace, h->geo_t.as<Geo64>(), h->geo_b.as<Geo64>(),
                      h->diag_a.as<int>(), h->diag_b.as<int>(), npairs, force_class, h->diag_c.as<double2>(), dcls,
                      h->err.as<int>(), h->num_sms, h->stream, h->ent_mask.as<int16_t>());
  // mixed: singular / near pairs through the double-float kernel (far pairs are replaced below)
  std::vector<float> dftab;
  if (precision == BGB_PREC_MIXED && df_singular_ok(opp, max_edge(test), max_edge(trial))) {
    DfTables M;
    build_df_tables(qsel, R, dftab, M);
    if ((rc = h->df_tab.ensure(sizeof(float) * dftab.size()))) return rc;
    BGB_CUDA(cudaMemcpyAsync(h->df_tab.p, dftab.data(), sizeof(float) * dftab.size(), cudaMemcpyHostToDevice, h->stream));
    if ((rc = h->geodf_t.ensure(sizeof(GeoDf) * std::max(1, test->nt))) ||
        (rc = h->geodf_b.ensure(sizeof(GeoDf) * std::max(1, trial->nt))))
      return rc;
    launch_prepare_geodf(h->geo_t.as<Geo64>(), test->nt, h->geodf_t.as<GeoDf>(), h->stream);
    launch_prepare_geodf(h->geo_b.as<Geo64>(), trial->nt, h->geodf_b.as<GeoDf>(), h->stream);
    launch_singular_df(opp.kind, make_opdf(opp), nullptr, nullptr, M, h->df_tab.as<float>(), h->geodf_t.as<GeoDf>(),
                       h->geodf_b.as<GeoDf>(), h->diag_a.as<int>(), h->diag_b.as<int>(), dcls,
                       h->ent_mask.as<int16_t>(), npairs, h->diag_c.as<double2>(), nullptr, h->num_sms, h->stream);
  }
  // far pairs through the far-kernel pair code of the requested precision
  FarConst K = make_farconst(opp, R, qsel);
  const int gen = far_generic_q(K.qt, K.qb);
  const int rst = rec_stride(precision, K.qt, gen), rsb = rec_stride(precision, K.qb, gen);
  const size_t esz = precision == BGB_PREC_MIXED ? sizeof(float) : sizeof(double);
  if ((rc = h->rec_t.ensure(esz * rst * std::max(1, test->nt))) || (rc = h->rec_b.ensure(esz * rsb * std::max(1, trial->nt))))
    return rc;
  launch_prepare_rec(precision, 0, gen ? BGB_MAXQ : K.qt, h->geo_t.as<Geo64>(), test->nt, R, qsel.far_t, 1.0, h->rec_t.p, h->stream);
  launch_prepare_rec(precision, 1, gen ? BGB_MAXQ : K.qb, h->geo_b.as<Geo64>(), trial->nt, R, qsel.far_b,
                     BGB_INV_4PI_D, h->rec_b.p, h->stream);
  if ((rc = launch_far_pairs_diag(precision, K, h->rec_t.p, h->rec_b.p, h->diag_a.as<int>(), h->diag_b.as<int>(), npairs,
                                  h->diag_d.as<double2>(), h->stream)))
    return rc;
  std::vector<double> far((size_t)npairs * 18);
  std::vector<int8_t> cls((size_t)npairs);
  int herr = 0;
  BGB_CUDA(cudaMemcpyAsync(out, h->diag_c.p, sizeof(double2) * 9 * npairs, cudaMemcpyDeviceToHost, h->stream));
  BGB_CUDA(cudaMemcpyAsync(far.data(), h->diag_d.p, sizeof(double2) * 9 * npairs, cudaMemcpyDeviceToHost, h->stream));
  BGB_CUDA(cudaMemcpyAsync(cls.data(), dcls, npairs, cudaMemcpyDeviceToHost, h->stream));
  BGB_CUDA(cudaMemcpyAsync(&herr, h->err.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  BGB_CUDA(cudaStreamSynchronize(h->stream));
  if (herr) { set_error("degenerate geometry: a triangle pair shares more than three vertices"); return BGB_ERR_INVALID; }
  for (int64_t p = 0; p < npairs; ++p) {
    if (cls[p] == BGB_CLASS_FAR) std::memcpy(out + 18 * p, far.data() + 18 * p, sizeof(double) * 18);
    if (cls_out) cls_out[p] = cls[p];
  }
  return 0;
}

int bgb_assemble(bgb_handle* h, const bgb_operator* op, const bgb_space* test, const bgb_space* trial,
                 const bgb_quadstrat* qs, int32_t precision, void* out, int32_t out_kind, int64_t ld, int64_t row0,
                 int64_t nrows, void* stream, bgb_stats* stats) {
  using clk = std::chrono::steady_clock;
  auto t_start = clk::now();
  if (!h) { set_error("invalid handle"); return BGB_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(h->mu);
  int rc;
  if ((rc = validate_space(test, "test")) || (rc = validate_space(trial, "trial"))) return rc;
  OpParams opp;
  QuadSel qsel;
  if ((rc = make_opparams(op, test, trial, &opp))) return rc;
  if (!qs) { set_error("quadstrat is NULL"); return BGB_ERR_INVALID; }
  if ((rc = make_quadsel(qs, &qsel))) return rc;
  if (precision != BGB_PREC_FP64 && precision != BGB_PREC_MIXED) { set_error("bad precision %d", precision); return BGB_ERR_INVALID; }
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
  cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
  const bool host_out = out_kind == BGB_OUT_HOST_C64 || out_kind == BGB_OUT_HOST_C32;
  const bool c64 = out_kind == BGB_OUT_HOST_C64 || out_kind == BGB_OUT_DEVICE_C64;
  const size_t esz = c64 ? 16 : 8;
  if (!host_out && s != h->stream) {
    // run the pipeline on the handle stream, ordered after the caller's stream
    BGB_CUDA(cudaEventRecord(h->ev[7], s));
    BGB_CUDA(cudaStreamWaitEvent(h->stream, h->ev[7], 0));
  }

  RuleTable R = make_rules();
  cudaEventRecord(h->ev[0], h->stream);
  int launches = 0;
  if ((rc = upload_space(h, test, h->verts_t, h->tris_t, h->geo_t))) return rc;
  launches += test->nt > 0;
  const bool same = same_space(test, trial);
  const Geo64* gt = h->geo_t.as<Geo64>();
  const Geo64* gb = gt;
  if (!same) {
    if ((rc = upload_space(h, trial, h->verts_b, h->tris_b, h->geo_b))) return rc;
    gb = h->geo_b.as<Geo64>();
    launches += trial->nt > 0;
  }
  // 1. classification
  int64_t nsing = 0;
  if ((rc = classify_all(h, test, trial, gt, gb, opp.k2, &nsing))) return rc;
  launches += 6;  // 2 bounds, 2 classify passes, scan (+1 singular below)
  cudaEventRecord(h->ev[1], h->stream);
  // 2. singular / near pairs: FP64 kernel (plain path), double-float kernel (mixed path)
  if ((rc = h->sing_L.ensure(sizeof(double2) * 9 * std::max<int64_t>(1, nsing)))) return rc;
  const bool use_df = precision == BGB_PREC_MIXED && df_singular_ok(opp, max_edge(test), same ? max_edge(test) : max_edge(trial));
  if (use_df) {
    std::vector<float> tab;
    DfTables M;
    build_df_tables(qsel, R, tab, M);
    if ((rc = h->df_tab.ensure(sizeof(float) * tab.size()))) return rc;
    BGB_CUDA(cudaMemcpyAsync(h->df_tab.p, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice, h->stream));
    if ((rc = h->geodf_t.ensure(sizeof(GeoDf) * std::max(1, test->nt))) ||
        (!same && (rc = h->geodf_b.ensure(sizeof(GeoDf) * std::max(1, trial->nt)))))
      return rc;
    launch_prepare_geodf(gt, test->nt, h->geodf_t.as<GeoDf>(), h->stream);
    if (!same) launch_prepare_geodf(gb, trial->nt, h->geodf_b.as<GeoDf>(), h->stream);
    const GeoDf* dgt = h->geodf_t.as<GeoDf>();
    const GeoDf* dgb = same ? dgt : h->geodf_b.as<GeoDf>();
    launch_singular_df(opp.kind, make_opdf(opp), nullptr, nullptr, M, h->df_tab.as<float>(), dgt, dgb,
                       h->ent_tau.as<int>(), h->ent_sigma.as<int>(), h->ent_cls.as<int8_t>(),
                       h->ent_mask.as<int16_t>(), nsing, h->sing_L.as<double2>(), h->abort_dev, h->num_sms, h->stream);
    launches += 1 + (same ? 0 : 1);
    BGB_CUDA(cudaStreamSynchronize(h->stream));  // the host table buffer goes out of scope
  } else {
    launch_singular(opp, qsel, R, test->refspace, trial->refspace, gt, gb, h->ent_tau.as<int>(), h->ent_sigma.as<int>(),
                    h->ent_cls.as<int8_t>(), nsing, h->sing_L.as<double2>(), h->abort_dev, h->num_sms, h->stream);
  }
  BGB_CUDA(cudaGetLastError());
  cudaEventRecord(h->ev[2], h->stream);
  if ((rc = check_abort(h))) return rc;
  // 3. far-pair records
  FarConst K = make_farconst(opp, R, qsel);
  const int gen = far_generic_q(K.qt, K.qb);
  const int rst = rec_stride(precision, K.qt, gen), rsb = rec_stride(precision, K.qb, gen);
  const size_t rsz = precision == BGB_PREC_MIXED ? sizeof(float) : sizeof(double);
  if ((rc = h->rec_t.ensure(rsz * rst * std::max(1, test->nt))) || (rc = h->rec_b.ensure(rsz * rsb * std::max(1, trial->nt))))
    return rc;
  launch_prepare_rec(precision, 0, gen ? BGB_MAXQ : K.qt, gt, test->nt, R, qsel.far_t, 1.0, h->rec_t.p, h->stream);
  launch_prepare_rec(precision, 1, gen ? BGB_MAXQ : K.qb, gb, trial->nt, R, qsel.far_b, BGB_INV_4PI_D, h->rec_b.p, h->stream);
  launches += 2;

  // 4. host plan
  const bool pinned_cfg = h->cfg.tile_config >= 0;
  if (pinned_cfg && h->cfg.tile_config >= kNumTileCfgs) { set_error("tile_config %d out of range", h->cfg.tile_config); return BGB_ERR_INVALID; }
  std::vector<int> prefs;
  if (pinned_cfg) prefs.push_back(h->cfg.tile_config);
  else if (precision == BGB_PREC_MIXED) prefs.assign(std::begin(kPrefMixed), std::end(kPrefMixed));
  else prefs.assign(std::begin(kPrefFp64), std::end(kPrefFp64));
  int smem_max = 0;
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  int cfg_id = -1;
  Supports St = build_supports(test);
  Supports Sb = same ? St : build_supports(trial);
  std::vector<int> rank_t = morton_rank(test);
  std::vector<int> rank_b = same ? rank_t : morton_rank(trial);
  std::vector<int> ord_b = order_functions(Sb, rank_b, 0, trial->nfun);

  // row blocks for out-of-core: bounded by the HBM budget
  size_t freeb = 0, totalb = 0;
  cudaMemGetInfo(&freeb, &totalb);
  int64_t budget = h->cfg.hbm_budget_bytes > 0 ? h->cfg.hbm_budget_bytes : (int64_t)(0.9 * (double)freeb);
  int64_t rows_per_block = nrows;
  if (host_out) {
    int64_t per_row = (int64_t)esz * trial->nfun;
    rows_per_block = std::max<int64_t>(1, (budget / 2) / std::max<int64_t>(1, per_row));
    rows_per_block = std::min(rows_per_block, nrows);
  }
  st.row_blocks = (int)((nrows + rows_per_block - 1) / rows_per_block);
  double ms_far = 0, ms_copy = 0;
  int64_t pairs_computed = 0;
  for (int64_t r0 = row0; r0 < row0 + nrows; r0 += rows_per_block) {
    const int64_t nr = std::min(rows_per_block, row0 + nrows - r0);
    HostPlan P;
    std::vector<int> ord_t = order_functions(St, rank_t, (int)r0, (int)(r0 + nr));
    TileCfg tc{};
    size_t smem = 0;
    for (size_t pi_ = 0; pi_ < prefs.size(); ++pi_) {
      if (cfg_id >= 0 && prefs[pi_] != cfg_id) continue;  // later row blocks keep the first block's choice
      tc = kTileCfgs[prefs[pi_]];
      P = HostPlan();
      plan_test_side(St, ord_t, tc.FM, host_out ? r0 : row0, P);
      plan_trial_side(Sb, ord_b, tc.FN, tc.SC, P);
      TilePlan probe{};
      probe.FM = tc.FM; probe.FN = tc.FN; probe.SC = tc.SC; probe.MAXS = P.MAXS;
      probe.gmax = P.gmax; probe.gsmax = P.gsmax;
      probe.tmax = std::max(1, P.tmax); probe.nmax = std::max(1, P.nmax);
      smem = far_smem_bytes(precision, K.qt, K.qb, probe);
      if (smem <= (size_t)smem_max) { cfg_id = prefs[pi_]; break; }
    }
    if (cfg_id < 0 || smem > (size_t)smem_max) {
      set_error("no tile configuration fits in %d B of shared memory (last tried needs %zu B)", smem_max, smem);
      return BGB_ERR_CAPACITY;
    }
    st.tile_config = cfg_id;
    for (size_t a = 0; a + 1 < P.tb_off.size(); ++a)
      for (size_t b = 0; b + 1 < P.bb_off.size(); ++b)
        pairs_computed += (int64_t)(P.tb_off[a + 1] - P.tb_off[a]) * (P.bb_off[b + 1] - P.bb_off[b]);
    // pack int arrays
    std::vector<int> I;
    std::vector<int64_t> Lg;
    std::vector<double> D;
    auto put_i = [&](const std::vector<int>& v) { size_t o = I.size(); I.insert(I.end(), v.begin(), v.end()); return o; };
    auto put_l = [&](const std::vector<int64_t>& v) { size_t o = Lg.size(); Lg.insert(Lg.end(), v.begin(), v.end()); return o; };
    auto put_d = [&](const std::vector<double>& v) { size_t o = D.size(); D.insert(D.end(), v.begin(), v.end()); return o; };
    size_t o_tb_off = put_i(P.tb_off), o_tb_tris = put_i(P.tb_tris), o_tb_fn = put_i(P.tb_fn_off), o_fs_off = put_i(P.fs_off),
           o_fs_code = put_i(P.fs_code), o_bb_off = put_i(P.bb_off), o_bb_tris = put_i(P.bb_tris), o_bb_fn = put_i(P.bb_fn_off),
           o_bb_ch = put_i(P.bb_chunk_off), o_ch_grp = put_i(P.ch_grp_off), o_grp_fn = put_i(P.grp_fn),
           o_grp_sup = put_i(P.grp_sup_off), o_gs_code = put_i(P.gs_code);
    size_t o_rows = put_l(P.rows), o_cols = put_l(P.cols);
    size_t o_fs_coef = put_d(P.fs_coef), o_gs_coef = put_d(P.gs_coef);
    std::vector<float> F32;
    F32.reserve(P.fs_coef.size() + P.gs_coef.size());
    for (double v : P.fs_coef) F32.push_back((float)v);
    const size_t o_gs32 = F32.size();
    for (double v : P.gs_coef) F32.push_back((float)v);
    if ((rc = h->plan_i.ensure(sizeof(int) * std::max<size_t>(1, I.size()))) ||
        (rc = h->plan_l.ensure(sizeof(int64_t) * std::max<size_t>(1, Lg.size()))) ||
        (rc = h->plan_d.ensure(sizeof(double) * std::max<size_t>(1, D.size()))) ||
        (rc = h->plan_f.ensure(sizeof(float) * std::max<size_t>(1, F32.size()))))
      return rc;
    BGB_CUDA(cudaStreamSynchronize(h->stream));  // previous block's plan arrays no longer in use
    if ((rc = upload(h, h->plan_i, I, 0)) || (rc = upload(h, h->plan_l, Lg, 0)) || (rc = upload(h, h->plan_d, D, 0)) ||
        (rc = upload(h, h->plan_f, F32, 0)))
      return rc;
    const int* pi = h->plan_i.as<int>();
    const int64_t* pl = h->plan_l.as<int64_t>();
    const double* pd = h->plan_d.as<double>();
    TilePlan T{};
    T.rec_t = h->rec_t.p;
    T.rec_b = h->rec_b.p;
    T.bnd_t = h->bnd_t.as<float4>();
    T.bnd_b = h->bnd_b.as<float4>();
    T.n_tblocks = (int)P.tb_off.size() - 1;
    T.tb_off = pi + o_tb_off;
    T.tb_tris = pi + o_tb_tris;
    T.tb_fn_off = pi + o_tb_fn;
    T.fs_off = pi + o_fs_off;
    T.fs_code = pi + o_fs_code;
    T.fs_coef = pd + o_fs_coef;
    T.rows = pl + o_rows;
    T.n_bblocks = (int)P.bb_off.size() - 1;
    T.bb_off = pi + o_bb_off;
    T.bb_tris = pi + o_bb_tris;
    T.bb_fn_off = pi + o_bb_fn;
    T.bb_chunk_off = pi + o_bb_ch;
    T.ch_grp_off = pi + o_ch_grp;
    T.grp_fn = pi + o_grp_fn;
    T.grp_sup_off = pi + o_grp_sup;
    T.gs_code = pi + o_gs_code;
    T.gs_coef = pd + o_gs_coef;
    T.fs_coef32 = h->plan_f.as<float>();
    T.gs_coef32 = h->plan_f.as<float>() + o_gs32;
    T.gmax = P.gmax;
    T.gsmax = P.gsmax;
    T.cols = pl + o_cols;
    T.sing_off = h->cls_off.as<int64_t>();
    T.sing_sigma = h->ent_sigma.as<int>();
    T.sing_L = h->sing_L.as<double2>();
    T.FM = tc.FM;
    T.FN = tc.FN;
    T.SC = tc.SC;
    T.MAXS = P.MAXS;
    T.tmax = std::max(1, P.tmax);
    T.nmax = std::max(1, P.nmax);
    T.out_c64 = c64;
    T.abort_flag = h->abort_dev;
    void* dst = out;
    int64_t dld = ld;
    if (host_out) {
      if ((rc = h->stage[0].ensure(esz * (size_t)nr * trial->nfun))) return rc;
      dst = h->stage[0].p;
      dld = nr;
    }
    T.out = dst;
    T.ld = dld;
    cudaEventRecord(h->ev[3], h->stream);
    // the single problem runs through the same persistent work-queue kernel as batches
    // (one far kernel, so batched and single assemblies are bit-identical); tiles are
    // queued row block fastest so concurrent CTAs write neighbouring rows of a column
    std::vector<int4> items;
    items.reserve((size_t)T.n_tblocks * T.n_bblocks);
    for (int bn = 0; bn < T.n_bblocks; ++bn)
      for (int bm = 0; bm < T.n_tblocks; ++bm) items.push_back(make_int4(0, bm, bn, 0));
    if ((rc = h->far_items.ensure(sizeof(int4) * std::max<size_t>(1, items.size()))) ||
        (rc = h->far_const.ensure(sizeof(FarConst) + sizeof(TilePlan) + sizeof(int) * 4)))
      return rc;
    FarConst* dK = (FarConst*)h->far_const.p;
    TilePlan* dT = (TilePlan*)((char*)h->far_const.p + sizeof(FarConst));
    int* dctr = (int*)((char*)h->far_const.p + sizeof(FarConst) + sizeof(TilePlan));
    BGB_CUDA(cudaMemcpyAsync(dK, &K, sizeof(FarConst), cudaMemcpyHostToDevice, h->stream));
    BGB_CUDA(cudaMemcpyAsync(dT, &T, sizeof(TilePlan), cudaMemcpyHostToDevice, h->stream));
    if (!items.empty())
      BGB_CUDA(cudaMemcpyAsync(h->far_items.p, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, h->stream));
    BGB_CUDA(cudaMemsetAsync(dctr, 0, sizeof(int), h->stream));
    int per_sm = 0;
    if ((rc = far_persistent_occupancy(precision, K.op_kind, gen, smem, &per_sm))) return rc;
    const int ctas = (int)std::min<int64_t>((int64_t)items.size(), (int64_t)std::max(1, per_sm) * h->num_sms);
    if ((rc = launch_far_persistent(precision, K.op_kind, gen, dK, dT, (const int4*)h->far_items.p, (int)items.size(),
                                    dctr, smem, std::max(1, ctas), h->abort_dev, h->stream)))
      return rc;
    ++launches;
    cudaEventRecord(h->ev[4], h->stream);
    BGB_CUDA(cudaStreamSynchronize(h->stream));  // plan, items and constants are reused by the next row block
    if (host_out) {
      char* hdst = (char*)out + (size_t)(r0 - row0) * esz;
      BGB_CUDA(cudaMemcpy2DAsync(hdst, (size_t)ld * esz, dst, (size_t)nr * esz, (size_t)nr * esz, (size_t)trial->nfun,
                                 cudaMemcpyDeviceToHost, h->stream));
    }
    cudaEventRecord(h->ev[5], h->stream);
    BGB_CUDA(cudaEventSynchronize(h->ev[5]));
    if ((rc = check_abort(h))) return rc;
    ms_far += event_ms(h->ev[3], h->ev[4]);
    ms_copy += event_ms(h->ev[4], h->ev[5]);
  }
  BGB_CUDA(cudaGetLastError());
  if (!host_out && s != h->stream) {
    BGB_CUDA(cudaEventRecord(h->ev[6], h->stream));
    BGB_CUDA(cudaStreamWaitEvent(s, h->ev[6], 0));
  }
  // statistics
  st.pairs_total = (int64_t)test->nt * trial->nt;
  st.pairs_computed = pairs_computed;
  st.ms_classify = event_ms(h->ev[0], h->ev[1]);
  st.ms_singular = event_ms(h->ev[1], h->ev[2]);
  st.ms_far = ms_far;
  st.ms_copy = ms_copy;
  if (stats) {
    std::vector<int8_t> cls((size_t)nsing);
    if (nsing) BGB_CUDA(cudaMemcpy(cls.data(), h->ent_cls.p, nsing, cudaMemcpyDeviceToHost));
    int64_t cnt[5] = {0, 0, 0, 0, 0};
    for (int8_t c : cls) cnt[(int)c]++;
    cnt[0] = st.pairs_total - nsing;
    for (int c = 0; c < 5; ++c) st.pairs_class[c] = cnt[c];
  }
  st.ms_total = std::chrono::duration<double, std::milli>(clk::now() - t_start).count();
  st.kernel_launches = launches;
  if (stats) *stats = st;
  return 0;
}

}  // extern "C"
