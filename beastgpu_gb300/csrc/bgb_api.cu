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

#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
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
void gauss_legendre01(int n, double* x, double* w) {
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
  if (op->kind == BGB_OP_HELMHOLTZ3D_SL || op->kind == BGB_OP_HELMHOLTZ3D_DL || op->kind == BGB_OP_HELMHOLTZ3D_DLT ||
      op->kind == BGB_OP_HELMHOLTZ3D_HS) {
    if (a->refspace != BGB_REFSPACE_LAGRANGE_C0D1 || b->refspace != BGB_REFSPACE_LAGRANGE_C0D1) {
      set_error("Helmholtz3D operators are implemented on lagrangec0d1 spaces");
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

FarConst make_farconst(const OpParams& op, const RuleTable& R, const QuadSel& qs, const bgb_space* test,
                       const bgb_space* trial, SpaceExtents* ext_t, SpaceExtents* ext_b) {
  FarConst k{};
  SpaceExtents et{}, eb{};
  if (test && trial) {
    et = space_extents(test);
    eb = same_space(test, trial) ? et : space_extents(trial);
  }
  if (ext_t) *ext_t = et;
  if (ext_b) *ext_b = eb;
  // |k delta| <= k (r_test + r_trial) < k (edge_test + edge_trial): within pi, the point-pair phase
  // phi0 + k delta stays in [-2 pi, 2 pi] and goes to sin / cos without a second reduction
  k.phase_direct = test && trial && std::fabs(op.gamma[1]) * (et.max_edge + eb.max_edge) <= 3.14159;
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
  // plain FP64 kernel: series for exp(-i k (R - R0)) when |k (R - R0)| <= k (r_test + r_trial) is small
  k.tay_n = 0;
  if (test && trial && op.gamma[1] != 0.0) {
    const double xmax = std::fabs(op.gamma[1]) * (et.max_centroid_radius + eb.max_centroid_radius);
    if (xmax <= 2.0) {
      double fs = 1.0, fc = 1.0;  // (2j+1)!, (2j)!
      int n = 1;
      for (; n <= BGB_TAYLOR_MAX; ++n) {
        // terms j < n kept: the first dropped terms are x^(2n) / (2n)! (cos) and x^(2n+1) / (2n+1)! (sin)
        double tc = 1.0, ts = xmax;
        for (int q = 1; q <= 2 * n; ++q) tc *= xmax / q;
        for (int q = 2; q <= 2 * n + 1; ++q) ts *= xmax / q;
        if (tc <= 0x1p-55 && ts <= 0x1p-55) break;
      }
      // measured on GB300: FP64 sincos of these small arguments costs about as much as 8 series terms
      // (cube of the reference's benchmark, 4 terms: far stage 16.0 -> 14.4 s; icosphere level 5 at
      // k = 8 pi, 11 terms: 1.13 -> 1.15 s), so the series is kept for short series only
      if (n <= 6) {
        k.tay_n = n;
        for (int j = 0; j < n; ++j) {
          if (j > 0) {
            fc *= (2.0 * j - 1.0) * (2.0 * j);
            fs *= (2.0 * j) * (2.0 * j + 1.0);
          }
          const double sg = (j & 1) ? -1.0 : 1.0;
          k.tay_c[j] = sg / fc;
          k.tay_s[j] = sg / fs;
        }
      }
    }
  }
  return k;
}

// ----------------------------------------------------------------------------------------
// Host planning: function blocks (bisection patches) and their triangle sets
// ----------------------------------------------------------------------------------------
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
    {24, 24, 4},    // 13: Lagrange
    {32, 32, 2},    // 14
    {40, 40, 4},    // 15
    {24, 24, 8},    // 16
    {60, 64, 5},    // 17: mixed, RWG (~50 test triangles x 5 = one round of 256 pairs per chunk)
    {32, 40, 5},    // 18: Lagrange
};
// Preference order when the caller does not pin a tile: the first whose shared memory fits.
// RWG: 60 x 64 tiles with 5-triangle chunks (C2 mixed far stage 28.6 ms against 31.1 ms for
// 64 x 64 x 4, whose ~53 test triangles x 4 leave a sixth of the 256 threads idle in each chunk).
const int kPrefMixed[] = {17, 4, 8, 1, 5, 6, 7};
const int kNumPrefMixed = sizeof(kPrefMixed) / sizeof(int);
// (60 x 64 x 5 gained 0.4% on the FP64 EFIE and lost 3.5% on the FP64 MFIE: the FP64 pipe, not the
// idle lanes, bounds the plain kernel)
const int kPrefFp64[] = {4, 8, 5, 6, 7};
const int kNumPrefFp64 = sizeof(kPrefFp64) / sizeof(int);
// Lagrange hats have ~6 supports: small function blocks keep the halo and the gather short
// (measured on the two-plate Helmholtz case: 32 x 32 tiles 6x faster than 64 x 64).
// d = 40 cube, mixed: 32 x 40 x 5 330 ms, 40 x 40 x 4 334 ms, 32 x 32 x 4 364 ms (with the FP32
// Lagrange kernels' per-chunk trial staging).
const int kPrefLagrange[] = {18, 6, 13, 15, 5, 7};
const int kNumPrefLagrange = sizeof(kPrefLagrange) / sizeof(int);
// The plain FP64 kernel (one CTA per SM, FP64-pipe bound) gains from fewer halo pairs more than
// from full chunks: d = 24 cube 48 x 48 x 4 1,537 ms, 40 x 40 x 4 1,629 ms, 32 x 40 x 5 1,693 ms.
const int kPrefLagrangeFp64[] = {9, 15, 18, 6, 13, 5, 7};
const int kNumPrefLagrangeFp64 = sizeof(kPrefLagrangeFp64) / sizeof(int);
const int kNumTileCfgs = sizeof(kTileCfgs) / sizeof(kTileCfgs[0]);

// ----------------------------------------------------------------------------------------
// Upload helpers
// ----------------------------------------------------------------------------------------
template <class T>
static int upload_on(cudaStream_t st, DevBuf& buf, const std::vector<T>& v) {
  if (v.empty()) return 0;
  BGB_CUDA(cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  return 0;
}

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

// Longest edge and largest vertex-to-centroid distance of a space, in one pass.
SpaceExtents space_extents(const bgb_space* s) {
  double me = 0.0, mc = 0.0;
  for (int64_t t = 0; t < s->nt; ++t) {
    const double* v[3];
    for (int a = 0; a < 3; ++a) v[a] = s->vertices + 3 * (int64_t)s->triangles[3 * t + a];
    double c[3];
    for (int k = 0; k < 3; ++k) c[k] = (v[0][k] + v[1][k] + v[2][k]) / 3.0;
    for (int a = 0; a < 3; ++a) {
      const double* q = v[(a + 1) % 3];
      double e2 = 0.0, d2 = 0.0;
      for (int k = 0; k < 3; ++k) {
        e2 += (v[a][k] - q[k]) * (v[a][k] - q[k]);
        d2 += (v[a][k] - c[k]) * (v[a][k] - c[k]);
      }
      me = std::max(me, e2);
      mc = std::max(mc, d2);
    }
  }
  return SpaceExtents{std::sqrt(me), std::sqrt(mc) * (1.0 + 1e-12)};
}

// Largest distance of a vertex from its triangle's centroid: bounds |x - c| for every rule point x.
double max_centroid_radius(const bgb_space* s) {
  double m = 0.0;
  for (int64_t t = 0; t < s->nt; ++t) {
    const double* v[3];
    for (int a = 0; a < 3; ++a) v[a] = s->vertices + 3 * (int64_t)s->triangles[3 * t + a];
    for (int a = 0; a < 3; ++a) {
      double d2 = 0.0;
      for (int c = 0; c < 3; ++c) {
        const double d = v[a][c] - (v[0][c] + v[1][c] + v[2][c]) / 3.0;
        d2 += d * d;
      }
      m = std::max(m, std::sqrt(d2));
    }
  }
  return m * (1.0 + 1e-12);
}

bool df_singular_ok(const OpParams& op, double edge_t, double edge_b) {
  // singular / near pairs have R <= (edge_t + edge_b) * 2 at most; df_sincos covers |k R| < 400
  // the double-float kernel covers the single layers and the Maxwell double layer
  return op.kind <= BGB_OP_MAXWELL3D_DL && op.gamma[0] == 0.0 &&
         std::fabs(op.gamma[1]) * 2.0 * (edge_t + edge_b) < 350.0;
}

int check_mixed_range(const bgb_operator* op, const bgb_space* a, const bgb_space* b) {
  // the mixed far kernels reduce k R0 modulo 2 pi with 2 pi split in three floats, exact for
  // k R0 < 4e5 (2^16 turns)
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (const bgb_space* sp : {a, b})
    for (int64_t v = 0; v < sp->nv; ++v)
      for (int c = 0; c < 3; ++c) {
        lo[c] = std::min(lo[c], sp->vertices[3 * v + c]);
        hi[c] = std::max(hi[c], sp->vertices[3 * v + c]);
      }
  const double diam = std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                                (hi[2] - lo[2]) * (hi[2] - lo[2]));
  const double kd = std::fabs(op->gamma[1]) * diam;
  if (kd > 3e5) {
    set_error("mixed precision covers k times the meshes' diameter up to 3e5 (got %.3g); use BGB_PREC_FP64", kd);
    return BGB_ERR_NOT_SUPPORTED;
  }
  return 0;
}

static int ensure_ring(bgb_handle* h, size_t bytes) {
  if (h->ring && h->ring_bytes >= bytes) return 0;
  if (h->ring) cudaFreeHost(h->ring);
  h->ring = nullptr;
  h->ring_bytes = 0;
  cudaError_t e = cudaHostAlloc(&h->ring, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    h->ring = nullptr;
    return cuda_fail(e, "cudaHostAlloc(pinned ring)");
  }
  h->ring_bytes = bytes;
  return 0;
}

// Copy ncols column segments (seg bytes each) from a contiguous source into a strided
// destination, split over host threads (by byte ranges when both sides are contiguous).
static void parallel_copy_columns(char* dst, size_t dpitch, const char* src, size_t spitch, size_t seg, int64_t ncols) {
  const int64_t total = (int64_t)seg * ncols;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nth = (int)std::min<int64_t>(std::min<unsigned>(16u, hw), std::max<int64_t>(1, total / ((int64_t)16 << 20)));
  const bool contiguous = dpitch == seg && spitch == seg;
  auto work = [&](int t) {
    if (contiguous) {
      const int64_t b0 = total * t / nth, b1 = total * (t + 1) / nth;
      std::memcpy(dst + b0, src + b0, (size_t)(b1 - b0));
      return;
    }
    const int64_t c0 = ncols * t / nth, c1 = ncols * (t + 1) / nth;
    for (int64_t c = c0; c < c1; ++c) std::memcpy(dst + (size_t)c * dpitch, src + (size_t)c * spitch, seg);
  };
  if (nth == 1) {
    work(0);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 1; t < nth; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& x : th) x.join();
}

// Fault in the pages of [p, p + n) that are not resident (mincore) by writing one byte inside
// the range per page, in host threads.  The range belongs to the output being assembled.
static void prefault_range(char* p, size_t n, int nth) {
  if (n == 0) return;
  static const size_t page = (size_t)sysconf(_SC_PAGESIZE);
  const uintptr_t a = (uintptr_t)p & ~(uintptr_t)(page - 1);
  const size_t len = (((uintptr_t)p + n - a) + page - 1) & ~(page - 1);
  const size_t np = len / page;
  std::vector<unsigned char> vec(np);
  const bool have = mincore((void*)a, len, vec.data()) == 0;
  if (have) {
    bool all = true;
    for (unsigned char v : vec) all = all && (v & 1);
    if (all) return;
  }
  nth = (int)std::max<size_t>(1, std::min<size_t>((size_t)nth, np / 64));
  auto work = [&](int t) {
    for (size_t k = np * t / nth; k < np * (t + 1) / nth; ++k) {
      if (have && (vec[k] & 1)) continue;
      char* q = std::max(p, (char*)(a + k * page));
      *(volatile char*)q = 0;
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nth; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& x : th) x.join();
}

// Progress of the host thread that faults in the pages of the output blocks in order.
struct PrefaultProgress {
  std::mutex m;
  std::condition_variable cv;
  int done = 0;
  std::atomic<bool> stop{false};
  void advance() {
    { std::lock_guard<std::mutex> g(m); ++done; }
    cv.notify_all();
  }
  void wait_for(int blocks) {
    std::unique_lock<std::mutex> g(m);
    cv.wait(g, [&] { return done >= blocks; });
  }
};

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
  if ((rc = h->bnd_c.ensure(sizeof(float4) * std::max(1, (nb + 31) / 32)))) return rc;
  if ((rc = h->cls_count.ensure(sizeof(int) * (size_t)(nt + 1)))) return rc;
  if ((rc = h->cls_off.ensure(sizeof(int64_t) * (size_t)(nt + 1)))) return rc;
  if ((rc = h->err.ensure(sizeof(int) * 4))) return rc;
  BGB_CUDA(cudaMemsetAsync(h->err.p, 0, sizeof(int) * 4, h->stream));
  launch_prepare_bounds(gt, nt, k2, 0, h->bnd_t.as<float4>(), h->stream);
  launch_prepare_bounds(gb, nb, k2, 1, h->bnd_b.as<float4>(), h->stream);
  launch_chunk_bounds(h->bnd_b.as<float4>(), nb, h->bnd_c.as<float4>(), h->stream);
  launch_classify(false, h->bnd_t.as<float4>(), h->bnd_b.as<float4>(), gt, gb, nt, nb, k2, h->cls_count.as<int>(),
                  nullptr, nullptr, nullptr, nullptr, h->err.as<int>(), h->num_sms, h->stream, nullptr,
                  h->bnd_c.as<float4>());
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
                  h->err.as<int>(), h->num_sms, h->stream, h->ent_mask.as<int16_t>(), h->bnd_c.as<float4>());
  BGB_CUDA(cudaGetLastError());
  *total = tot;
  return 0;
}

__global__ void k_publish(const int* __restrict__ src, int n, volatile int* dst) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
  __threadfence_system();
}

void launch_publish(const int* src, int n, int* mbox_dev, cudaStream_t st) {
  if (n > 0) k_publish<<<1, 64, 0, st>>>(src, n, mbox_dev);
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
      (e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&h->stream_sing, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&h->stream_up, cudaStreamNonBlocking)) != cudaSuccess) {
    rc = cuda_fail(e, "cudaStreamCreate");
  }
  for (int i = 0; i < 8 && !rc; ++i)
    if ((e = cudaEventCreate(&h->ev[i])) != cudaSuccess) rc = cuda_fail(e, "cudaEventCreate");
  for (int i = 0; i < 4 * bgb_handle::kSlots && !rc; ++i)
    if ((e = cudaEventCreate(&h->ev2[i])) != cudaSuccess) rc = cuda_fail(e, "cudaEventCreate");
  for (int i = 0; i < 2 && !rc; ++i)
    if ((e = cudaEventCreateWithFlags(&h->ring_ev[i], cudaEventDisableTiming)) != cudaSuccess) rc = cuda_fail(e, "cudaEventCreate");
  for (int i = 0; i <= bgb_handle::kSlots && !rc; ++i)
    if ((e = cudaEventCreateWithFlags(&h->ev_up[i], cudaEventDisableTiming)) != cudaSuccess) rc = cuda_fail(e, "cudaEventCreate");
  if (!rc) {
    // the abort flag and, 64 bytes further, the mailbox
    int* p = nullptr;
    if ((e = cudaHostAlloc((void**)&p, sizeof(int) * (16 + bgb_handle::kMbox), cudaHostAllocMapped)) != cudaSuccess)
      rc = cuda_fail(e, "cudaHostAlloc");
    else {
      std::memset(p, 0, sizeof(int) * (16 + bgb_handle::kMbox));
      h->abort_host = p;
      h->mbox_host = p + 16;
      if ((e = cudaHostGetDevicePointer((void**)&h->abort_dev, p, 0)) != cudaSuccess) rc = cuda_fail(e, "cudaHostGetDevicePointer");
      else h->mbox_dev = h->abort_dev + 16;
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
  if (h->stream2) cudaStreamSynchronize(h->stream2);
  if (h->stream_sing) cudaStreamSynchronize(h->stream_sing);
  if (h->stream_up) cudaStreamSynchronize(h->stream_up);
  DevBuf* bufs[] = {&h->verts_t, &h->tris_t, &h->verts_b, &h->tris_b, &h->geo_t, &h->geo_b, &h->bnd_t, &h->bnd_b, &h->bnd_c,
                    &h->rec_t, &h->rec_b, &h->cls_count, &h->cls_off, &h->ent_tau, &h->ent_sigma, &h->ent_cls, &h->ent_mask, &h->geodf_t, &h->geodf_b,
                    &h->sing_L, &h->err, &h->df_tab, &h->tplan_i, &h->tplan_l, &h->tplan_d, &h->tplan_f,
                    &h->diag_a, &h->diag_b, &h->diag_c, &h->diag_d, &h->grp_tri, &h->grp_cnt, &h->grp_off, &h->grp_perm, &h->cls_hist};
  for (DevBuf* b : bufs) b->release();
  h->curve.release();
  for (int k = 0; k < bgb_handle::kSlots; ++k) {
    DevBuf* slot_bufs[] = {&h->plan_i[k], &h->plan_l[k], &h->plan_d[k], &h->plan_f[k], &h->far_const[k],
                           &h->stage[k]};
    for (DevBuf* b : slot_bufs) b->release();
  }
  for (int i = 0; i < 8; ++i)
    if (h->ev[i]) cudaEventDestroy(h->ev[i]);
  for (int i = 0; i < 4 * bgb_handle::kSlots; ++i)
    if (h->ev2[i]) cudaEventDestroy(h->ev2[i]);
  for (cudaEvent_t x : h->grp_ev) cudaEventDestroy(x);
  for (int i = 0; i <= bgb_handle::kSlots; ++i)
    if (h->ev_up[i]) cudaEventDestroy(h->ev_up[i]);
  for (int i = 0; i < 2; ++i)
    if (h->ring_ev[i]) cudaEventDestroy(h->ring_ev[i]);
  if (h->ring) cudaFreeHost(h->ring);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  if (h->stream2) cudaStreamDestroy(h->stream2);
  if (h->stream_sing) cudaStreamDestroy(h->stream_sing);
  if (h->stream_up) cudaStreamDestroy(h->stream_up);
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

int bgb_plan_order(const bgb_space* s, int32_t f_begin, int32_t f_end, int32_t width, int32_t* order,
                   int64_t* slots) {
  int rc;
  if (!s || !order || !slots || width < 1) { set_error("bgb_plan_order: invalid argument"); return BGB_ERR_INVALID; }
  if ((rc = validate_space(s, "space"))) return rc;
  if (f_begin < 0 || f_end < f_begin || f_end > s->nfun) {
    set_error("bgb_plan_order: function range [%d, %d) outside [0, %d)", f_begin, f_end, s->nfun);
    return BGB_ERR_INVALID;
  }
  const Supports S = build_supports(s);
  const std::vector<int> ord = order_functions(S, function_centres(s, S), f_begin, f_end, width, planner_threads());
  HostPlan P;
  plan_test_side(S, ord, width, 0, P);
  std::copy(ord.begin(), ord.end(), order);
  *slots = (int64_t)P.tb_tris.size();
  return 0;
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
  if (precision == BGB_PREC_MIXED && (rc = check_mixed_range(op, test, trial))) return rc;
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
  FarConst K = make_farconst(opp, R, qsel, test, trial);
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
  SpaceExtents ext_t{}, ext_b{};
  const FarConst K = make_farconst(opp, R, qsel, test, trial, &ext_t, &ext_b);
  const int gen = far_generic_q(K.qt, K.qb);
  const bool same = same_space(test, trial);
  const int64_t ncols = trial->nfun;

  // Output blocks.  A device output is one block.  A host output is produced in blocks of
  // columns (trial functions): the output is column-major, so each block is one contiguous
  // range of the host matrix (when ld == nrows) and its copy one linear DMA.  Blocks are sized
  // to the HBM budget with two device staging buffers, and a large output is cut into about
  // 16 blocks (of at least 64 MiB) so that every copy but the last overlaps the far kernel of
  // the next block.
  const int64_t per_col = (int64_t)esz * nrows;
  int64_t cols_per_block = ncols;
  if (host_out) {
    size_t freeb = 0, totalb = 0;
    if (h->cfg.hbm_budget_bytes <= 0) cudaMemGetInfo(&freeb, &totalb);
    const int64_t budget = h->cfg.hbm_budget_bytes > 0 ? h->cfg.hbm_budget_bytes : (int64_t)(0.9 * (double)freeb);
    cols_per_block = std::max<int64_t>(1, budget / std::max<int64_t>(1, 4 * per_col));
    const int64_t overlap_cols = std::max<int64_t>((ncols + 15) / 16, ((int64_t)64 << 20) / std::max<int64_t>(1, per_col));
    cols_per_block = std::min(std::min(cols_per_block, overlap_cols), ncols);
  }
  // Block b covers columns [col_start[b], col_start[b + 1]).  With several blocks the first and the
  // last are cut to about a quarter: the copies, which bound the pipeline when they are as fast as
  // the fill, start sooner, and the last copy (the only one not hidden behind a far kernel) is short.
  std::vector<int64_t> col_start;
  for (int64_t c = 0; c < ncols; c += cols_per_block) col_start.push_back(c);
  if (host_out && col_start.size() >= 4) {
    const int64_t quarter = std::max<int64_t>(1, (cols_per_block + 3) / 4);
    col_start.push_back(std::min(quarter, ncols - 1));
    col_start.push_back(std::max<int64_t>(1, ncols - quarter));
    std::sort(col_start.begin(), col_start.end());
    col_start.erase(std::unique(col_start.begin(), col_start.end()), col_start.end());
  }
  col_start.push_back(ncols);
  const int nblocks = (int)col_start.size() - 1;
  st.out_blocks = nblocks;

  // Host tile planning depends on the spaces only: it runs on worker threads while the device
  // uploads, classifies and integrates the singular pairs.
  const bool pinned_cfg = h->cfg.tile_config >= 0;
  if (pinned_cfg && h->cfg.tile_config >= kNumTileCfgs) { set_error("tile_config %d out of range", h->cfg.tile_config); return BGB_ERR_INVALID; }
  std::vector<int> prefs;
  if (pinned_cfg) prefs.push_back(h->cfg.tile_config);
  else if (test->refspace == BGB_REFSPACE_LAGRANGE_C0D1 && precision == BGB_PREC_MIXED)
    prefs.assign(kPrefLagrange, kPrefLagrange + kNumPrefLagrange);
  else if (test->refspace == BGB_REFSPACE_LAGRANGE_C0D1)
    prefs.assign(kPrefLagrangeFp64, kPrefLagrangeFp64 + kNumPrefLagrangeFp64);
  else if (precision == BGB_PREC_MIXED) prefs.assign(kPrefMixed, kPrefMixed + kNumPrefMixed);
  else prefs.assign(kPrefFp64, kPrefFp64 + kNumPrefFp64);
  int smem_max = 0;
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  struct Plans {
    HostPlan test;                 // test side, all rows of the window
    std::vector<HostPlan> trial;   // trial side per output block
    TileCfg tc{};
    int cfg_id = -1;
    size_t smem = 0;
    std::string err;
    double ms = 0;
  } PL;
  const int nth = planner_threads();
  const int target_occ = far_target_ctas_per_sm(precision);
  auto plan_all = [&]() {
    const auto t0 = clk::now();
    cudaSetDevice(h->device);  // occupancy queries from this thread
    const Supports St = build_supports(test);
    const Supports Sb_own = same ? Supports() : build_supports(trial);
    const Supports& Sb = same ? St : Sb_own;
    const std::vector<double> cent_t = function_centres(test, St);
    const std::vector<double> cent_b_own = same ? std::vector<double>() : function_centres(trial, Sb);
    const std::vector<double>& cent_b = same ? cent_t : cent_b_own;
    // function orders in runs of the tile widths (recomputed only when a width changes)
    std::vector<int> ord_t;
    std::vector<std::vector<int>> ord_b(nblocks);
    int ord_fm = -1, ord_fn = -1;
    // per output block: function order and trial-side plan, blocks spread over the planner's threads
    auto over_blocks = [&](auto fn) {
      if (nblocks == 1) {
        fn(0, nth);
        return;
      }
      std::vector<std::thread> th;
      const int nt = std::min(nth, nblocks);
      for (int t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
          for (int b = t; b < nblocks; b += nt) fn(b, 1);
        });
      for (auto& x : th) x.join();
    };
    size_t smem = 0;
    for (int id : prefs) {
      const TileCfg tc = kTileCfgs[id];
      if (tc.FM != ord_fm) {
        ord_t = order_functions(St, cent_t, (int)row0, (int)(row0 + nrows), tc.FM, nth);
        // rows of a tile in ascending order: the tile's output stores of one column then fall in
        // fewer 32-byte sectors (C2: 23 instead of 60 per column)
        for (size_t b = 0; b < ord_t.size(); b += (size_t)tc.FM)
          std::sort(ord_t.begin() + b, ord_t.begin() + std::min(ord_t.size(), b + (size_t)tc.FM));
        ord_fm = tc.FM;
      }
      if (tc.FN != ord_fn) {
        if (same && nblocks == 1 && row0 == 0 && nrows == ncols && tc.FN == tc.FM)
          ord_b[0] = ord_t;  // the same functions and width: the same order
        else
          over_blocks([&](int b, int threads) {
            ord_b[b] = order_functions(Sb, cent_b, (int)col_start[b], (int)col_start[b + 1], tc.FN, threads);
          });
        ord_fn = tc.FN;
      }
      PL.test = HostPlan();
      plan_test_side_par(St, ord_t, tc.FM, row0, PL.test, nth);
      PL.trial.assign(nblocks, HostPlan());
      TilePlan probe{};
      probe.FM = tc.FM; probe.FN = tc.FN; probe.SC = tc.SC; probe.MAXS = PL.test.MAXS;
      probe.tmax = std::max(1, PL.test.tmax);
      over_blocks([&](int b, int threads) { plan_trial_side_par(Sb, ord_b[b], tc.FN, tc.SC, PL.trial[b], threads); });
      for (int b = 0; b < nblocks; ++b) {
        probe.gmax = std::max(probe.gmax, PL.trial[b].gmax);
        probe.gsmax = std::max(probe.gsmax, PL.trial[b].gsmax);
        probe.nmax = std::max(probe.nmax, std::max(1, PL.trial[b].nmax));
      }
      smem = far_smem_bytes(precision, K.op_kind, K.qt, K.qb, probe);
      // Occupancy: when the widest test tile pushes shared memory past what the kernel's
      // CTAs per SM allow, cap the triangles per test tile at the largest count that fits.
      int occ = 0;
      if (smem <= (size_t)smem_max && far_persistent_occupancy(precision, K.op_kind, gen, smem, &occ) == 0 &&
          occ >= 1 && occ < target_occ) {
        int cap = -1;
        for (int t = probe.tmax - 1; t >= std::max(1, PL.test.MAXS); --t) {
          TilePlan q = probe;
          q.tmax = t;
          const size_t sm = far_smem_bytes(precision, K.op_kind, K.qt, K.qb, q);
          int o = 0;
          if (far_persistent_occupancy(precision, K.op_kind, gen, sm, &o) == 0 && o >= target_occ) {
            cap = t;
            break;
          }
        }
        if (cap > 0) {
          PL.test = HostPlan();
          plan_test_side_par(St, ord_t, tc.FM, row0, PL.test, nth, cap);
          probe.MAXS = PL.test.MAXS;
          probe.tmax = std::max(1, PL.test.tmax);
          smem = far_smem_bytes(precision, K.op_kind, K.qt, K.qb, probe);
        }
      }
      occ = 0;
      if (smem <= (size_t)smem_max && far_persistent_occupancy(precision, K.op_kind, gen, smem, &occ) == 0 && occ >= 1) {
        PL.cfg_id = id;
        PL.tc = tc;
        PL.smem = smem;
        break;
      }
    }
    if (PL.cfg_id < 0) {
      char buf[160];
      snprintf(buf, sizeof buf, "no tile configuration fits in %d B of shared memory (last tried needs %zu B)",
               smem_max, smem);
      PL.err = buf;
    }
    PL.ms = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
  };
  struct Joiner {
    std::thread& t;
    ~Joiner() {
      if (t.joinable()) t.join();
    }
  };
  std::thread planner(plan_all);
  Joiner join_planner{planner};

  // Host destination: pinned memory (cudaHostAlloc or registered) is copied into directly, and
  // so is pageable memory when the GPU reaches it through the host page tables (a Grace host),
  // after a host thread has faulted its pages in block by block (a DMA that faults pages runs
  // several times slower than one into resident pages); other pageable memory goes through a
  // pinned ring.
  enum { DST_PINNED, DST_PAGEABLE, DST_RING } dst_kind = DST_PINNED;
  if (host_out) {
    cudaPointerAttributes attr{};
    const bool pinned = cudaPointerGetAttributes(&attr, out) == cudaSuccess && attr.type == cudaMemoryTypeHost;
    cudaGetLastError();
    int ats = 0;
    cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, h->device);
    dst_kind = pinned ? DST_PINNED : (ats && !(h->cfg.flags & BGB_CFG_PAGEABLE_VIA_RING) ? DST_PAGEABLE : DST_RING);
  }
  PrefaultProgress PF;
  std::thread prefaulter;
  if (dst_kind == DST_PAGEABLE) {
    prefaulter = std::thread([&] {
      const int nth = (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
      for (int b = 0; b < nblocks && !PF.stop; ++b) {
        const int64_t c0 = col_start[b], nc = col_start[b + 1] - c0;
        char* base = (char*)out + (size_t)c0 * ld * esz;
        if (ld == nrows) {
          prefault_range(base, (size_t)nc * nrows * esz, nth);
        } else {
          for (int64_t c = 0; c < nc && !PF.stop; ++c) prefault_range(base + (size_t)c * ld * esz, (size_t)nrows * esz, 1);
        }
        PF.advance();
      }
    });
  }
  struct StopJoin {
    PrefaultProgress& pf;
    std::thread& t;
    ~StopJoin() {
      pf.stop = true;
      if (t.joinable()) t.join();
    }
  } join_prefault{PF, prefaulter};

  cudaEventRecord(h->ev[0], h->stream);
  int launches = 0;
  if ((rc = upload_space(h, test, h->verts_t, h->tris_t, h->geo_t))) return rc;
  launches += test->nt > 0;
  const Geo64* gt = h->geo_t.as<Geo64>();
  const Geo64* gb = gt;
  if (!same) {
    if ((rc = upload_space(h, trial, h->verts_b, h->tris_b, h->geo_b))) return rc;
    gb = h->geo_b.as<Geo64>();
    launches += trial->nt > 0;
  }
  // 1. classification
  auto host_ms = [&]() { return std::chrono::duration<double, std::milli>(clk::now() - t_start).count(); };
  double hm[6] = {host_ms(), 0, 0, 0, 0, 0};  // host marks for BGB_TRACE
  int64_t nsing = 0;
  if ((rc = classify_all(h, test, trial, gt, gb, opp.k2, &nsing))) return rc;
  hm[1] = host_ms();
  launches += 6;  // 2 bounds, 2 classify passes, scan (+1 singular below)
  if (stats) {  // entries per class, published to the mailbox (read after the final synchronisation)
    if ((rc = h->cls_hist.ensure(sizeof(unsigned long long) * 5))) return rc;
    launch_class_hist(h->ent_cls.as<int8_t>(), nsing, h->cls_hist.as<unsigned long long>(), h->num_sms, h->stream);
    launch_publish(h->cls_hist.as<int>(), 10, h->mbox_dev, h->stream);
    launches += nsing > 0 ? 2 : 1;
  }
  cudaEventRecord(h->ev[1], h->stream);
  // 2. singular / near pairs: FP64 kernel (plain path), double-float kernel (mixed path)
  if ((rc = h->sing_L.ensure(sizeof(double2) * 9 * std::max<int64_t>(1, nsing)))) return rc;
  const bool use_df = precision == BGB_PREC_MIXED && df_singular_ok(opp, ext_t.max_edge, ext_b.max_edge);
  std::vector<float> df_host;  // uploaded asynchronously: lives until the end of the call
  DfTables M{};
  const GeoDf* dgt = nullptr;
  const GeoDf* dgb = nullptr;
  // the singular kernels over all entries (perm null) or over the entries perm[range[0] .. range[1])
  auto launch_sing = [&](const int* perm, const int64_t* range, cudaStream_t st) {
    if (use_df) {
      launch_singular_df(opp.kind, make_opdf(opp), nullptr, nullptr, M, h->df_tab.as<float>(), dgt, dgb,
                         h->ent_tau.as<int>(), h->ent_sigma.as<int>(), h->ent_cls.as<int8_t>(),
                         h->ent_mask.as<int16_t>(), nsing, h->sing_L.as<double2>(), h->abort_dev, h->num_sms, st, perm,
                         range);
      // near pairs (singularity extraction: logarithms and arctangents) in FP64
      launch_singular(opp, qsel, R, test->refspace, trial->refspace, gt, gb, h->ent_tau.as<int>(),
                      h->ent_sigma.as<int>(), h->ent_cls.as<int8_t>(), nsing, h->sing_L.as<double2>(), h->abort_dev,
                      h->num_sms, st, true, perm, range);
      return 2;
    }
    launch_singular(opp, qsel, R, test->refspace, trial->refspace, gt, gb, h->ent_tau.as<int>(), h->ent_sigma.as<int>(),
                    h->ent_cls.as<int8_t>(), nsing, h->sing_L.as<double2>(), h->abort_dev, h->num_sms, st, false, perm,
                    range);
    return 1;
  };
  // A host output in several blocks integrates its singular entries in groups on a stream of their
  // own: group b holds the entries whose trial triangle first appears in block b, the groups run in
  // block order from the end of the classification on (while the host still plans the tiles), and
  // block b's far kernel waits for group b only.  Block 0's far kernel and copy then start after a
  // fraction of the singular stage instead of all of it.
  const bool grouped = host_out && nblocks > 1 && nsing > 0;
  std::vector<int> tri_group;  // uploaded asynchronously: lives until the end of the call
  if (grouped) {
    tri_group.assign((size_t)std::max(1, trial->nt), nblocks - 1);
    for (int t = 0; t < trial->nt; ++t)
      for (int i = 0; i < 3; ++i) {
        const int f = trial->fn_index[3 * t + i];
        if (f < 0) continue;
        const int g = (int)(std::upper_bound(col_start.begin(), col_start.end(), (int64_t)f) - col_start.begin()) - 1;
        tri_group[(size_t)t] = std::min(tri_group[(size_t)t], std::max(0, g));
      }
    if ((rc = h->grp_tri.ensure(sizeof(int) * tri_group.size())) || (rc = h->grp_cnt.ensure(sizeof(int) * nblocks)) ||
        (rc = h->grp_off.ensure(sizeof(int64_t) * (nblocks + 1))) || (rc = h->grp_perm.ensure(sizeof(int) * nsing)))
      return rc;
    if ((rc = upload(h, h->grp_tri, tri_group, 0))) return rc;
    launch_group_entries(h->ent_sigma.as<int>(), nsing, h->grp_tri.as<int>(), nblocks, h->grp_cnt.as<int>(),
                         h->grp_off.as<int64_t>(), h->grp_perm.as<int>(), h->num_sms, h->stream);
    launches += 3;
    while ((int)h->grp_ev.size() < nblocks) {
      cudaEvent_t x = nullptr;
      BGB_CUDA(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
      h->grp_ev.push_back(x);
    }
  }
  if (use_df) {
    build_df_tables(qsel, R, df_host, M);
    if ((rc = h->df_tab.ensure(sizeof(float) * df_host.size()))) return rc;
    BGB_CUDA(cudaMemcpyAsync(h->df_tab.p, df_host.data(), sizeof(float) * df_host.size(), cudaMemcpyHostToDevice, h->stream));
    if ((rc = h->geodf_t.ensure(sizeof(GeoDf) * std::max(1, test->nt))) ||
        (!same && (rc = h->geodf_b.ensure(sizeof(GeoDf) * std::max(1, trial->nt)))))
      return rc;
    launch_prepare_geodf(gt, test->nt, h->geodf_t.as<GeoDf>(), h->stream);
    if (!same) launch_prepare_geodf(gb, trial->nt, h->geodf_b.as<GeoDf>(), h->stream);
    dgt = h->geodf_t.as<GeoDf>();
    dgb = same ? dgt : h->geodf_b.as<GeoDf>();
    launches += 1 + (same ? 0 : 1);
  }
  struct SyncOnExit {  // singular groups still in flight when the call returns early
    cudaStream_t st;
    ~SyncOnExit() {
      if (st) cudaStreamSynchronize(st);
    }
  } sync_sing{grouped ? h->stream_sing : nullptr};
  if (grouped) {
    BGB_CUDA(cudaEventRecord(h->ev[4], h->stream));
    BGB_CUDA(cudaStreamWaitEvent(h->stream_sing, h->ev[4], 0));
    for (int b = 0; b < nblocks; ++b) {
      launches += launch_sing(h->grp_perm.as<int>(), h->grp_off.as<int64_t>() + b, h->stream_sing);
      BGB_CUDA(cudaEventRecord(h->grp_ev[(size_t)b], h->stream_sing));
    }
    BGB_CUDA(cudaEventRecord(h->ev[5], h->stream_sing));
  } else {
    launches += launch_sing(nullptr, nullptr, h->stream);
  }
  BGB_CUDA(cudaGetLastError());
  cudaEventRecord(h->ev[2], h->stream);
  hm[2] = host_ms();
  // 3. far-pair records
  const int rst = rec_stride(precision, K.qt, gen), rsb = rec_stride(precision, K.qb, gen);
  const size_t rsz = precision == BGB_PREC_MIXED ? sizeof(float) : sizeof(double);
  if ((rc = h->rec_t.ensure(rsz * rst * std::max(1, test->nt))) || (rc = h->rec_b.ensure(rsz * rsb * std::max(1, trial->nt))))
    return rc;
  launch_prepare_rec(precision, 0, gen ? BGB_MAXQ : K.qt, gt, test->nt, R, qsel.far_t, 1.0, h->rec_t.p, h->stream);
  launch_prepare_rec(precision, 1, gen ? BGB_MAXQ : K.qb, gb, trial->nt, R, qsel.far_b, BGB_INV_4PI_D, h->rec_b.p, h->stream);
  launches += 2;

  // 4. the host plan (joined here) and the test-side tables, uploaded once
  planner.join();
  hm[3] = host_ms();
  st.ms_plan = PL.ms;
  if (PL.cfg_id < 0) {
    cudaStreamSynchronize(h->stream);
    set_error("%s", PL.err.c_str());
    return BGB_ERR_CAPACITY;
  }
  st.tile_config = PL.cfg_id;
  const TileCfg tc = PL.tc;
  const size_t smem = PL.smem;
  const HostPlan& PT = PL.test;
  std::vector<int> TI;
  std::vector<float> TF;
  auto cat_i = [&](std::vector<int>& dst, const std::vector<int>& v) { size_t o = dst.size(); dst.insert(dst.end(), v.begin(), v.end()); return o; };
  const size_t o_tb_off = cat_i(TI, PT.tb_off), o_tb_tris = cat_i(TI, PT.tb_tris), o_tb_fn = cat_i(TI, PT.tb_fn_off),
               o_fs_off = cat_i(TI, PT.fs_off), o_fs_code = cat_i(TI, PT.fs_code);
  TF.reserve(PT.fs_coef.size());
  for (double v : PT.fs_coef) TF.push_back((float)v);
  if ((rc = h->tplan_i.ensure(sizeof(int) * std::max<size_t>(1, TI.size()))) ||
      (rc = h->tplan_l.ensure(sizeof(int64_t) * std::max<size_t>(1, PT.rows.size()))) ||
      (rc = h->tplan_d.ensure(sizeof(double) * std::max<size_t>(1, PT.fs_coef.size()))) ||
      (rc = h->tplan_f.ensure(sizeof(float) * std::max<size_t>(1, TF.size()))))
    return rc;
  // uploads on their own stream: a pageable upload queued behind the singular kernels would hold
  // the host until they end
  if ((rc = upload_on(h->stream_up, h->tplan_i, TI)) || (rc = upload_on(h->stream_up, h->tplan_l, PT.rows)) ||
      (rc = upload_on(h->stream_up, h->tplan_d, PT.fs_coef)) || (rc = upload_on(h->stream_up, h->tplan_f, TF)))
    return rc;
  BGB_CUDA(cudaEventRecord(h->ev_up[bgb_handle::kSlots], h->stream_up));
  int per_sm = 0;
  if ((rc = far_persistent_occupancy(precision, K.op_kind, gen, smem, &per_sm))) return rc;
  const int ntb = (int)PT.tb_off.size() - 1;

  double ms_far = 0, ms_copy = 0;
  int64_t pairs_computed = 0;
  constexpr int NS = bgb_handle::kSlots;
  bool pending[NS] = {};
  // BGB_TRACE set: one line per output block on stderr (far kernel and copy in ms from the call's
  // first event, host time spent enqueueing the block)
  const bool trace = std::getenv("BGB_TRACE") != nullptr;
  int slot_block[NS] = {};
  std::vector<double> enq_ms((size_t)nblocks, 0.0);
  auto harvest = [&](int slot) {  // times of the block that last used `slot` (complete)
    if (!pending[slot]) return;
    ms_far += event_ms(h->ev2[slot * 4 + 0], h->ev2[slot * 4 + 1]);
    if (host_out) ms_copy += event_ms(h->ev2[slot * 4 + 2], h->ev2[slot * 4 + 3]);
    if (trace)
      fprintf(stderr, "bgb trace block %d: far %.3f .. %.3f  copy %.3f .. %.3f  enqueue %.3f ms\n", slot_block[slot],
              event_ms(h->ev[0], h->ev2[slot * 4 + 0]), event_ms(h->ev[0], h->ev2[slot * 4 + 1]),
              host_out ? event_ms(h->ev[0], h->ev2[slot * 4 + 2]) : 0.0,
              host_out ? event_ms(h->ev[0], h->ev2[slot * 4 + 3]) : 0.0, enq_ms[(size_t)slot_block[slot]]);
    pending[slot] = false;
  };
  struct SlotHost {  // host copies of a block's tables, alive until the slot is reused
    std::vector<int> I;
    std::vector<int64_t> L;
    std::vector<float> F;
    TilePlan T;
  };
  SlotHost slot_host[NS];
  // upload the trial-side tables of block b into its slot and launch the far kernel
  auto enqueue_block = [&](int b) -> int {
    const auto t_enq = clk::now();
    const int slot = b % NS;
    cudaStream_t cst = (b & 1) ? h->stream2 : h->stream;  // consecutive blocks alternate compute streams
    const int64_t c0 = col_start[b];
    const int64_t nc = col_start[b + 1] - c0;
    const HostPlan& PB = PL.trial[b];
    if (pending[slot]) {  // block b - NS used this slot: its kernel and copy must be complete
      BGB_CUDA(cudaEventSynchronize(h->ev2[slot * 4 + (host_out ? 3 : 1)]));
      harvest(slot);
    }
    SlotHost& H = slot_host[slot];
    H.I.clear();
    H.L.clear();
    H.F.clear();
    const size_t o_bb_off = cat_i(H.I, PB.bb_off), o_bb_tris = cat_i(H.I, PB.bb_tris), o_bb_fn = cat_i(H.I, PB.bb_fn_off),
                 o_bb_ch = cat_i(H.I, PB.bb_chunk_off), o_ch_grp = cat_i(H.I, PB.ch_grp_off),
                 o_grp_fn = cat_i(H.I, PB.grp_fn), o_grp_sup = cat_i(H.I, PB.grp_sup_off),
                 o_gs_code = cat_i(H.I, PB.gs_code);
    H.L.reserve(PB.cols.size());
    for (int64_t c : PB.cols) H.L.push_back(c - (host_out ? c0 : 0));  // staging columns start at c0
    H.F.reserve(PB.gs_coef.size());
    for (double v : PB.gs_coef) H.F.push_back((float)v);
    const size_t o_gs_coef = 0;
    pairs_computed += (int64_t)PT.tb_tris.size() * (int64_t)PB.bb_tris.size();
    const int nbb = (int)PB.bb_off.size() - 1;
    // tiles t = bn * ntb + bm (row block fastest: neighbouring rows of a column together); the
    // kernel derives (bm, bn) from t, no item list
    const int64_t ntiles = (int64_t)ntb * nbb;
    int rc2;
    if ((rc2 = h->plan_i[slot].ensure(sizeof(int) * std::max<size_t>(1, H.I.size()))) ||
        (rc2 = h->plan_l[slot].ensure(sizeof(int64_t) * std::max<size_t>(1, H.L.size()))) ||
        (rc2 = h->plan_d[slot].ensure(sizeof(double) * std::max<size_t>(1, PB.gs_coef.size()))) ||
        (rc2 = h->plan_f[slot].ensure(sizeof(float) * std::max<size_t>(1, H.F.size()))) ||
        (rc2 = h->far_const[slot].ensure(sizeof(FarConst) + sizeof(TilePlan) + sizeof(int) * 4)))
      return rc2;
    if (ntiles > INT32_MAX) {
      set_error("%lld tiles in one output block", (long long)ntiles);
      return BGB_ERR_CAPACITY;
    }
    if (host_out && (rc2 = h->stage[slot].ensure(esz * (size_t)cols_per_block * nrows))) return rc2;
    cudaStream_t up = h->stream_up;
    if ((rc2 = upload_on(up, h->plan_i[slot], H.I)) || (rc2 = upload_on(up, h->plan_l[slot], H.L)) ||
        (rc2 = upload_on(up, h->plan_d[slot], PB.gs_coef)) || (rc2 = upload_on(up, h->plan_f[slot], H.F)))
      return rc2;
    const int* ti = h->tplan_i.as<int>();
    const int* bi = h->plan_i[slot].as<int>();
    TilePlan& T = H.T;
    T = TilePlan{};
    T.rec_t = h->rec_t.p;
    T.rec_b = h->rec_b.p;
    T.bnd_t = h->bnd_t.as<float4>();
    T.bnd_b = h->bnd_b.as<float4>();
    T.n_tblocks = ntb;
    T.tb_off = ti + o_tb_off;
    T.tb_tris = ti + o_tb_tris;
    T.tb_fn_off = ti + o_tb_fn;
    T.fs_off = ti + o_fs_off;
    T.fs_code = ti + o_fs_code;
    T.fs_coef = h->tplan_d.as<double>();
    T.fs_coef32 = h->tplan_f.as<float>();
    T.rows = h->tplan_l.as<int64_t>();
    T.n_bblocks = nbb;
    T.bb_off = bi + o_bb_off;
    T.bb_tris = bi + o_bb_tris;
    T.bb_fn_off = bi + o_bb_fn;
    T.bb_chunk_off = bi + o_bb_ch;
    T.ch_grp_off = bi + o_ch_grp;
    T.grp_fn = bi + o_grp_fn;
    T.grp_sup_off = bi + o_grp_sup;
    T.gs_code = bi + o_gs_code;
    T.gs_coef = h->plan_d[slot].as<double>() + o_gs_coef;
    T.gs_coef32 = h->plan_f[slot].as<float>();
    T.cols = h->plan_l[slot].as<int64_t>();
    T.gmax = PB.gmax;
    T.gsmax = PB.gsmax;
    T.sing_off = h->cls_off.as<int64_t>();
    T.sing_sigma = h->ent_sigma.as<int>();
    T.sing_L = h->sing_L.as<double2>();
    T.FM = tc.FM;
    T.FN = tc.FN;
    T.SC = tc.SC;
    T.MAXS = PT.MAXS;
    T.tmax = std::max(1, PT.tmax);
    T.nmax = std::max(1, PB.nmax);
    T.out_c64 = c64;
    T.abort_flag = h->abort_dev;
    T.out = host_out ? h->stage[slot].p : out;
    T.ld = host_out ? nrows : ld;
    FarConst* dK = (FarConst*)h->far_const[slot].p;
    TilePlan* dT = (TilePlan*)((char*)h->far_const[slot].p + sizeof(FarConst));
    int* dctr = (int*)((char*)h->far_const[slot].p + sizeof(FarConst) + sizeof(TilePlan));
    BGB_CUDA(cudaMemcpyAsync(dK, &K, sizeof(FarConst), cudaMemcpyHostToDevice, up));
    BGB_CUDA(cudaMemcpyAsync(dT, &T, sizeof(TilePlan), cudaMemcpyHostToDevice, up));
    BGB_CUDA(cudaMemsetAsync(dctr, 0, sizeof(int), up));
    BGB_CUDA(cudaEventRecord(h->ev_up[slot], up));
    BGB_CUDA(cudaStreamWaitEvent(cst, h->ev_up[slot], 0));
    BGB_CUDA(cudaStreamWaitEvent(cst, h->ev_up[NS], 0));  // test-side tables
    const int ctas = (int)std::min<int64_t>(ntiles, (int64_t)std::max(1, per_sm) * h->num_sms);
    if (grouped) BGB_CUDA(cudaStreamWaitEvent(cst, h->grp_ev[(size_t)b], 0));  // singular groups 0 .. b
    BGB_CUDA(cudaEventRecord(h->ev2[slot * 4 + 0], cst));
    if ((rc2 = launch_far_persistent(precision, K.op_kind, gen, dK, dT, nullptr, (int)ntiles, dctr, smem,
                                     std::max(1, ctas), h->abort_dev, cst)))
      return rc2;
    ++launches;
    BGB_CUDA(cudaEventRecord(h->ev2[slot * 4 + 1], cst));
    pending[slot] = true;
    slot_block[slot] = b;
    enq_ms[(size_t)b] = std::chrono::duration<double, std::milli>(clk::now() - t_enq).count();
    (void)nc;
    return 0;
  };
  // copy block b to the host on the side stream; pageable destinations go through the pinned ring
  auto copy_block = [&](int b) -> int {
    const int slot = b % NS;
    const int64_t c0 = col_start[b];
    const int64_t nc = col_start[b + 1] - c0;
    cudaStream_t cs = h->copy_stream;
    if (dst_kind == DST_PAGEABLE) PF.wait_for(b + 1);  // pages of this block are resident
    BGB_CUDA(cudaStreamWaitEvent(cs, h->ev2[slot * 4 + 1], 0));
    BGB_CUDA(cudaEventRecord(h->ev2[slot * 4 + 2], cs));
    char* hdst = (char*)out + (size_t)c0 * ld * esz;
    const char* src = (const char*)h->stage[slot].p;
    const size_t seg = (size_t)nrows * esz;  // one column of the block
    const size_t dpitch = (size_t)ld * esz;
    if (dst_kind != DST_RING) {
      if (dpitch == seg)
        BGB_CUDA(cudaMemcpyAsync(hdst, src, seg * nc, cudaMemcpyDeviceToHost, cs));
      else
        BGB_CUDA(cudaMemcpy2DAsync(hdst, dpitch, src, seg, seg, (size_t)nc, cudaMemcpyDeviceToHost, cs));
    } else {
      int rc2;
      const size_t ring_half =
          std::max(seg, (size_t)(h->cfg.pinned_ring_bytes > 0 ? h->cfg.pinned_ring_bytes : ((int64_t)512 << 20)));
      if ((rc2 = ensure_ring(h, 2 * ring_half))) return rc2;
      const int64_t cols_per_chunk = std::max<int64_t>(1, (int64_t)(ring_half / seg));
      const int64_t nchunks = (nc + cols_per_chunk - 1) / cols_per_chunk;
      auto host_copy = [&](int64_t k) {
        const int64_t k0 = k * cols_per_chunk, kn = std::min(cols_per_chunk, nc - k0);
        const char* r = (const char*)h->ring + (size_t)(k & 1) * ring_half;
        parallel_copy_columns(hdst + (size_t)k0 * dpitch, dpitch, r, seg, seg, kn);
      };
      for (int64_t k = 0; k < nchunks; ++k) {
        const int64_t k0 = k * cols_per_chunk, kn = std::min(cols_per_chunk, nc - k0);
        BGB_CUDA(cudaMemcpyAsync((char*)h->ring + (size_t)(k & 1) * ring_half, src + (size_t)k0 * seg, seg * kn,
                                 cudaMemcpyDeviceToHost, cs));
        BGB_CUDA(cudaEventRecord(h->ring_ev[k & 1], cs));
        if (k > 0) {  // copy out the previous chunk while this one is in flight
          BGB_CUDA(cudaEventSynchronize(h->ring_ev[(k - 1) & 1]));
          host_copy(k - 1);
        }
      }
      BGB_CUDA(cudaEventSynchronize(h->ring_ev[(nchunks - 1) & 1]));
      host_copy(nchunks - 1);
    }
    BGB_CUDA(cudaEventRecord(h->ev2[slot * 4 + 3], cs));
    return 0;
  };
  hm[4] = host_ms();
  const auto t_pipe = clk::now();
  // the second compute stream starts after everything enqueued so far (classification, singular
  // pairs, records, test-side tables)
  BGB_CUDA(cudaEventRecord(h->ev[3], h->stream));
  BGB_CUDA(cudaStreamWaitEvent(h->stream2, h->ev[3], 0));
  auto drain = [&](int code) {  // the slots' host tables must outlive uploads still in flight
    cudaStreamSynchronize(h->stream);
    cudaStreamSynchronize(h->stream2);
    cudaStreamSynchronize(h->stream_sing);
    cudaStreamSynchronize(h->stream_up);
    cudaStreamSynchronize(h->copy_stream);
    return code;
  };
  if ((rc = enqueue_block(0))) return drain(rc);
  for (int b = 0; b < nblocks; ++b) {
    if (b + 1 < nblocks && (rc = enqueue_block(b + 1))) return drain(rc);
    if (host_out && (rc = copy_block(b))) return drain(rc);
    if ((rc = check_abort(h))) return drain(rc);
  }
  BGB_CUDA(cudaStreamSynchronize(h->stream));
  BGB_CUDA(cudaStreamSynchronize(h->stream2));
  BGB_CUDA(cudaStreamSynchronize(h->stream_sing));
  BGB_CUDA(cudaStreamSynchronize(h->stream_up));
  BGB_CUDA(cudaStreamSynchronize(h->copy_stream));
  for (int k = 0; k < NS; ++k) harvest(k);
  const double ms_pipe = std::chrono::duration<double, std::milli>(clk::now() - t_pipe).count();
  if ((rc = check_abort(h))) return rc;
  st.ms_copy = ms_copy;
  st.ms_pipeline = ms_pipe;
  BGB_CUDA(cudaGetLastError());
  if (!host_out && s != h->stream) {
    BGB_CUDA(cudaEventRecord(h->ev[6], h->stream));
    BGB_CUDA(cudaStreamWaitEvent(s, h->ev[6], 0));
  }
  // statistics
  st.pairs_total = (int64_t)test->nt * trial->nt;
  st.pairs_computed = pairs_computed;
  st.ms_classify = event_ms(h->ev[0], h->ev[1]);
  if (trace)
    fprintf(stderr, "bgb trace host: upload %.3f classified %.3f singular enqueued %.3f planner joined %.3f tables %.3f ms\n",
            hm[0], hm[1], hm[2], hm[3], hm[4]);
  if (trace)
    fprintf(stderr, "bgb trace: classify end %.3f, singular end %.3f, pipeline start %.3f (host) ms\n",
            event_ms(h->ev[0], h->ev[1]), event_ms(h->ev[0], grouped ? h->ev[5] : h->ev[2]),
            std::chrono::duration<double, std::milli>(t_pipe - t_start).count());
  // grouped: the classification-side preparation plus the span of the groups (beside far kernels)
  st.ms_singular = event_ms(h->ev[1], h->ev[2]) + (grouped ? event_ms(h->ev[4], h->ev[5]) : 0.0);
  st.ms_far = ms_far;
  if (stats) {
    for (int c = 1; c < 5; ++c)
      st.pairs_class[c] = (int64_t)(((uint64_t)(uint32_t)h->mbox_host[2 * c + 1] << 32) | (uint32_t)h->mbox_host[2 * c]);
    st.pairs_class[0] = st.pairs_total - nsing;
  }
  st.ms_total = std::chrono::duration<double, std::milli>(clk::now() - t_start).count();
  st.kernel_launches = launches;
  if (stats) *stats = st;
  return 0;
}

}  // extern "C"
