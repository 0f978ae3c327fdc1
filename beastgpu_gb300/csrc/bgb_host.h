// Host-side declarations shared by the C-ABI translation units (handle, buffers, planning).
#pragma once

#include "bgb_kernels.cuh"

#include <mutex>
#include <vector>

namespace bgb {

// ----------------------------------------------------------------------------------------
// Device buffers (grow-only, owned by the handle)
// ----------------------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap && p) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      return cuda_fail(e, "cudaMalloc");
    }
    cap = want;
    return 0;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* as() const { return (T*)p; }
};

// Scratch of the curve (2-D) path.
struct CurveBufs {
  DevBuf verts_t, segs_t, geo_t, geof_t, verts_b, segs_b, geo_b, geof_b, rules, rulesdf, L, list, counts, mask, tsup_i,
      tsup_c, tsup_off, bsup_i, bsup_c, bsup_off, T, S, own, pairs, out, stage, stage2;
  void release() {
    DevBuf* all[] = {&verts_t, &segs_t, &geo_t, &geof_t, &verts_b, &segs_b, &geo_b, &geof_b, &rules, &rulesdf, &L, &list,
                     &counts,
                     &mask, &tsup_i, &tsup_c, &tsup_off, &bsup_i, &bsup_c, &bsup_off, &T, &S, &own, &pairs, &out, &stage,
                     &stage2};
    for (DevBuf* b : all) b->release();
  }
};

}  // namespace bgb

struct bgb_handle {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;
  cudaStream_t stream2 = nullptr;  // second compute stream: consecutive output blocks alternate, so one
                                   // block's far kernel starts while the previous one drains
  bgb_config cfg{};
  volatile int* abort_host = nullptr;
  int* abort_dev = nullptr;
  // small counts that kernels publish to the host (mapped pinned memory, beside the abort flag): a
  // device-to-host copy of a few bytes would queue behind an output block's copy on the copy engine
  volatile int* mbox_host = nullptr;
  int* mbox_dev = nullptr;
  static constexpr int kMbox = 64;
  std::mutex mu;
  // buffers
  bgb::DevBuf verts_t, tris_t, verts_b, tris_b, geo_t, geo_b, bnd_t, bnd_b, bnd_c, rec_t, rec_b;
  bgb::DevBuf cls_count, cls_off, ent_tau, ent_sigma, ent_cls, ent_mask, sing_L, err, geodf_t, geodf_b;
  bgb::DevBuf grp_tri, grp_cnt, grp_off, grp_perm;  // singular entries grouped by output block
  bgb::DevBuf cls_hist;                             // entries per class (statistics)
  static constexpr int kSlots = 3;  // output-block slots in flight (staging, plan tables, events)
  bgb::DevBuf plan_i[kSlots], plan_l[kSlots], plan_d[kSlots], plan_f[kSlots], far_const[kSlots], df_tab;
  bgb::DevBuf tplan_i, tplan_l, tplan_d, tplan_f;  // test-side tile tables (shared by all output blocks)
  bgb::DevBuf stage[kSlots];
  bgb::DevBuf diag_a, diag_b, diag_c, diag_d;
  bgb::CurveBufs curve;
  cudaEvent_t ev[8] = {};
  cudaEvent_t ev2[4 * kSlots] = {};  // per output-block slot: far start / end, copy start / end
  cudaStream_t stream_sing = nullptr;  // singular groups of a host output in blocks
  cudaStream_t stream_up = nullptr;    // uploads of the far kernels' tile tables (never behind a kernel)
  cudaEvent_t ev_up[kSlots + 1] = {};  // per slot: its block's tables uploaded; [kSlots]: test-side tables
  std::vector<cudaEvent_t> grp_ev;     // end of each singular group (grown on demand)
  cudaEvent_t ring_ev[2] = {};
  void* ring = nullptr;      // pinned host staging ring
  size_t ring_bytes = 0;
};


namespace bgb {

struct Supports {
  std::vector<int64_t> off;  // [nfun + 1]
  std::vector<int> tri, loc;
  std::vector<double> coef;
};

struct HostPlan {
  std::vector<int> tb_off, tb_tris, tb_fn_off, fs_off, fs_code;
  std::vector<double> fs_coef;
  std::vector<int64_t> rows;
  std::vector<int> bb_off, bb_tris, bb_fn_off, bb_chunk_off, ch_grp_off, grp_fn, grp_sup_off, gs_code;
  std::vector<double> gs_coef;
  std::vector<int64_t> cols;
  int tmax = 0, nmax = 0, MAXS = 1, gmax = 1, gsmax = 1;
  int64_t pairs = 0;
};

struct TileCfg { int FM, FN, SC; };
extern const TileCfg kTileCfgs[];
extern const int kNumTileCfgs;
extern const int kPrefMixed[];
extern const int kNumPrefMixed;
extern const int kPrefFp64[];
extern const int kNumPrefFp64;
extern const int kPrefLagrange[];
extern const int kNumPrefLagrange;
extern const int kPrefLagrangeFp64[];
extern const int kNumPrefLagrangeFp64;

int validate_space(const bgb_space* s, const char* name);
int make_quadsel(const bgb_quadstrat* qs, QuadSel* out);
int make_opparams(const bgb_operator* op, const bgb_space* a, const bgb_space* b, OpParams* out);
RuleTable make_rules();
struct SpaceExtents {
  double max_edge = 0.0, max_centroid_radius = 0.0;
};
// Far-kernel constants; with both spaces given, also decides whether the point-pair phase needs
// no second reduction (phase_direct), and returns the spaces' extents (ext_t, ext_b if given).
FarConst make_farconst(const OpParams& op, const RuleTable& R, const QuadSel& qs, const bgb_space* test = nullptr,
                       const bgb_space* trial = nullptr, SpaceExtents* ext_t = nullptr,
                       SpaceExtents* ext_b = nullptr);
Supports build_supports(const bgb_space* s);
std::vector<double> function_centres(const bgb_space* s, const Supports& S);
// Functions [f_begin, f_end) in recursive-bisection order of their centres, in compact runs of `leaf`.
std::vector<int> order_functions(const Supports& S, const std::vector<double>& centre, int f_begin, int f_end,
                                 int leaf, int nth = 1);
// Test-side tiles: up to FM functions and at most tcap distinct triangles per tile.
void plan_test_side(const Supports& S, const std::vector<int>& order, int FM, int64_t row0, HostPlan& P,
                    int tcap = 1 << 30);
void plan_trial_side(const Supports& S, const std::vector<int>& order, int FN, int SC, HostPlan& P);
// The same plans built over ranges of blocks in up to nth threads (identical results).
void plan_test_side_par(const Supports& S, const std::vector<int>& order, int FM, int64_t row0, HostPlan& P, int nth,
                        int tcap = 1 << 30);
void plan_trial_side_par(const Supports& S, const std::vector<int>& order, int FN, int SC, HostPlan& P, int nth);
int planner_threads();
bool same_space(const bgb_space* a, const bgb_space* b);
// Largest triangle edge of a space (host), for the argument range of the double-float sincos.
SpaceExtents space_extents(const bgb_space* s);
double max_edge(const bgb_space* s);
double max_centroid_radius(const bgb_space* s);
// True when the mixed path may integrate singular / near pairs in double-float: no lossy
// wave number and k R below the range of the df sin / cos.
bool df_singular_ok(const OpParams& op, double edge_t, double edge_b);
double event_ms(cudaEvent_t a, cudaEvent_t b);
// Copy n ints from device memory into the handle's mapped mailbox (read after a stream sync).
void launch_publish(const int* src, int n, int* mbox_dev, cudaStream_t st);
// BGB_ERR_NOT_SUPPORTED when k times the diameter of the two meshes exceeds 3e5, the range of the
// mixed far kernels' phase reduction.
int check_mixed_range(const bgb_operator* op, const bgb_space* a, const bgb_space* b);
// Gauss-Legendre rule on [0, 1], nodes ascending (n <= 64).
void gauss_legendre01(int n, double* x, double* w);

}  // namespace bgb
