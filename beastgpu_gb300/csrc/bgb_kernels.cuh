// Kernel launch interfaces shared by the translation units of libbeastgb.
#pragma once

#include "bgb_common.cuh"
#include "bgb_df.cuh"

#include <vector>

namespace bgb {

// ---- bgb_singular.cu -------------------------------------------------------------------
void launch_prepare_geo64(const double* verts, const int32_t* tris, int nt, Geo64* out, cudaStream_t st);
void launch_prepare_bounds(const Geo64* g, int nt, double k2, int trial_side, float4* out, cudaStream_t st);
// Bounding spheres of chunks of 32 consecutive trial triangles (out: (nb + 31) / 32 entries).
void launch_chunk_bounds(const float4* b, int nb, float4* out, cudaStream_t st);
// cb (optional): the trial chunk spheres; whole chunks are skipped by one test.
void launch_classify(bool fill, const float4* tb, const float4* bb, const Geo64* tg, const Geo64* bg, int nt, int nb,
                     double k2, int* count, const int64_t* offset, int* out_tau, int* out_sigma, int8_t* out_cls,
                     int* err, int num_sms, cudaStream_t st, int16_t* out_mask = nullptr, const float4* cb = nullptr);
void launch_scan(const int* counts, int n, int64_t* offsets, cudaStream_t st);
// Entries per class of the non-far list: hist[5] (64-bit counts).
void launch_class_hist(const int8_t* cls, int64_t n, unsigned long long* hist, int num_sms, cudaStream_t st);
// Singular entries sorted by group: perm[off[g] .. off[g + 1]) are the entries e with
// tri_group[sigma[e]] == g (out of range: the last group).  counts: ngroups ints, off: ngroups + 1.
void launch_group_entries(const int* sigma, int64_t n, const int* tri_group, int ngroups, int* counts, int64_t* off,
                          int* perm, int num_sms, cudaStream_t st);
void launch_classify_dense(const Geo64* tg, const Geo64* bg, int t0, int t1, int s0, int s1, double k2, int8_t* out,
                           int* err, cudaStream_t st);
// near_only: integrate only the near pairs of the list (the mixed path's double-float kernel skips them).
// perm (device, optional): integrate only the entries perm[range[0] .. range[1]) (range: device int64[2]).
void launch_singular(const OpParams& op, const QuadSel& qs, const RuleTable& rules, int rsA, int rsB, const Geo64* tg,
                     const Geo64* bg, const int* et, const int* es, const int8_t* ec, int64_t n, double2* out,
                     const volatile int* abort_flag, int num_sms, cudaStream_t st, bool near_only = false,
                     const int* perm = nullptr, const int64_t* range = nullptr);
void launch_local_diag64(const OpParams& op, const QuadSel& qs, const RuleTable& rules, int rsA, int rsB,
                         const Geo64* tg, const Geo64* bg, const int* tau, const int* sigma, int64_t n, int force,
                         double2* out, int8_t* cls, int* err, int num_sms, cudaStream_t st, int16_t* mask = nullptr);

void launch_prepare_bounds_batched(const Geo64* g, int nt, const int* tri_problem, const double* prob_k2, int trial_side,
                                   float4* out, cudaStream_t st);
void launch_classify_batched(bool fill, const float4* tb, const float4* bb, const Geo64* tg, const Geo64* bg, int nt,
                             const int* tri_problem, const int2* prob_trial, const double* prob_k2, int* count,
                             const int64_t* offset, int* out_tau, int* out_sigma, int8_t* out_cls, int* err,
                             int num_sms, cudaStream_t st, int16_t* out_mask = nullptr, const float4* cb = nullptr);
void launch_singular_batched(int op_kind, const OpParams* ops, const QuadSel& qs, const RuleTable& rules,
                             const Geo64* tg, const Geo64* bg, const int* tri_problem, const int* et, const int* es,
                             const int8_t* ec, int64_t n, double2* out, const volatile int* abort_flag, int num_sms,
                             cudaStream_t st, bool near_only = false);

// ---- bgb_singular_df.cu ----------------------------------------------------------------
// Host-built tables of the double-float singular kernel (one float buffer): Sauter-Schwab
// region points (u1, u2, v1, v2, weight as df) per class, near-rule points (u, v, w as df) and
// the sin / cos table.
struct DfTables {
  int ss_off[4], ss_cnt[4];
  int near_t_off, near_b_off, near_qt, near_qb;
  int trig_off, total_floats;
  DfTrig trig;
};
void build_df_tables(const QuadSel& qs, const RuleTable& R, std::vector<float>& buf, DfTables& M);
// Per-triangle double-float geometry: vertices (df), area and 1 / area (df).
struct GeoDf {
  float v[3][3][2];
  float area[2], inv_area[2];
};
void launch_prepare_geodf(const Geo64* g, int nt, GeoDf* out, cudaStream_t st);
// Operator constants as df: alpha, beta (complex), k = Im gamma.
struct OpDf {
  float alpha[2][2], beta[2][2], k[2];
  int kind, oscill;
};
OpDf make_opdf(const OpParams& op);
// opdf_array / tri_problem non-NULL: batched (constants of the test triangle's problem).
void launch_singular_df(int op_kind, const OpDf& op, const OpDf* opdf_array, const int* tri_problem,
                        const DfTables& M, const float* dtab, const GeoDf* tg, const GeoDf* bg, const int* et,
                        const int* es, const int8_t* ec, const int16_t* emask, int64_t n, double2* out,
                        const volatile int* abort_flag, int num_sms, cudaStream_t st, const int* perm = nullptr,
                        const int64_t* range = nullptr);

// ---- bgb_far.cu ------------------------------------------------------------------------
// Constants of the far-pair kernels (passed by value).
struct FarConst {
  int op_kind;
  int qt, qb;                  // rule points (runtime, <= template maxima)
  int lossy;                   // gamma has a real part
  int phase_direct;            // k (r_test + r_trial) <= pi: the point-pair phase needs no reduction
  double alpha[2], beta[2], gamma[2];
  float alpha32[2], beta32[2];
  float k_hi, k_lo, gre;       // gamma_im as double-float, gamma_re
  float shpT[BGB_MAXQ][3], shpB[BGB_MAXQ][3];     // Lagrange hats at rule points
  double shpT64[BGB_MAXQ][3], shpB64[BGB_MAXQ][3];
  // Plain FP64 kernel: with tay_n > 0 the phase of a point pair is k R = k R0 + k (R - R0), R0 the
  // centroid distance, and exp(-i k (R - R0)) comes from the first tay_n <= 6 terms of the series of
  // sin and cos (|k (R - R0)| <= k (r_test + r_trial), truncation below 2^-55); tay_s[j] =
  // (-1)^j / (2j + 1)!, tay_c[j] = (-1)^j / (2j)!.  tay_n = 0: sincos at every point pair.
  int tay_n;
  double tay_s[BGB_TAYLOR_MAX], tay_c[BGB_TAYLOR_MAX];
};

// The scalar constants of a far launch, copied into registers per tile.
struct FarScalars {
  int qt, qb, lossy, phase_direct, tay_n;
  float k_hi, k_lo, gre;
  float alpha32[2], beta32[2];
  double alpha[2], beta[2], gamma[2];
};

// Device-side plan of one tiled assembly (all arrays device pointers).
struct TilePlan {
  // records
  const void* rec_t;           // test records (float or double, stride rec_stride_t)
  const void* rec_b;
  const float4* bnd_t;         // bounding spheres (classification radii)
  const float4* bnd_b;
  // test blocks
  int n_tblocks;
  const int* tb_off;           // [n_tblocks + 1] into tb_tris
  const int* tb_tris;          // global test triangle ids, sorted ascending per block
  const int* tb_fn_off;        // [n_tblocks + 1] into internal test function list
  const int* fs_off;           // [n_tfun + 1] support entries of internal test function m
  const int* fs_code;          // slot << 2 | local
  const double* fs_coef;
  const int64_t* rows;         // output row (relative to the window) of internal test function m
  // trial blocks
  int n_bblocks;
  const int* bb_off;           // [n_bblocks + 1] into bb_tris
  const int* bb_tris;          // global trial triangle ids, sorted ascending per block
  const int* bb_fn_off;        // [n_bblocks + 1] into internal trial function list
  const int* bb_chunk_off;     // [n_bblocks + 1] into chunk list
  const int* ch_grp_off;       // [n_chunks + 1] into group list
  const int* grp_fn;           // local trial function (within block)
  const int* grp_sup_off;      // [n_groups + 1] into group support entries
  const int* gs_code;          // slot (within block's triangle list) << 2 | local
  const double* gs_coef;
  const float* gs_coef32;      // float copy for the mixed kernel
  const float* fs_coef32;
  int gmax, gsmax;             // max groups / group supports per trial block
  const int64_t* cols;         // output column of internal trial function n
  // singular / near overrides (CSR over global test triangles, sorted by trial triangle)
  const int64_t* sing_off;
  const int* sing_sigma;
  const double2* sing_L;
  // shapes
  int FM, FN, SC, MAXS;        // block sizes, chunk, max supports per test function
  int tmax, nmax;              // max triangles per test / trial block
  // output
  void* out;
  int out_c64;                 // 1: complex double, 0: complex float
  int64_t ld;
  const volatile int* abort_flag;
};

size_t far_smem_bytes(int precision, int op_kind, int qt, int qb, const TilePlan& p);
// CTAs per SM the far kernel is compiled for (__launch_bounds__ minimum blocks).
int far_target_ctas_per_sm(int precision);
// Persistent batched launch over a work queue of (problem, bm, bn) items (device arrays).
int launch_far_persistent(int precision, int op_kind, int generic, const FarConst* Ks, const TilePlan* plans,
                          const int4* items, int nitems, int* counter, size_t smem_bytes, int ctas,
                          const volatile int* abort_flag, cudaStream_t st);
int far_persistent_occupancy(int precision, int op_kind, int generic, size_t smem_bytes, int* per_sm);
void launch_prepare_rec(int precision, int side, int q, const Geo64* g, int nt, const RuleTable& rules, int rule,
                        double wscale, void* out, cudaStream_t st);
int far_generic_q(int qt, int qb);  // 1 when the (qt, qb) pair uses the generic instance
int rec_stride(int precision, int q, int generic);

// Diagnostic: far-pair local matrices of explicit pairs with the tile kernels' pair code.
int launch_far_pairs_diag(int precision, const FarConst& k, const void* rec_t, const void* rec_b, const int* tau,
                          const int* sigma, int64_t n, double2* out, cudaStream_t st);

// ---- bgb_peaks.cu ----------------------------------------------------------------------
int measure_issue_peaks(int num_sms, double* fp32, double* fp64, double* mufu);

}  // namespace bgb
