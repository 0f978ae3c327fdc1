// Batched assembly of many independent problems (scatterers of uneven size and wave number).
//
// bgb_batch_create concatenates the problems' geometry, classifies all their pairs with one
// launch (each test triangle sweeps only its own problem), integrates all singular / near
// pairs with one launch, and plans every problem's output tiles.  The far pairs of all
// problems are then done by ONE persistent launch: CTAs pull (problem, row block, column
// block) tiles from a work queue (an atomic counter), ordered by the schedule the autotuner
// picked (largest tiles first, or problem-major).  The autotuner times the candidate tile
// shapes and schedules on the batch itself and keeps the fastest.  The whole device sequence
// is captured once in a CUDA graph; bgb_batch_run replays it.  Results are bit-identical to
// assembling each problem alone with bgb_assemble (same kernels, same accumulation order).
#include "bgb_host.h"

#include <algorithm>
#include <cstring>
#include <numeric>

struct bgb_batch {
  bgb_handle* h = nullptr;
  int n = 0, precision = 0, out_kind = 0, op_kind = 0, generic = 0;
  int cfg_id = -1, schedule = 0, ctas = 0;
  size_t smem = 0;
  bool host_out = false, c64 = false;
  // device buffers
  bgb::DevBuf verts_t, tris_t, verts_b, tris_b, geo_t, geo_b, bnd_t, bnd_b, bnd_c, rec_t, rec_b;
  bgb::DevBuf tri_problem, prob_trial, prob_k2, ops, Ks, plans, items, counter;
  bgb::DevBuf cls_count, cls_off, ent_tau, ent_sigma, ent_cls, ent_mask, sing_L, err, geodf_t, geodf_b, opdf;
  bgb::DevBuf plan_i, plan_l, plan_d, plan_f, stage, df_tab;
  bool use_df = false;
  bgb::DfTables dfm{};
  int nt_t = 0, nt_b = 0, nv_t = 0, nv_b = 0, nitems = 0;
  bool shared_trial = false;
  int64_t nsing = 0;
  std::vector<void*> outs;
  std::vector<int64_t> lds, nrows, ncols, stage_off;
  bgb::QuadSel qsel{};
  bgb::RuleTable rules{};
  bgb_stats stats{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev[2] = {};

  ~bgb_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
    bgb::DevBuf* bufs[] = {&verts_t, &verts_b, &tris_t, &tris_b, &geo_t, &geo_b, &bnd_t, &bnd_b, &bnd_c, &rec_t, &rec_b,
                           &tri_problem, &prob_trial, &prob_k2, &ops, &Ks, &plans, &items, &counter, &cls_count,
                           &cls_off, &ent_tau, &ent_sigma, &ent_cls, &ent_mask, &sing_L, &err, &geodf_t, &geodf_b, &opdf, &plan_i, &plan_l, &plan_d,
                           &plan_f, &stage, &df_tab};
    for (auto* b : bufs) b->release();
  }
};

namespace bgb {
namespace {

bool same_quadstrat(const bgb_quadstrat& a, const bgb_quadstrat& b) {
  return a.far_test == b.far_test && a.far_trial == b.far_trial && a.near_test == b.near_test &&
         a.near_trial == b.near_trial && a.ss_cf == b.ss_cf && a.ss_ce == b.ss_ce && a.ss_cv == b.ss_cv;
}

template <class T>
int put(cudaStream_t st, DevBuf& buf, const std::vector<T>& v) {
  int rc;
  if ((rc = buf.ensure(sizeof(T) * std::max<size_t>(1, v.size())))) return rc;
  if (!v.empty()) BGB_CUDA(cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  return 0;
}

// Device stages that can be replayed: geometry, classification, singular pairs, records,
// far tiles.  Enqueued on `st` (also used while capturing the graph).
int enqueue_device_work(bgb_batch* B, cudaStream_t st, bool far_only) {
  bgb_handle* h = B->h;
  if (!far_only) {
    BGB_CUDA(cudaMemsetAsync(B->err.p, 0, sizeof(int) * 4, st));
    launch_prepare_geo64(B->verts_t.as<double>(), B->tris_t.as<int32_t>(), B->nt_t, B->geo_t.as<Geo64>(), st);
    if (!B->shared_trial)
      launch_prepare_geo64(B->verts_b.as<double>(), B->tris_b.as<int32_t>(), B->nt_b, B->geo_b.as<Geo64>(), st);
    const Geo64* gt = B->geo_t.as<Geo64>();
    const Geo64* gb = B->shared_trial ? gt : B->geo_b.as<Geo64>();
    // the trial-side problem of a trial triangle: trial ranges are per problem; bounds need
    // the problem of each trial triangle, stored after the test ones in tri_problem
    const int* tp_t = B->tri_problem.as<int>();
    const int* tp_b = B->tri_problem.as<int>() + B->nt_t;
    launch_prepare_bounds_batched(gt, B->nt_t, tp_t, B->prob_k2.as<double>(), 0, B->bnd_t.as<float4>(), st);
    launch_prepare_bounds_batched(gb, B->nt_b, tp_b, B->prob_k2.as<double>(), 1, B->bnd_b.as<float4>(), st);
    launch_chunk_bounds(B->bnd_b.as<float4>(), B->nt_b, B->bnd_c.as<float4>(), st);
    launch_classify_batched(false, B->bnd_t.as<float4>(), B->bnd_b.as<float4>(), gt, gb, B->nt_t, tp_t,
                            B->prob_trial.as<int2>(), B->prob_k2.as<double>(), B->cls_count.as<int>(), nullptr,
                            nullptr, nullptr, nullptr, B->err.as<int>(), h->num_sms, st, nullptr, B->bnd_c.as<float4>());
    launch_scan(B->cls_count.as<int>(), B->nt_t, B->cls_off.as<int64_t>(), st);
    launch_classify_batched(true, B->bnd_t.as<float4>(), B->bnd_b.as<float4>(), gt, gb, B->nt_t, tp_t,
                            B->prob_trial.as<int2>(), B->prob_k2.as<double>(), B->cls_count.as<int>(),
                            B->cls_off.as<int64_t>(), B->ent_tau.as<int>(), B->ent_sigma.as<int>(),
                            B->ent_cls.as<int8_t>(), B->err.as<int>(), h->num_sms, st, B->ent_mask.as<int16_t>(),
                            B->bnd_c.as<float4>());
    if (B->use_df) {
      launch_prepare_geodf(gt, B->nt_t, B->geodf_t.as<GeoDf>(), st);
      if (!B->shared_trial) launch_prepare_geodf(gb, B->nt_b, B->geodf_b.as<GeoDf>(), st);
      const GeoDf* dgt = B->geodf_t.as<GeoDf>();
      const GeoDf* dgb = B->shared_trial ? dgt : B->geodf_b.as<GeoDf>();
      launch_singular_df(B->op_kind, OpDf{}, B->opdf.as<OpDf>(), tp_t, B->dfm, B->df_tab.as<float>(), dgt, dgb,
                         B->ent_tau.as<int>(), B->ent_sigma.as<int>(), B->ent_cls.as<int8_t>(),
                         B->ent_mask.as<int16_t>(), B->nsing, B->sing_L.as<double2>(), h->abort_dev, h->num_sms, st);
      launch_singular_batched(B->op_kind, B->ops.as<OpParams>(), B->qsel, B->rules, gt, gb, tp_t, B->ent_tau.as<int>(),
                              B->ent_sigma.as<int>(), B->ent_cls.as<int8_t>(), B->nsing, B->sing_L.as<double2>(),
                              h->abort_dev, h->num_sms, st, true);  // near pairs in FP64
    } else
      launch_singular_batched(B->op_kind, B->ops.as<OpParams>(), B->qsel, B->rules, gt, gb, tp_t, B->ent_tau.as<int>(),
                              B->ent_sigma.as<int>(), B->ent_cls.as<int8_t>(), B->nsing, B->sing_L.as<double2>(),
                              h->abort_dev, h->num_sms, st);
    const int qt = B->rules.npoints[B->qsel.far_t], qb = B->rules.npoints[B->qsel.far_b];
    launch_prepare_rec(B->precision, 0, B->generic ? BGB_MAXQ : qt, gt, B->nt_t, B->rules, B->qsel.far_t, 1.0,
                       B->rec_t.p, st);
    launch_prepare_rec(B->precision, 1, B->generic ? BGB_MAXQ : qb, gb, B->nt_b, B->rules, B->qsel.far_b,
                       BGB_INV_4PI_D, B->rec_b.p, st);
  }
  BGB_CUDA(cudaMemsetAsync(B->counter.p, 0, sizeof(int), st));
  return launch_far_persistent(B->precision, B->op_kind, B->generic, B->Ks.as<FarConst>(), B->plans.as<TilePlan>(),
                               B->items.as<int4>(), B->nitems, B->counter.as<int>(), B->smem, B->ctas, h->abort_dev,
                               st);
}

// Plans of every problem for tile configuration `cfg`; uploads them and the work items.
int build_plans(bgb_batch* B, const bgb_problem* pr, const std::vector<Supports>& St, const std::vector<Supports>& Sb,
                const std::vector<std::vector<double>>& cent_t, const std::vector<std::vector<double>>& cent_b,
                const std::vector<int>& tbase, const std::vector<int>& bbase, int cfg, int schedule, bool upload_all,
                size_t* smem_out) {
  const TileCfg tc = kTileCfgs[cfg];
  const int n = B->n;
  std::vector<HostPlan> P(n);
  // one shared-memory layout for the whole launch: the batch-wide maxima
  int tmax = 1, nmax = 1, MAXS = 1, gmax = 1, gsmax = 1;
  for (int p = 0; p < n; ++p) {
    // function orders in runs of this configuration's tile widths
    plan_test_side(St[p], order_functions(St[p], cent_t[p], 0, pr[p].test.nfun, tc.FM), tc.FM, 0, P[p]);
    plan_trial_side(Sb[p], order_functions(Sb[p], cent_b[p], 0, pr[p].trial.nfun, tc.FN), tc.FN, tc.SC, P[p]);
    for (int& t : P[p].tb_tris) t += tbase[p];
    for (int& t : P[p].bb_tris) t += bbase[p];
    tmax = std::max(tmax, P[p].tmax); nmax = std::max(nmax, P[p].nmax); MAXS = std::max(MAXS, P[p].MAXS);
    gmax = std::max(gmax, P[p].gmax); gsmax = std::max(gsmax, P[p].gsmax);
  }
  TilePlan probe{};
  probe.FM = tc.FM; probe.FN = tc.FN; probe.SC = tc.SC; probe.MAXS = MAXS;
  probe.gmax = gmax; probe.gsmax = gsmax; probe.tmax = tmax; probe.nmax = nmax;
  *smem_out = far_smem_bytes(B->precision, B->op_kind, B->rules.npoints[B->qsel.far_t], B->rules.npoints[B->qsel.far_b],
                             probe);
  if (!upload_all) return 0;
  // concatenate
  std::vector<int> I;
  std::vector<int64_t> Lg;
  std::vector<double> D;
  std::vector<float> F;
  struct Off { size_t tb_off, tb_tris, tb_fn, fs_off, fs_code, bb_off, bb_tris, bb_fn, bb_ch, ch_grp, grp_fn, grp_sup,
               gs_code, rows, cols, fs_coef, gs_coef, fs32, gs32; };
  std::vector<Off> off(n);
  auto pi = [&](const std::vector<int>& v) { size_t o = I.size(); I.insert(I.end(), v.begin(), v.end()); return o; };
  auto pl = [&](const std::vector<int64_t>& v) { size_t o = Lg.size(); Lg.insert(Lg.end(), v.begin(), v.end()); return o; };
  auto pd = [&](const std::vector<double>& v) { size_t o = D.size(); D.insert(D.end(), v.begin(), v.end()); return o; };
  auto pf = [&](const std::vector<double>& v) { size_t o = F.size(); for (double x : v) F.push_back((float)x); return o; };
  for (int p = 0; p < n; ++p) {
    Off& o = off[p];
    o.tb_off = pi(P[p].tb_off); o.tb_tris = pi(P[p].tb_tris); o.tb_fn = pi(P[p].tb_fn_off); o.fs_off = pi(P[p].fs_off);
    o.fs_code = pi(P[p].fs_code); o.bb_off = pi(P[p].bb_off); o.bb_tris = pi(P[p].bb_tris); o.bb_fn = pi(P[p].bb_fn_off);
    o.bb_ch = pi(P[p].bb_chunk_off); o.ch_grp = pi(P[p].ch_grp_off); o.grp_fn = pi(P[p].grp_fn);
    o.grp_sup = pi(P[p].grp_sup_off); o.gs_code = pi(P[p].gs_code);
    o.rows = pl(P[p].rows); o.cols = pl(P[p].cols);
    o.fs_coef = pd(P[p].fs_coef); o.gs_coef = pd(P[p].gs_coef);
    o.fs32 = pf(P[p].fs_coef); o.gs32 = pf(P[p].gs_coef);
  }
  cudaStream_t st = B->h->stream;
  BGB_CUDA(cudaStreamSynchronize(st));  // the previous plan arrays may still be read by a tuning launch
  int rc;
  if ((rc = put(st, B->plan_i, I)) || (rc = put(st, B->plan_l, Lg)) || (rc = put(st, B->plan_d, D)) ||
      (rc = put(st, B->plan_f, F)))
    return rc;
  std::vector<TilePlan> T(n);
  std::vector<int4> items;
  std::vector<int64_t> cost;
  const int* di = B->plan_i.as<int>();
  const int64_t* dl = B->plan_l.as<int64_t>();
  const double* dd = B->plan_d.as<double>();
  const float* df = B->plan_f.as<float>();
  for (int p = 0; p < n; ++p) {
    const Off& o = off[p];
    TilePlan& t = T[p];
    t.rec_t = B->rec_t.p;
    t.rec_b = B->rec_b.p;
    t.bnd_t = B->bnd_t.as<float4>();
    t.bnd_b = B->bnd_b.as<float4>();
    t.n_tblocks = (int)P[p].tb_off.size() - 1;
    t.tb_off = di + o.tb_off; t.tb_tris = di + o.tb_tris; t.tb_fn_off = di + o.tb_fn; t.fs_off = di + o.fs_off;
    t.fs_code = di + o.fs_code; t.fs_coef = dd + o.fs_coef; t.fs_coef32 = df + o.fs32; t.rows = dl + o.rows;
    t.n_bblocks = (int)P[p].bb_off.size() - 1;
    t.bb_off = di + o.bb_off; t.bb_tris = di + o.bb_tris; t.bb_fn_off = di + o.bb_fn; t.bb_chunk_off = di + o.bb_ch;
    t.ch_grp_off = di + o.ch_grp; t.grp_fn = di + o.grp_fn; t.grp_sup_off = di + o.grp_sup; t.gs_code = di + o.gs_code;
    t.gs_coef = dd + o.gs_coef; t.gs_coef32 = df + o.gs32; t.cols = dl + o.cols;
    t.sing_off = B->cls_off.as<int64_t>();
    t.sing_sigma = B->ent_sigma.as<int>();
    t.sing_L = B->sing_L.as<double2>();
    t.FM = tc.FM; t.FN = tc.FN; t.SC = tc.SC;
    t.MAXS = MAXS; t.tmax = tmax; t.nmax = nmax; t.gmax = gmax; t.gsmax = gsmax;
    t.out_c64 = B->c64;
    t.abort_flag = B->h->abort_dev;
    if (B->host_out) {
      t.out = (char*)B->stage.p + B->stage_off[p];
      t.ld = std::max<int64_t>(1, B->nrows[p]);
    } else {
      t.out = B->outs[p];
      t.ld = B->lds[p];
    }
    for (int bm = 0; bm < t.n_tblocks; ++bm)
      for (int bn = 0; bn < t.n_bblocks; ++bn) {
        items.push_back(make_int4(p, bm, bn, 0));
        cost.push_back((int64_t)(P[p].tb_off[bm + 1] - P[p].tb_off[bm]) * (P[p].bb_off[bn + 1] - P[p].bb_off[bn]));
      }
  }
  if (schedule == 1) {  // largest tiles first (LPT), ties by problem, block
    std::vector<size_t> idx(items.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<int4> sorted(items.size());
    for (size_t i = 0; i < idx.size(); ++i) sorted[i] = items[idx[i]];
    items.swap(sorted);
  }
  B->nitems = (int)items.size();
  if ((rc = put(st, B->plans, T)) || (rc = put(st, B->items, items))) return rc;
  return 0;
}

}  // namespace
}  // namespace bgb

using namespace bgb;

static int batch_copy_out(bgb_batch* B, cudaStream_t s) {
  const size_t esz = B->c64 ? 16 : 8;
  for (int p = 0; p < B->n; ++p) {
    if (B->nrows[p] == 0 || B->ncols[p] == 0) continue;
    BGB_CUDA(cudaMemcpy2DAsync(B->outs[p], (size_t)B->lds[p] * esz, (char*)B->stage.p + B->stage_off[p],
                               (size_t)B->nrows[p] * esz, (size_t)B->nrows[p] * esz, (size_t)B->ncols[p],
                               cudaMemcpyDeviceToHost, s));
  }
  BGB_CUDA(cudaStreamSynchronize(s));
  return 0;
}

extern "C" {

int bgb_batch_destroy(bgb_batch* b) {
  if (!b) return 0;
  cudaSetDevice(b->h->device);
  cudaStreamSynchronize(b->h->stream);
  delete b;
  return 0;
}

int bgb_batch_create(bgb_handle* h, int32_t n, const bgb_problem* problems, int32_t precision, int32_t out_kind,
                     int32_t flags, bgb_batch** out, bgb_stats* stats) {
  if (!h || !out || n < 1 || !problems) { set_error("bgb_batch_create: invalid argument"); return BGB_ERR_INVALID; }
  *out = nullptr;
  if (precision != BGB_PREC_FP64 && precision != BGB_PREC_MIXED) { set_error("bad precision %d", precision); return BGB_ERR_INVALID; }
  if (out_kind < BGB_OUT_HOST_C64 || out_kind > BGB_OUT_DEVICE_C32) { set_error("bad out_kind %d", out_kind); return BGB_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(h->mu);
  int rc;
  for (int p = 0; p < n; ++p) {
    const bgb_problem& q = problems[p];
    if ((rc = validate_space(&q.test, "test")) || (rc = validate_space(&q.trial, "trial"))) return rc;
    if (q.op.kind != problems[0].op.kind || q.test.refspace != problems[0].test.refspace ||
        q.trial.refspace != problems[0].trial.refspace || !same_quadstrat(q.qs, problems[0].qs)) {
      set_error("bgb_batch_create: all problems of a batch share the operator kind, the spaces' kind and the "
                "quadrature strategy (problem %d differs)", p);
      return BGB_ERR_NOT_SUPPORTED;
    }
    if (!q.out && q.test.nfun > 0 && q.trial.nfun > 0) { set_error("problem %d: out is NULL", p); return BGB_ERR_INVALID; }
    if (precision == BGB_PREC_MIXED && (rc = check_mixed_range(&q.op, &q.test, &q.trial))) return rc;
    if (q.ld < std::max(1, q.test.nfun)) { set_error("problem %d: ld < number of rows", p); return BGB_ERR_INVALID; }
  }
  cudaSetDevice(h->device);
  *h->abort_host = 0;
  bgb_batch* B = new bgb_batch();
  B->h = h;
  B->n = n;
  B->precision = precision;
  B->out_kind = out_kind;
  B->op_kind = problems[0].op.kind;
  B->host_out = out_kind == BGB_OUT_HOST_C64 || out_kind == BGB_OUT_HOST_C32;
  B->c64 = out_kind == BGB_OUT_HOST_C64 || out_kind == BGB_OUT_DEVICE_C64;
  B->rules = make_rules();
  auto fail = [&](int code) { delete B; return code; };
  if ((rc = make_quadsel(&problems[0].qs, &B->qsel))) return fail(rc);
  cudaStream_t st = h->stream;
  cudaEventCreate(&B->ev[0]);
  cudaEventCreate(&B->ev[1]);

  // concatenated geometry and per-problem tables
  std::vector<double> vt, vb;
  std::vector<int32_t> tt, tb;
  std::vector<int> tri_problem, tbase(n), bbase(n);
  std::vector<int2> prob_trial(n);
  std::vector<double> prob_k2(n);
  std::vector<OpParams> ops(n);
  std::vector<FarConst> Ks(n);
  B->shared_trial = true;
  for (int p = 0; p < n; ++p) B->shared_trial &= same_space(&problems[p].test, &problems[p].trial);
  int64_t pairs_total = 0;
  for (int p = 0; p < n; ++p) {
    const bgb_problem& q = problems[p];
    if ((rc = make_opparams(&q.op, &q.test, &q.trial, &ops[p]))) return fail(rc);
    Ks[p] = make_farconst(ops[p], B->rules, B->qsel, &q.test, &q.trial);
    prob_k2[p] = ops[p].k2;
    tbase[p] = (int)(tt.size() / 3);
    const int vo = (int)(vt.size() / 3);
    vt.insert(vt.end(), q.test.vertices, q.test.vertices + 3 * (size_t)q.test.nv);
    for (int64_t i = 0; i < 3 * (int64_t)q.test.nt; ++i) tt.push_back(q.test.triangles[i] + vo);
    for (int t = 0; t < q.test.nt; ++t) tri_problem.push_back(p);
    if (!B->shared_trial) {
      bbase[p] = (int)(tb.size() / 3);
      const int wo = (int)(vb.size() / 3);
      vb.insert(vb.end(), q.trial.vertices, q.trial.vertices + 3 * (size_t)q.trial.nv);
      for (int64_t i = 0; i < 3 * (int64_t)q.trial.nt; ++i) tb.push_back(q.trial.triangles[i] + wo);
    } else {
      bbase[p] = tbase[p];
    }
    prob_trial[p] = make_int2(bbase[p], bbase[p] + q.trial.nt);
    pairs_total += (int64_t)q.test.nt * q.trial.nt;
  }
  if (precision == BGB_PREC_MIXED) {
    B->use_df = true;
    for (int p = 0; p < n; ++p)
      B->use_df &= df_singular_ok(ops[p], max_edge(&problems[p].test), max_edge(&problems[p].trial));
    if (B->use_df) {
      std::vector<float> tab;
      build_df_tables(B->qsel, B->rules, tab, B->dfm);
      std::vector<OpDf> od(n);
      for (int p = 0; p < n; ++p) od[p] = make_opdf(ops[p]);
      if ((rc = put(st, B->df_tab, tab)) || (rc = put(st, B->opdf, od))) return fail(rc);
      BGB_CUDA(cudaStreamSynchronize(st));
    }
  }
  B->nt_t = (int)(tt.size() / 3);
  B->nv_t = (int)(vt.size() / 3);
  B->nt_b = B->shared_trial ? B->nt_t : (int)(tb.size() / 3);
  B->nv_b = B->shared_trial ? B->nv_t : (int)(vb.size() / 3);
  // problem of every trial triangle, after the test ones
  std::vector<int> tp_all = tri_problem;
  if (B->shared_trial) {
    tp_all.insert(tp_all.end(), tri_problem.begin(), tri_problem.end());
  } else {
    for (int p = 0; p < n; ++p)
      for (int t = 0; t < problems[p].trial.nt; ++t) tp_all.push_back(p);
  }
  if ((rc = put(st, B->verts_t, vt)) || (rc = put(st, B->tris_t, tt)) || (rc = put(st, B->tri_problem, tp_all)) ||
      (rc = put(st, B->prob_trial, prob_trial)) || (rc = put(st, B->prob_k2, prob_k2)) || (rc = put(st, B->ops, ops)) ||
      (rc = put(st, B->Ks, Ks)))
    return fail(rc);
  if (!B->shared_trial && ((rc = put(st, B->verts_b, vb)) || (rc = put(st, B->tris_b, tb)))) return fail(rc);
  const int qt = B->rules.npoints[B->qsel.far_t], qb = B->rules.npoints[B->qsel.far_b];
  B->generic = far_generic_q(qt, qb);
  const size_t rsz = precision == BGB_PREC_MIXED ? sizeof(float) : sizeof(double);
  if ((rc = B->geo_t.ensure(sizeof(Geo64) * std::max(1, B->nt_t))) ||
      (!B->shared_trial && (rc = B->geo_b.ensure(sizeof(Geo64) * std::max(1, B->nt_b)))) ||
      (rc = B->bnd_t.ensure(sizeof(float4) * std::max(1, B->nt_t))) || (rc = B->bnd_b.ensure(sizeof(float4) * std::max(1, B->nt_b))) ||
      (rc = B->bnd_c.ensure(sizeof(float4) * std::max(1, (B->nt_b + 31) / 32))) ||
      (rc = B->cls_count.ensure(sizeof(int) * (B->nt_t + 1))) || (rc = B->cls_off.ensure(sizeof(int64_t) * (B->nt_t + 1))) ||
      (rc = B->err.ensure(sizeof(int) * 4)) || (rc = B->counter.ensure(sizeof(int) * 4)) ||
      (rc = B->rec_t.ensure(rsz * rec_stride(precision, qt, B->generic) * std::max(1, B->nt_t))) ||
      (rc = B->rec_b.ensure(rsz * rec_stride(precision, qb, B->generic) * std::max(1, B->nt_b))))
    return fail(rc);
  if (B->shared_trial) {  // alias the trial geometry to the test geometry
    B->geo_b.p = nullptr;
  }
  // eager classification count to size the pair list (the graph replays the same sizes)
  const Geo64* gt = B->geo_t.as<Geo64>();
  launch_prepare_geo64(B->verts_t.as<double>(), B->tris_t.as<int32_t>(), B->nt_t, B->geo_t.as<Geo64>(), st);
  if (!B->shared_trial)
    launch_prepare_geo64(B->verts_b.as<double>(), B->tris_b.as<int32_t>(), B->nt_b, B->geo_b.as<Geo64>(), st);
  const Geo64* gb = B->shared_trial ? gt : B->geo_b.as<Geo64>();
  BGB_CUDA(cudaMemsetAsync(B->err.p, 0, sizeof(int) * 4, st));
  launch_prepare_bounds_batched(gt, B->nt_t, B->tri_problem.as<int>(), B->prob_k2.as<double>(), 0, B->bnd_t.as<float4>(), st);
  launch_prepare_bounds_batched(gb, B->nt_b, B->tri_problem.as<int>() + B->nt_t, B->prob_k2.as<double>(), 1,
                                B->bnd_b.as<float4>(), st);
  launch_chunk_bounds(B->bnd_b.as<float4>(), B->nt_b, B->bnd_c.as<float4>(), st);
  launch_classify_batched(false, B->bnd_t.as<float4>(), B->bnd_b.as<float4>(), gt, gb, B->nt_t, B->tri_problem.as<int>(),
                          B->prob_trial.as<int2>(), B->prob_k2.as<double>(), B->cls_count.as<int>(), nullptr, nullptr,
                          nullptr, nullptr, B->err.as<int>(), h->num_sms, st, nullptr, B->bnd_c.as<float4>());
  launch_scan(B->cls_count.as<int>(), B->nt_t, B->cls_off.as<int64_t>(), st);
  int herr = 0;
  int64_t tot = 0;
  BGB_CUDA(cudaMemcpyAsync(&tot, B->cls_off.as<int64_t>() + B->nt_t, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  BGB_CUDA(cudaMemcpyAsync(&herr, B->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  BGB_CUDA(cudaStreamSynchronize(st));
  if (herr) { set_error("degenerate geometry: a triangle pair shares more than three vertices"); return fail(BGB_ERR_INVALID); }
  B->nsing = tot;
  if ((rc = B->ent_tau.ensure(sizeof(int) * std::max<int64_t>(1, tot))) ||
      (rc = B->ent_sigma.ensure(sizeof(int) * std::max<int64_t>(1, tot))) ||
      (rc = B->ent_cls.ensure(std::max<int64_t>(1, tot))) ||
      (rc = B->ent_mask.ensure(sizeof(int16_t) * std::max<int64_t>(1, tot))) ||
      (B->use_df && (rc = B->geodf_t.ensure(sizeof(GeoDf) * std::max(1, B->nt_t)))) ||
      (B->use_df && !B->shared_trial && (rc = B->geodf_b.ensure(sizeof(GeoDf) * std::max(1, B->nt_b)))) ||
      (rc = B->sing_L.ensure(sizeof(double2) * 9 * std::max<int64_t>(1, tot))))
    return fail(rc);
  // outputs
  size_t stage_bytes = 0;
  const size_t esz = B->c64 ? 16 : 8;
  for (int p = 0; p < n; ++p) {
    B->outs.push_back(problems[p].out);
    B->lds.push_back(problems[p].ld);
    B->nrows.push_back(problems[p].test.nfun);
    B->ncols.push_back(problems[p].trial.nfun);
    B->stage_off.push_back((int64_t)stage_bytes);
    stage_bytes += esz * (size_t)std::max(1, problems[p].test.nfun) * (size_t)problems[p].trial.nfun;
    stage_bytes = (stage_bytes + 255) & ~(size_t)255;
  }
  if (B->host_out && (rc = B->stage.ensure(stage_bytes))) return fail(rc);
  // all device stages once, eagerly (sizes the pair list, and is the first assembly)
  // host plans
  std::vector<Supports> St(n), Sb(n);
  std::vector<std::vector<double>> cent_t(n), cent_b(n);
  for (int p = 0; p < n; ++p) {
    St[p] = build_supports(&problems[p].test);
    cent_t[p] = function_centres(&problems[p].test, St[p]);
    if (same_space(&problems[p].test, &problems[p].trial)) {
      Sb[p] = St[p];
      cent_b[p] = cent_t[p];
    } else {
      Sb[p] = build_supports(&problems[p].trial);
      cent_b[p] = function_centres(&problems[p].trial, Sb[p]);
    }
  }
  int smem_max = 0;
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  const bool lagrange = problems[0].test.refspace == BGB_REFSPACE_LAGRANGE_C0D1;
  const bool mixed = precision == BGB_PREC_MIXED;
  const int* prefs = lagrange ? (mixed ? kPrefLagrange : kPrefLagrangeFp64) : mixed ? kPrefMixed : kPrefFp64;
  const int nprefs = lagrange ? (mixed ? kNumPrefLagrange : kNumPrefLagrangeFp64) : mixed ? kNumPrefMixed : kNumPrefFp64;
  std::vector<int> cands;
  if (h->cfg.tile_config >= 0) cands.push_back(h->cfg.tile_config);
  else
    for (int i = 0; i < nprefs; ++i) cands.push_back(prefs[i]);
  const bool autotune = (flags & 1) && cands.size() > 1;
  // first full run (records + singular) with the first fitting candidate
  int first = -1;
  size_t smem = 0;
  for (int c : cands) {
    if ((rc = build_plans(B, problems, St, Sb, cent_t, cent_b, tbase, bbase, c, 1, false, &smem))) return fail(rc);
    if (smem <= (size_t)smem_max) { first = c; break; }
  }
  if (first < 0) { set_error("bgb_batch_create: no tile shape fits shared memory"); return fail(BGB_ERR_CAPACITY); }
  if ((rc = build_plans(B, problems, St, Sb, cent_t, cent_b, tbase, bbase, first, 1, true, &smem))) return fail(rc);
  auto set_cfg = [&](int cfg, size_t sm) -> int {
    B->cfg_id = cfg;
    B->smem = sm;
    int per_sm = 0;
    int r = far_persistent_occupancy(precision, B->op_kind, B->generic, sm, &per_sm);
    if (r) return r;
    B->ctas = std::max(1, per_sm) * h->num_sms;
    return 0;
  };
  if ((rc = set_cfg(first, smem))) return fail(rc);
  cudaEventRecord(B->ev[0], st);
  if ((rc = enqueue_device_work(B, st, false))) return fail(rc);
  cudaEventRecord(B->ev[1], st);
  BGB_CUDA(cudaStreamSynchronize(st));
  double best_ms = event_ms(B->ev[0], B->ev[1]);
  if (B->host_out && (rc = batch_copy_out(B, st))) return fail(rc);
  int best_cfg = first, best_sched = 1;
  if (autotune) {
    // time the far launch alone for every fitting (shape, schedule)
    best_ms = 1e30;
    for (int c : cands)
      for (int sched = 0; sched < 2; ++sched) {
        if ((rc = build_plans(B, problems, St, Sb, cent_t, cent_b, tbase, bbase, c, sched, false, &smem))) return fail(rc);
        if (smem > (size_t)smem_max) continue;
        if ((rc = build_plans(B, problems, St, Sb, cent_t, cent_b, tbase, bbase, c, sched, true, &smem)) || (rc = set_cfg(c, smem)))
          return fail(rc);
        if ((rc = enqueue_device_work(B, st, true))) return fail(rc);  // warm-up
        cudaEventRecord(B->ev[0], st);
        if ((rc = enqueue_device_work(B, st, true))) return fail(rc);
        cudaEventRecord(B->ev[1], st);
        BGB_CUDA(cudaStreamSynchronize(st));
        const double ms = event_ms(B->ev[0], B->ev[1]);
        if (ms < best_ms) { best_ms = ms; best_cfg = c; best_sched = sched; }
      }
    if ((rc = build_plans(B, problems, St, Sb, cent_t, cent_b, tbase, bbase, best_cfg, best_sched, true, &smem)) ||
        (rc = set_cfg(best_cfg, smem)))
      return fail(rc);
  }
  B->schedule = best_sched;
  // capture the whole device sequence in a CUDA graph
  BGB_CUDA(cudaStreamSynchronize(st));
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) { cuda_fail(e, "cudaStreamBeginCapture"); return fail(BGB_ERR_CUDA); }
  rc = enqueue_device_work(B, st, false);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(st, &g);
  if (rc) { if (g) cudaGraphDestroy(g); return fail(rc); }
  if (e != cudaSuccess) { cuda_fail(e, "cudaStreamEndCapture"); return fail(BGB_ERR_CUDA); }
  B->graph = g;
  e = cudaGraphInstantiate(&B->exec, g, 0);
  if (e != cudaSuccess) { cuda_fail(e, "cudaGraphInstantiate"); return fail(BGB_ERR_CUDA); }
  bgb_stats s{};
  s.pairs_total = pairs_total;
  s.tile_config = best_cfg;
  s.schedule = best_sched;
  s.ms_far = best_ms;
  s.kernel_launches = 0;
  B->stats = s;
  if (stats) *stats = s;
  *out = B;
  return 0;
}

int bgb_batch_run(bgb_batch* B, void* stream, bgb_stats* stats) {
  if (!B) { set_error("invalid batch"); return BGB_ERR_INVALID; }
  bgb_handle* h = B->h;
  std::lock_guard<std::mutex> lk(h->mu);
  cudaSetDevice(h->device);
  *h->abort_host = 0;
  cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
  BGB_CUDA(cudaEventRecord(B->ev[0], s));
  BGB_CUDA(cudaGraphLaunch(B->exec, s));
  BGB_CUDA(cudaEventRecord(B->ev[1], s));
  if (B->host_out) {
    int rc = batch_copy_out(B, s);
    if (rc) return rc;
  }
  if (h->abort_host && *h->abort_host) {
    BGB_CUDA(cudaStreamSynchronize(s));
    set_error("aborted by bgb_abort");
    return BGB_ERR_ABORTED;
  }
  if (stats) {
    BGB_CUDA(cudaEventSynchronize(B->ev[1]));
    bgb_stats st = B->stats;
    st.ms_total = event_ms(B->ev[0], B->ev[1]);
    st.kernel_launches = 1;  // one graph launch (device work: ~11 kernels, one persistent far kernel)
    *stats = st;
  }
  return 0;
}

int bgb_assemble_batch(bgb_handle* h, int32_t n, const bgb_problem* problems, int32_t precision, int32_t out_kind,
                       void* stream, bgb_stats* stats) {
  bgb_batch* B = nullptr;
  int rc = bgb_batch_create(h, n, problems, precision, out_kind, 0, &B, stats);
  if (rc) return rc;
  // bgb_batch_create already ran every stage once and copied host outputs
  if (!B->host_out && stream) {
    cudaEvent_t ev;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess) {
      cudaEventRecord(ev, h->stream);
      cudaStreamWaitEvent((cudaStream_t)stream, ev, 0);
      cudaEventDestroy(ev);
    }
  }
  bgb_batch_destroy(B);
  return rc;
}

}  // extern "C"
