// Host-side tile planning of the far-pair kernel: bisection order of the functions, supports,
// and the per-tile tables (triangles of a block of test / trial functions, the slot and local
// shape of each support, the trial-side groups per chunk).  The plan of one side is built in
// parallel over ranges of function blocks and merged by shifting offsets, so the result does
// not depend on the number of threads.
#include "bgb_host.h"

#include <algorithm>
#include <cstdint>
#include <thread>
#include <vector>

namespace bgb {

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

// Centre of every function: the mean of the centroids of its support triangles.
std::vector<double> function_centres(const bgb_space* s, const Supports& S) {
  std::vector<double> tc(3 * (size_t)s->nt);
  for (int64_t t = 0; t < s->nt; ++t)
    for (int k = 0; k < 3; ++k) {
      double v = 0;
      for (int a = 0; a < 3; ++a) v += s->vertices[3 * (int64_t)s->triangles[3 * t + a] + k];
      tc[3 * (size_t)t + k] = v / 3.0;
    }
  std::vector<double> fc(3 * (size_t)s->nfun, 0.0);
  for (int f = 0; f < s->nfun; ++f) {
    const int64_t n = S.off[f + 1] - S.off[f];
    if (n == 0) continue;
    for (int64_t k = S.off[f]; k < S.off[f + 1]; ++k)
      for (int c = 0; c < 3; ++c) fc[3 * (size_t)f + c] += tc[3 * (size_t)S.tri[k] + c];
    for (int c = 0; c < 3; ++c) fc[3 * (size_t)f + c] /= (double)n;
  }
  return fc;
}

// Functions [f_begin, f_end) in the order of a recursive coordinate bisection of their centres:
// a range is split across its longest extent at a multiple of `leaf` functions near its middle,
// down to ranges of at most `leaf`, so every aligned run of `leaf` functions (a tile of the far
// kernel) is a compact patch and the triangles its supports share are few.  Ties go by function
// index, each leaf is in index order (the order does not depend on the sort's implementation),
// and functions without supports come last.  The first levels are split on the calling thread,
// the ranges below them on up to nth threads; the result does not depend on nth.
std::vector<int> order_functions(const Supports& S, const std::vector<double>& centre, int f_begin, int f_end,
                                 int leaf, int nth) {
  leaf = std::max(1, leaf);
  std::vector<int> idx, none;
  idx.reserve((size_t)std::max(0, f_end - f_begin));
  for (int f = f_begin; f < f_end; ++f) (S.off[f + 1] > S.off[f] ? idx : none).push_back(f);
  struct Range { size_t lo, hi; };
  // one bisection step of r (n > leaf) into its two halves
  auto split = [&](const Range& r, Range& a, Range& b) {
    const size_t n = r.hi - r.lo;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (size_t i = r.lo; i < r.hi; ++i)
      for (int c = 0; c < 3; ++c) {
        const double v = centre[3 * (size_t)idx[i] + c];
        lo[c] = std::min(lo[c], v);
        hi[c] = std::max(hi[c], v);
      }
    int ax = 0;
    for (int c = 1; c < 3; ++c)
      if (hi[c] - lo[c] > hi[ax] - lo[ax]) ax = c;
    size_t nl = (n / 2 + (size_t)leaf / 2) / (size_t)leaf * (size_t)leaf;
    nl = std::min(std::max(nl, (size_t)leaf), n - 1);
    std::nth_element(idx.begin() + (std::ptrdiff_t)r.lo, idx.begin() + (std::ptrdiff_t)(r.lo + nl),
                     idx.begin() + (std::ptrdiff_t)r.hi, [&](int x, int y) {
                       const double vx = centre[3 * (size_t)x + ax], vy = centre[3 * (size_t)y + ax];
                       return vx < vy || (vx == vy && x < y);
                     });
    a = {r.lo, r.lo + nl};
    b = {r.lo + nl, r.hi};
  };
  // the whole bisection below r
  auto finish = [&](const Range& root) {
    std::vector<Range> stack{root};
    while (!stack.empty()) {
      const Range r = stack.back();
      stack.pop_back();
      if (r.hi - r.lo <= (size_t)leaf) {
        std::sort(idx.begin() + (std::ptrdiff_t)r.lo, idx.begin() + (std::ptrdiff_t)r.hi);
        continue;
      }
      Range a, b;
      split(r, a, b);
      stack.push_back(a);
      stack.push_back(b);
    }
  };
  nth = std::max(1, nth);
  std::vector<Range> level{{0, idx.size()}};
  while (nth > 1 && level.size() < 4 * (size_t)nth) {
    std::vector<Range> next;
    bool any = false;
    for (const Range& r : level) {
      if (r.hi - r.lo <= (size_t)leaf) {
        next.push_back(r);
        continue;
      }
      Range a, b;
      split(r, a, b);
      next.push_back(a);
      next.push_back(b);
      any = true;
    }
    level.swap(next);
    if (!any) break;
  }
  if (nth == 1 || level.size() == 1) {
    for (const Range& r : level) finish(r);
  } else {
    std::vector<std::thread> th;
    const int nt = (int)std::min<size_t>((size_t)nth, level.size());
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&, t] {
        for (size_t i = (size_t)t; i < level.size(); i += (size_t)nt) finish(level[i]);
      });
    for (auto& x : th) x.join();
  }
  idx.insert(idx.end(), none.begin(), none.end());
  return idx;
}

void plan_test_side(const Supports& S, const std::vector<int>& order, int FM, int64_t row0, HostPlan& P, int tcap) {
  P.tb_off.push_back(0);
  P.tb_fn_off.push_back(0);
  P.fs_off.push_back(0);
  std::vector<int> tris;
  // stamp[t] == b0: triangle t is already in the block starting at b0; slot[t]: its position
  // in the block's sorted triangles
  int ntri = 0;
  size_t nsup = 0;
  for (size_t i = 0; i < order.size(); ++i) {
    for (int64_t k = S.off[order[i]]; k < S.off[order[i] + 1]; ++k) ntri = std::max(ntri, S.tri[k] + 1);
    nsup += (size_t)(S.off[order[i] + 1] - S.off[order[i]]);
  }
  std::vector<int64_t> stamp((size_t)ntri, -1);
  std::vector<int> slot_of((size_t)ntri, 0);
  P.fs_code.reserve(P.fs_code.size() + nsup);
  P.fs_coef.reserve(P.fs_coef.size() + nsup);
  P.rows.reserve(P.rows.size() + order.size());
  P.fs_off.reserve(P.fs_off.size() + order.size());
  size_t b0 = 0;
  while (b0 < order.size()) {
    // a block takes up to FM functions while its distinct triangles stay within tcap
    size_t b1 = b0;
    tris.clear();
    while (b1 < order.size() && b1 - b0 < (size_t)FM) {
      const int f = order[b1];
      int fresh = 0;
      for (int64_t k = S.off[f]; k < S.off[f + 1]; ++k)
        if (stamp[(size_t)S.tri[k]] != (int64_t)b0) ++fresh;
      if (b1 > b0 && (int)tris.size() + fresh > tcap) break;
      for (int64_t k = S.off[f]; k < S.off[f + 1]; ++k)
        if (stamp[(size_t)S.tri[k]] != (int64_t)b0) {
          stamp[(size_t)S.tri[k]] = (int64_t)b0;
          tris.push_back(S.tri[k]);
        }
      ++b1;
    }
    std::sort(tris.begin(), tris.end());
    for (size_t i = 0; i < tris.size(); ++i) slot_of[(size_t)tris[i]] = (int)i;
    for (size_t i = b0; i < b1; ++i) {
      int f = order[i];
      int cnt = 0;
      for (int64_t k = S.off[f]; k < S.off[f + 1]; ++k) {
        const int slot = slot_of[(size_t)S.tri[k]];
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
    b0 = b1;
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
  std::vector<Ent> ents, sorted;
  std::vector<int> ccnt;
  // stamp[t] == b0: triangle t is already in the block starting at b0; slot_of[t]: its position
  // in the block's sorted triangles
  int ntri = 0;
  size_t nsup = 0;
  for (size_t i = 0; i < order.size(); ++i) {
    for (int64_t k = S.off[order[i]]; k < S.off[order[i] + 1]; ++k) ntri = std::max(ntri, S.tri[k] + 1);
    nsup += (size_t)(S.off[order[i] + 1] - S.off[order[i]]);
  }
  std::vector<int64_t> stamp((size_t)ntri, -1);
  std::vector<int> slot_of((size_t)ntri, 0);
  P.gs_code.reserve(P.gs_code.size() + nsup);
  P.gs_coef.reserve(P.gs_coef.size() + nsup);
  P.cols.reserve(P.cols.size() + order.size());
  for (size_t b0 = 0; b0 < order.size(); b0 += FN) {
    size_t b1 = std::min(order.size(), b0 + FN);
    tris.clear();
    for (size_t i = b0; i < b1; ++i) {
      int f = order[i];
      for (int64_t k = S.off[f]; k < S.off[f + 1]; ++k)
        if (stamp[(size_t)S.tri[k]] != (int64_t)b0) {
          stamp[(size_t)S.tri[k]] = (int64_t)b0;
          tris.push_back(S.tri[k]);
        }
    }
    std::sort(tris.begin(), tris.end());
    for (size_t i = 0; i < tris.size(); ++i) slot_of[(size_t)tris[i]] = (int)i;
    ents.clear();
    for (size_t i = b0; i < b1; ++i) {
      int f = order[i];
      for (int64_t k = S.off[f]; k < S.off[f + 1]; ++k) {
        const int slot = slot_of[(size_t)S.tri[k]];
        ents.push_back({slot / SC, (int)(i - b0), slot, S.loc[k], S.coef[k]});
      }
    }
    // groups: per chunk, per local function, supports by slot (= trial triangle) ascending.
    // The entries were made in (local function, slot) order (supports are sorted by triangle),
    // so a stable counting sort by chunk orders them by (chunk, local function, slot).
    int nchunks = ((int)tris.size() + SC - 1) / SC;
    ccnt.assign((size_t)nchunks + 1, 0);
    for (const Ent& x : ents) ++ccnt[(size_t)x.chunk + 1];
    for (int c = 0; c < nchunks; ++c) ccnt[(size_t)c + 1] += ccnt[(size_t)c];
    sorted.resize(ents.size());
    for (const Ent& x : ents) sorted[(size_t)ccnt[(size_t)x.chunk]++] = x;
    ents.swap(sorted);
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


int planner_threads() {
  const unsigned hw = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(8u, hw ? hw / 2 : 1u));
}

// Plans are built over fixed ranges of kRangeFns functions (tiles never straddle a range),
// in parallel threads, and merged in range order: the result is the same for any thread count.
static constexpr size_t kRangeFns = 6720;  // a multiple of every tile width (16 .. 96)

template <class F>
static void for_ranges(size_t nfun, int nth, F fn) {
  const size_t nr = (nfun + kRangeFns - 1) / kRangeFns;
  const int nt = (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(1, nth), nr));
  auto work = [&](int t) {
    for (size_t r = t; r < nr; r += nt) fn(r, r * kRangeFns, std::min(nfun, (r + 1) * kRangeFns));
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& x : th) x.join();
}

void plan_test_side_par(const Supports& S, const std::vector<int>& order, int FM, int64_t row0, HostPlan& P, int nth,
                        int tcap) {
  const size_t nr = std::max<size_t>(1, (order.size() + kRangeFns - 1) / kRangeFns);
  std::vector<HostPlan> sub(nr);
  for_ranges(order.size(), nth, [&](size_t r, size_t f0, size_t f1) {
    std::vector<int> ord(order.begin() + f0, order.begin() + f1);
    plan_test_side(S, ord, FM, row0, sub[r], tcap);
  });
  if (order.empty()) plan_test_side(S, order, FM, row0, sub[0], tcap);
  P.tb_off.push_back(0);
  P.tb_fn_off.push_back(0);
  P.fs_off.push_back(0);
  for (size_t t = 0; t < nr; ++t) {
    const HostPlan& Q = sub[t];
    const int tb_base = (int)P.tb_tris.size(), fs_base = (int)P.fs_code.size(), fn_base = (int)(t * kRangeFns);
    for (size_t i = 1; i < Q.tb_off.size(); ++i) P.tb_off.push_back(Q.tb_off[i] + tb_base);
    for (size_t i = 1; i < Q.tb_fn_off.size(); ++i) P.tb_fn_off.push_back(Q.tb_fn_off[i] + fn_base);
    for (size_t i = 1; i < Q.fs_off.size(); ++i) P.fs_off.push_back(Q.fs_off[i] + fs_base);
    P.tb_tris.insert(P.tb_tris.end(), Q.tb_tris.begin(), Q.tb_tris.end());
    P.fs_code.insert(P.fs_code.end(), Q.fs_code.begin(), Q.fs_code.end());
    P.fs_coef.insert(P.fs_coef.end(), Q.fs_coef.begin(), Q.fs_coef.end());
    P.rows.insert(P.rows.end(), Q.rows.begin(), Q.rows.end());
    P.MAXS = std::max(P.MAXS, Q.MAXS);
    P.tmax = std::max(P.tmax, Q.tmax);
  }
}

void plan_trial_side_par(const Supports& S, const std::vector<int>& order, int FN, int SC, HostPlan& P, int nth) {
  const size_t nr = std::max<size_t>(1, (order.size() + kRangeFns - 1) / kRangeFns);
  std::vector<HostPlan> sub(nr);
  for_ranges(order.size(), nth, [&](size_t r, size_t f0, size_t f1) {
    std::vector<int> ord(order.begin() + f0, order.begin() + f1);
    plan_trial_side(S, ord, FN, SC, sub[r]);
  });
  if (order.empty()) plan_trial_side(S, order, FN, SC, sub[0]);
  const int parts = (int)nr;
  std::vector<size_t> first(nr);
  for (size_t r = 0; r < nr; ++r) first[r] = r * kRangeFns;
  P.bb_off.push_back(0);
  P.bb_fn_off.push_back(0);
  P.bb_chunk_off.push_back(0);
  P.ch_grp_off.push_back(0);
  P.grp_sup_off.push_back(0);
  for (int t = 0; t < parts; ++t) {
    const HostPlan& Q = sub[t];
    const int bb_base = (int)P.bb_tris.size(), fn_base = (int)first[t], ch_base = P.bb_chunk_off.back(),
              grp_base = (int)P.grp_fn.size(), gs_base = (int)P.gs_code.size();
    for (size_t i = 1; i < Q.bb_off.size(); ++i) P.bb_off.push_back(Q.bb_off[i] + bb_base);
    for (size_t i = 1; i < Q.bb_fn_off.size(); ++i) P.bb_fn_off.push_back(Q.bb_fn_off[i] + fn_base);
    for (size_t i = 1; i < Q.bb_chunk_off.size(); ++i) P.bb_chunk_off.push_back(Q.bb_chunk_off[i] + ch_base);
    for (size_t i = 1; i < Q.ch_grp_off.size(); ++i) P.ch_grp_off.push_back(Q.ch_grp_off[i] + grp_base);
    for (size_t i = 1; i < Q.grp_sup_off.size(); ++i) P.grp_sup_off.push_back(Q.grp_sup_off[i] + gs_base);
    P.bb_tris.insert(P.bb_tris.end(), Q.bb_tris.begin(), Q.bb_tris.end());
    P.grp_fn.insert(P.grp_fn.end(), Q.grp_fn.begin(), Q.grp_fn.end());
    P.gs_code.insert(P.gs_code.end(), Q.gs_code.begin(), Q.gs_code.end());
    P.gs_coef.insert(P.gs_coef.end(), Q.gs_coef.begin(), Q.gs_coef.end());
    P.cols.insert(P.cols.end(), Q.cols.begin(), Q.cols.end());
    P.gmax = std::max(P.gmax, Q.gmax);
    P.gsmax = std::max(P.gsmax, Q.gsmax);
    P.nmax = std::max(P.nmax, Q.nmax);
  }
}

}  // namespace bgb
