// Far-pair dispatch (precision x operator x rule instance) and record preparation.
#include "bgb_far_impl.cuh"

namespace bgb {
namespace farimpl {
BGB_FAR_EXTERN(PMixed, 0)
BGB_FAR_EXTERN(PMixed, 1)
BGB_FAR_EXTERN(PMixed, 2)
BGB_FAR_EXTERN(PMixed, 3)
BGB_FAR_EXTERN(PMixed, 4)
BGB_FAR_EXTERN(PMixed, 5)
BGB_FAR_EXTERN(PFp64, 0)
BGB_FAR_EXTERN(PFp64, 1)
BGB_FAR_EXTERN(PFp64, 2)
BGB_FAR_EXTERN(PFp64, 3)
BGB_FAR_EXTERN(PFp64, 4)
BGB_FAR_EXTERN(PFp64, 5)

template <class P, int QT, int QB>
static int dispatch_diag(const FarConst& K, const void* rt, const void* rb, const int* tau, const int* sigma,
                         int64_t n, double2* out, cudaStream_t st) {
  switch (K.op_kind) {
    case BGB_OP_HELMHOLTZ3D_SL: return launch_diag_t<P, BGB_OP_HELMHOLTZ3D_SL, QT, QB>(K, rt, rb, tau, sigma, n, out, st);
    case BGB_OP_MAXWELL3D_SL: return launch_diag_t<P, BGB_OP_MAXWELL3D_SL, QT, QB>(K, rt, rb, tau, sigma, n, out, st);
    case BGB_OP_MAXWELL3D_DL: return launch_diag_t<P, BGB_OP_MAXWELL3D_DL, QT, QB>(K, rt, rb, tau, sigma, n, out, st);
    case BGB_OP_HELMHOLTZ3D_DL: return launch_diag_t<P, BGB_OP_HELMHOLTZ3D_DL, QT, QB>(K, rt, rb, tau, sigma, n, out, st);
    case BGB_OP_HELMHOLTZ3D_DLT: return launch_diag_t<P, BGB_OP_HELMHOLTZ3D_DLT, QT, QB>(K, rt, rb, tau, sigma, n, out, st);
    case BGB_OP_HELMHOLTZ3D_HS: return launch_diag_t<P, BGB_OP_HELMHOLTZ3D_HS, QT, QB>(K, rt, rb, tau, sigma, n, out, st);
  }
  set_error("unknown operator kind %d", K.op_kind);
  return BGB_ERR_INVALID;
}
template <class P, int QT, int QB>
static int dispatch_persistent(int op_kind, const FarConst* Ks, const TilePlan* plans, const int4* items, int nitems,
                               int* counter, size_t smem, int ctas, const volatile int* ab, cudaStream_t st) {
  switch (op_kind) {
    case BGB_OP_HELMHOLTZ3D_SL:
      return launch_persistent_t<P, BGB_OP_HELMHOLTZ3D_SL, QT, QB>(Ks, plans, items, nitems, counter, smem, ctas, ab, st);
    case BGB_OP_MAXWELL3D_SL:
      return launch_persistent_t<P, BGB_OP_MAXWELL3D_SL, QT, QB>(Ks, plans, items, nitems, counter, smem, ctas, ab, st);
    case BGB_OP_MAXWELL3D_DL:
      return launch_persistent_t<P, BGB_OP_MAXWELL3D_DL, QT, QB>(Ks, plans, items, nitems, counter, smem, ctas, ab, st);
    case BGB_OP_HELMHOLTZ3D_DL:
      return launch_persistent_t<P, BGB_OP_HELMHOLTZ3D_DL, QT, QB>(Ks, plans, items, nitems, counter, smem, ctas, ab, st);
    case BGB_OP_HELMHOLTZ3D_DLT:
      return launch_persistent_t<P, BGB_OP_HELMHOLTZ3D_DLT, QT, QB>(Ks, plans, items, nitems, counter, smem, ctas, ab, st);
    case BGB_OP_HELMHOLTZ3D_HS:
      return launch_persistent_t<P, BGB_OP_HELMHOLTZ3D_HS, QT, QB>(Ks, plans, items, nitems, counter, smem, ctas, ab, st);
  }
  set_error("unknown operator kind %d", op_kind);
  return BGB_ERR_INVALID;
}

template <class P, int QT, int QB>
static int dispatch_occupancy(int op_kind, size_t smem, int* per_sm) {
  switch (op_kind) {
    case BGB_OP_HELMHOLTZ3D_SL: return occupancy_t<P, BGB_OP_HELMHOLTZ3D_SL, QT, QB>(smem, per_sm);
    case BGB_OP_MAXWELL3D_SL: return occupancy_t<P, BGB_OP_MAXWELL3D_SL, QT, QB>(smem, per_sm);
    case BGB_OP_MAXWELL3D_DL: return occupancy_t<P, BGB_OP_MAXWELL3D_DL, QT, QB>(smem, per_sm);
    case BGB_OP_HELMHOLTZ3D_DL: return occupancy_t<P, BGB_OP_HELMHOLTZ3D_DL, QT, QB>(smem, per_sm);
    case BGB_OP_HELMHOLTZ3D_DLT: return occupancy_t<P, BGB_OP_HELMHOLTZ3D_DLT, QT, QB>(smem, per_sm);
    case BGB_OP_HELMHOLTZ3D_HS: return occupancy_t<P, BGB_OP_HELMHOLTZ3D_HS, QT, QB>(smem, per_sm);
  }
  set_error("unknown operator kind %d", op_kind);
  return BGB_ERR_INVALID;
}
}  // namespace farimpl

using namespace farimpl;

int launch_far_persistent(int precision, int op_kind, int generic, const FarConst* Ks, const TilePlan* plans,
                          const int4* items, int nitems, int* counter, size_t smem_bytes, int ctas,
                          const volatile int* abort_flag, cudaStream_t st) {
  if (precision == BGB_PREC_MIXED)
    return generic ? dispatch_persistent<PMixed, BGB_MAXQ, BGB_MAXQ>(op_kind, Ks, plans, items, nitems, counter, smem_bytes, ctas, abort_flag, st)
                   : dispatch_persistent<PMixed, 3, 4>(op_kind, Ks, plans, items, nitems, counter, smem_bytes, ctas, abort_flag, st);
  return generic ? dispatch_persistent<PFp64, BGB_MAXQ, BGB_MAXQ>(op_kind, Ks, plans, items, nitems, counter, smem_bytes, ctas, abort_flag, st)
                 : dispatch_persistent<PFp64, 3, 4>(op_kind, Ks, plans, items, nitems, counter, smem_bytes, ctas, abort_flag, st);
}

int far_persistent_occupancy(int precision, int op_kind, int generic, size_t smem_bytes, int* per_sm) {
  if (precision == BGB_PREC_MIXED)
    return generic ? dispatch_occupancy<PMixed, BGB_MAXQ, BGB_MAXQ>(op_kind, smem_bytes, per_sm)
                   : dispatch_occupancy<PMixed, 3, 4>(op_kind, smem_bytes, per_sm);
  return generic ? dispatch_occupancy<PFp64, BGB_MAXQ, BGB_MAXQ>(op_kind, smem_bytes, per_sm)
                 : dispatch_occupancy<PFp64, 3, 4>(op_kind, smem_bytes, per_sm);
}

int far_generic_q(int qt, int qb) { return !(qt == 3 && qb == 4); }

int far_target_ctas_per_sm(int precision) {
  return precision == BGB_PREC_MIXED ? PMixed::kMinBlocks : PFp64::kMinBlocks;
}

int rec_stride(int precision, int q, int generic) {
  const int Q = generic ? BGB_MAXQ : q;
  return precision == BGB_PREC_MIXED ? farimpl::off32_size(Q) : 13 + 4 * Q;
}

size_t far_smem_bytes(int precision, int op_kind, int qt, int qb, const TilePlan& p) {
  const bool gen = far_generic_q(qt, qb);
  // the layout depends on the operator only through chunk_trial_records (Lagrange or RWG)
  const bool lag = is_lagrange_op(op_kind);
  if (precision == BGB_PREC_MIXED)
    return gen ? (lag ? smem_t<PMixed, BGB_OP_HELMHOLTZ3D_SL, BGB_MAXQ, BGB_MAXQ>(p)
                      : smem_t<PMixed, BGB_OP_MAXWELL3D_SL, BGB_MAXQ, BGB_MAXQ>(p))
               : (lag ? smem_t<PMixed, BGB_OP_HELMHOLTZ3D_SL, 3, 4>(p) : smem_t<PMixed, BGB_OP_MAXWELL3D_SL, 3, 4>(p));
  return gen ? smem_t<PFp64, 0, BGB_MAXQ, BGB_MAXQ>(p) : smem_t<PFp64, 0, 3, 4>(p);
}

int launch_far_pairs_diag(int precision, const FarConst& k, const void* rt, const void* rb, const int* tau,
                          const int* sigma, int64_t n, double2* out, cudaStream_t st) {
  const bool gen = far_generic_q(k.qt, k.qb);
  if (precision == BGB_PREC_MIXED)
    return gen ? dispatch_diag<PMixed, BGB_MAXQ, BGB_MAXQ>(k, rt, rb, tau, sigma, n, out, st)
               : dispatch_diag<PMixed, 3, 4>(k, rt, rb, tau, sigma, n, out, st);
  return gen ? dispatch_diag<PFp64, BGB_MAXQ, BGB_MAXQ>(k, rt, rb, tau, sigma, n, out, st)
             : dispatch_diag<PFp64, 3, 4>(k, rt, rb, tau, sigma, n, out, st);
}

void launch_prepare_rec(int precision, int side, int q, const Geo64* g, int nt, const RuleTable& rules, int rule,
                        double wscale, void* out, cudaStream_t st) {
  (void)side;
  if (nt <= 0) return;
  const int blocks = (nt + 127) / 128;
  const bool gen = (q == BGB_MAXQ);
  if (precision == BGB_PREC_MIXED) {
    if (gen) k_prepare_rec32<BGB_MAXQ><<<blocks, 128, 0, st>>>(g, nt, rules, rule, wscale, (float*)out);
    else if (q == 3) k_prepare_rec32<3><<<blocks, 128, 0, st>>>(g, nt, rules, rule, wscale, (float*)out);
    else k_prepare_rec32<4><<<blocks, 128, 0, st>>>(g, nt, rules, rule, wscale, (float*)out);
  } else {
    if (gen) k_prepare_rec64<BGB_MAXQ><<<blocks, 128, 0, st>>>(g, nt, rules, rule, wscale, (double*)out);
    else if (q == 3) k_prepare_rec64<3><<<blocks, 128, 0, st>>>(g, nt, rules, rule, wscale, (double*)out);
    else k_prepare_rec64<4><<<blocks, 128, 0, st>>>(g, nt, rules, rule, wscale, (double*)out);
  }
}

}  // namespace bgb
