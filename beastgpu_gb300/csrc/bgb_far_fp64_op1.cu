// Explicit instantiation of the far-pair tile and diagnostic kernels (PFp64, operator 1).
// Split per precision and operator so nvcc compiles the instances in parallel.
#include "bgb_far_impl.cuh"

namespace bgb {
namespace farimpl {
template int launch_tiles_t<PFp64, 1, 3, 4>(const FarConst&, const TilePlan&, cudaStream_t);
template int launch_tiles_t<PFp64, 1, BGB_MAXQ, BGB_MAXQ>(const FarConst&, const TilePlan&, cudaStream_t);
template int launch_diag_t<PFp64, 1, 3, 4>(const FarConst&, const void*, const void*, const int*, const int*, int64_t, double2*, cudaStream_t);
template int launch_diag_t<PFp64, 1, BGB_MAXQ, BGB_MAXQ>(const FarConst&, const void*, const void*, const int*, const int*, int64_t, double2*, cudaStream_t);
}  // namespace farimpl
}  // namespace bgb
