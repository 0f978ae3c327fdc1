// Explicit instantiation of the far-pair tile and diagnostic kernels (PFp64, operator 3).
// Split per precision and operator so nvcc compiles the instances in parallel.
#include "bgb_far_impl.cuh"

namespace bgb {
namespace farimpl {
template int launch_diag_t<PFp64, 3, 3, 4>(const FarConst&, const void*, const void*, const int*, const int*, int64_t, double2*, cudaStream_t);
template int launch_diag_t<PFp64, 3, BGB_MAXQ, BGB_MAXQ>(const FarConst&, const void*, const void*, const int*, const int*, int64_t, double2*, cudaStream_t);
template int launch_persistent_t<PFp64, 3, 3, 4>(const FarConst*, const TilePlan*, const int4*, int, int*, size_t, int, const volatile int*, cudaStream_t);
template int launch_persistent_t<PFp64, 3, BGB_MAXQ, BGB_MAXQ>(const FarConst*, const TilePlan*, const int4*, int, int*, size_t, int, const volatile int*, cudaStream_t);
template int occupancy_t<PFp64, 3, 3, 4>(size_t, int*);
template int occupancy_t<PFp64, 3, BGB_MAXQ, BGB_MAXQ>(size_t, int*);
}  // namespace farimpl
}  // namespace bgb
