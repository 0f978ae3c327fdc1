// Pair classification into a CSR without any device allocation.
//
// Some callers cannot let a library call cudaMalloc: a Julia (CUDA.jl) or PyTorch process
// whose own pool has already reserved the device memory, or an embedding that hands out
// memory through its own allocator and forbids allocations behind its back.  For them
// bgb_classify_csr_noalloc runs the same count -> scan -> fill classification as
// bgb_assemble, but its scratch (FP64 triangle data, bounding spheres, per-triangle counts)
// lives in one file-scope device array of fixed size; the caller passes the inputs and the
// output buffers, all in device memory.
//
// The array is a per-device global: every device on which the library is loaded holds it
// until the process exits, and every call on that device reuses it.  Calls whose GPU work
// overlaps (different streams, different host threads) race on it and must be serialised by
// the caller.
#include "bgb_kernels.cuh"

#include <cmath>

namespace bgb {
namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)16 << 20;  // 16 MiB per device
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the scratch array on the current device.  Looked up on every call, with
// the caller's device current: the address belongs to the device's current context, and a
// cached address would dangle after the context is reset (cudaDeviceReset, CUDA.jl's
// device_reset!).  The lookup costs far less than the pair-count read-back of every call.
int scratch_address(void** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
  *out = p;
  return 0;
}

// Geometry preparation that checks the caller's vertex indices (device input) and flags a
// bad index instead of reading out of bounds.
__global__ void k_prepare_geo64_checked(const double* __restrict__ verts, const int32_t* __restrict__ tris, int nt,
                                        int nv, Geo64* __restrict__ out, int* __restrict__ err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  Geo64 g;
  for (int a = 0; a < 3; ++a) {
    const int vi = tris[3 * t + a];
    if (vi < 0 || vi >= nv) {  // flagged, and no vertex is read: the triangle gets zero coordinates
      atomicOr(err, 2);
      for (int c = 0; c < 3; ++c) g.v[a][c] = 0.0;
      continue;
    }
    for (int c = 0; c < 3; ++c) g.v[a][c] = verts[3 * (int64_t)vi + c];
  }
  for (int k = 0; k < 2; ++k)
    for (int c = 0; c < 3; ++c) g.t[k][c] = __dsub_rn(g.v[k][c], g.v[2][c]);
  const double n0 = __dsub_rn(__dmul_rn(g.t[0][1], g.t[1][2]), __dmul_rn(g.t[0][2], g.t[1][1]));
  const double n1 = __dsub_rn(__dmul_rn(g.t[0][2], g.t[1][0]), __dmul_rn(g.t[0][0], g.t[1][2]));
  const double n2 = __dsub_rn(__dmul_rn(g.t[0][0], g.t[1][1]), __dmul_rn(g.t[0][1], g.t[1][0]));
  const double s = __dadd_rn(__dadd_rn(__dmul_rn(n0, n0), __dmul_rn(n1, n1)), __dmul_rn(n2, n2));
  g.area = __ddiv_rn(__dsqrt_rn(s), 2.0);
  g.pad = 0.0;
  out[t] = g;
}

inline size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace
}  // namespace bgb

using namespace bgb;

extern "C" int bgb_classify_csr_noalloc(const double* d_vertices_test, const int32_t* d_triangles_test,
                                        int32_t nv_test, int32_t nt_test, const double* d_vertices_trial,
                                        const int32_t* d_triangles_trial, int32_t nv_trial, int32_t nt_trial,
                                        double k2, int64_t* d_offsets, int32_t* d_tau, int32_t* d_sigma,
                                        int8_t* d_class, int64_t capacity, int64_t* total, void* stream) {
  if (!total || nv_test < 0 || nt_test < 0 || nv_trial < 0 || nt_trial < 0 || capacity < 0 || !(k2 >= 0.0) ||
      !std::isfinite(k2)) {
    set_error("bgb_classify_csr_noalloc: invalid sizes, k2 or NULL total");
    return BGB_ERR_INVALID;
  }
  *total = 0;
  // scratch layout: error flag | test Geo64 | trial Geo64 | test bounds | trial bounds | counts
  const size_t need = up256(sizeof(int) * 4) + up256(sizeof(Geo64) * (size_t)nt_test) +
                      up256(sizeof(Geo64) * (size_t)nt_trial) + up256(sizeof(float4) * (size_t)nt_test) +
                      up256(sizeof(float4) * (size_t)nt_trial) + up256(sizeof(int) * ((size_t)nt_test + 1));
  if (need > kNoAllocScratchBytes) {
    set_error("bgb_classify_csr_noalloc: %d test + %d trial triangles need %zu bytes of scratch, more than the "
              "fixed %zu bytes (156 bytes per test and 152 per trial triangle: about 54,000 triangles per side "
              "when both sides are equal); use bgb_assemble / bgb_classify_block",
              nt_test, nt_trial, need, kNoAllocScratchBytes);
    return BGB_ERR_CAPACITY;
  }
  if ((nt_test > 0 && nv_test == 0) || (nt_trial > 0 && nv_trial == 0)) {
    set_error("bgb_classify_csr_noalloc: triangles without vertices (nt > 0 and nv == 0)");
    return BGB_ERR_INVALID;
  }
  if (!d_offsets || (nt_test > 0 && (!d_vertices_test || !d_triangles_test)) ||
      (nt_trial > 0 && (!d_vertices_trial || !d_triangles_trial))) {
    set_error("bgb_classify_csr_noalloc: NULL device input or output");
    return BGB_ERR_INVALID;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  void* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  int num_sms = 0;
  cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  unsigned char* p = (unsigned char*)base;
  int* err = (int*)p;
  p += up256(sizeof(int) * 4);
  Geo64* gt = (Geo64*)p;
  p += up256(sizeof(Geo64) * (size_t)nt_test);
  Geo64* gb = (Geo64*)p;
  p += up256(sizeof(Geo64) * (size_t)nt_trial);
  float4* bt = (float4*)p;
  p += up256(sizeof(float4) * (size_t)nt_test);
  float4* bb = (float4*)p;
  p += up256(sizeof(float4) * (size_t)nt_trial);
  int* counts = (int*)p;

  // the array keeps the previous call's contents: clear the error flag
  BGB_CUDA(cudaMemsetAsync(err, 0, sizeof(int) * 4, st));
  if (nt_test > 0) k_prepare_geo64_checked<<<(nt_test + 255) / 256, 256, 0, st>>>(d_vertices_test, d_triangles_test, nt_test, nv_test, gt, err);
  if (nt_trial > 0) k_prepare_geo64_checked<<<(nt_trial + 255) / 256, 256, 0, st>>>(d_vertices_trial, d_triangles_trial, nt_trial, nv_trial, gb, err);
  launch_prepare_bounds(gt, nt_test, k2, 0, bt, st);
  launch_prepare_bounds(gb, nt_trial, k2, 1, bb, st);
  launch_classify(false, bt, bb, gt, gb, nt_test, nt_trial, k2, counts, nullptr, nullptr, nullptr, nullptr, err,
                  num_sms, st);
  launch_scan(counts, nt_test, d_offsets, st);
  BGB_CUDA(cudaGetLastError());
  int herr = 0;
  int64_t tot = 0;
  BGB_CUDA(cudaMemcpyAsync(&tot, d_offsets + nt_test, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  BGB_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  BGB_CUDA(cudaStreamSynchronize(st));
  *total = tot;
  if (herr & 2) {
    set_error("bgb_classify_csr_noalloc: a triangle has a vertex index outside [0, nv)");
    return BGB_ERR_INVALID;
  }
  if (herr) {
    set_error("bgb_classify_csr_noalloc: degenerate geometry: a triangle pair shares more than three vertices");
    return BGB_ERR_INVALID;
  }
  if (tot > capacity) {
    set_error("bgb_classify_csr_noalloc: %lld non-far pairs do not fit the output capacity %lld", (long long)tot,
              (long long)capacity);
    return BGB_ERR_CAPACITY;
  }
  if (tot > 0 && (!d_tau || !d_sigma || !d_class)) {
    set_error("bgb_classify_csr_noalloc: NULL pair outputs");
    return BGB_ERR_INVALID;
  }
  launch_classify(true, bt, bb, gt, gb, nt_test, nt_trial, k2, counts, d_offsets, d_tau, d_sigma, d_class, err,
                  num_sms, st);
  BGB_CUDA(cudaGetLastError());
  return 0;
}
