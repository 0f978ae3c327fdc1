// Issue-rate probes for roofline denominators: FP32 FMA, FP64 FMA and MUFU (sin) throughput
// of the current device, measured with independent dependency chains per thread (no memory
// traffic).  The far-pair kernels are bound by these pipes, not by HBM or tensor cores.
#include "bgb_kernels.cuh"

namespace bgb {
namespace {

template <int CH>
__global__ void k_fma32(float* out, int iters, float a, float b) {
  float x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = threadIdx.x * 1e-3f + c;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < CH; ++c) x[c] = fmaf(x[c], a, b);
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  if (s == 1234.5f) out[0] = s;
}

template <int CH>
__global__ void k_fma64(double* out, int iters, double a, double b) {
  double x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = threadIdx.x * 1e-3 + c;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < CH; ++c) x[c] = fma(x[c], a, b);
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  if (s == 1234.5) out[0] = s;
}

template <int CH>
__global__ void k_mufu(float* out, int iters) {
  float x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = 0.5f + threadIdx.x * 1e-5f + c * 1e-3f;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < CH; ++c) x[c] = __sinf(x[c]);
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  if (s == 1234.5f) out[0] = s;
}

}  // namespace

int measure_issue_peaks(int num_sms, double* fp32, double* fp64, double* mufu) {
  float* o32 = nullptr;
  double* o64 = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  BGB_CUDA(cudaMalloc(&o32, 64));
  BGB_CUDA(cudaMalloc(&o64, 64));
  BGB_CUDA(cudaEventCreate(&e0));
  BGB_CUDA(cudaEventCreate(&e1));
  const int blocks = num_sms * 8, threads = 256;
  double best32 = 0, best64 = 0, bestm = 0;
  for (int rep = 0; rep < 3; ++rep) {
    float ms = 0.f;
    const int it32 = 20000, it64 = 2000;
    cudaEventRecord(e0);
    k_fma32<8><<<blocks, threads>>>(o32, it32, 0.999f, 0.001f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    best32 = fmax(best32, 2.0 * 8 * (double)it32 * blocks * threads / (ms * 1e-3) / 1e12);
    cudaEventRecord(e0);
    k_fma64<8><<<blocks, threads>>>(o64, it64, 0.999, 0.001);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    best64 = fmax(best64, 2.0 * 8 * (double)it64 * blocks * threads / (ms * 1e-3) / 1e12);
    cudaEventRecord(e0);
    k_mufu<8><<<blocks, threads>>>(o32, it32);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    bestm = fmax(bestm, 8.0 * it32 * blocks * threads / (ms * 1e-3) / 1e12);
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(o32);
  cudaFree(o64);
  if (err != cudaSuccess) return cuda_fail(err, "issue-peak probes");
  *fp32 = best32;
  *fp64 = best64;
  *mufu = bestm;
  return 0;
}

}  // namespace bgb
