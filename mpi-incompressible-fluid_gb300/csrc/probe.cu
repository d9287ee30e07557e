// Instrumentation: the FP64 fused multiply-add rate of the current device.
// The plain FP64 step does its arithmetic on the FP64 pipe, whose rate on
// GB300 is a small fraction of the FP32 one; this rate is the step's second
// roofline, beside HBM bandwidth.
#include <cuda_runtime.h>

#include "../../include/mifgpu.h"

namespace {

constexpr int kChains = 8;    // independent FMA chains per thread
constexpr int kThreads = 256;
constexpr int kBlocksPerSm = 8;

// Every thread runs kChains independent chains x = fma(x, a, b); a and b keep
// the values bounded. The sum is stored only if it equals -1, which never
// happens for these inputs, but the compiler cannot drop the chains.
__global__ void __launch_bounds__(kThreads) fp64_fma_probe_kernel(double *sink, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = 1e-3 * (double)(threadIdx.x + c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == -1.0) sink[blockIdx.x] = s;
}

}  // namespace

extern "C" int mifgpu_probe_fp64_fma(double *tflops) {
  if (!tflops) return MIFGPU_EINVAL;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
    return MIFGPU_ECUDA;
  const int blocks = sms * kBlocksPerSm, iters = 4096;
  double *sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = MIFGPU_ECUDA;
  if (cudaMalloc(&sink, sizeof(double) * blocks) == cudaSuccess && cudaEventCreate(&e0) == cudaSuccess &&
      cudaEventCreate(&e1) == cudaSuccess) {
    fp64_fma_probe_kernel<<<blocks, kThreads>>>(sink, iters, 0.9999999, 1e-9);  // warm-up
    cudaEventRecord(e0);
    fp64_fma_probe_kernel<<<blocks, kThreads>>>(sink, iters, 0.9999999, 1e-9);
    cudaEventRecord(e1);
    float ms = 0.f;
    if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.f) {
      const double flops = 2.0 * kChains * (double)iters * blocks * kThreads;
      *tflops = flops / (ms * 1e-3) / 1e12;
      rc = MIFGPU_OK;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (sink) cudaFree(sink);
  return rc;
}
