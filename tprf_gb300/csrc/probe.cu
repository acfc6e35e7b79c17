// Device-capability probe: sustained FP64 FMA throughput of the current GPU.
//
// The bubble / RPA kernels are bound by the FP64 pipe on GB300, so the
// benchmark reports their FP64 fraction against this number, measured live
// on the same device. Every thread runs 8 independent FMA chains; the loop
// count is fixed, so the kernel always terminates.
#include <algorithm>

#include "common.cuh"

namespace tprf {
namespace {

constexpr int kProbeIters = 4096;

__global__ void __launch_bounds__(256) fp64_fma_probe(double *out, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
#pragma unroll 4
  for (int i = 0; i < kProbeIters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * (long)blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace
}  // namespace tprf

extern "C" int tprf_measure_fp64_tflops(double *tflops, void *scratch, size_t scratch_bytes, void *stream) {
  using namespace tprf;
  if (!tflops || !scratch) return set_error(TPRF_ERR_INVALID_ARGUMENT, "measure_fp64_tflops: null pointer");
  const int threads = 256, blocks = num_sms() * 8;
  if (scratch_bytes < (size_t)threads * blocks * sizeof(double))
    return set_error(TPRF_ERR_ALLOC, "measure_fp64_tflops: scratch needs 2048 doubles per SM");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  TPRF_CUDA(cudaEventCreate(&e0));
  TPRF_CUDA(cudaEventCreate(&e1));
  double best = 0.0;
  for (int rep = 0; rep < 3; ++rep) {
    TPRF_CUDA(cudaEventRecord(e0, s));
    fp64_fma_probe<<<blocks, threads, 0, s>>>(static_cast<double *>(scratch), 1.0000001, 1e-9);
    TPRF_CUDA(cudaEventRecord(e1, s));
    TPRF_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    TPRF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    const double flops = 2.0 * 8.0 * kProbeIters * (double)threads * blocks;
    if (ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  TPRF_KERNEL_LAUNCHED("fp64_fma_probe");
  *tflops = best;
  return TPRF_OK;
}
