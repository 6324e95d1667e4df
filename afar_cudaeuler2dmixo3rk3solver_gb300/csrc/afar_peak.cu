// afar_measure_fp64_peak: the FP64 fused multiply-add rate of the device, measured.
//
// The fp64 policy's face flux and update are bound by the FP64 pipe, not by HBM (GB300 runs FP64
// at a small fraction of its FP32 rate), so their roofline is the measured DFMA rate.  The kernel
// keeps eight independent FMA chains per thread over a grid of several blocks per SM, so the pipe
// never waits on a dependency; each DFMA counts as two floating-point operations.  The chains stay
// bounded (x <- x a + b with |a| < 1) and their sum is stored, so nothing is optimised away.
#include <cuda_runtime.h>

#include "afar_internal.h"

namespace {

constexpr int kPeakThreads = 256;
constexpr int kChains = 8;

__global__ void __launch_bounds__(kPeakThreads) k_dfma_loop(double* sink, const int iters, const double a,
                                                            const double b) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) x[k] = 1e-3 * (threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += x[k];
  sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

using afar::set_error;

#define PEAK_CUDA(call)                                          \
  do {                                                           \
    cudaError_t e_ = (call);                                     \
    if (e_ != cudaSuccess) {                                     \
      set_error("%s failed: %s", #call, cudaGetErrorString(e_)); \
      if (sink) cudaFree(sink);                                  \
      if (ev[0]) cudaEventDestroy(ev[0]);                        \
      if (ev[1]) cudaEventDestroy(ev[1]);                        \
      return AFAR_ERR_CUDA;                                      \
    }                                                            \
  } while (0)

extern "C" afar_status afar_measure_fp64_peak(int device, double* gflops, float* ms) {
  double* sink = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  if (!gflops) {
    set_error("afar_measure_fp64_peak: null output");
    return AFAR_ERR_ARGUMENT;
  }
  PEAK_CUDA(cudaSetDevice(device));
  int sms = 0;
  PEAK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int blocks = sms * 8;  // 8 blocks of 256 threads: 64 warps, a full SM
  const int iters = 1 << 14;
  PEAK_CUDA(cudaMalloc(&sink, sizeof(double) * (size_t)blocks * kPeakThreads));
  PEAK_CUDA(cudaEventCreate(&ev[0]));
  PEAK_CUDA(cudaEventCreate(&ev[1]));
  k_dfma_loop<<<blocks, kPeakThreads>>>(sink, iters / 16, 0.999999, 1e-6);  // warm-up (clocks, module load)
  PEAK_CUDA(cudaGetLastError());
  float best = 0.f;
  for (int rep = 0; rep < 5; ++rep) {
    PEAK_CUDA(cudaEventRecord(ev[0]));
    k_dfma_loop<<<blocks, kPeakThreads>>>(sink, iters, 0.999999, 1e-6);
    PEAK_CUDA(cudaEventRecord(ev[1]));
    PEAK_CUDA(cudaEventSynchronize(ev[1]));
    float t = 0.f;
    PEAK_CUDA(cudaEventElapsedTime(&t, ev[0], ev[1]));
    if (rep == 0 || t < best) best = t;
  }
  const double flops = 2.0 * kChains * (double)iters * blocks * kPeakThreads;
  *gflops = flops / (best * 1e-3) / 1e9;
  if (ms) *ms = best;
  cudaFree(sink);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  return AFAR_OK;
}
