// k_probe.cu -- FP64 FMA throughput probe.
//
// The engine's FP64 kernels (integral builders, element-wise gam_4) are
// bound by the FP64 pipe, which the measured-peaks file of the GPU pool does
// not cover.  This probe measures it on the device at hand: every thread
// runs eight independent DFMA chains, the grid fills all SMs, and the
// sustained rate (2 FLOP per FMA) is timed with CUDA events.
#include <cuda_runtime.h>

#include "../../include/neoxc.h"

namespace {
__global__ void __launch_bounds__(256) fp64_fma_kernel(int iters, double* out) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  double a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const double m = 0.999999, c = 1e-7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 16; k++) {
      a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
      a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
  }
  double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678) out[0] = s;   // keeps the chains live; never true
}
}  // namespace

extern "C" int neoxc_probe_fp64(double* tflops) {
  if (!tflops) return NEOXC_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return NEOXC_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return NEOXC_ERR_CUDA;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) return NEOXC_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256, iters = 2048;
  fp64_fma_kernel<<<blocks, threads>>>(16, d);          // warm-up
  cudaEventRecord(e0);
  fp64_fma_kernel<<<blocks, threads>>>(iters, d);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (err != cudaSuccess || ms <= 0.f) return NEOXC_ERR_CUDA;
  const double flops = 2.0 * 8.0 * 16.0 * (double)iters * blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return NEOXC_OK;
}
