// Measurement helpers used by the benchmark: the FP64 fused-multiply-add
// throughput of the device (the arithmetic roofline of the FP64 mLW step).
#include <cuda_runtime.h>

#include "cans_gpu.h"
#include "cans_internal.h"

namespace cans {

// Eight independent FMA chains per thread; `iters` rounds.  The result is
// written so the compiler keeps every operation.
__global__ void k_fp64_fma(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = threadIdx.x * 1e-3 + k;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  if (s == 1234.5678) out[0] = s;  // practically never taken
}

}  // namespace cans

// Measured FP64 FMA rate in TFLOP/s (2 flops per FMA), on the library
// stream.  Synchronous.
extern "C" int cans_measure_fp64_tflops(double *tflops) {
  if (!tflops) return CANS_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CANS_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return CANS_ERR_CUDA;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return CANS_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 4, threads = 256, iters = 4096;
  cans::k_fp64_fma<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  cans::k_fp64_fma<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cans::count_launch(2);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return CANS_ERR_CUDA;
  const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return CANS_OK;
}
