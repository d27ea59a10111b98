// Arithmetic peaks of the device for the benchmark's rooflines: the FP64
// and FP32 fused-multiply-add throughput.  Built into its own library,
// libcansprobe.so, beside libcansgpu.so: it is measurement tooling for
// bench.py, not part of the C ABI of the solver.
#include <cuda_runtime.h>

namespace {

// Eight independent FMA chains per thread; `iters` rounds.  The result is
// written so the compiler keeps every operation.
template <class T>
__global__ void k_fma_chains(T *out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = (T)(threadIdx.x * 1e-3 + k);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  if (s == (T)1234.5678) out[0] = s;  // practically never taken
}

template <class T>
int measure(double *tflops, int iters, T a, T b) {
  if (!tflops) return 1;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 2;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 2;
  T *out = nullptr;
  if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return 2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256;
  k_fma_chains<T><<<blocks, threads>>>(out, 64, a, b);  // warm-up
  cudaEventRecord(e0);
  k_fma_chains<T><<<blocks, threads>>>(out, iters, a, b);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return 2;
  const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return 0;
}

}  // namespace

// Measured FMA rates in TFLOP/s (2 flops per FMA), on the default stream.
// Synchronous; 0 on success.
extern "C" int cans_probe_fp64_tflops(double *tflops) {
  return measure<double>(tflops, 4096, 0.999999, 1e-7);
}
extern "C" int cans_probe_fp32_tflops(double *tflops) {
  return measure<float>(tflops, 65536, 0.999999f, 1e-7f);
}
