// cfl_m3 (2-D) on device-resident arrays with no allocation by the library.
//
// Some callers cannot call cudaMalloc: a solver embedded in a host code that
// hands all device memory to its own pool and forbids other allocators, a
// driver that runs inside a memory budget fixed at start-up, or a caller that
// must not allocate between the steps it times.  They hold the state in device
// memory already and need only the CFL time step of it.  The entry point
// below serves them: the caller passes its device arrays in and receives dt
// and merr on the host, and the only scratch the reduction needs -- one
// partial minimum per block of 256 cells plus the final minimum -- lives in a
// file-scope __device__ array that every GPU loading this library holds until
// the process exits.
//
// That array is shared by every call: it keeps the last call's contents and
// two calls that overlap on the GPU (on different streams, or from different
// host threads) race on it.  Nothing in it has to start at zero: each call
// writes every partial it reads.
#include <cuda_runtime.h>

#include <cstring>

#include "cans_gpu.h"
#include "cans_internal.h"

namespace cans {

// Largest grid the allocation-free CFL accepts: one partial per block of
// 256 cells, at most kNoAllocBlocks blocks.
constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocBlocks = 4096;
constexpr long long kNoAllocMaxCells = (long long)kNoAllocBlocks * kNoAllocThreads;

// partials[0..nblocks-1], then the reduced minimum at index kNoAllocBlocks
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocBlocks + 1];

// Per-cell time step of cfl_m3 (cans2d/common/cfl_m3.f:46-55), in the
// reference's operation order:
// dtq = safety * min(dx, dy) / sqrt(v^2 + gm p / ro + B^2 / (4 pi ro)).
template <bool E>
__device__ __forceinline__ double cfl_m3_cell(double ro_, double pr_, double vx_,
                                              double vy_, double vz_, double bx_,
                                              double by_, double bz_, double dx_,
                                              double dy_, double gm_, double pi4i_,
                                              double safety) {
  using FT = F<E>;
  const FT ro(ro_), pr(pr_), vx(vx_), vy(vy_), vz(vz_), bx(bx_), by(by_), bz(bz_);
  const FT b2 = bx * bx + by * by + bz * bz;
  const FT ca2 = b2 * FT(pi4i_) / ro;
  const FT cs2 = FT(gm_) * pr / ro;
  const FT v2 = vx * vx + vy * vy + vz * vz;
  const FT dtcfl = fmin_(FT(dx_), FT(dy_)) / fsqrt(v2 + cs2 + ca2);
  return (FT(safety) * dtcfl).v;
}

// Pass 1: one thread per cell, one partial minimum per block, no atomics.
template <bool E>
__global__ void __launch_bounds__(kNoAllocThreads)
    k_cfl_m3_partials(const double *__restrict__ ro, const double *__restrict__ pr,
                      const double *__restrict__ vx, const double *__restrict__ vy,
                      const double *__restrict__ vz, const double *__restrict__ bx,
                      const double *__restrict__ by, const double *__restrict__ bz,
                      const double *__restrict__ dx, const double *__restrict__ dy,
                      int ix, int jx, double gm, double pi4i, double safety,
                      double *scratch) {
  __shared__ double red[32];
  const long long n = (long long)ix * jx;
  const long long g = (long long)blockIdx.x * kNoAllocThreads + threadIdx.x;
  double v = __longlong_as_double(0x7ff0000000000000LL);
  if (g < n) {
    const int i = (int)(g % ix), j = (int)(g / ix);
    const double d = cfl_m3_cell<E>(ro[g], pr[g], vx[g], vy[g], vz[g], bx[g],
                                        by[g], bz[g], dx[i], dy[j], gm, pi4i, safety);
    if (d < v) v = d;  // as cfl_m3.f's `if (dtq .lt. dt)`: a NaN never becomes the minimum
  }
  const double m = block_min(v, red, threadIdx.x, kNoAllocThreads);
  if (threadIdx.x == 0) scratch[blockIdx.x] = m;
}

// Pass 2: one block folds the partials, starting from the reference's
// dt = 1.e20 (real*4).
__global__ void __launch_bounds__(1024) k_cfl_m3_final(double *scratch, int nblocks) {
  __shared__ double red[32];
  double v = (double)1.e20f;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const double x = scratch[b];
    if (x < v) v = x;
  }
  const double m = block_min(v, red, threadIdx.x, blockDim.x);
  if (threadIdx.x == 0) scratch[kNoAllocBlocks] = m;
}

namespace {
// Device address of the scratch array on the current device.  It is looked
// up on every call: the lookup allocates nothing and does no device work once
// the module is loaded, and a cached address would go stale if the host
// reset the device between calls.  The first call on a device loads the
// module, so it should come before any stream capture.
int noalloc_scratch(double **out) {
  double *p = nullptr;
  if (cudaGetSymbolAddress((void **)&p, g_noalloc_scratch) != cudaSuccess || !p)
    return CANS_ERR_CUDA;
  *out = p;
  return CANS_OK;
}
}  // namespace

}  // namespace cans

using namespace cans;

// No counterpart in the reference: cfl_m3 (cans2d/common/cfl_m3.f) on arrays
// that already live in device memory, for callers that cannot allocate.
extern "C" int cans_cfl_m3_2d_noalloc(double *dt, const double *safety,
                                      const double *dtmin, int *merr,
                                      const double *gm, const double *ro,
                                      const double *pr, const double *vx,
                                      const double *vy, const double *vz,
                                      const double *bx, const double *by,
                                      const double *bz, const double *dx,
                                      const int *ix, const double *dy,
                                      const int *jx) {
  if (!dt || !safety || !dtmin || !merr || !gm || !ix || !jx) return CANS_ERR_ARG;
  if (!ro || !pr || !vx || !vy || !vz || !bx || !by || !bz || !dx || !dy)
    return CANS_ERR_ARG;
  const long long n = (long long)*ix * (long long)*jx;
  if (*ix < 1 || *jx < 1 || n > kNoAllocMaxCells) return CANS_ERR_ARG;
  double *scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  const cudaStream_t s = configured_stream();  // never creates one
  const int nblocks = (int)((n + kNoAllocThreads - 1) / kNoAllocThreads);
  const Phys ph = make_phys(*gm, 0.0);
  if (cans_get_exact())
    k_cfl_m3_partials<true><<<nblocks, kNoAllocThreads, 0, s>>>(
        ro, pr, vx, vy, vz, bx, by, bz, dx, dy, *ix, *jx, ph.gm, ph.pi4i, *safety, scratch);
  else
    k_cfl_m3_partials<false><<<nblocks, kNoAllocThreads, 0, s>>>(
        ro, pr, vx, vy, vz, bx, by, bz, dx, dy, *ix, *jx, ph.gm, ph.pi4i, *safety, scratch);
  k_cfl_m3_final<<<1, 1024, 0, s>>>(scratch, nblocks);
  count_launch(2);
  if (cudaGetLastError() != cudaSuccess) return CANS_ERR_CUDA;
  double out = 0.0;
  if (cudaMemcpyAsync(&out, scratch + kNoAllocBlocks, sizeof out, cudaMemcpyDeviceToHost,
                      s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return CANS_ERR_CUDA;
  *dt = out;
  *merr = (out < *dtmin) ? 9001 : 0;
  return CANS_OK;
}
