// On-device ghost-cell fill (the reference bd* routines) and the run-start
// kernel of the device time loop.
//
// Every bd* routine applies one rule to each grid line that runs along its
// axis (cans2d/bc/bdperx.f:33-46, bdsppx.f:31-47, bdsmnx.f:31-55, bdfrex.f,
// bdcnsx.f, bdfrdx.f and their y/z and 1-D/3-D twins), so one device function
// serves every family and dimension.  A boundary program (BcTable) applies
// the rules of all variables axis by axis, x first, as the model packages'
// bnd routines do (cans2d/md_mhdkh/hdmlw/bnd.f:11-39).
#include <cuda_runtime.h>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "bc_line.cuh"

namespace cans {

// Boundary program of one axis over all variables: thread per (var, line).
__global__ void k_bc_axis(int nvar, double *S, int n0, int n1, int n2,
                          int axis, BcTable bc, const double *dxm,
                          const Ctl *ctl) {
  if (ctl != nullptr) {
    if (ctl->done | ctl->pause) return;
    S = ctl->buf[ctl->cur ^ 1];  // the state the step just wrote
  }
  const int dims[3] = {n0, n1, n2};
  const int n = dims[axis];
  const size_t stride = axis == 0 ? 1 : (axis == 1 ? (size_t)n0 : (size_t)n0 * n1);
  const long long nlines = (long long)n0 * n1 * n2 / n;
  const size_t nall = (size_t)n0 * n1 * n2;
  const long long total = nlines * nvar;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       t < total; t += (long long)gridDim.x * blockDim.x) {
    const int v = (int)(t / nlines);
    const long long line = t % nlines;
    double *q = S + (size_t)v * nall + line_base(axis, line, n0, n1);
    const int klo = bc.kind[v][2 * axis], khi = bc.kind[v][2 * axis + 1];
    if (klo >= 0)
      bd_line(klo, 0, bc.margin, bc.margin, q, n, stride, bc.q0[v][2 * axis], dxm);
    if (khi >= 0)
      bd_line(khi, 1, bc.margin, bc.margin, q, n, stride, bc.q0[v][2 * axis + 1], dxm);
  }
}

static cudaError_t bc_axis(int nvar, double *S, int n0, int n1, int n2,
                           int axis, const BcTable &bc, const double *dxm,
                           const Ctl *ctl, cudaStream_t s) {
  const int dims[3] = {n0, n1, n2};
  const long long total = (long long)n0 * n1 * n2 / dims[axis] * nvar;
  int blocks = (int)((total + 255) / 256);
  if (blocks < 1) blocks = 1;
  if (blocks > 152 * 4) blocks = 152 * 4;
  k_bc_axis<<<blocks, 256, 0, s>>>(nvar, S, n0, n1, n2, axis, bc, dxm, ctl);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_bc2d(int nvar, double *S, int ix, int jx, const Axis &ax,
                        const Axis &ay, const BcTable &bc, const Ctl *ctl,
                        cudaStream_t s) {
  cudaError_t e = bc_axis(nvar, S, ix, jx, 1, 0, bc, ax.dm, ctl, s);
  if (e != cudaSuccess) return e;
  return bc_axis(nvar, S, ix, jx, 1, 1, bc, ay.dm, ctl, s);
}

cudaError_t launch_bc3d(int nvar, double *S, int ix, int jx, int kx,
                        const Axis &ax, const Axis &ay, const Axis &az,
                        const BcTable &bc, const Ctl *ctl, cudaStream_t s) {
  cudaError_t e = bc_axis(nvar, S, ix, jx, kx, 0, bc, ax.dm, ctl, s);
  if (e != cudaSuccess) return e;
  e = bc_axis(nvar, S, ix, jx, kx, 1, bc, ay.dm, ctl, s);
  if (e != cudaSuccess) return e;
  return bc_axis(nvar, S, ix, jx, kx, 2, bc, az.dm, ctl, s);
}

// A single reference bd* call on one array: thread per line.
__global__ void k_bd_one(int kind, int axis, int mbnd, int m0, int m1,
                         double *q, double q0, const double *dxm, int n0,
                         int n1, int n2) {
  const int dims[3] = {n0, n1, n2};
  const int n = dims[axis];
  const size_t stride = axis == 0 ? 1 : (axis == 1 ? (size_t)n0 : (size_t)n0 * n1);
  const long long nlines = (long long)n0 * n1 * n2 / n;
  for (long long line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       line < nlines; line += (long long)gridDim.x * blockDim.x) {
    bd_line(kind, mbnd, m0, m1, q + line_base(axis, line, n0, n1), n, stride,
            q0, dxm);
  }
}

cudaError_t launch_bd_one(int kind, int axis, int mbnd, int margin0,
                          int margin1, double *q, double q0, const double *dxm,
                          int n0, int n1, int n2, cudaStream_t s) {
  const int dims[3] = {n0, n1, n2};
  const long long nlines = (long long)n0 * n1 * n2 / dims[axis];
  int blocks = (int)((nlines + 255) / 256);
  if (blocks < 1) blocks = 1;
  if (blocks > 152 * 4) blocks = 152 * 4;
  k_bd_one<<<blocks, 256, 0, s>>>(kind, axis, mbnd, margin0, margin1, q, q0,
                                  dxm, n0, n1, n2);
  count_launch();
  return cudaGetLastError();
}

// Start of the first loop iteration (main.f:161-173): ns+=1, dt from the CFL
// minimum already reduced into ctl->cfl_bits, the dtmin test, tp=t, t+=dt.
__global__ void k_prepare(Ctl *ctl) {
  // The reference loop tests its condition at the end of the body, so the
  // first iteration always starts.
  // It also restarts a loop paused at an output time.
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (ctl->done || ctl->pause) return;
  start_iteration(ctl);
}

cudaError_t launch_prepare(Ctl *ctl, cudaStream_t s) {
  k_prepare<<<1, 32, 0, s>>>(ctl);
  count_launch();
  return cudaGetLastError();
}

}  // namespace cans
