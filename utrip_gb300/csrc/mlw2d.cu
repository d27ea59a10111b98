// Fused 2-D modified Lax-Wendroff step (sm_103a, FP64): the single-grid
// kernel, the CFL kernels and the frame kernel.  The tile body itself
// (phases 1-3, one TX x TY tile) is in mlw2d_tile.cuh.
#include <cuda_runtime.h>

#include "bc_line.cuh"
#include "cans_common.cuh"
#include "cans_internal.h"
#include "mlw2d_tile.cuh"

namespace cans {

// One tile per block.  With a control block the step takes dt and the
// buffers from it, does nothing once the run is done or paused, and reduces
// the CFL of the cells inside `box`.
template <bool E, bool M3, int TX, int TY, int RPT>
__global__ void __launch_bounds__(TX *TY / RPT, 1)
    k_mlw2d(const double *__restrict__ A, double *__restrict__ B, int ix,
            int jx, Axis ax, Axis ay, Phys ph, double dt_arg,
            Ctl *__restrict__ ctl, Box3 box) {
  extern __shared__ double smem[];
  double dt = dt_arg, safety = 0.0;
  unsigned long long *cfl = nullptr;
  if (ctl != nullptr) {
    if (ctl->done | ctl->pause) return;
    A = ctl->buf[ctl->cur];
    B = ctl->buf[ctl->cur ^ 1];
    dt = ctl->dt;
    safety = ctl->safety;
    cfl = &ctl->cfl_bits;
  }
  tile_step<E, M3, TX, TY, RPT>(A, B, ix, jx, ax, ay, ph, dt, safety, cfl, box,
                                blockIdx.x, blockIdx.y, gridDim.x, gridDim.y, smem,
                                nullptr, nullptr, ctl ? &ctl->nonfinite : nullptr);
}

// The mlw_m3 step with the artificial viscosity's branch recorded (AVF = 1)
// or held at the recorded one (AVF = 2): the forward of the adjoint's
// finite-difference check (see tile_step).  32 x 8 tiles, no control block.
template <bool E, int AVF>
__global__ void __launch_bounds__(128, 1)
    k_mlw2d_av(const double *__restrict__ A, double *__restrict__ B, int ix, int jx, Axis ax,
               Axis ay, Phys ph, double dt, unsigned char *avb, unsigned long long *nflip) {
  extern __shared__ double smem[];
  tile_step<E, true, 32, 8, 2, false, false, AVF>(
      A, B, ix, jx, ax, ay, ph, dt, 0.0, nullptr, Box3{}, blockIdx.x, blockIdx.y, gridDim.x,
      gridDim.y, smem, nullptr, nullptr, nullptr, avb, nflip);
}

cudaError_t launch_mlw2d_av(bool exact, int mode, const double *A, double *B, int ix, int jx,
                            const Axis &ax, const Axis &ay, const Phys &ph, double dt,
                            unsigned char *avb, unsigned long long *nflip, cudaStream_t s) {
  if (ix < 3 || jx < 3 || (mode != 1 && mode != 2) || !avb || (mode == 2 && !nflip))
    return cudaErrorInvalidValue;
  using T = Tile<32, 8, true, 2>;
  void (*k)(const double *, double *, int, int, Axis, Axis, Phys, double, unsigned char *,
            unsigned long long *) =
      exact ? (mode == 1 ? k_mlw2d_av<true, 1> : k_mlw2d_av<true, 2>)
            : (mode == 1 ? k_mlw2d_av<false, 1> : k_mlw2d_av<false, 2>);
  cudaError_t e =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
  if (e != cudaSuccess) return e;
  dim3 grid((ix - 2 + 31) / 32, (jx - 2 + 7) / 8);
  k<<<grid, T::NT, T::smem_bytes, s>>>(A, B, ix, jx, ax, ay, ph, dt, avb, nflip);
  count_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Tile configurations offered to the autotuner: (TX, TY).
namespace {
template <bool E, bool M3, int TX, int TY, int RPT = 2>
cudaError_t launch_tile(const double *A, double *B, int ix, int jx,
                        const Axis &ax, const Axis &ay, const Phys &ph,
                        double dt, Ctl *ctl, Box3 box, cudaStream_t s) {
  using T = Tile<TX, TY, M3, RPT>;
  static bool attr_set = false;  // per template instance
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(
        k_mlw2d<E, M3, TX, TY, RPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)T::smem_bytes);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  dim3 grid((ix - 2 + TX - 1) / TX, (jx - 2 + TY - 1) / TY);
  k_mlw2d<E, M3, TX, TY, RPT><<<grid, T::NT, T::smem_bytes, s>>>(A, B, ix, jx, ax,
                                                                ay, ph, dt, ctl, box);
  count_launch();
  return cudaGetLastError();
}

template <bool E, bool M3>
cudaError_t launch_sel(int tile, const double *A, double *B, int ix, int jx,
                       const Axis &ax, const Axis &ay, const Phys &ph,
                       double dt, Ctl *ctl, Box3 box, cudaStream_t s) {
  // 32 x 9 and 32 x 10 give tile counts that fill whole waves of two blocks
  // per SM on grids where 32 x 8 leaves a partly empty last wave (512^2:
  // 1024 tiles = 3.4 waves of 304 blocks, 32 x 9: 912 = 3.0 waves)
  switch (tile) {
    case 1: return launch_tile<E, M3, 32, 8>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
    case 2: return launch_tile<E, M3, 16, 16>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
    case 3: return launch_tile<E, M3, 64, 8>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
    case 4: return launch_tile<E, M3, 32, 9, 1>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
    case 5: return launch_tile<E, M3, 32, 10>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
    default: return launch_tile<E, M3, 32, 16>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
  }
}
}  // namespace

// tile 6: the y-marching kernel of the fast mlw_m3 step (mlw2d_df.cu); the
// exact policy and mlw_m take the 32 x 9 tile in its place
int mlw2d_tile_count() { return 8; }

cudaError_t launch_mlw2d(int solver, bool exact, int tile, const double *A,
                         double *B, int ix, int jx, const Axis &ax,
                         const Axis &ay, const Phys &ph, double dt, Ctl *ctl,
                         Box3 box, cudaStream_t s) {
  if (ix < 3 || jx < 3) return cudaErrorInvalidValue;
  if (tile >= 6) {  // the y-marching tile (segments balanced per SM, or by waves)
    if (solver == 1 && !exact)
      return launch_mlw2d_march_fast(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s, tile == 7);
    tile = 4;
  }
  if (solver == 1) {
    return exact ? launch_sel<true, true>(tile, A, B, ix, jx, ax, ay, ph, dt, ctl, box, s)
                 : launch_sel<false, true>(tile, A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
  }
  return exact ? launch_sel<true, false>(tile, A, B, ix, jx, ax, ay, ph, dt, ctl, box, s)
               : launch_sel<false, false>(tile, A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
}

// ---------------------------------------------------------------------------
// Standalone CFL over all cells (cfl_m3.f:46-65, cfl_m.f:46-65).
template <bool E, bool M3>
__global__ void k_cfl2d_full(const double *__restrict__ S, int ix, int jx,
                             Axis ax, Axis ay, Phys ph, double safety,
                             unsigned long long *out) {
  using FT = F<E>;
  using P = Prim<M3>;
  __shared__ double red[32];
  const size_t n = (size_t)ix * jx;
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  const FT gm(ph.gm), pi4i(ph.pi4i);
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n;
       g += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(g % ix), j = (int)(g / ix);
    const FT ro(S[P::RO * n + g]), pr(S[P::PR * n + g]);
    const FT vx(S[P::VX * n + g]), vy(S[P::VY * n + g]);
    const FT bx(S[P::BX * n + g]), by(S[P::BY * n + g]);
    FT b2, v2;
    if constexpr (M3) {
      const FT vz(S[P::VZ * n + g]), bz(S[P::BZ * n + g]);
      b2 = bx * bx + by * by + bz * bz;
      v2 = vx * vx + vy * vy + vz * vz;
    } else {
      b2 = bx * bx + by * by;
      v2 = vx * vx + vy * vy;
    }
    const FT ca2 = b2 * pi4i / ro;
    const FT cs2 = gm * pr / ro;
    const FT dtcfl = fmin_(FT(ax.d[i]), FT(ay.d[j])) / fsqrt(v2 + cs2 + ca2);
    const double dtq = (FT(safety) * dtcfl).v;
    if (dtq < dmin) dmin = dtq;
  }
  block_min_to(out, dmin, red, threadIdx.x, blockDim.x);
}

cudaError_t launch_cfl2d_full(int solver, bool exact, const double *S, int ix,
                              int jx, const Axis &ax, const Axis &ay,
                              const Phys &ph, double safety,
                              unsigned long long *out_bits, cudaStream_t s) {
  const size_t n = (size_t)ix * jx;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (solver == 1) {
    if (exact) k_cfl2d_full<true, true><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, safety, out_bits);
    else k_cfl2d_full<false, true><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, safety, out_bits);
  } else {
    if (exact) k_cfl2d_full<true, false><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, safety, out_bits);
    else k_cfl2d_full<false, false><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, safety, out_bits);
  }
  count_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// CFL over the frame of cells the boundary fill may have rewritten (ghost
// layers plus the first interior layer), then the start of the next loop
// iteration by the last block to finish.
// With all = 1 the CFL covers every cell: a loop whose chkdav changes cells
// after the step reduces its CFL here alone.

// Cell (i, j) of frame index f: rows j < w or j >= jx-w (all i), then
// columns i < w or i >= ix-w of the remaining rows (every cell with all).
__device__ __forceinline__ void frame_cell(long long f, int ix, int jx, int w, int all,
                                           int &i, int &j) {
  const long long nrow = 2LL * w * ix;
  if (all) {
    i = (int)(f % ix);
    j = (int)(f / ix);
  } else if (f < nrow) {
    const long long r = f / ix;
    i = (int)(f % ix);
    j = (r < w) ? (int)r : (int)(jx - 2 * w + r);
  } else {
    const long long q = f - nrow;
    const long long r = q / (2 * w);
    const int cidx = (int)(q % (2 * w));
    j = (int)(w + r);
    i = (cidx < w) ? cidx : (ix - 2 * w + cidx);
  }
}
__host__ __device__ __forceinline__ long long frame_cells(int ix, int jx, int w, int all) {
  const long long inner_rows = jx - 2LL * w;
  return all ? (long long)ix * jx
             : 2LL * w * ix + (inner_rows > 0 ? inner_rows * 2LL * w : 0);
}

// cfl_m3 (cfl_m for the 7-array layout) of one cell from its values q[v]:
// safety * the cell's time-step limit; bad is set for a cell the CFL cannot
// use.
template <bool E, bool M3>
__device__ __forceinline__ double cell_dtq(const double *q, int i, int j, const Axis &ax,
                                           const Axis &ay, const Phys &ph, double safety,
                                           bool &bad) {
  using FT = F<E>;
  using P = Prim<M3>;
  const FT gm(ph.gm), pi4i(ph.pi4i);
  const FT ro(q[P::RO]), pr(q[P::PR]);
  const FT vx(q[P::VX]), vy(q[P::VY]);
  const FT bx(q[P::BX]), by(q[P::BY]);
  FT b2, v2;
  if constexpr (M3) {
    const FT vz(q[P::VZ]), bz(q[P::BZ]);
    b2 = bx * bx + by * by + bz * bz;
    v2 = vx * vx + vy * vy + vz * vz;
  } else {
    b2 = bx * bx + by * by;
    v2 = vx * vx + vy * vy;
  }
  const FT ca2 = b2 * pi4i / ro;
  const FT cs2 = gm * pr / ro;
  const FT dtcfl = fmin_(FT(ax.d[i]), FT(ay.d[j])) / fsqrt(v2 + cs2 + ca2);
  const double dtq = (FT(safety) * dtcfl).v;
  bad |= bad_cell(ro.v, pr.v, dtq);
  return dtq;
}
template <bool E, bool M3>
__device__ __forceinline__ double frame_dtq(const double *__restrict__ S, size_t n, int i,
                                            int j, int ix, const Axis &ax, const Axis &ay,
                                            const Phys &ph, double safety, bool &bad) {
  using P = Prim<M3>;
  const size_t g = (size_t)i + (size_t)j * ix;
  double q[P::N];
#pragma unroll
  for (int v = 0; v < P::N; v++) q[v] = (v == P::AZ) ? 0.0 : S[(size_t)v * n + g];
  return cell_dtq<E, M3>(q, i, j, ax, ay, ph, safety, bad);
}

template <bool E, bool M3>
__global__ void k_frame2d(const double *__restrict__ S, int ix, int jx,
                          Axis ax, Axis ay, Phys ph, int w, int all, Ctl *ctl) {
  __shared__ double red[32];
  if (ctl->done | ctl->pause) return;
  S = ctl->buf[ctl->cur ^ 1];  // the state the step just wrote
  const size_t n = (size_t)ix * jx;
  const long long total = frame_cells(ix, jx, w, all);
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  bool bad = false;
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       f < total; f += (long long)gridDim.x * blockDim.x) {
    int i, j;
    frame_cell(f, ix, jx, w, all, i, j);
    const double dtq = frame_dtq<E, M3>(S, n, i, j, ix, ax, ay, ph, ctl->safety, bad);
    if (dtq < dmin) dmin = dtq;
  }
  count_bad_block(bad, &ctl->nonfinite, threadIdx.x);
  block_min_to(&ctl->cfl_bits, dmin, red, threadIdx.x, blockDim.x);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(&ctl->frame_blocks_done, 1u);
    if (prev == gridDim.x - 1) {
      __threadfence();
      finish_iteration(ctl);
    }
  }
}

// The value at 1-based position l of row `row` after the x rules.  Not
// inlined: bc_xy_value calls it from each of its rule cases.
__device__ __noinline__ double bc_x_value(const double *row, int ix, int m, int kxl, int kxh,
                                          double q0l, double q0h, const double *dxm, int l) {
  return bd_value(kxl, kxh, m, ix, q0l, q0h, dxm, l, [&](int p) { return row[p - 1]; });
}
// The value at 1-based (i, j) of one variable's array after the x rules of
// every row and then (cy: where they change the cell) the y rules of column i.
__device__ __noinline__ double bc_xy_value(const double *sv, int ix, int jx, int m, int kxl,
                                           int kxh, int kyl, int kyh, double qxl, double qxh,
                                           double qyl, double qyh, const double *dxmx,
                                           const double *dxmy, int i, int j, bool cy) {
  auto xval = [&](int j1) {
    return bc_x_value(sv + (size_t)(j1 - 1) * ix, ix, m, kxl, kxh, qxl, qxh, dxmx, i);
  };
  if (!cy) return xval(j);
  return bd_value(kyl, kyh, m, jx, qyl, qyh, dxmy, j, xval);
}

// The boundary program and the frame CFL of one loop iteration in one
// launch, for a 2-D loop without chkdav.  A thread owns one frame cell and
// computes each variable's value there as the x rules and then the y rules
// of the program leave it (bd_value of the y rules over a column whose values
// are bd_value of the x rules over their rows): the same operations as
// k_bc_axis (x), k_bc_axis (y), so the same bits, with no barrier between the
// axes.  A thread reads only cells that no rule changes (the step's output)
// and writes only its own cell, so the threads are independent.  It then
// reduces the CFL over the frame as k_frame2d does, from the values in
// registers, and the last block ends the iteration.
template <bool E, bool M3>
__global__ void __launch_bounds__(32 * Prim<M3>::N)
    k_bcframe2d(int ix, int jx, Axis ax, Axis ay, Phys ph, BcTable bc, Ctl *ctl) {
  using P = Prim<M3>;
  // a block takes 32 frame cells; thread (c, v) = (lane, warp) evaluates
  // variable v of cell c, and the first warp reduces the CFL of the 32 cells
  __shared__ double q[P::N][32];
  __shared__ double red[32];
  if (ctl->done | ctl->pause) return;
  double *S = ctl->buf[ctl->cur ^ 1];  // the state the step just wrote
  const size_t n = (size_t)ix * jx;
  const int m = bc.margin, w = m + 1;
  const long long total = frame_cells(ix, jx, w, 0);
  const int c = threadIdx.x & 31, v = threadIdx.x >> 5;
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  bool bad = false;
  for (long long f0 = blockIdx.x * 32LL; f0 < total; f0 += gridDim.x * 32LL) {
    const long long f = f0 + c;
    int i = 0, j = 0;
    if (f < total) {
      frame_cell(f, ix, jx, w, 0, i, j);
      const double *sv = S + (size_t)v * n;
      const int kxl = bc.kind[v][0], kxh = bc.kind[v][1];
      const int kyl = bc.kind[v][2], kyh = bc.kind[v][3];
      const bool cx = bd_changes(kxl, kxh, m, ix, i + 1);
      const bool cy = bd_changes(kyl, kyh, m, jx, j + 1);
      const double val = bc_xy_value(sv, ix, jx, m, kxl, kxh, kyl, kyh, bc.q0[v][0],
                                     bc.q0[v][1], bc.q0[v][2], bc.q0[v][3], ax.dm, ay.dm,
                                     i + 1, j + 1, cy);
      if (cx || cy) S[(size_t)v * n + (size_t)i + (size_t)j * ix] = val;
      q[v][c] = val;
    }
    __syncthreads();
    if (v == 0 && f < total) {
      double qc[P::N];
#pragma unroll
      for (int u = 0; u < P::N; u++) qc[u] = q[u][c];
      const double dtq = cell_dtq<E, M3>(qc, i, j, ax, ay, ph, ctl->safety, bad);
      if (dtq < dmin) dmin = dtq;
    }
    __syncthreads();
  }
  count_bad_block(bad, &ctl->nonfinite, threadIdx.x);
  block_min_to(&ctl->cfl_bits, dmin, red, threadIdx.x, blockDim.x);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(&ctl->frame_blocks_done, 1u);
    if (prev == gridDim.x - 1) {
      __threadfence();
      finish_iteration(ctl);
    }
  }
}

cudaError_t launch_bcframe2d(int solver, bool exact, int nvar, int ix, int jx, const Axis &ax,
                             const Axis &ay, const Phys &ph, const BcTable &bc, Ctl *ctl,
                             cudaStream_t s) {
  const int need = solver == 1 ? 9 : 7;
  if (nvar != need || ix < 2 * bc.margin + 3 || jx < 2 * bc.margin + 3)
    return cudaErrorInvalidValue;
  const int w = bc.margin + 1;
  int blocks = (int)((frame_cells(ix, jx, w, 0) + 31) / 32);
  if (blocks < 1) blocks = 1;
  if (blocks > 152 * 4) blocks = 152 * 4;
  const int nt = 32 * nvar;
  if (solver == 1) {
    if (exact) k_bcframe2d<true, true><<<blocks, nt, 0, s>>>(ix, jx, ax, ay, ph, bc, ctl);
    else k_bcframe2d<false, true><<<blocks, nt, 0, s>>>(ix, jx, ax, ay, ph, bc, ctl);
  } else {
    if (exact) k_bcframe2d<true, false><<<blocks, nt, 0, s>>>(ix, jx, ax, ay, ph, bc, ctl);
    else k_bcframe2d<false, false><<<blocks, nt, 0, s>>>(ix, jx, ax, ay, ph, bc, ctl);
  }
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_frame2d(int solver, bool exact, const double *S, int ix,
                           int jx, const Axis &ax, const Axis &ay,
                           const Phys &ph, int margin, Ctl *ctl,
                           cudaStream_t s, int all) {
  const int w = margin + 1;
  const long long total = frame_cells(ix, jx, w, all);
  int blocks = (int)((total + 255) / 256);
  if (blocks < 1) blocks = 1;
  if (blocks > (all ? 152 * 4 : 152)) blocks = all ? 152 * 4 : 152;
  if (solver == 1) {
    if (exact) k_frame2d<true, true><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, w, all, ctl);
    else k_frame2d<false, true><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, w, all, ctl);
  } else {
    if (exact) k_frame2d<true, false><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, w, all, ctl);
    else k_frame2d<false, false><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, w, all, ctl);
  }
  count_launch();
  return cudaGetLastError();
}

}  // namespace cans
