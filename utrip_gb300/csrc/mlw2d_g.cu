// Fused 2-D modified Lax-Wendroff step with gravity (sm_103a, FP64):
// mlw_m3_g (cans2d/hdmlw/mlw_m3_g.f) and mlw_m_g (cans2d/hdmlw/mlw_m_g.f),
// the tile body of mlw2d_tile.cuh with its gravity sources switched on.  The
// md_mhdgwave, md_parkerinst and md_efr packages call these steps.
//
// The gravity fields gx, gxm, gy, gym (ix*jx each, gxm and gym at the cell
// corners) are read from global memory once per tile; the six source arrays
// add 17 KB of shared memory per 32 x 8 tile, so two tile shapes are offered.
#include <cuda_runtime.h>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "mlw2d_tile.cuh"

namespace cans {

template <bool E, bool M3, int TX, int TY, int RPT>
__global__ void __launch_bounds__(TX *TY / RPT, 1)
    k_mlw2d_g(const double *__restrict__ A, double *__restrict__ B, int ix, int jx,
              Axis ax, Axis ay, Phys ph, const double *__restrict__ grav,
              double dt_arg, Ctl *__restrict__ ctl, Box3 box) {
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
  tile_step<E, M3, TX, TY, RPT, true>(A, B, ix, jx, ax, ay, ph, dt, safety, cfl, box,
                                      blockIdx.x, blockIdx.y, gridDim.x, gridDim.y,
                                      smem, grav, nullptr,
                                      ctl ? &ctl->nonfinite : nullptr);
}

namespace {
template <bool E, bool M3, int TX, int TY, int RPT = 2>
cudaError_t launch_tile_g(const double *A, double *B, int ix, int jx, const Axis &ax,
                          const Axis &ay, const Phys &ph, const double *grav, double dt,
                          Ctl *ctl, Box3 box, cudaStream_t s) {
  using T = Tile<TX, TY, M3, RPT, true>;
  static bool attr_set = false;  // per template instance
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_mlw2d_g<E, M3, TX, TY, RPT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)T::smem_bytes);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  dim3 grid((ix - 2 + TX - 1) / TX, (jx - 2 + TY - 1) / TY);
  k_mlw2d_g<E, M3, TX, TY, RPT><<<grid, T::NT, T::smem_bytes, s>>>(A, B, ix, jx, ax, ay,
                                                                  ph, grav, dt, ctl, box);
  count_launch();
  return cudaGetLastError();
}

template <bool E, bool M3>
cudaError_t launch_sel_g(int tile, const double *A, double *B, int ix, int jx,
                         const Axis &ax, const Axis &ay, const Phys &ph,
                         const double *grav, double dt, Ctl *ctl, Box3 box,
                         cudaStream_t s) {
  if (tile == 1)
    return launch_tile_g<E, M3, 16, 16>(A, B, ix, jx, ax, ay, ph, grav, dt, ctl, box, s);
  return launch_tile_g<E, M3, 32, 8>(A, B, ix, jx, ax, ay, ph, grav, dt, ctl, box, s);
}
}  // namespace

int mlw2d_g_tile_count() { return 2; }

cudaError_t launch_mlw2d_g(int solver, bool exact, int tile, const double *A, double *B,
                           int ix, int jx, const Axis &ax, const Axis &ay,
                           const Phys &ph, const double *grav, double dt, Ctl *ctl,
                           Box3 box, cudaStream_t s) {
  if (ix < 3 || jx < 3 || grav == nullptr) return cudaErrorInvalidValue;
  if (solver == 1)
    return exact ? launch_sel_g<true, true>(tile, A, B, ix, jx, ax, ay, ph, grav, dt, ctl,
                                            box, s)
                 : launch_sel_g<false, true>(tile, A, B, ix, jx, ax, ay, ph, grav, dt, ctl,
                                             box, s);
  return exact ? launch_sel_g<true, false>(tile, A, B, ix, jx, ax, ay, ph, grav, dt, ctl,
                                           box, s)
               : launch_sel_g<false, false>(tile, A, B, ix, jx, ax, ay, ph, grav, dt, ctl,
                                            box, s);
}

}  // namespace cans
