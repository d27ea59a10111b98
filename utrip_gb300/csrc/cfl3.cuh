// Per-cell CFL time step of the 3-D solvers (cans3d/common/cfl_m.f:39-85),
// shared by the mLW and the Roe-MUSCL kernels so that both reduce the same
// expression: safety * min(dx, dy, dz) / sqrt(v^2 + cs^2 + ca^2) with
// ca^2 = b^2 / (4 pi rho) taken with the single-precision pi of cfl_m.f.
#pragma once
#include "cans_common.cuh"
#include "cans_internal.h"

namespace cans {

// primitive arrays of a 3-D state in global memory
struct P3 {
  static constexpr int RO = 0, PR = 1, VX = 2, VY = 3, VZ = 4, BX = 5, BY = 6,
                       BZ = 7, N = 8;
};

template <bool E>
__device__ __forceinline__ double cfl3_cell(const double *__restrict__ S,
                                            size_t n, size_t g, int i, int j,
                                            int k, const Axis &ax,
                                            const Axis &ay, const Axis &az,
                                            const Phys &ph, double safety) {
  using FT = F<E>;
  const FT ro(S[P3::RO * n + g]), pr(S[P3::PR * n + g]);
  const FT vx(S[P3::VX * n + g]), vy(S[P3::VY * n + g]), vz(S[P3::VZ * n + g]);
  const FT bx(S[P3::BX * n + g]), by(S[P3::BY * n + g]), bz(S[P3::BZ * n + g]);
  const FT b2 = bx * bx + by * by + bz * bz;
  const FT ca2 = b2 * FT(ph.pi4i_cfl) / ro;
  const FT cs2 = FT(ph.gm) * pr / ro;
  const FT v2 = vx * vx + vy * vy + vz * vz;
  const FT dmn = fmin_(fmin_(FT(ax.d[i]), FT(ay.d[j])), FT(az.d[k]));
  return (FT(safety) * (dmn / fsqrt(v2 + cs2 + ca2))).v;
}

}  // namespace cans
