// Resistive 3-D modified Lax-Wendroff step (sm_103a, FP64):
//   mlw_m_e   cans3d/hdmlw/mlw_m_e.f  (md_recon 3-D)
// and the diffusion limit of its time step, cfl_m_e (cans3d/common/cfl_m_e.f).
//
// The step adds eta J to the electric field twice: et*J at the cells
// (mlw_m_e.f:103-115, J from bbtocx/bbtocy/bbtocz, a one-neighbour central
// difference of B) and etm*Jh at the corners (mlw_m_e.f:257-270, the same
// difference of the half-step B at the neighbouring corners).  The z-marching
// kernel of mlw3d.cu sees only its own corner, so three kernels run before it:
//   k_res3_cells   one thread per cell: et*J at the cells
//   k_bh3          one thread per corner: the half-step B (mlwhalf, with the
//                  cell E that includes et*J, in the reference order)
//   k_res3_corners one thread per corner: etm*Jh
// and k_mlw3d<..., R = true> adds both fields where the reference adds them.
// The half-step B of k_bh3 is the one the step computes (same operations,
// same order), so in the exact policy the step equals the reference.
//
// The reference leaves J undefined on the outer layer of cells (bbtocx writes
// 2..ix-1, 2..jx-1, 2..kx-1) and reads, for the corners ix-1, jx-1, kx-1, the
// half-step B of corners ix, jx, kx, which mlwhalf never sets.  Both are taken
// as zero (the reference reads uninitialised memory there).
//
// Scratch (mlw3d_e_scratch_doubles): res = et*J at the cells (x, y, z), etm*Jh
// at the corners (x, y, z), then the half-step B (x, y, z), ix*jx*kx each.
#include <cuda_runtime.h>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "cfl3.cuh"

namespace cans {

namespace {

// bbtocx (cans3d/common/bbtocx.f:29-35) and its cyclic permutations bbtocy,
// bbtocz at one point: (b2(+s1) - b2(-s1)) / d1 / 2 - (b1(+s2) - b1(-s2)) / d2 / 2.
// Every operation rounds once (no contraction): the exact policy's form.
__device__ __forceinline__ double bbtoc(const double *__restrict__ b1,
                                        const double *__restrict__ b2, size_t g, size_t s1,
                                        size_t s2, double d1, double d2) {
  const double t1 = __dmul_rn(__ddiv_rn(__dsub_rn(b2[g + s1], b2[g - s1]), d1), 0.5);
  const double t2 = __dmul_rn(__ddiv_rn(__dsub_rn(b1[g + s2], b1[g - s2]), d2), 0.5);
  return __dsub_rn(t1, t2);
}

// The fast policy's form: the same difference times half the reciprocal
// spacings h1 = 0.5/d1, h2 = 0.5/d2 (no division).
__device__ __forceinline__ double bbtoc_fast(const double *__restrict__ b1,
                                             const double *__restrict__ b2, size_t g,
                                             size_t s1, size_t s2, double h1, double h2) {
  return (b2[g + s1] - b2[g - s1]) * h1 - (b1[g + s2] - b1[g - s2]) * h2;
}

__device__ __forceinline__ void split3(size_t g, int ix, size_t plane, int &i, int &j,
                                       int &k) {
  k = (int)(g / plane);
  const size_t r = g % plane;
  j = (int)(r / ix);
  i = (int)(r % ix);
}

__device__ __forceinline__ bool inner3(int i, int j, int k, int ix, int jx, int kx) {
  return i >= 1 && i <= ix - 2 && j >= 1 && j <= jx - 2 && k >= 1 && k <= kx - 2;
}

// et*J at every cell (zero on the outer layer).
template <bool E>
__global__ void k_res3_cells(const double *__restrict__ S, int ix, int jx, int kx,
                             Axis ax, Axis ay, Axis az, const double *__restrict__ et,
                             double *__restrict__ res, const Ctl *__restrict__ ctl) {
  if (ctl != nullptr) {
    if (ctl->done | ctl->pause) return;
    S = ctl->buf[ctl->cur];
  }
  const size_t plane = (size_t)ix * jx, n = plane * kx;
  const double *bx = S + P3::BX * n, *by = S + P3::BY * n, *bz = S + P3::BZ * n;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n;
       g += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    split3(g, ix, plane, i, j, k);
    double cx = 0.0, cy = 0.0, cz = 0.0;
    if (inner3(i, j, k, ix, jx, kx)) {
      const double e = et[g];
      if constexpr (E) {
        cx = __dmul_rn(e, bbtoc(by, bz, g, ix, plane, ay.d[j], az.d[k]));
        cy = __dmul_rn(e, bbtoc(bz, bx, g, plane, 1, az.d[k], ax.d[i]));
        cz = __dmul_rn(e, bbtoc(bx, by, g, 1, ix, ax.d[i], ay.d[j]));
      } else {
        const double hx = 0.5 * ax.di[i], hy = 0.5 * ay.di[j], hz = 0.5 * az.di[k];
        cx = e * bbtoc_fast(by, bz, g, ix, plane, hy, hz);
        cy = e * bbtoc_fast(bz, bx, g, plane, 1, hz, hx);
        cz = e * bbtoc_fast(bx, by, g, 1, ix, hx, hy);
      }
    }
    res[g] = cx;
    res[n + g] = cy;
    res[2 * n + g] = cz;
  }
}

// The half-step B at every corner (zero on corners ix, jx, kx): the corner
// predictor of the exact 3-D step (mlwhalf, mlw_m.f:203-260) for bx, by, bz.
template <bool E>
__global__ void k_bh3(const double *__restrict__ S, const double *__restrict__ res,
                      double *__restrict__ bh, int ix, int jx, int kx, Axis ax, Axis ay,
                      Axis az, double dt_arg, const Ctl *__restrict__ ctl) {
  using FT = F<E>;
  if (ctl != nullptr) {
    if (ctl->done | ctl->pause) return;
    S = ctl->buf[ctl->cur];
  }
  const FT dt((ctl != nullptr) ? ctl->dt : dt_arg);
  const size_t plane = (size_t)ix * jx, n = plane * kx;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n;
       g += (size_t)gridDim.x * blockDim.x) {
    int a, b, k;
    split3(g, ix, plane, a, b, k);
    if (a > ix - 2 || b > jx - 2 || k > kx - 2) {
      bh[g] = 0.0;
      bh[n + g] = 0.0;
      bh[2 * n + g] = 0.0;
      continue;
    }
    // the eight cells: q = (di) + 2 (dj) + 4 (dk); L = plane k, U = plane k+1
    FT B[3][8], Ef[3][8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const size_t c = g + (size_t)(q & 1) + ((q >> 1) & 1) * (size_t)ix +
                       ((q >> 2) & 1) * plane;
      const FT vx(S[P3::VX * n + c]), vy(S[P3::VY * n + c]), vz(S[P3::VZ * n + c]);
      const FT bx(S[P3::BX * n + c]), by(S[P3::BY * n + c]), bz(S[P3::BZ * n + c]);
      B[0][q] = bx;
      B[1][q] = by;
      B[2][q] = bz;
      FT ex = -vy * bz + vz * by;  // mlw_m_e.f:110-115
      FT ey = -vz * bx + vx * bz;
      FT ez = -vx * by + vy * bx;
      Ef[0][q] = ex + FT(res[c]);
      Ef[1][q] = ey + FT(res[n + c]);
      Ef[2][q] = ez + FT(res[2 * n + c]);
    }
    // corner positions of the step's predictor: p00 (a,b), p10 (a+1,b),
    // p01 (a,b+1), p11 (a+1,b+1); L(q) plane k, U(q) plane k+1
    constexpr int p00 = 0, p10 = 1, p01 = 2, p11 = 3;
    const FT dxim(ax.dim[a]), dyim(ay.dim[b]), dzim(az.dim[k]);
    auto avg = [&](const FT *u) {
      return (u[p10] + u[p00] + u[p11] + u[p01] + u[4 + p10] + u[4 + p00] + u[4 + p11] +
              u[4 + p01]) * 0.125;
    };
    auto dif_x = [&](const FT *f, bool ng) {
      auto v = [&](int q) { return ng ? -f[q] : f[q]; };
      return (v(p10) - v(p00) + v(p11) - v(p01) + v(4 + p10) - v(4 + p00) + v(4 + p11) -
              v(4 + p01)) * 0.25 * dxim;
    };
    auto dif_y = [&](const FT *f, bool ng) {
      auto v = [&](int q) { return ng ? -f[q] : f[q]; };
      return (v(p01) - v(p00) + v(p11) - v(p10) + v(4 + p01) - v(4 + p00) + v(4 + p11) -
              v(4 + p10)) * 0.25 * dyim;
    };
    auto dif_z = [&](const FT *f, bool ng) {
      auto v = [&](int q) { return ng ? -f[q] : f[q]; };
      return (v(4 + p00) - v(p00) + v(4 + p10) - v(p10) + v(4 + p01) - v(p01) + v(4 + p11) -
              v(p11)) * 0.25 * dzim;
    };
    // bx: y flux ez, z flux -ey; by: x flux -ez, z flux ex; bz: x flux ey,
    // y flux -ex (the induction equation in the step's flux table)
    FT r = avg(B[0]);
    r = r - dt * dif_y(Ef[2], false);
    r = r - dt * dif_z(Ef[1], true);
    bh[g] = r.v;
    r = avg(B[1]);
    r = r - dt * dif_x(Ef[2], true);
    r = r - dt * dif_z(Ef[0], false);
    bh[n + g] = r.v;
    r = avg(B[2]);
    r = r - dt * dif_x(Ef[1], false);
    r = r - dt * dif_y(Ef[0], true);
    bh[2 * n + g] = r.v;
  }
}

// etm*Jh at every corner (zero on the outer layer), Jh from the half-step B
// at the neighbouring corners and the corner spacings dxm, dym, dzm.
template <bool E>
__global__ void k_res3_corners(const double *__restrict__ bh, int ix, int jx, int kx,
                               Axis ax, Axis ay, Axis az, const double *__restrict__ etm,
                               double *__restrict__ resc, const Ctl *__restrict__ ctl) {
  if (ctl != nullptr && (ctl->done | ctl->pause)) return;
  const size_t plane = (size_t)ix * jx, n = plane * kx;
  const double *bxh = bh, *byh = bh + n, *bzh = bh + 2 * n;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n;
       g += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    split3(g, ix, plane, i, j, k);
    double cx = 0.0, cy = 0.0, cz = 0.0;
    if (inner3(i, j, k, ix, jx, kx)) {
      const double e = etm[g];
      if constexpr (E) {
        cx = __dmul_rn(e, bbtoc(byh, bzh, g, ix, plane, ay.dm[j], az.dm[k]));
        cy = __dmul_rn(e, bbtoc(bzh, bxh, g, plane, 1, az.dm[k], ax.dm[i]));
        cz = __dmul_rn(e, bbtoc(bxh, byh, g, 1, ix, ax.dm[i], ay.dm[j]));
      } else {
        const double hx = 0.5 * ax.dim[i], hy = 0.5 * ay.dim[j], hz = 0.5 * az.dim[k];
        cx = e * bbtoc_fast(byh, bzh, g, ix, plane, hy, hz);
        cy = e * bbtoc_fast(bzh, bxh, g, plane, 1, hz, hx);
        cz = e * bbtoc_fast(bxh, byh, g, 1, ix, hx, hy);
      }
    }
    resc[g] = cx;
    resc[n + g] = cy;
    resc[2 * n + g] = cz;
  }
}

// cfl_m_e (cans3d/common/cfl_m_e.f:47-67): min over the cells of
// min(wave limit, safety*0.5*dmesh**2/max(et, 1.d-10)); with wave = 0 the
// diffusion limit alone.
template <bool E>
__global__ void k_cfl3d_e(const double *__restrict__ S, int ix, int jx, int kx, Axis ax,
                          Axis ay, Axis az, Phys ph, const double *__restrict__ et,
                          double safety, int wave, unsigned long long *out) {
  using FT = F<E>;
  __shared__ double red[32];
  const size_t plane = (size_t)ix * jx, n = plane * kx;
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  const FT sf(safety);
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n;
       g += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    split3(g, ix, plane, i, j, k);
    const FT dmesh = fmin_(fmin_(FT(ax.d[i]), FT(ay.d[j])), FT(az.d[k]));
    const double e = et[g] > 1.e-10 ? et[g] : 1.e-10;
    const FT dtdif = sf * 0.5 * (dmesh * dmesh) / FT(e);
    double dtq = dtdif.v;
    if (wave) {
      const double dtwav = cfl3_cell<E>(S, n, g, i, j, k, ax, ay, az, ph, safety);
      dtq = dtwav < dtdif.v ? dtwav : dtdif.v;  // min(dtwav, dtdif)
    }
    if (dtq < dmin) dmin = dtq;
  }
  block_min_to(out, dmin, red, threadIdx.x, blockDim.x);
}

int grid_for(size_t n) {
  int blocks = (int)((n + 255) / 256);
  if (blocks < 1) blocks = 1;
  if (blocks > 152 * 8) blocks = 152 * 8;
  return blocks;
}

}  // namespace

size_t mlw3d_e_scratch_doubles(int ix, int jx, int kx) {
  return (size_t)9 * (size_t)ix * (size_t)jx * (size_t)kx;
}

cudaError_t launch_mlw3d_e(bool exact, int tile, const double *A, double *B, int ix, int jx,
                           int kx, const Axis &ax, const Axis &ay, const Axis &az,
                           const Phys &ph, const double *eta, double *res, double dt,
                           Ctl *ctl, Box3 box, cudaStream_t s) {
  if (ix < 3 || jx < 3 || kx < 3 || eta == nullptr || res == nullptr)
    return cudaErrorInvalidValue;
  const size_t n = (size_t)ix * jx * kx;
  const int blocks = grid_for(n);
  if (exact)
    k_res3_cells<true><<<blocks, 256, 0, s>>>(A, ix, jx, kx, ax, ay, az, eta, res, ctl);
  else
    k_res3_cells<false><<<blocks, 256, 0, s>>>(A, ix, jx, kx, ax, ay, az, eta, res, ctl);
  count_launch();
  if (exact)
    k_bh3<true><<<blocks, 256, 0, s>>>(A, res, res + 6 * n, ix, jx, kx, ax, ay, az, dt, ctl);
  else
    k_bh3<false><<<blocks, 256, 0, s>>>(A, res, res + 6 * n, ix, jx, kx, ax, ay, az, dt, ctl);
  count_launch();
  if (exact)
    k_res3_corners<true><<<blocks, 256, 0, s>>>(res + 6 * n, ix, jx, kx, ax, ay, az,
                                                eta + n, res + 3 * n, ctl);
  else
    k_res3_corners<false><<<blocks, 256, 0, s>>>(res + 6 * n, ix, jx, kx, ax, ay, az,
                                                 eta + n, res + 3 * n, ctl);
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_mlw3d_res(exact, tile, A, B, ix, jx, kx, ax, ay, az, ph, res, dt, ctl, box, s);
}

cudaError_t launch_cfl3d_e(bool exact, const double *S, int ix, int jx, int kx,
                           const Axis &ax, const Axis &ay, const Axis &az, const Phys &ph,
                           const double *et, double safety, int wave,
                           unsigned long long *out_bits, cudaStream_t s) {
  const int blocks = grid_for((size_t)ix * jx * kx);
  if (exact)
    k_cfl3d_e<true><<<blocks, 256, 0, s>>>(S, ix, jx, kx, ax, ay, az, ph, et, safety, wave,
                                          out_bits);
  else
    k_cfl3d_e<false><<<blocks, 256, 0, s>>>(S, ix, jx, kx, ax, ay, az, ph, et, safety, wave,
                                           out_bits);
  count_launch();
  return cudaGetLastError();
}

}  // namespace cans
