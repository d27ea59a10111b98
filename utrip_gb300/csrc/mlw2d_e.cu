// Resistive 2-D modified Lax-Wendroff steps (sm_103a, FP64):
//   mlw_m_e   cans2d/hdmlw/mlw_m_e.f    (md_recon)
//   mlw_m3_e  cans2d/hdmlw/mlw_m3_e.f   (md_reccnd, md_flare)
//   mlw_m_ge, mlw_m3_ge  cans2d/hdmlw/mlw_m_ge.f, mlw_m3_ge.f (with gravity)
// and the diffusion limit of their time step, cfl_m_e / cfl_m3_e
// (cans2d/common/cfl_m_e.f, cfl_m3_e.f).
//
// The resistive step adds eta J to the electric field twice: et*J at the
// cells, J from a 3x3 stencil of B (bbtocz, bbtocx, bbtocy), and etm*Jh at
// the corners, Jh from a 3x3 stencil of the half-step B at the neighbouring
// corners.  The fused tile of mlw2d_tile.cuh keeps a one-cell halo, so it
// cannot see the half-step B of the neighbouring corners; instead two small
// kernels run before it:
//   k_res_cells    one thread per cell: et*J at the cells
//   k_res_corners  16 x 16 corners per block: E at the 19 x 19 cells around
//                  them (with et*J), the half-step B at 18 x 18 corners
//                  (mlwhalf, in the reference order), then etm*Jh
// and the tile adds both fields where the reference adds them.  The
// half-step B computed here is the one the tile computes (same operations,
// same order), so in the exact policy the step equals the reference.
//
// The reference leaves J undefined on the outer ring of cells (bbtocz
// writes 2..ix-1, 2..jx-1) and reads, for corner ix-1, the half-step B of
// corner ix, which mlwhalf never sets.  Both are taken as zero (the
// reference reads uninitialised memory there).
#include <cuda_runtime.h>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "mlw2d_tile.cuh"

namespace cans {

namespace {

// bbtocz at one point (cans2d/common/bbtocz.f:34-39): b(dx, dy) reads the
// field at offset (dx, dy); hx, hy are the spacings of the point.
template <bool E, class BX, class BY>
__device__ __forceinline__ F<E> curl_z(BX bx, BY by, F<E> hx, F<E> hy) {
  using FT = F<E>;
  const FT t1 = (by(1, 0) - by(-1, 0)) / hx * 0.5 * 0.5;
  const FT t2 = (by(1, 1) - by(-1, 1)) / hx * 0.5 * 0.25;
  const FT t3 = (by(1, -1) - by(-1, -1)) / hx * 0.5 * 0.25;
  const FT t4 = (bx(0, 1) - bx(0, -1)) / hy * 0.5 * 0.5;
  const FT t5 = (bx(1, 1) - bx(1, -1)) / hy * 0.5 * 0.25;
  const FT t6 = (bx(-1, 1) - bx(-1, -1)) / hy * 0.5 * 0.25;
  return t1 + t2 + t3 - t4 - t5 - t6;
}

// The same current with the reciprocal spacings hxi = 1/hx, hyi = 1/hy and
// the stencil regrouped (fast policy: no division).
template <class BX, class BY>
__device__ __forceinline__ double curl_z_fast(BX bx, BY by, double hxi, double hyi) {
  const double sx = fma(0.25, by(1, 0) - by(-1, 0),
                        0.125 * ((by(1, 1) - by(-1, 1)) + (by(1, -1) - by(-1, -1))));
  const double sy = fma(0.25, bx(0, 1) - bx(0, -1),
                        0.125 * ((bx(1, 1) - bx(1, -1)) + (bx(-1, 1) - bx(-1, -1))));
  return fma(hxi, sx, -hyi * sy);
}

template <bool M3> struct NRes { static constexpr int value = M3 ? 3 : 1; };

// et*J at the cells (mlw_m_e.f:125-129, mlw_m3_e.f:124-132).
template <bool E, bool M3>
__global__ void __launch_bounds__(256)
    k_res_cells(const double *__restrict__ A, int ix, int jx, Axis ax, Axis ay,
                const double *__restrict__ et, double *__restrict__ res,
                const Ctl *__restrict__ ctl) {
  using FT = F<E>;
  using P = Prim<M3>;
  if (ctl != nullptr) {
    if (ctl->done | ctl->pause) return;
    A = ctl->buf[ctl->cur];
  }
  const size_t n = (size_t)ix * jx;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= ix || j >= jx) return;
  const size_t g = (size_t)i + (size_t)j * ix;
  {
    double rx = 0.0, ry = 0.0, rz = 0.0;
    if (i >= 1 && i <= ix - 2 && j >= 1 && j <= jx - 2) {
      const double *bxa = A + P::BX * n + g, *bya = A + P::BY * n + g;
      auto bx = [&](int di, int dj) { return bxa[di + (long long)dj * ix]; };
      auto by = [&](int di, int dj) { return bya[di + (long long)dj * ix]; };
      const double *bz = A + (M3 ? P::BZ : 0) * n;  // read by mlw_m3_e only
      if constexpr (E) {
        const FT hx(ax.d[i]), hy(ay.d[j]);
        const FT e(et[g]);
        auto fbx = [&](int di, int dj) { return FT(bx(di, dj)); };
        auto fby = [&](int di, int dj) { return FT(by(di, dj)); };
        rz = (e * curl_z<E>(fbx, fby, hx, hy)).v;
        if constexpr (M3) {
          // bbtocx.f:31, bbtocy.f:31
          const FT cx = (FT(bz[g + ix]) - FT(bz[g - ix])) / hy * 0.5;
          const FT cy = -((FT(bz[g + 1]) - FT(bz[g - 1])) / hx * 0.5);
          rx = (e * cx).v;
          ry = (e * cy).v;
        }
      } else {
        const double hxi = ax.di[i], hyi = ay.di[j], e = et[g];
        rz = e * curl_z_fast(bx, by, hxi, hyi);
        if constexpr (M3) {
          rx = e * (0.5 * hyi) * (bz[g + ix] - bz[g - ix]);
          ry = -e * (0.5 * hxi) * (bz[g + 1] - bz[g - 1]);
        }
      }
    }
    if constexpr (M3) {
      res[g] = rx;
      res[n + g] = ry;
      res[2 * n + g] = rz;
    } else {
      res[g] = rz;
    }
  }
}

constexpr int KT = 16;           // corners per block edge
constexpr int KC = KT + 3;       // cells per block edge
constexpr int KH = KT + 2;       // half-step corners per block edge

// etm*Jh at the corners (mlw_m_e.f:216-220, mlw_m3_e.f:236-244).
template <bool E, bool M3>
__global__ void __launch_bounds__(KT *KT)
    k_res_corners(const double *__restrict__ A, int ix, int jx, Axis ax, Axis ay,
                  const double *__restrict__ etm, double *__restrict__ res,
                  double dt_arg, const Ctl *__restrict__ ctl) {
  using FT = F<E>;
  using P = Prim<M3>;
  constexpr int NE = NRes<M3>::value;
  // cells: bx, by, ez (+ bz, ex, ey); half-step corners: bxh, byh (+ bzh)
  __shared__ double sc[(M3 ? 6 : 3) * KC * KC];
  __shared__ double sh[(M3 ? 3 : 2) * KH * KH];
  double dtv = dt_arg;
  if (ctl != nullptr) {
    if (ctl->done | ctl->pause) return;
    A = ctl->buf[ctl->cur];
    dtv = ctl->dt;
  }
  const FT dt(dtv);
  const size_t n = (size_t)ix * jx;
  const int k0 = blockIdx.x * KT, l0 = blockIdx.y * KT;
  const int tid = threadIdx.x;
  // cells k0-1 .. k0+KT+1 (x) and l0-1 .. l0+KT+1 (y)
  for (int c = tid; c < KC * KC; c += KT * KT) {
    const int ci = k0 - 1 + c % KC, cj = l0 - 1 + c / KC;
    double vbx = 0.0, vby = 0.0, vez = 0.0, vbz = 0.0, vex = 0.0, vey = 0.0;
    if (ci >= 0 && ci < ix && cj >= 0 && cj < jx) {
      const size_t g = (size_t)ci + (size_t)cj * ix;
      const FT vx(A[P::VX * n + g]), vy(A[P::VY * n + g]);
      const FT bx(A[P::BX * n + g]), by(A[P::BY * n + g]);
      vbx = bx.v;
      vby = by.v;
      if constexpr (M3) {
        const FT vz(A[P::VZ * n + g]), bz(A[P::BZ * n + g]);
        vbz = bz.v;
        vex = (-vy * bz + vz * by + FT(res[g])).v;
        vey = (-vz * bx + vx * bz + FT(res[n + g])).v;
        vez = (-vx * by + vy * bx + FT(res[2 * n + g])).v;
      } else {
        vez = (-vx * by + vy * bx + FT(res[g])).v;
      }
    }
    sc[c] = vbx;
    sc[KC * KC + c] = vby;
    sc[2 * KC * KC + c] = vez;
    if constexpr (M3) {
      sc[3 * KC * KC + c] = vbz;
      sc[4 * KC * KC + c] = vex;
      sc[5 * KC * KC + c] = vey;
    }
  }
  __syncthreads();
  // half-step B at corners k0-1 .. k0+KT (mlwhalf.f:45-52); corners outside
  // 0..ix-2, 0..jx-2 are never set by the reference and are zero here
  for (int c = tid; c < KH * KH; c += KT * KT) {
    const int hx = c % KH, hy = c / KH;
    const int ki = k0 - 1 + hx, kj = l0 - 1 + hy;
    double hbx = 0.0, hby = 0.0, hbz = 0.0;
    if (ki >= 0 && ki <= ix - 2 && kj >= 0 && kj <= jx - 2) {
      const int a = hx + hy * KC, b = a + 1, cc = a + 1 + KC, d = a + KC;
      const FT dxim(ax.dim[ki]), dyim(ay.dim[kj]);
      auto S = [&](int slot, int at) { return FT(sc[slot * KC * KC + at]); };
      auto avg = [&](int slot) {
        return 0.25 * (S(slot, b) + S(slot, a) + S(slot, cc) + S(slot, d));
      };
      // bx: fx = 0, fy = ez
      const FT dfy_bx = dyim * (S(2, d) - S(2, a) + S(2, cc) - S(2, b)) * 0.5;
      hbx = (avg(0) - dt * dfy_bx).v;
      // by: fx = -ez, fy = 0
      const FT dfx_by = dxim * (-S(2, b) - -S(2, a) + -S(2, cc) - -S(2, d)) * 0.5;
      hby = (avg(1) - dt * dfx_by).v;
      if constexpr (M3) {
        // bz: fx = ey, fy = -ex
        const FT dfx = dxim * (S(5, b) - S(5, a) + S(5, cc) - S(5, d)) * 0.5;
        const FT dfy = dyim * (-S(4, d) - -S(4, a) + -S(4, cc) - -S(4, b)) * 0.5;
        hbz = (avg(3) - dt * dfx - dt * dfy).v;
      }
    }
    sh[c] = hbx;
    sh[KH * KH + c] = hby;
    if constexpr (M3) sh[2 * KH * KH + c] = hbz;
  }
  __syncthreads();
  const int lx = tid % KT, ly = tid / KT;
  const int ki = k0 + lx, kj = l0 + ly;
  if (ki > ix - 2 || kj > jx - 2) return;
  const size_t gk = (size_t)ki + (size_t)kj * ix;
  double rx = 0.0, ry = 0.0, rz = 0.0;
  if (ki >= 1 && kj >= 1) {
    const int h = (lx + 1) + (ly + 1) * KH;
    auto bxh = [&](int di, int dj) { return sh[h + di + dj * KH]; };
    auto byh = [&](int di, int dj) { return sh[KH * KH + h + di + dj * KH]; };
    const double *bzh = sh + 2 * KH * KH;
    if constexpr (E) {
      const FT hxm(ax.dm[ki]), hym(ay.dm[kj]);
      const FT e(etm[gk]);
      auto fbx = [&](int di, int dj) { return FT(bxh(di, dj)); };
      auto fby = [&](int di, int dj) { return FT(byh(di, dj)); };
      rz = (e * curl_z<E>(fbx, fby, hxm, hym)).v;
      if constexpr (M3) {
        const FT cx = (FT(bzh[h + KH]) - FT(bzh[h - KH])) / hym * 0.5;
        const FT cy = -((FT(bzh[h + 1]) - FT(bzh[h - 1])) / hxm * 0.5);
        rx = (e * cx).v;
        ry = (e * cy).v;
      }
    } else {
      const double hxi = ax.dim[ki], hyi = ay.dim[kj], e = etm[gk];
      rz = e * curl_z_fast(bxh, byh, hxi, hyi);
      if constexpr (M3) {
        rx = e * (0.5 * hyi) * (bzh[h + KH] - bzh[h - KH]);
        ry = -e * (0.5 * hxi) * (bzh[h + 1] - bzh[h - 1]);
      }
    }
  }
  if constexpr (M3) {
    res[NE * n + gk] = rx;
    res[(NE + 1) * n + gk] = ry;
    res[(NE + 2) * n + gk] = rz;
  } else {
    res[NE * n + gk] = rz;
  }
}

constexpr int ETX = 32, ETY = 8, ERPT = 2;

template <bool E, bool M3, bool G>
__global__ void __launch_bounds__(ETX *ETY / ERPT, 1)
    k_mlw2d_e(const double *__restrict__ A, double *__restrict__ B, int ix, int jx,
              Axis ax, Axis ay, Phys ph, const double *__restrict__ grav,
              const double *__restrict__ res, double dt_arg, Ctl *__restrict__ ctl,
              Box3 box) {
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
  tile_step<E, M3, ETX, ETY, ERPT, G, true>(A, B, ix, jx, ax, ay, ph, dt, safety, cfl,
                                            box, blockIdx.x, blockIdx.y, gridDim.x,
                                            gridDim.y, smem, grav, res,
                                            ctl ? &ctl->nonfinite : nullptr);
}

template <bool E, bool M3, bool G>
cudaError_t launch_e(const double *A, double *B, int ix, int jx, const Axis &ax,
                     const Axis &ay, const Phys &ph, const double *grav,
                     const double *eta, double *res, double dt, Ctl *ctl, Box3 box,
                     cudaStream_t s) {
  using T = Tile<ETX, ETY, M3, ERPT, G>;
  static bool attr_set = false;  // per template instance
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_mlw2d_e<E, M3, G>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)T::smem_bytes);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const size_t n = (size_t)ix * jx;
  dim3 gc((ix + 31) / 32, (jx + 7) / 8);
  k_res_cells<E, M3><<<gc, dim3(32, 8), 0, s>>>(A, ix, jx, ax, ay, eta, res, ctl);
  count_launch();
  dim3 gk((ix - 1 + KT - 1) / KT, (jx - 1 + KT - 1) / KT);
  k_res_corners<E, M3><<<gk, KT * KT, 0, s>>>(A, ix, jx, ax, ay, eta + n, res, dt, ctl);
  count_launch();
  dim3 grid((ix - 2 + ETX - 1) / ETX, (jx - 2 + ETY - 1) / ETY);
  k_mlw2d_e<E, M3, G><<<grid, T::NT, T::smem_bytes, s>>>(A, B, ix, jx, ax, ay, ph, grav,
                                                          res, dt, ctl, box);
  count_launch();
  return cudaGetLastError();
}

template <bool E, bool M3>
cudaError_t launch_e_g(const double *A, double *B, int ix, int jx, const Axis &ax,
                       const Axis &ay, const Phys &ph, const double *grav,
                       const double *eta, double *res, double dt, Ctl *ctl, Box3 box,
                       cudaStream_t s) {
  if (grav != nullptr)
    return launch_e<E, M3, true>(A, B, ix, jx, ax, ay, ph, grav, eta, res, dt, ctl, box, s);
  return launch_e<E, M3, false>(A, B, ix, jx, ax, ay, ph, grav, eta, res, dt, ctl, box, s);
}

// cfl_m_e / cfl_m3_e (cfl_m_e.f:47-63, cfl_m3_e.f:49-65): the wave limit and
// the diffusion limit safety*0.5*dmesh**2/max(et,etmin) per cell.
template <bool E, bool M3>
__global__ void k_cfl2d_e(const double *__restrict__ S, int ix, int jx, Axis ax, Axis ay,
                          Phys ph, const double *__restrict__ et, double safety,
                          int wave, unsigned long long *out) {
  using FT = F<E>;
  using P = Prim<M3>;
  __shared__ double red[32];
  const size_t n = (size_t)ix * jx;
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  const FT gm(ph.gm), pi4i(ph.pi4i), sf(safety);
  const double etmin = (double)1.e-5f;  // the single-precision literal 1.e-5
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n;
       g += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(g % ix), j = (int)(g / ix);
    const FT dmesh = fmin_(FT(ax.d[i]), FT(ay.d[j]));
    const double e = et[g] > etmin ? et[g] : etmin;
    const FT dtdif = sf * 0.5 * (dmesh * dmesh) / FT(e);
    double dtq = dtdif.v;
    if (wave) {
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
      const FT dtcfl = dmesh / fsqrt(v2 + cs2 + ca2);
      const double dtwav = (sf * dtcfl).v;
      dtq = dtwav < dtdif.v ? dtwav : dtdif.v;  // min(dtwav, dtdif)
    }
    if (dtq < dmin) dmin = dtq;
  }
  block_min_to(out, dmin, red, threadIdx.x, blockDim.x);
}

}  // namespace

size_t mlw2d_e_scratch_doubles(int solver, int ix, int jx) {
  return (size_t)2 * (solver == 1 ? 3 : 1) * (size_t)ix * (size_t)jx;
}

cudaError_t launch_mlw2d_e(int solver, bool exact, const double *A, double *B, int ix,
                           int jx, const Axis &ax, const Axis &ay, const Phys &ph,
                           const double *grav, const double *eta, double *res,
                           double dt, Ctl *ctl, Box3 box, cudaStream_t s) {
  if (ix < 3 || jx < 3 || eta == nullptr || res == nullptr) return cudaErrorInvalidValue;
  if (solver == 1)
    return exact ? launch_e_g<true, true>(A, B, ix, jx, ax, ay, ph, grav, eta, res, dt, ctl,
                                          box, s)
                 : launch_e_g<false, true>(A, B, ix, jx, ax, ay, ph, grav, eta, res, dt,
                                           ctl, box, s);
  return exact ? launch_e_g<true, false>(A, B, ix, jx, ax, ay, ph, grav, eta, res, dt, ctl,
                                         box, s)
               : launch_e_g<false, false>(A, B, ix, jx, ax, ay, ph, grav, eta, res, dt, ctl,
                                          box, s);
}

cudaError_t launch_cfl2d_e(int solver, bool exact, const double *S, int ix, int jx,
                           const Axis &ax, const Axis &ay, const Phys &ph,
                           const double *et, double safety, int wave,
                           unsigned long long *out_bits, cudaStream_t s) {
  const size_t n = (size_t)ix * jx;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (solver == 1) {
    if (exact)
      k_cfl2d_e<true, true><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, et, safety, wave,
                                                  out_bits);
    else
      k_cfl2d_e<false, true><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, et, safety, wave,
                                                   out_bits);
  } else {
    if (exact)
      k_cfl2d_e<true, false><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, et, safety, wave,
                                                   out_bits);
    else
      k_cfl2d_e<false, false><<<blocks, 256, 0, s>>>(S, ix, jx, ax, ay, ph, et, safety,
                                                    wave, out_bits);
  }
  count_launch();
  return cudaGetLastError();
}

}  // namespace cans
