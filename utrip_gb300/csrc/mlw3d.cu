// Fused 3-D modified Lax-Wendroff step (sm_103a, FP64).
//
// Replaces the body of cans3d/hdmlw/mlw_m.f:2-453 with its primitives
// mlwhalf (cans3d/hdmlw/mlwhalf.f:38-65), mlwfull (mlwfull.f:34-52) and
// mlwartv (mlwartv.f), and the CFL of cans3d/common/cfl_m.f:39-85.
//
// Each thread block owns a TX x TY column of cells and marches along z over
// a chunk of planes.  One thread per cell of the (TX+2) x (TY+2) halo tile.
// Shared memory holds a two-plane ring of cell data (conserved variables,
// fluxes, E, velocity) and a two-plane ring of corner (half-step) fluxes;
// the z-neighbour data of a thread's own column for plane k-1 stays in
// registers.  Per plane k:
//   (a) cells of plane k+1 (whole halo tile)               -> ring slot
//   (b) corners of plane k+1/2 from planes k, k+1; AV faces of plane k
//   (c) full step of plane k: central differences (mlwhalf part 1),
//       corrector from corner planes k-1/2 and k+1/2 (mlwfull), artificial
//       viscosity (mlwartv), update, back to primitives, CFL, write.
// The state crosses HBM once in and once out: 8 arrays, 128 B per zone.
//
// With G the kernel is mlw_m_g (cans3d/hdmlw/mlw_m_g.f:2-469): the gravity
// sources ro (v.g), ro gx, ro gy, ro gz of each cell plane (mlw_m_g.f:135-196)
// and the same of each half-step corner plane (:289-350) get two-plane rings
// of their own and enter the energy and the three momenta through mlwsrch
// (cans3d/hdmlw/mlwsrch.f:32-50) and mlwsrcf (mlwsrcf.f:35-45).  grav holds
// gx, gxm, gy, gym, gz, gzm (ix*jx*kx each; the *m fields at the corners).
//
// With R the kernel is mlw_m_e (cans3d/hdmlw/mlw_m_e.f:103-115, 257-270): res
// holds eta J at the cells (x, y, z) and at the corners (x, y, z), ix*jx*kx
// each, computed beforehand by the kernels of mlw3d_e.cu, and each is added
// to E = -v x B where the reference adds et*c and etm*ch.
#include <cuda_runtime.h>

#include <mutex>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "cfl3.cuh"

namespace cans {

namespace {

// cell fields of one ring slot
struct C3 {
  static constexpr int RO = 0, EE = 1, RX = 2, RY = 3, RZ = 4, BX = 5, BY = 6,
                       BZ = 7;
  static constexpr int FXE = 8, FXRX = 9, FXRY = 10, FXRZ = 11;
  static constexpr int FYE = 12, FYRX = 13, FYRY = 14, FYRZ = 15;
  static constexpr int FZE = 16, FZRX = 17, FZRY = 18, FZRZ = 19;
  static constexpr int EX = 20, EY = 21, EZ = 22, VX = 23, VY = 24, VZ = 25;
  static constexpr int N = 26;
};
// corner fields of one ring slot
struct K3 {
  static constexpr int XRO = 0, YRO = 1, ZRO = 2, XEE = 3, YEE = 4, ZEE = 5;
  static constexpr int XRX = 6, YRX = 7, ZRX = 8, XRY = 9, YRY = 10, ZRY = 11;
  static constexpr int XRZ = 12, YRZ = 13, ZRZ = 14, EX = 15, EY = 16, EZ = 17;
  static constexpr int N = 18;
};
template <int TX, int TY, bool G = false> struct Tile3 {
  static constexpr int CX = TX + 2, CY = TY + 2, NC = CX * CY;
  static constexpr int KX = TX + 1, KY = TY + 1, NK = KX * KY;
  static constexpr int NQX = (TX + 1) * TY, NQY = TX * (TY + 1);
  // one thread per halo-tile cell, rounded up to whole warps so that every
  // warp-level reduction sees 32 live lanes; the extra threads own no cell
  static constexpr int NT = (NC + 31) / 32 * 32;
  // gravity: four source fields per cell plane and per corner plane
  static constexpr size_t smem_doubles =
      2 * (size_t)C3::N * NC + 2 * (size_t)K3::N * NK + NQX + NQY + 32 +
      (G ? 2 * 4 * ((size_t)NC + NK) : 0);
  static constexpr size_t smem_bytes = smem_doubles * sizeof(double);
};

constexpr int NOF = -1;  // no flux in this direction

// Flux sources of the 8 conserved variables, per direction: cell field
// index (or NOF) and whether the stored value is negated.
__device__ __forceinline__ void cell_flux_src(int v, int dir, int &f, bool &neg) {
  // v: 0 ro 1 ee 2 rx 3 ry 4 rz 5 bx 6 by 7 bz
  neg = false;
  switch (v) {
    case 0: f = dir == 0 ? C3::RX : dir == 1 ? C3::RY : C3::RZ; break;
    case 1: f = dir == 0 ? C3::FXE : dir == 1 ? C3::FYE : C3::FZE; break;
    case 2: f = dir == 0 ? C3::FXRX : dir == 1 ? C3::FYRX : C3::FZRX; break;
    case 3: f = dir == 0 ? C3::FXRY : dir == 1 ? C3::FYRY : C3::FZRY; break;
    case 4: f = dir == 0 ? C3::FXRZ : dir == 1 ? C3::FYRZ : C3::FZRZ; break;
    case 5: f = dir == 0 ? NOF : dir == 1 ? C3::EZ : C3::EY; neg = (dir == 2); break;
    case 6: f = dir == 0 ? C3::EZ : dir == 1 ? NOF : C3::EX; neg = (dir == 0); break;
    default: f = dir == 0 ? C3::EY : dir == 1 ? C3::EX : NOF; neg = (dir == 1); break;
  }
}
__device__ __forceinline__ void corner_flux_src(int v, int dir, int &f, bool &neg) {
  neg = false;
  switch (v) {
    case 0: f = dir == 0 ? K3::XRO : dir == 1 ? K3::YRO : K3::ZRO; break;
    case 1: f = dir == 0 ? K3::XEE : dir == 1 ? K3::YEE : K3::ZEE; break;
    case 2: f = dir == 0 ? K3::XRX : dir == 1 ? K3::YRX : K3::ZRX; break;
    case 3: f = dir == 0 ? K3::XRY : dir == 1 ? K3::YRY : K3::ZRY; break;
    case 4: f = dir == 0 ? K3::XRZ : dir == 1 ? K3::YRZ : K3::ZRZ; break;
    case 5: f = dir == 0 ? NOF : dir == 1 ? K3::EZ : K3::EY; neg = (dir == 2); break;
    case 6: f = dir == 0 ? K3::EZ : dir == 1 ? NOF : K3::EX; neg = (dir == 0); break;
    default: f = dir == 0 ? K3::EY : dir == 1 ? K3::EX : NOF; neg = (dir == 1); break;
  }
}

// Cell stage: primitives of one cell -> conserved variables, E and the
// cell fluxes of cans3d/hdmlw/mlw_m.f:74-202, into one ring slot.
template <bool E, bool R = false>
__device__ __forceinline__ void cell_stage(const double *__restrict__ A,
                                           size_t n, size_t g, double *sl,
                                           int NC, int c, const Phys &ph,
                                           const double *__restrict__ res = nullptr) {
  using FT = F<E>;
  const FT gm(ph.gm), gm1(ph.gm1), pi8i(ph.pi8i), pi4i(ph.pi4i);
  const FT ro(A[P3::RO * n + g]), pr(A[P3::PR * n + g]);
  const FT vx(A[P3::VX * n + g]), vy(A[P3::VY * n + g]), vz(A[P3::VZ * n + g]);
  const FT bx(A[P3::BX * n + g]), by(A[P3::BY * n + g]), bz(A[P3::BZ * n + g]);
  const FT vv = vx * vx + vy * vy + vz * vz;
  const FT bb = bx * bx + by * by + bz * bz;
  FT ee, ep;
  if constexpr (E) {
    ee = pr / gm1 + 0.5 * ro * vv + pi8i * bb;
    ep = pr * gm / gm1 + 0.5 * ro * vv;
  } else {
    ee = pr * ph.gm1i + 0.5 * ro * vv + pi8i * bb;
    ep = pr * ph.ggm1 + 0.5 * ro * vv;
  }
  FT ex = -vy * bz + vz * by;
  FT ey = -vz * bx + vx * bz;
  FT ez = -vx * by + vy * bx;
  if constexpr (R) {  // mlw_m_e.f:110-115
    ex = ex + FT(res[g]);
    ey = ey + FT(res[n + g]);
    ez = ez + FT(res[2 * n + g]);
  }
#define S(f) sl[(size_t)(f) * NC + c]
  S(C3::RO) = ro.v; S(C3::EE) = ee.v;
  S(C3::RX) = (ro * vx).v; S(C3::RY) = (ro * vy).v; S(C3::RZ) = (ro * vz).v;
  S(C3::BX) = bx.v; S(C3::BY) = by.v; S(C3::BZ) = bz.v;
  S(C3::EX) = ex.v; S(C3::EY) = ey.v; S(C3::EZ) = ez.v;
  S(C3::VX) = vx.v; S(C3::VY) = vy.v; S(C3::VZ) = vz.v;
  S(C3::FXE) = (ep * vx + (bz * ey - by * ez) * pi4i).v;
  S(C3::FYE) = (ep * vy + (bx * ez - bz * ex) * pi4i).v;
  S(C3::FZE) = (ep * vz + (by * ex - bx * ey) * pi4i).v;
  S(C3::FXRX) = (ro * (vx * vx) + pr + pi8i * (by * by + bz * bz - bx * bx)).v;
  S(C3::FYRX) = (ro * vx * vy - pi4i * bx * by).v;
  S(C3::FZRX) = (ro * vx * vz - pi4i * bx * bz).v;
  S(C3::FXRY) = (ro * vy * vx - pi4i * by * bx).v;
  S(C3::FYRY) = (ro * (vy * vy) + pr + pi8i * (bx * bx + bz * bz - by * by)).v;
  S(C3::FZRY) = (ro * vy * vz - pi4i * by * bz).v;
  S(C3::FXRZ) = (ro * vz * vx - pi4i * bz * bx).v;
  S(C3::FYRZ) = (ro * vz * vy - pi4i * bz * by).v;
  S(C3::FZRZ) = (ro * (vz * vz) + pr + pi8i * (bx * bx + by * by - bz * bz)).v;
#undef S
}

}  // namespace

template <bool E, int TX, int TY, bool G = false, bool R = false>
__global__ void __launch_bounds__(((TX + 2) * (TY + 2) + 31) / 32 * 32, 1)
    k_mlw3d(const double *__restrict__ A, double *__restrict__ B, int ix,
            int jx, int kx, Axis ax, Axis ay, Axis az, Phys ph, double dt_arg,
            Ctl *__restrict__ ctl, Box3 box, int kchunk,
            const double *__restrict__ grav = nullptr,
            const double *__restrict__ res = nullptr) {
  using T = Tile3<TX, TY, G>;
  using FT = F<E>;
  extern __shared__ double smem[];
  double *scell = smem;                                   // [2][C3::N][NC]
  double *scorn = scell + 2 * (size_t)C3::N * T::NC;      // [2][K3::N][NK]
  double *sqx = scorn + 2 * (size_t)K3::N * T::NK;        // q*dxim of plane k
  double *sqy = sqx + T::NQX;                             // q*dyim of plane k
  double *sred = sqy + T::NQY;
  double *sgc = sred + 32;                                // G: [2][4][NC]
  double *sgk = sgc + 2 * 4 * (size_t)T::NC;              // G: [2][4][NK]

  if (ctl != nullptr) {
    if (ctl->done | ctl->pause) return;
    A = ctl->buf[ctl->cur];
    B = ctl->buf[ctl->cur ^ 1];
  }
  const FT dt((ctl != nullptr) ? ctl->dt : dt_arg);
  const size_t n = (size_t)ix * jx * kx;
  const size_t plane = (size_t)ix * jx;
  const int tid = threadIdx.x;
  const bool cell = tid < T::NC;                 // this thread owns a cell
  const int hx = tid % T::CX, hy = tid / T::CX;  // halo-tile coordinates
  const int i0 = 1 + blockIdx.x * TX, j0 = 1 + blockIdx.y * TY;
  const int gi = i0 - 1 + hx, gj = j0 - 1 + hy;
  const bool in_arr = cell && (gi < ix) && (gj < jx);
  const bool interior = cell && hx >= 1 && hx <= TX && hy >= 1 && hy <= TY &&
                        gi <= ix - 2 && gj <= jx - 2;
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kx - 2, kb + kchunk - 1);
  if (kb > ke) return;
  const FT gm(ph.gm), gm1(ph.gm1), pi8i(ph.pi8i), pi4i(ph.pi4i);

  auto cslot = [&](int k) { return scell + (size_t)(k & 1) * C3::N * T::NC; };
  auto kslot = [&](int k) { return scorn + (size_t)(k & 1) * K3::N * T::NK; };
  auto gcslot = [&](int k) { return sgc + (size_t)(k & 1) * 4 * T::NC; };
  auto gkslot = [&](int k) { return sgk + (size_t)(k & 1) * 4 * T::NK; };

  auto load_plane = [&](int k) {
    double *sl = cslot(k);
    if (in_arr) {
      const size_t g = (size_t)gi + (size_t)gj * ix + (size_t)k * plane;
      cell_stage<E, R>(A, n, g, sl, T::NC, tid, ph, res);
      if constexpr (G) {  // mlw_m_g.f:135-136, 154, 172, 190
        const FT ro(sl[(size_t)C3::RO * T::NC + tid]);
        const FT vx(sl[(size_t)C3::VX * T::NC + tid]), vy(sl[(size_t)C3::VY * T::NC + tid]);
        const FT vz(sl[(size_t)C3::VZ * T::NC + tid]);
        const FT gx(grav[g]), gy(grav[2 * n + g]), gz(grav[4 * n + g]);
        double *gs = gcslot(k);
        gs[tid] = (ro * (vx * gx + vy * gy + vz * gz)).v;
        gs[T::NC + tid] = (ro * gx).v;
        gs[2 * T::NC + tid] = (ro * gy).v;
        gs[3 * T::NC + tid] = (ro * gz).v;
      }
    } else if (cell) {
#pragma unroll 1
      for (int f = 0; f < C3::N; f++) sl[(size_t)f * T::NC + tid] = 0.0;
      if constexpr (G) {
        double *gs = gcslot(k);
        for (int f = 0; f < 4; f++) gs[f * T::NC + tid] = 0.0;
      }
    }
  };

  // corner plane k+1/2 from cell planes k (lower) and k+1 (upper)
  auto corner_plane = [&](int k) {
    if (tid >= T::NK) return;
    const int cx = tid % T::KX, cy = tid / T::KX;
    const int a = i0 - 1 + cx, b = j0 - 1 + cy;  // lower corner cell
    double *ks = kslot(k);
#define KS(f) ks[(size_t)(f) * T::NK + tid]
    if (a > ix - 2 || b > jx - 2) {
#pragma unroll 1
      for (int f = 0; f < K3::N; f++) KS(f) = 0.0;
      if constexpr (G) {
        double *gk = gkslot(k);
        for (int f = 0; f < 4; f++) gk[f * T::NK + tid] = 0.0;
      }
      return;
    }
    const double *L = cslot(k), *U = cslot(k + 1);
    const int p00 = cx + cy * T::CX, p10 = p00 + 1, p01 = p00 + T::CX,
              p11 = p01 + 1;
    // global operands of this corner, loaded before the predictor so that
    // their latency overlaps its arithmetic
    const size_t gc = (size_t)a + (size_t)b * ix + (size_t)k * plane;
    double rq[3] = {0.0, 0.0, 0.0}, gq[3] = {0.0, 0.0, 0.0};
    if constexpr (R) {
      rq[0] = res[3 * n + gc];
      rq[1] = res[4 * n + gc];
      rq[2] = res[5 * n + gc];
    }
    if constexpr (G) {
      gq[0] = grav[n + gc];
      gq[1] = grav[3 * n + gc];
      gq[2] = grav[5 * n + gc];
    }
    const FT dxim(ax.dim[a]), dyim(ay.dim[b]), dzim(az.dim[k]);
    FT un[8];
    if constexpr (!E) {  // same predictor, fewer rounded operations
      const double cxk = dt.v * dxim.v * 0.25, cyk = dt.v * dyim.v * 0.25,
                   czk = dt.v * dzim.v * 0.25;
#pragma unroll
      for (int v = 0; v < 8; v++) {
        const double *Lv = L + (size_t)v * T::NC, *Uv = U + (size_t)v * T::NC;
        double r = 0.125 * (((Lv[p10] + Lv[p00]) + (Lv[p11] + Lv[p01])) +
                            ((Uv[p10] + Uv[p00]) + (Uv[p11] + Uv[p01])));
        int f;
        bool ng;
        cell_flux_src(v, 0, f, ng);
        if (f != NOF) {
          const double *a = L + (size_t)f * T::NC, *b = U + (size_t)f * T::NC;
          const double s = ((a[p10] - a[p00]) + (a[p11] - a[p01])) +
                           ((b[p10] - b[p00]) + (b[p11] - b[p01]));
          r = fma(ng ? cxk : -cxk, s, r);
        }
        cell_flux_src(v, 1, f, ng);
        if (f != NOF) {
          const double *a = L + (size_t)f * T::NC, *b = U + (size_t)f * T::NC;
          const double s = ((a[p01] - a[p00]) + (a[p11] - a[p10])) +
                           ((b[p01] - b[p00]) + (b[p11] - b[p10]));
          r = fma(ng ? cyk : -cyk, s, r);
        }
        cell_flux_src(v, 2, f, ng);
        if (f != NOF) {
          const double *a = L + (size_t)f * T::NC, *b = U + (size_t)f * T::NC;
          const double s = ((b[p00] - a[p00]) + (b[p10] - a[p10])) +
                           ((b[p01] - a[p01]) + (b[p11] - a[p11]));
          r = fma(ng ? czk : -czk, s, r);
        }
        un[v] = FT(r);
      }
    } else {
#pragma unroll
    for (int v = 0; v < 8; v++) {
      const int su = v;  // conserved fields are 0..7
      auto uL = [&](int p) { return FT(L[(size_t)su * T::NC + p]); };
      auto uU = [&](int p) { return FT(U[(size_t)su * T::NC + p]); };
      const FT uh = (uL(p10) + uL(p00) + uL(p11) + uL(p01) + uU(p10) + uU(p00) +
                     uU(p11) + uU(p01)) * 0.125;
      FT r = uh;
      int f;
      bool ng;
      cell_flux_src(v, 0, f, ng);
      if (f != NOF) {
        auto fL = [&](int p) { FT x(L[(size_t)f * T::NC + p]); return ng ? -x : x; };
        auto fU = [&](int p) { FT x(U[(size_t)f * T::NC + p]); return ng ? -x : x; };
        const FT d = (fL(p10) - fL(p00) + fL(p11) - fL(p01) + fU(p10) - fU(p00) +
                      fU(p11) - fU(p01)) * 0.25 * dxim;
        r = r - dt * d;
      }
      cell_flux_src(v, 1, f, ng);
      if (f != NOF) {
        auto fL = [&](int p) { FT x(L[(size_t)f * T::NC + p]); return ng ? -x : x; };
        auto fU = [&](int p) { FT x(U[(size_t)f * T::NC + p]); return ng ? -x : x; };
        const FT d = (fL(p01) - fL(p00) + fL(p11) - fL(p10) + fU(p01) - fU(p00) +
                      fU(p11) - fU(p10)) * 0.25 * dyim;
        r = r - dt * d;
      }
      cell_flux_src(v, 2, f, ng);
      if (f != NOF) {
        auto fL = [&](int p) { FT x(L[(size_t)f * T::NC + p]); return ng ? -x : x; };
        auto fU = [&](int p) { FT x(U[(size_t)f * T::NC + p]); return ng ? -x : x; };
        const FT d = (fU(p00) - fL(p00) + fU(p10) - fL(p10) + fU(p01) - fL(p01) +
                      fU(p11) - fL(p11)) * 0.25 * dzim;
        r = r - dt * d;
      }
      un[v] = r;
    }
    }
    if constexpr (G) {
      // mlwsrch part 2 (mlwsrch.f:41-47): un += dt * (average of the eight
      // cell sources around the corner), energy and the three momenta
      const double *gL = gcslot(k), *gU = gcslot(k + 1);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const double *l = gL + q * T::NC, *u = gU + q * T::NC;
        if constexpr (E) {
          const FT sh = (FT(l[p10]) + FT(l[p00]) + FT(l[p11]) + FT(l[p01]) + FT(u[p10]) +
                         FT(u[p00]) + FT(u[p11]) + FT(u[p01])) * 0.125;
          un[1 + q] = un[1 + q] + dt * sh;
        } else {
          const double sh = ((l[p10] + l[p00]) + (l[p11] + l[p01])) +
                            ((u[p10] + u[p00]) + (u[p11] + u[p01]));
          un[1 + q] = FT(fma(dt.v * 0.125, sh, un[1 + q].v));
        }
      }
    }
    const FT roh = un[0], eeh = un[1], rxh = un[2], ryh = un[3], rzh = un[4];
    const FT bxh = un[5], byh = un[6], bzh = un[7];
    FT vxh, vyh, vzh;
    if constexpr (E) {
      vxh = rxh / roh;
      vyh = ryh / roh;
      vzh = rzh / roh;
    } else {
      const FT rinv(1.0 / roh.v);
      vxh = rxh * rinv;
      vyh = ryh * rinv;
      vzh = rzh * rinv;
    }
    const FT vv = vxh * vxh + vyh * vyh + vzh * vzh;
    const FT bb = bxh * bxh + byh * byh + bzh * bzh;
    const FT prh = gm1 * (eeh - 0.5 * roh * vv - pi8i * bb);
    FT exh = -vyh * bzh + vzh * byh;
    FT eyh = -vzh * bxh + vxh * bzh;
    FT ezh = -vxh * byh + vyh * bxh;
    if constexpr (R) {  // mlw_m_e.f:264-269
      exh = exh + FT(rq[0]);
      eyh = eyh + FT(rq[1]);
      ezh = ezh + FT(rq[2]);
    }
    FT ep;
    if constexpr (E) ep = prh * gm / gm1 + 0.5 * roh * vv;
    else ep = prh * ph.ggm1 + 0.5 * roh * vv;
    KS(K3::XRO) = (roh * vxh).v;
    KS(K3::YRO) = (roh * vyh).v;
    KS(K3::ZRO) = (roh * vzh).v;
    KS(K3::XEE) = (ep * vxh + (bzh * eyh - byh * ezh) * pi4i).v;
    KS(K3::YEE) = (ep * vyh + (bxh * ezh - bzh * exh) * pi4i).v;
    KS(K3::ZEE) = (ep * vzh + (byh * exh - bxh * eyh) * pi4i).v;
    KS(K3::XRX) = (roh * (vxh * vxh) + prh + pi8i * (byh * byh + bzh * bzh - bxh * bxh)).v;
    KS(K3::YRX) = (roh * vxh * vyh - pi4i * bxh * byh).v;
    KS(K3::ZRX) = (roh * vxh * vzh - pi4i * bxh * bzh).v;
    KS(K3::XRY) = (roh * vyh * vxh - pi4i * byh * bxh).v;
    KS(K3::YRY) = (roh * (vyh * vyh) + prh + pi8i * (bxh * bxh + bzh * bzh - byh * byh)).v;
    KS(K3::ZRY) = (roh * vyh * vzh - pi4i * byh * bzh).v;
    KS(K3::XRZ) = (roh * vzh * vxh - pi4i * bzh * bxh).v;
    KS(K3::YRZ) = (roh * vzh * vyh - pi4i * bzh * byh).v;
    KS(K3::ZRZ) = (roh * (vzh * vzh) + prh + pi8i * (bxh * bxh + byh * byh - bzh * bzh)).v;
    KS(K3::EX) = exh.v;
    KS(K3::EY) = eyh.v;
    KS(K3::EZ) = ezh.v;
    if constexpr (G) {  // corner sources (mlw_m_g.f:289-290, 308, 326, 344)
      const FT gxm(gq[0]), gym(gq[1]), gzm(gq[2]);
      double *gk = gkslot(k);
      gk[tid] = (roh * (vxh * gxm + vyh * gym + vzh * gzm)).v;
      gk[T::NK + tid] = (roh * gxm).v;
      gk[2 * T::NK + tid] = (roh * gym).v;
      gk[3 * T::NK + tid] = (roh * gzm).v;
    }
#undef KS
  };

  // own-column data of plane k-1 kept for the z terms of plane k
  double pu[8], pfz[8], pvz = 0.0;
  auto save_prev = [&](int k) {
    const double *sl = cslot(k);
#pragma unroll
    for (int v = 0; v < 8; v++) {
      pu[v] = sl[(size_t)v * T::NC + tid];
      int f;
      bool ng;
      cell_flux_src(v, 2, f, ng);
      double x = (f != NOF) ? sl[(size_t)f * T::NC + tid] : 0.0;
      pfz[v] = ng ? -x : x;
    }
    pvz = sl[(size_t)C3::VZ * T::NC + tid];
  };

  // ---- prologue: planes kb-1 and kb, corner plane kb-1/2 -------------------
  load_plane(kb - 1);
  load_plane(kb);
  __syncthreads();
  if (interior) save_prev(kb - 1);
  corner_plane(kb - 1);
  __syncthreads();

  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  bool bad = false;  // a cell of the new state the CFL cannot use
  const FT qav(ph.qav);

  for (int k = kb; k <= ke; k++) {
    // (a) cell plane k+1 (overwrites plane k-1, whose own-column data is saved)
    load_plane(k + 1);
    __syncthreads();
    // (b) corner plane k+1/2 and the AV faces of plane k
    corner_plane(k);
    {
      const double *sl = cslot(k);
      for (int f = tid; f < T::NQX; f += T::NT) {
        const int fx = f % (TX + 1), r = f / (TX + 1);
        const int a = i0 - 1 + fx, b = j0 + r;
        double v = 0.0;
        if (a + 1 < ix && b < jx) {
          const int cl = fx + (r + 1) * T::CX;
          const FT q = qav * FT(ax.dm[a]) *
                       max0(fabs_(FT(sl[(size_t)C3::VX * T::NC + cl + 1]) -
                                  FT(sl[(size_t)C3::VX * T::NC + cl])) - CANS_AV_EPS);
          v = (q * FT(ax.dim[a])).v;
        }
        sqx[f] = v;
      }
      for (int f = tid; f < T::NQY; f += T::NT) {
        const int fx = f % TX, r = f / TX;
        const int a = i0 + fx, b = j0 - 1 + r;
        double v = 0.0;
        if (a < ix && b + 1 < jx) {
          const int cl = (fx + 1) + r * T::CX;
          const FT q = qav * FT(ay.dm[b]) *
                       max0(fabs_(FT(sl[(size_t)C3::VY * T::NC + cl + T::CX]) -
                                  FT(sl[(size_t)C3::VY * T::NC + cl])) - CANS_AV_EPS);
          v = (q * FT(ay.dim[b])).v;
        }
        sqy[f] = v;
      }
    }
    __syncthreads();
    // (c) full step of plane k
    if (interior) {
      const double *S0 = cslot(k), *S1 = cslot(k + 1);
      const double *KL = kslot(k - 1), *KU = kslot(k);
      const int c = tid, cE = c + 1, cW = c - 1, cN = c + T::CX, cS = c - T::CX;
      const int lx = hx, ly = hy;
      const int kSW = (lx - 1) + (ly - 1) * T::KX, kSE = kSW + 1;
      const int kNW = kSW + T::KX, kNE = kNW + 1;
      const FT hdt = 0.5 * dt;
      const FT dxi(ax.di[gi]), dyi(ay.di[gj]), dzi(az.di[k]);
      const FT hdx = 0.5 * dxi, hdy = 0.5 * dyi, hdz = 0.5 * dzi;
      const FT ux0(ax.u0[gi]), ux1(ax.u1[gi]), uy0(ay.u0[gj]), uy1(ay.u1[gj]);
      const FT uz0(az.u0[k]), uz1(az.u1[k]);
      const FT qxe(sqx[lx + (ly - 1) * (TX + 1)]), qxw(sqx[lx - 1 + (ly - 1) * (TX + 1)]);
      const FT qyn(sqy[(lx - 1) + ly * TX]), qys(sqy[(lx - 1) + (ly - 1) * TX]);
      const FT vz0(S0[(size_t)C3::VZ * T::NC + c]), vz1(S1[(size_t)C3::VZ * T::NC + c]);
      const FT qzu = qav * FT(az.dm[k]) * max0(fabs_(vz1 - vz0) - CANS_AV_EPS) * FT(az.dim[k]);
      const FT qzd = qav * FT(az.dm[k - 1]) * max0(fabs_(vz0 - FT(pvz)) - CANS_AV_EPS) *
                     FT(az.dim[k - 1]);
      FT unew[8];
      if constexpr (!E) {
        // Fast policy: each new conserved value is a linear combination of
        // 37 stencil values with per-cell coefficients, one chain of FMAs.
        const double h = hdt.v;
        const double fcx = h * hdx.v, fcy = h * hdy.v, fcz = h * hdz.v;
        const double hx_ = h * dxi.v, hy_ = h * dyi.v, hz_ = h * dzi.v;
        const double wxL0 = hx_ * uz0.v * uy0.v, wxL1 = hx_ * uz0.v * uy1.v;
        const double wxU0 = hx_ * uz1.v * uy0.v, wxU1 = hx_ * uz1.v * uy1.v;
        const double wyL0 = hy_ * ux0.v * uz0.v, wyU0 = hy_ * ux0.v * uz1.v;
        const double wyL1 = hy_ * ux1.v * uz0.v, wyU1 = hy_ * ux1.v * uz1.v;
        const double wzSW = hz_ * uy0.v * ux0.v, wzSE = hz_ * uy0.v * ux1.v;
        const double wzNW = hz_ * uy1.v * ux0.v, wzNE = hz_ * uy1.v * ux1.v;
        const double ae = dt.v * dxi.v * qxe.v, aw = dt.v * dxi.v * qxw.v;
        const double an = dt.v * dyi.v * qyn.v, as = dt.v * dyi.v * qys.v;
        const double au = dt.v * dzi.v * qzu.v, ad = dt.v * dzi.v * qzd.v;
        const double a1 = 1.0 - (((ae + aw) + (an + as)) + (au + ad));
#pragma unroll
        for (int v = 0; v < 8; v++) {
          const double *Sv = S0 + (size_t)v * T::NC;
          double r = a1 * Sv[c];
          r = fma(ae, Sv[cE], r);
          r = fma(aw, Sv[cW], r);
          r = fma(an, Sv[cN], r);
          r = fma(as, Sv[cS], r);
          r = fma(au, S1[(size_t)v * T::NC + c], r);
          r = fma(ad, pu[v], r);
          int f;
          bool ng;
          cell_flux_src(v, 0, f, ng);
          if (f != NOF)
            r = fma(ng ? fcx : -fcx, S0[(size_t)f * T::NC + cE] - S0[(size_t)f * T::NC + cW], r);
          cell_flux_src(v, 1, f, ng);
          if (f != NOF)
            r = fma(ng ? fcy : -fcy, S0[(size_t)f * T::NC + cN] - S0[(size_t)f * T::NC + cS], r);
          cell_flux_src(v, 2, f, ng);
          if (f != NOF) {
            const double up = ng ? -S1[(size_t)f * T::NC + c] : S1[(size_t)f * T::NC + c];
            r = fma(-fcz, up - pfz[v], r);
          }
          corner_flux_src(v, 0, f, ng);
          if (f != NOF) {
            const double *L = KL + (size_t)f * T::NK, *U = KU + (size_t)f * T::NK;
            const double sg = ng ? 1.0 : -1.0;
            r = fma(sg * wxL0, L[kSE] - L[kSW], r);
            r = fma(sg * wxL1, L[kNE] - L[kNW], r);
            r = fma(sg * wxU0, U[kSE] - U[kSW], r);
            r = fma(sg * wxU1, U[kNE] - U[kNW], r);
          }
          corner_flux_src(v, 1, f, ng);
          if (f != NOF) {
            const double *L = KL + (size_t)f * T::NK, *U = KU + (size_t)f * T::NK;
            const double sg = ng ? 1.0 : -1.0;
            r = fma(sg * wyL0, L[kNW] - L[kSW], r);
            r = fma(sg * wyU0, U[kNW] - U[kSW], r);
            r = fma(sg * wyL1, L[kNE] - L[kSE], r);
            r = fma(sg * wyU1, U[kNE] - U[kSE], r);
          }
          corner_flux_src(v, 2, f, ng);
          if (f != NOF) {
            const double *L = KL + (size_t)f * T::NK, *U = KU + (size_t)f * T::NK;
            const double sg = ng ? 1.0 : -1.0;
            r = fma(sg * wzSW, U[kSW] - L[kSW], r);
            r = fma(sg * wzSE, U[kSE] - L[kSE], r);
            r = fma(sg * wzNW, U[kNW] - L[kNW], r);
            r = fma(sg * wzNE, U[kNE] - L[kNE], r);
          }
          if constexpr (G) {
            if (v >= 1 && v <= 4) {  // mlwsrch part 1 and mlwsrcf
              const int q = v - 1;
              r = fma(h, gcslot(k)[q * T::NC + c], r);
              const double *gl = gkslot(k - 1) + q * T::NK, *gu = gkslot(k) + q * T::NK;
              const double sl_ = fma(uy0.v, fma(ux0.v, gl[kSW], ux1.v * gl[kSE]),
                                     uy1.v * fma(ux0.v, gl[kNW], ux1.v * gl[kNE]));
              const double su_ = fma(uy0.v, fma(ux0.v, gu[kSW], ux1.v * gu[kSE]),
                                     uy1.v * fma(ux0.v, gu[kNW], ux1.v * gu[kNE]));
              r = fma(h, fma(uz0.v, sl_, uz1.v * su_), r);
            }
          }
          unew[v] = FT(r);
        }
      } else {
#pragma unroll
      for (int v = 0; v < 8; v++) {
        FT du(0.0);
        int f;
        bool ng;
        // mlwhalf part 1: x, y, z central differences
        cell_flux_src(v, 0, f, ng);
        if (f != NOF) {
          FT a(S0[(size_t)f * T::NC + cE]), b(S0[(size_t)f * T::NC + cW]);
          if (ng) { a = -a; b = -b; }
          du = du - hdt * (hdx * (a - b));
        }
        cell_flux_src(v, 1, f, ng);
        if (f != NOF) {
          FT a(S0[(size_t)f * T::NC + cN]), b(S0[(size_t)f * T::NC + cS]);
          if (ng) { a = -a; b = -b; }
          du = du - hdt * (hdy * (a - b));
        }
        cell_flux_src(v, 2, f, ng);
        if (f != NOF) {
          FT a(S1[(size_t)f * T::NC + c]);
          if (ng) a = -a;
          du = du - hdt * (hdz * (a - FT(pfz[v])));
        }
        // mlwsrch part 1 (mlwsrch.f:35): du += 0.5*dt*s
        if (G && v >= 1 && v <= 4) du = du + hdt * FT(gcslot(k)[(v - 1) * T::NC + c]);
        // mlwfull: corner planes k-1/2 (L) and k+1/2 (U)
        corner_flux_src(v, 0, f, ng);
        if (f != NOF) {
          auto L = [&](int p) { FT x(KL[(size_t)f * T::NK + p]); return ng ? -x : x; };
          auto U = [&](int p) { FT x(KU[(size_t)f * T::NK + p]); return ng ? -x : x; };
          const FT dfdx = dxi * (uz0 * (uy0 * (L(kSE) - L(kSW)) + uy1 * (L(kNE) - L(kNW))) +
                                 uz1 * (uy0 * (U(kSE) - U(kSW)) + uy1 * (U(kNE) - U(kNW))));
          du = du - hdt * dfdx;
        }
        corner_flux_src(v, 1, f, ng);
        if (f != NOF) {
          auto L = [&](int p) { FT x(KL[(size_t)f * T::NK + p]); return ng ? -x : x; };
          auto U = [&](int p) { FT x(KU[(size_t)f * T::NK + p]); return ng ? -x : x; };
          const FT dfdy = dyi * (ux0 * (uz0 * (L(kNW) - L(kSW)) + uz1 * (U(kNW) - U(kSW))) +
                                 ux1 * (uz0 * (L(kNE) - L(kSE)) + uz1 * (U(kNE) - U(kSE))));
          du = du - hdt * dfdy;
        }
        corner_flux_src(v, 2, f, ng);
        if (f != NOF) {
          auto L = [&](int p) { FT x(KL[(size_t)f * T::NK + p]); return ng ? -x : x; };
          auto U = [&](int p) { FT x(KU[(size_t)f * T::NK + p]); return ng ? -x : x; };
          const FT dfdz = dzi * (uy0 * (ux0 * (U(kSW) - L(kSW)) + ux1 * (U(kSE) - L(kSE))) +
                                 uy1 * (ux0 * (U(kNW) - L(kNW)) + ux1 * (U(kNE) - L(kNE))));
          du = du - hdt * dfdz;
        }
        // mlwsrcf (mlwsrcf.f:38-42): du += 0.5*dt*(corner sources to the cell)
        if (G && v >= 1 && v <= 4) {
          const double *gl = gkslot(k - 1) + (v - 1) * T::NK, *gu = gkslot(k) + (v - 1) * T::NK;
          const FT sh = uz0 * (uy0 * (ux0 * FT(gl[kSW]) + ux1 * FT(gl[kSE])) +
                               uy1 * (ux0 * FT(gl[kNW]) + ux1 * FT(gl[kNE]))) +
                        uz1 * (uy0 * (ux0 * FT(gu[kSW]) + ux1 * FT(gu[kSE])) +
                               uy1 * (ux0 * FT(gu[kNW]) + ux1 * FT(gu[kNE])));
          du = du + hdt * sh;
        }
        // mlwartv
        const FT u(S0[(size_t)v * T::NC + c]);
        du = du + dt * (dxi * (qxe * (FT(S0[(size_t)v * T::NC + cE]) - u) -
                               qxw * (u - FT(S0[(size_t)v * T::NC + cW])))) +
             dt * (dyi * (qyn * (FT(S0[(size_t)v * T::NC + cN]) - u) -
                          qys * (u - FT(S0[(size_t)v * T::NC + cS])))) +
             dt * (dzi * (qzu * (FT(S1[(size_t)v * T::NC + c]) - u) - qzd * (u - FT(pu[v]))));
        unew[v] = u + du;
      }
      }
      const FT ro = unew[0], ee = unew[1], rx = unew[2], ry = unew[3], rz = unew[4];
      const FT bx = unew[5], by = unew[6], bz = unew[7];
      FT vx, vy, vz;
      if constexpr (E) {
        vx = rx / ro;
        vy = ry / ro;
        vz = rz / ro;
      } else {
        const FT rinv(1.0 / ro.v);
        vx = rx * rinv;
        vy = ry * rinv;
        vz = rz * rinv;
      }
      const FT vv = vx * vx + vy * vy + vz * vz;
      const FT bb = bx * bx + by * by + bz * bz;
      const FT pr = gm1 * (ee - 0.5 * ro * vv - pi8i * bb);
      const size_t g = (size_t)gi + (size_t)gj * ix + (size_t)k * plane;
      B[P3::RO * n + g] = ro.v;
      B[P3::PR * n + g] = pr.v;
      B[P3::VX * n + g] = vx.v;
      B[P3::VY * n + g] = vy.v;
      B[P3::VZ * n + g] = vz.v;
      B[P3::BX * n + g] = bx.v;
      B[P3::BY * n + g] = by.v;
      B[P3::BZ * n + g] = bz.v;
      if (ctl != nullptr && gi >= box.lo[0] && gi <= box.hi[0] && gj >= box.lo[1] &&
          gj <= box.hi[1] && k >= box.lo[2] && k <= box.hi[2]) {
        // cans3d/common/cfl_m.f:52-59 (pi in single precision)
        const FT b2 = bx * bx + by * by + bz * bz;
        const FT v2 = vx * vx + vy * vy + vz * vz;
        if constexpr (E) {
          const FT ca2 = b2 * FT(ph.pi4i_cfl) / ro;
          const FT cs2 = gm * pr / ro;
          const FT dmn = fmin_(fmin_(FT(ax.d[gi]), FT(ay.d[gj])), FT(az.d[k]));
          const double dtq = (FT(ctl->safety) * (dmn / fsqrt(v2 + cs2 + ca2))).v;
          if (dtq < dmin) dmin = dtq;
          bad |= bad_cell(ro.v, pr.v, dtq);
        } else {
          // largest S*max(1/dx^2,1/dy^2,1/dz^2) gives the smallest dt; dmin
          // holds minus that key (see the block reduction below)
          const double rinv = 1.0 / ro.v;
          const double s = v2.v + fma(gm.v, pr.v, ph.pi4i_cfl * b2.v) * rinv;
          const double kk = s * fmax(fmax(dxi.v * dxi.v, dyi.v * dyi.v), dzi.v * dzi.v);
          if (-kk < dmin) dmin = -kk;
          bad |= bad_cell(ro.v, pr.v, kk);
        }
      }
      save_prev(k);
    }
    // ghost cells keep their input values (cans3d/hdmlw/mlw_m.f updates
    // only 2..n-1); each is copied by the block owning its nearest interior
    // cell, plane by plane, plus the z ghost planes at the chunk ends.
    if (in_arr) {
      const int ci = min(max(gi, 1), ix - 2), cj = min(max(gj, 1), jx - 2);
      const bool owner = ci >= i0 && ci < i0 + TX && cj >= j0 && cj < j0 + TY;
      if (owner) {
        const bool xy_ghost = (gi == 0 || gi == ix - 1 || gj == 0 || gj == jx - 1);
        auto copy = [&](int kk) {
          const size_t g = (size_t)gi + (size_t)gj * ix + (size_t)kk * plane;
#pragma unroll
          for (int v = 0; v < P3::N; v++) B[v * n + g] = A[v * n + g];
        };
        if (xy_ghost) copy(k);
        if (k == 1) copy(0);
        if (k == kx - 2) copy(kx - 1);
      }
    }
    __syncthreads();
  }
  if (ctl != nullptr) {
    count_bad_block(bad, &ctl->nonfinite, tid);
    if constexpr (E) {
      block_min_to(&ctl->cfl_bits, dmin, sred, tid, T::NT);
    } else {
      const double m = block_min(dmin, sred, tid, T::NT);  // -(largest key)
      if (tid == 0 && m < 0.0) atomic_min_pos(&ctl->cfl_bits, ctl->safety / sqrt(-m));
    }
  }
}

namespace {
// The z chunk (at most kmax planes) that fills the GPU best: a launch of b
// blocks with `slots` resident at a time takes ceil(b / slots) waves, and a
// block of kc planes costs about kc + 1 plane steps (its prologue loads two
// planes).  The partition into chunks does not change any result.
int balance_kchunk(long long bxy, int nz, int kmax, int slots) {
  if (nz < 1 || kmax < 1 || slots < 1) return kmax;
  const int c0 = (nz + kmax - 1) / kmax;
  int best = kmax;
  long long best_cost = -1;
  for (int c = c0; c <= nz && c <= 4 * c0 + 8; c++) {
    const int kc = (nz + c - 1) / c;
    const long long chunks = (nz + kc - 1) / kc;
    const long long waves = (bxy * chunks + slots - 1) / slots;
    const long long cost = waves * (kc + 1);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = kc;
    }
  }
  return best;
}

constexpr int kMaxDevices3 = 64;

template <bool E, int TX, int TY, bool G = false, bool R = false>
cudaError_t launch3(const double *A, double *B, int ix, int jx, int kx,
                    const Axis &ax, const Axis &ay, const Axis &az,
                    const Phys &ph, double dt, Ctl *ctl, Box3 box, int kchunk,
                    cudaStream_t s, const double *grav = nullptr,
                    const double *res = nullptr) {
  using T = Tile3<TX, TY, G>;
  // per device: the shared-memory attribute is set and the resident blocks
  // on the whole GPU counted once, under a lock (launches may come from
  // several host threads and devices)
  static std::mutex mu;
  static int slots_of[kMaxDevices3] = {};
  int dev = 0, slots = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices3) return cudaErrorInvalidDevice;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!slots_of[dev]) {
      e = cudaFuncSetAttribute(k_mlw3d<E, TX, TY, G, R>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
      if (e != cudaSuccess) return e;
      int sms = 0, per_sm = 0;
      if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return e;
      if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
               &per_sm, k_mlw3d<E, TX, TY, G, R>, T::NT, T::smem_bytes)) != cudaSuccess)
        return e;
      slots_of[dev] = sms * (per_sm > 0 ? per_sm : 1);
    }
    slots = slots_of[dev];
  }
  const int bx = (ix - 2 + TX - 1) / TX, by = (jx - 2 + TY - 1) / TY;
  kchunk = balance_kchunk((long long)bx * by, kx - 2, kchunk, slots);
  dim3 grid(bx, by, (kx - 2 + kchunk - 1) / kchunk);
  dim3 block(T::NT);
  k_mlw3d<E, TX, TY, G, R><<<grid, block, T::smem_bytes, s>>>(
      A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl, box, kchunk, grav, res);
  count_launch();
  return cudaGetLastError();
}
}  // namespace

// mlw_m_g: the gravity rings do not fit beside a 16 x 16 tile (222 KB), so
// the step with gravity runs 16 x 8 tiles (143 KB, 6 warps; z chunks of 64
// or 32), 16 x 12 tiles (202 KB, 8 warps) or 24 x 8 tiles (208 KB, 9 warps;
// chunks of 32).
int mlw3d_g_tile_count() { return 4; }

cudaError_t launch_mlw3d_g(bool exact, int tile, const double *A, double *B, int ix,
                           int jx, int kx, const Axis &ax, const Axis &ay, const Axis &az,
                           const Phys &ph, const double *grav, double dt, Ctl *ctl,
                           Box3 box, cudaStream_t s) {
  if (ix < 3 || jx < 3 || kx < 3 || grav == nullptr) return cudaErrorInvalidValue;
  const int kchunk = (tile == 1 || tile == 3) ? 32 : 64;
  if (tile == 3)
    return exact ? launch3<true, 24, 8, true>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl, box,
                                              kchunk, s, grav)
                 : launch3<false, 24, 8, true>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl,
                                               box, kchunk, s, grav);
  if (tile == 2)
    return exact ? launch3<true, 16, 12, true>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl, box,
                                               kchunk, s, grav)
                 : launch3<false, 16, 12, true>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl,
                                                box, kchunk, s, grav);
  return exact ? launch3<true, 16, 8, true>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl, box,
                                            kchunk, s, grav)
               : launch3<false, 16, 8, true>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl, box,
                                             kchunk, s, grav);
}

int mlw3d_tile_count() { return 3; }

// The step of mlw_m_e given the eta J fields res (6 arrays): the plain step's
// tiles (no extra shared memory).
cudaError_t launch_mlw3d_res(bool exact, int tile, const double *A, double *B, int ix,
                             int jx, int kx, const Axis &ax, const Axis &ay, const Axis &az,
                             const Phys &ph, const double *res, double dt, Ctl *ctl,
                             Box3 box, cudaStream_t s) {
  const int kchunk = (tile == 1) ? 32 : 64;
  if (tile == 2)
    return exact ? launch3<true, 16, 8, false, true>(A, B, ix, jx, kx, ax, ay, az, ph, dt,
                                                     ctl, box, kchunk, s, nullptr, res)
                 : launch3<false, 16, 8, false, true>(A, B, ix, jx, kx, ax, ay, az, ph, dt,
                                                      ctl, box, kchunk, s, nullptr, res);
  return exact ? launch3<true, 16, 16, false, true>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl,
                                                    box, kchunk, s, nullptr, res)
               : launch3<false, 16, 16, false, true>(A, B, ix, jx, kx, ax, ay, az, ph, dt,
                                                     ctl, box, kchunk, s, nullptr, res);
}

cudaError_t launch_mlw3d(bool exact, int tile, const double *A, double *B,
                         int ix, int jx, int kx, const Axis &ax,
                         const Axis &ay, const Axis &az, const Phys &ph,
                         double dt, Ctl *ctl, Box3 box, cudaStream_t s) {
  if (ix < 3 || jx < 3 || kx < 3) return cudaErrorInvalidValue;
  // tile: 0 = 16x16 tiles, z chunks of 64; 1 = 16x16, chunks of 32;
  //       2 = 16x8 tiles, chunks of 64
  const int kchunk = (tile == 1) ? 32 : 64;
  if (tile == 2)
    return exact ? launch3<true, 16, 8>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl, box, kchunk, s)
                 : launch3<false, 16, 8>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl, box, kchunk, s);
  return exact ? launch3<true, 16, 16>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl, box, kchunk, s)
               : launch3<false, 16, 16>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl, box, kchunk, s);
}

// ---------------------------------------------------------------------------
// CFL over all cells (cans3d/common/cfl_m.f:39-85) and over the frame of cells
// the boundary fill may rewrite, with the start of the next iteration
// (per-cell expression in cfl3.cuh).
template <bool E>
__global__ void k_cfl3d_full(const double *__restrict__ S, int ix, int jx,
                             int kx, Axis ax, Axis ay, Axis az, Phys ph,
                             double safety, unsigned long long *out) {
  __shared__ double red[32];
  const size_t plane = (size_t)ix * jx, n = plane * kx;
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n;
       g += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(g / plane);
    const size_t r = g % plane;
    const int j = (int)(r / ix), i = (int)(r % ix);
    const double d = cfl3_cell<E>(S, n, g, i, j, k, ax, ay, az, ph, safety);
    if (d < dmin) dmin = d;
  }
  block_min_to(out, dmin, red, threadIdx.x, blockDim.x);
}

cudaError_t launch_cfl3d_full(bool exact, const double *S, int ix, int jx,
                              int kx, const Axis &ax, const Axis &ay,
                              const Axis &az, const Phys &ph, double safety,
                              unsigned long long *out_bits, cudaStream_t s) {
  const size_t n = (size_t)ix * jx * kx;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (exact) k_cfl3d_full<true><<<blocks, 256, 0, s>>>(S, ix, jx, kx, ax, ay, az, ph, safety, out_bits);
  else k_cfl3d_full<false><<<blocks, 256, 0, s>>>(S, ix, jx, kx, ax, ay, az, ph, safety, out_bits);
  count_launch();
  return cudaGetLastError();
}

// Frame: cells with any index within w of its faces, enumerated as z slabs,
// then y slabs of the remaining planes, then x slabs of the remaining rows.
__device__ __forceinline__ void frame3_index(long long f, int ix, int jx, int kx,
                                             int w, int &i, int &j, int &k) {
  const long long zs = 2LL * w * ix * jx;
  if (f < zs) {
    const long long p = f / ((long long)ix * jx), r = f % ((long long)ix * jx);
    k = (p < w) ? (int)p : (int)(kx - 2 * w + p);
    j = (int)(r / ix);
    i = (int)(r % ix);
    return;
  }
  f -= zs;
  const long long kin = kx - 2LL * w;
  const long long ys = 2LL * w * ix * kin;
  if (f < ys) {
    const long long per = 2LL * w * ix;
    k = (int)(w + f / per);
    const long long r = f % per, jr = r / ix;
    i = (int)(r % ix);
    j = (jr < w) ? (int)jr : (int)(jx - 2 * w + jr);
    return;
  }
  f -= ys;
  const long long jin = jx - 2LL * w;
  const long long per = 2LL * w * jin;
  k = (int)(w + f / per);
  const long long r = f % per;
  j = (int)(w + r / (2 * w));
  const int c = (int)(r % (2 * w));
  i = (c < w) ? c : (ix - 2 * w + c);
}

// With all = 1 the CFL covers every cell (a loop with chkdav after the fill).
template <bool E>
__global__ void k_frame3d(int ix, int jx, int kx, Axis ax, Axis ay, Axis az,
                          Phys ph, int w, int all, Ctl *ctl) {
  __shared__ double red[32];
  if (ctl->done | ctl->pause) return;
  const double *S = ctl->buf[ctl->cur ^ 1];
  const size_t plane = (size_t)ix * jx, n = plane * kx;
  const long long total = all ? (long long)n
                              : 2LL * w * ix * jx + 2LL * w * ix * (kx - 2LL * w) +
                                    2LL * w * (jx - 2LL * w) * (kx - 2LL * w);
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  bool bad = false;
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < total;
       f += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    if (all) {
      i = (int)(f % ix);
      j = (int)((f / ix) % jx);
      k = (int)(f / ((long long)ix * jx));
    } else {
      frame3_index(f, ix, jx, kx, w, i, j, k);
    }
    const size_t g = (size_t)i + (size_t)j * ix + (size_t)k * plane;
    const double d = cfl3_cell<E>(S, n, g, i, j, k, ax, ay, az, ph, ctl->safety);
    if (d < dmin) dmin = d;
    bad |= bad_cell(S[P3::RO * n + g], S[P3::PR * n + g], d);
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

cudaError_t launch_frame3d(bool exact, int ix, int jx, int kx, const Axis &ax,
                           const Axis &ay, const Axis &az, const Phys &ph,
                           int margin, Ctl *ctl, cudaStream_t s, int all) {
  const int w = margin + 1;
  const long long total = all ? (long long)ix * jx * kx
                              : 2LL * w * ix * jx + 2LL * w * ix * (kx - 2LL * w) +
                                    2LL * w * (jx - 2LL * w) * (kx - 2LL * w);
  int blocks = (int)((total + 255) / 256);
  if (blocks < 1) blocks = 1;
  if (blocks > 152 * 4) blocks = 152 * 4;
  if (exact) k_frame3d<true><<<blocks, 256, 0, s>>>(ix, jx, kx, ax, ay, az, ph, w, all, ctl);
  else k_frame3d<false><<<blocks, 256, 0, s>>>(ix, jx, kx, ax, ay, az, ph, w, all, ctl);
  count_launch();
  return cudaGetLastError();
}

}  // namespace cans
