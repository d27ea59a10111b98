// Fused 2-D modified Lax-Wendroff step (sm_103a, FP64): the tile body.
//
// One kernel replaces the whole body of the reference routines
//   mlw_m3  cans2d/hdmlw/mlw_m3.f:64-374  (ro,pr,vx,vy,vz,bx,by,bz + az)
//   mlw_m   cans2d/hdmlw/mlw_m.f          (ro,pr,vx,vy,bx,by + az)
// with their primitives mlwhalf (cans2d/hdmlw/mlwhalf.f:36-52), mlwsrch
// (mlwsrch.f:87-102), mlwfull (mlwfull.f:136-146), mlwsrcf (mlwsrcf.f:182-189)
// and mlwartv (mlwartv.f:225-233).  The reference makes ~30 sweeps over ~37
// full-grid temporaries; here each thread block stages a TX x TY tile plus a
// one-cell halo in shared memory and makes three passes over it:
//   phase 1  cells (TX+2)(TY+2): conserved variables, cell fluxes, E = -v x B
//   phase 2  corners (TX+1)(TY+1): half-step predictor (mlwhalf part 2,
//            mlwsrch), half-step primitives and corner fluxes; and the
//            artificial-viscosity face coefficients q*dxim
//   phase 3  cells TX x TY: du = central-difference half-step term
//            (mlwhalf part 1) + corrector (mlwfull, mlwsrcf) + artificial
//            viscosity (mlwartv); u += du; back to primitives; write out.
// The state crosses HBM once in and once out (9 arrays for mlw_m3).
//
// With G the tile is mlw_m3_g / mlw_m_g (cans2d/hdmlw/mlw_m3_g.f:95-121,
// 194-220; mlw_m_g.f:96-122, 175-201): gravity sources ro (v.g), ro gx, ro gy
// at the cells and the same of the half-step state at the corners enter the
// energy and the x, y momenta through mlwsrch and mlwsrcf.  grav holds gx,
// gxm, gy, gym (ix*jx each; gxm, gym at the corner (i+1/2, j+1/2)).
//
// With R the tile is the resistive step mlw_m3_e / mlw_m_e (and with G as
// well mlw_m3_ge / mlw_m_ge; cans2d/hdmlw/mlw_m3_e.f:124-132, 236-244,
// mlw_m_e.f:125-129, 216-220): res holds eta J at the cells and at the
// corners, computed beforehand by the kernels of mlw2d_e.cu, and each is
// added to E = -v x B where the reference adds et*c and etm*ch.  res is
// [x, y, z at the cells, x, y, z at the corners] (ix*jx each) for mlw_m3 and
// [z at the cells, z at the corners] for mlw_m.
//
// With AVF the artificial viscosity's branch is recorded (AVF = 1) or held
// (AVF = 2), for the finite-difference check of the discrete adjoint: the
// coefficient q = qav dxm max(0, |dv| - 1e-4) of mlw_m3.f:325-334 is
// piecewise affine in dv, and the adjoint is the derivative of the branch
// the base run took.  Per face one byte: bit 0 = |dv| - 1e-4 > 0 (active),
// bit 1 = dv < 0.  Recording leaves every result unchanged; holding takes
// q = qav dxm (s dv - 1e-4) on the faces recorded active (s the recorded
// sign) and 0 on the others, and counts the faces whose own branch differs
// from the recorded one (each face once).  avb holds the x faces (i, j)
// between cells i and i+1, then the y faces (i, j) between rows j and j+1,
// ix*jx bytes each.
//
// In the exact policy every operation is the reference's, in its order, so
// the result equals a -ffp-contract=off CPU build of the Fortran bit for bit.
// Terms whose flux is identically zero (fx of bx, fy of by) are skipped: the
// reference adds dt*(+0) to them, which leaves every value unchanged.
#pragma once
#include <cuda_runtime.h>

#include "cans_common.cuh"
#include "cans_internal.h"

namespace cans {

namespace {

// Cell-array slots in shared memory (per cell of the halo tile).
template <bool M3> struct CellSlots;
template <> struct CellSlots<true> {
  // conserved: ro ee rx ry rz bx by bz
  static constexpr int RO = 0, EE = 1, RX = 2, RY = 3, RZ = 4, BX = 5, BY = 6,
                       BZ = 7;
  static constexpr int FXE = 8, FXRX = 9, FXRY = 10, FXRZ = 11;
  static constexpr int FYE = 12, FYRX = 13, FYRY = 14, FYRZ = 15;
  static constexpr int EX = 16, EY = 17, EZ = 18, VX = 19, VY = 20;
  static constexpr int N = 21, NU = 8;
};
template <> struct CellSlots<false> {
  static constexpr int RO = 0, EE = 1, RX = 2, RY = 3, BX = 4, BY = 5;
  static constexpr int FXE = 6, FXRX = 7, FXRY = 8;
  static constexpr int FYE = 9, FYRX = 10, FYRY = 11;
  static constexpr int EZ = 12, VX = 13, VY = 14;
  static constexpr int N = 15, NU = 6;
  // unused in 2-D, kept so generic code compiles
  static constexpr int RZ = -1, BZ = -1, FXRZ = -1, FYRZ = -1, EX = -1, EY = -1;
};
// Corner-array slots (half-step fluxes at the cell corners).
template <bool M3> struct CornerSlots;
template <> struct CornerSlots<true> {
  static constexpr int XRO = 0, XEE = 1, XRX = 2, XRY = 3, XRZ = 4;
  static constexpr int YRO = 5, YEE = 6, YRX = 7, YRY = 8, YRZ = 9;
  static constexpr int EX = 10, EY = 11, EZ = 12, N = 13;
};
template <> struct CornerSlots<false> {
  static constexpr int XRO = 0, XEE = 1, XRX = 2, XRY = 3;
  static constexpr int YRO = 4, YEE = 5, YRX = 6, YRY = 7;
  static constexpr int EZ = 8, N = 9;
  static constexpr int XRZ = -1, YRZ = -1, EX = -1, EY = -1;
};
// Primitive-array order in global memory.
template <bool M3> struct Prim;
template <> struct Prim<true> {
  static constexpr int RO = 0, PR = 1, VX = 2, VY = 3, VZ = 4, BX = 5, BY = 6,
                       BZ = 7, AZ = 8, N = 9;
};
template <> struct Prim<false> {
  static constexpr int RO = 0, PR = 1, VX = 2, VY = 3, BX = 4, BY = 5, AZ = 6,
                       N = 7;
  static constexpr int VZ = -1, BZ = -1;
};

// TX x TY interior cells per tile; each thread updates RPT of them (rows
// RPT apart), so a block has TX*TY/RPT threads.
template <int TX, int TY, bool M3, int RPT = 2, bool G = false> struct Tile {
  static constexpr int CX = TX + 2, CY = TY + 2, NC = CX * CY;
  static constexpr int KX = TX + 1, KY = TY + 1, NK = KX * KY;
  static constexpr int NQX = (TX + 1) * TY, NQY = TX * (TY + 1);
  static constexpr int NT = TX * TY / RPT;
  // gravity: three source arrays at the cells and three at the corners
  static constexpr size_t smem_doubles =
      (size_t)CellSlots<M3>::N * NC + (size_t)CornerSlots<M3>::N * NK + NQX +
      NQY + 32 + (G ? 3 * ((size_t)NC + NK) : 0);
  static constexpr size_t smem_bytes = smem_doubles * sizeof(double);
};

// Zero-flux marker for the corrector / central-difference helpers.
constexpr int NOFLUX = -1;

// Branch byte of one viscosity face (see tile_step): the face's own branch
// from dv and a = |dv| - 1e-4 is recorded (AVF = 1) and returned, or
// compared with the recorded one, which is returned (AVF = 2); a face a
// tile owns counts a flip of its active bit (or of its sign while active).
template <int AVF, class FT>
__device__ __forceinline__ unsigned char av_branch(double dv, FT a, unsigned char *slot,
                                                   unsigned long long *nflip, bool owned) {
  const unsigned char mine = (unsigned char)((a.v > 0.0 ? 1 : 0) | (dv < 0.0 ? 2 : 0));
  if constexpr (AVF == 1) {
    *slot = mine;
    return mine;
  } else {
    const unsigned char rec = *slot;
    const unsigned char x = rec ^ mine;
    if (owned && ((x & 1) || ((rec & mine & 1) && (x & 2)))) atomicAdd(nflip, 1ull);
    return rec;
  }
}

}  // namespace

// One TX x TY tile of one grid: the whole fused step.  Called by the
// single-grid kernel (one tile per block) and by the batched kernel (tiles
// of many grids pulled from a work queue by persistent blocks).  If cfl_out
// is non-null the CFL of the written cells inside `box` is reduced into it.
template <bool E, bool M3, int TX, int TY, int RPT, bool G = false, bool R = false,
          int AVF = 0>
__device__ __forceinline__ void tile_step(
    const double *__restrict__ A, double *__restrict__ B, int ix, int jx,
    const Axis &ax, const Axis &ay, const Phys &ph, double dtv, double safety,
    unsigned long long *cfl_out, const Box3 &box, int tile_x, int tile_y,
    int ntiles_x, int ntiles_y, double *smem,
    const double *__restrict__ grav = nullptr,
    const double *__restrict__ res = nullptr, int *bad_out = nullptr,
    unsigned char *avb = nullptr, unsigned long long *nflip = nullptr) {
  using T = Tile<TX, TY, M3, RPT, G>;
  using C = CellSlots<M3>;
  using K = CornerSlots<M3>;
  using P = Prim<M3>;
  using FT = F<E>;
  double *sc = smem;                            // cells   [C::N][NC]
  double *sk = sc + (size_t)C::N * T::NC;       // corners [K::N][NK]
  double *sqx = sk + (size_t)K::N * T::NK;      // q*dxim  [TY][TX+1]
  double *sqy = sqx + T::NQX;                   // q*dyim  [TY+1][TX]
  double *sred = sqy + T::NQY;                  // reduction scratch (32)
  double *sgc = sred + 32;                      // G: cell sources   [3][NC]
  double *sgk = sgc + 3 * T::NC;                // G: corner sources [3][NK]

  // a persistent block may come here from another tile: its reads of
  // shared memory must be over before this tile writes it
  __syncthreads();
  const FT dt(dtv);
  const size_t n = (size_t)ix * (size_t)jx;
  const int i0 = 1 + tile_x * TX;  // first interior cell of the tile
  const int j0 = 1 + tile_y * TY;
  const int tid = threadIdx.x;
  const FT gm(ph.gm), gm1(ph.gm1), pi8i(ph.pi8i), pi4i(ph.pi4i);

#define SC(slot, c) sc[(size_t)(slot) * T::NC + (c)]
#define SK(slot, c) sk[(size_t)(slot) * T::NK + (c)]
#define SGC(slot, c) sgc[(size_t)(slot) * T::NC + (c)]
#define SGK(slot, c) sgk[(size_t)(slot) * T::NK + (c)]

  // ---------------- phase 1: cells of the halo tile ------------------------
  for (int c = tid; c < T::NC; c += T::NT) {
    const int lx = c % T::CX, ly = c / T::CX;
    const int gi = i0 - 1 + lx, gj = j0 - 1 + ly;
    if (gi < ix && gj < jx) {
      const size_t g = (size_t)gi + (size_t)gj * ix;
      const FT ro(A[P::RO * n + g]), pr(A[P::PR * n + g]);
      const FT vx(A[P::VX * n + g]), vy(A[P::VY * n + g]);
      const FT bx(A[P::BX * n + g]), by(A[P::BY * n + g]);
      FT vz(0.0), bz(0.0);
      if constexpr (M3) { vz = FT(A[P::VZ * n + g]); bz = FT(A[P::BZ * n + g]); }
      FT vv, bb;
      if constexpr (M3) {
        vv = vx * vx + vy * vy + vz * vz;
        bb = bx * bx + by * by + bz * bz;
      } else {
        vv = vx * vx + vy * vy;
        bb = bx * bx + by * by;
      }
      FT ee, ep;
      if constexpr (E) {
        ee = pr / gm1 + 0.5 * ro * vv + pi8i * bb;     // mlw_m3.f:111
        ep = pr * gm / gm1 + 0.5 * ro * vv;            // mlw_m3.f:141
      } else {
        ee = pr * ph.gm1i + 0.5 * ro * vv + pi8i * bb;
        ep = pr * ph.ggm1 + 0.5 * ro * vv;
      }
      const FT rx = ro * vx, ry = ro * vy;
      if constexpr (G) {  // mlw_m3_g.f:95, 106, 117
        const FT gxc(grav[g]), gyc(grav[2 * n + g]);
        SGC(0, c) = (ro * (vx * gxc + vy * gyc)).v;
        SGC(1, c) = (ro * gxc).v;
        SGC(2, c) = (ro * gyc).v;
      }
      SC(C::RO, c) = ro.v; SC(C::EE, c) = ee.v;
      SC(C::RX, c) = rx.v; SC(C::RY, c) = ry.v;
      SC(C::BX, c) = bx.v; SC(C::BY, c) = by.v;
      SC(C::VX, c) = vx.v; SC(C::VY, c) = vy.v;
      if constexpr (M3) {
        const FT rz = ro * vz;
        FT ex = -vy * bz + vz * by;                    // mlw_m3.f:119-121
        FT ey = -vz * bx + vx * bz;
        FT ez = -vx * by + vy * bx;
        if constexpr (R) {                             // mlw_m3_e.f:130-132
          ex = ex + FT(res[g]);
          ey = ey + FT(res[n + g]);
          ez = ez + FT(res[2 * n + g]);
        }
        SC(C::RZ, c) = rz.v; SC(C::BZ, c) = bz.v;
        SC(C::EX, c) = ex.v; SC(C::EY, c) = ey.v; SC(C::EZ, c) = ez.v;
        // energy flux (:141-143)
        SC(C::FXE, c) = (ep * vx + (bz * ey - by * ez) * pi4i).v;
        SC(C::FYE, c) = (ep * vy + (bx * ez - bz * ex) * pi4i).v;
        // momentum fluxes (:151-153, :161-163, :171-172)
        SC(C::FXRX, c) = (ro * (vx * vx) + pr + pi8i * (by * by + bz * bz - bx * bx)).v;
        SC(C::FYRX, c) = (ro * vx * vy - pi4i * bx * by).v;
        SC(C::FXRY, c) = (ro * vy * vx - pi4i * by * bx).v;
        SC(C::FYRY, c) = (ro * (vy * vy) + pr + pi8i * (bx * bx + bz * bz - by * by)).v;
        SC(C::FXRZ, c) = (ro * vz * vx - pi4i * bz * bx).v;
        SC(C::FYRZ, c) = (ro * vz * vy - pi4i * bz * by).v;
      } else {
        FT ez = -vx * by + vy * bx;                    // mlw_m.f:70
        if constexpr (R) ez = ez + FT(res[g]);         // mlw_m_e.f:129
        SC(C::EZ, c) = ez.v;
        SC(C::FXE, c) = (ep * vx - by * ez * pi4i).v;  // mlw_m.f:85-86
        SC(C::FYE, c) = (ep * vy + bx * ez * pi4i).v;
        SC(C::FXRX, c) = (ro * (vx * vx) + pr + pi8i * (by * by - bx * bx)).v;
        SC(C::FYRX, c) = (ro * vx * vy - pi4i * bx * by).v;
        SC(C::FXRY, c) = (ro * vy * vx - pi4i * by * bx).v;
        SC(C::FYRY, c) = (ro * (vy * vy) + pr + pi8i * (bx * bx - by * by)).v;
      }
    } else {
#pragma unroll 1
      for (int s = 0; s < C::N; s++) SC(s, c) = 0.0;
      if constexpr (G) {
        SGC(0, c) = 0.0; SGC(1, c) = 0.0; SGC(2, c) = 0.0;
      }
    }
  }
  __syncthreads();

  // ---------------- phase 2: corners and viscosity faces -------------------
  for (int c = tid; c < T::NK; c += T::NT) {
    const int kx = c % T::KX, ky = c / T::KX;
    const int gi = i0 - 1 + kx, gj = j0 - 1 + ky;  // lower-left cell of corner
    if (gi <= ix - 2 && gj <= jx - 2) {
      const int a = kx + ky * T::CX;      // (i  ,j  )
      const int b = a + 1;                // (i+1,j  )
      const int cc = a + 1 + T::CX;       // (i+1,j+1)
      const int d = a + T::CX;            // (i  ,j+1)
      const FT dxim(ax.dim[gi]), dyim(ay.dim[gj]);
      // mlwhalf part 2: un = avg4(u) - dt*dfdx - dt*dfdy   (mlwhalf.f:45-52)
      const double cxk = dt.v * dxim.v * 0.5, cyk = dt.v * dyim.v * 0.5;
      auto pred = [&](int su, int sfx, int sfy, bool negx, bool negy) -> FT {
        if constexpr (!E) {  // same predictor, fewer rounded operations
          double r = 0.25 * ((SC(su, b) + SC(su, a)) + (SC(su, cc) + SC(su, d)));
          if (sfx != NOFLUX) {
            const double s = (SC(sfx, b) - SC(sfx, a)) + (SC(sfx, cc) - SC(sfx, d));
            r = fma(negx ? cxk : -cxk, s, r);
          }
          if (sfy != NOFLUX) {
            const double s = (SC(sfy, d) - SC(sfy, a)) + (SC(sfy, cc) - SC(sfy, b));
            r = fma(negy ? cyk : -cyk, s, r);
          }
          return FT(r);
        }
        const FT uh = 0.25 * (FT(SC(su, b)) + FT(SC(su, a)) + FT(SC(su, cc)) +
                              FT(SC(su, d)));
        FT un = uh;
        if (sfx != NOFLUX) {
          FT fb(SC(sfx, b)), fa(SC(sfx, a)), fc(SC(sfx, cc)), fd(SC(sfx, d));
          if (negx) { fb = -fb; fa = -fa; fc = -fc; fd = -fd; }
          const FT dfdx = dxim * (fb - fa + fc - fd) * 0.5;
          un = un - dt * dfdx;
        }
        if (sfy != NOFLUX) {
          FT fd(SC(sfy, d)), fa(SC(sfy, a)), fc(SC(sfy, cc)), fb(SC(sfy, b));
          if (negy) { fd = -fd; fa = -fa; fc = -fc; fb = -fb; }
          const FT dfdy = dyim * (fd - fa + fc - fb) * 0.5;
          un = un - dt * dfdy;
        }
        return un;
      };
      const FT roh = pred(C::RO, C::RX, C::RY, false, false);
      FT eeh = pred(C::EE, C::FXE, C::FYE, false, false);
      FT rxh = pred(C::RX, C::FXRX, C::FYRX, false, false);
      FT ryh = pred(C::RY, C::FXRY, C::FYRY, false, false);
      if constexpr (G) {
        // mlwsrch part 2: un += dt * (average of the four cell sources)
        auto srch = [&](int k, FT un) -> FT {
          if constexpr (E) {
            const FT sh = (FT(SGC(k, b)) + FT(SGC(k, a)) + FT(SGC(k, cc)) + FT(SGC(k, d))) /
                          FT(4.0);
            return un + dt * sh;
          } else {
            return FT(fma(dt.v, 0.25 * ((SGC(k, b) + SGC(k, a)) + (SGC(k, cc) + SGC(k, d))),
                          un.v));
          }
        };
        eeh = srch(0, eeh);
        rxh = srch(1, rxh);
        ryh = srch(2, ryh);
      }
      const FT bxh = pred(C::BX, NOFLUX, C::EZ, false, false);
      const FT byh = pred(C::BY, C::EZ, NOFLUX, true, false);
      FT rzh(0.0), bzh(0.0);
      if constexpr (M3) {
        rzh = pred(C::RZ, C::FXRZ, C::FYRZ, false, false);
        bzh = pred(C::BZ, C::EY, C::EX, false, true);
      }
      // half-step primitives (mlw_m3.f:214-230)
      FT vxh, vyh, vzh(0.0);
      if constexpr (E) {
        vxh = rxh / roh;
        vyh = ryh / roh;
        if constexpr (M3) vzh = rzh / roh;
      } else {
        const FT rinv(1.0 / roh.v);
        vxh = rxh * rinv;
        vyh = ryh * rinv;
        if constexpr (M3) vzh = rzh * rinv;
      }
      FT vv, bb;
      if constexpr (M3) {
        vv = vxh * vxh + vyh * vyh + vzh * vzh;
        bb = bxh * bxh + byh * byh + bzh * bzh;
      } else {
        vv = vxh * vxh + vyh * vyh;
        bb = bxh * bxh + byh * byh;
      }
      const FT prh = gm1 * (eeh - 0.5 * roh * vv - pi8i * bb);
      FT ep;
      if constexpr (E) ep = prh * gm / gm1 + 0.5 * roh * vv;
      else ep = prh * ph.ggm1 + 0.5 * roh * vv;
      if constexpr (G) {  // corner sources (mlw_m3_g.f:194, 205, 216)
        const size_t gk = (size_t)gi + (size_t)gj * ix;
        const FT gxk(grav[n + gk]), gyk(grav[3 * n + gk]);
        SGK(0, c) = (roh * (vxh * gxk + vyh * gyk)).v;
        SGK(1, c) = (roh * gxk).v;
        SGK(2, c) = (roh * gyk).v;
      }
      SK(K::XRO, c) = (roh * vxh).v;
      SK(K::YRO, c) = (roh * vyh).v;
      [[maybe_unused]] const size_t gk = (size_t)gi + (size_t)gj * ix;
      if constexpr (M3) {
        FT exh = -vyh * bzh + vzh * byh;
        FT eyh = -vzh * bxh + vxh * bzh;
        FT ezh = -vxh * byh + vyh * bxh;
        if constexpr (R) {                             // mlw_m3_e.f:242-244
          exh = exh + FT(res[3 * n + gk]);
          eyh = eyh + FT(res[4 * n + gk]);
          ezh = ezh + FT(res[5 * n + gk]);
        }
        SK(K::EX, c) = exh.v; SK(K::EY, c) = eyh.v; SK(K::EZ, c) = ezh.v;
        SK(K::XEE, c) = (ep * vxh + (bzh * eyh - byh * ezh) * pi4i).v;
        SK(K::YEE, c) = (ep * vyh + (bxh * ezh - bzh * exh) * pi4i).v;
        SK(K::XRX, c) = (roh * (vxh * vxh) + prh + pi8i * (byh * byh + bzh * bzh - bxh * bxh)).v;
        SK(K::YRX, c) = (roh * vxh * vyh - pi4i * bxh * byh).v;
        SK(K::XRY, c) = (roh * vyh * vxh - pi4i * byh * bxh).v;
        SK(K::YRY, c) = (roh * (vyh * vyh) + prh + pi8i * (bxh * bxh + bzh * bzh - byh * byh)).v;
        SK(K::XRZ, c) = (roh * vzh * vxh - pi4i * bzh * bxh).v;
        SK(K::YRZ, c) = (roh * vzh * vyh - pi4i * bzh * byh).v;
      } else {
        FT ezh = -vxh * byh + vyh * bxh;
        if constexpr (R) ezh = ezh + FT(res[n + gk]);  // mlw_m_e.f:220
        SK(K::EZ, c) = ezh.v;
        SK(K::XEE, c) = (ep * vxh - byh * ezh * pi4i).v;
        SK(K::YEE, c) = (ep * vyh + bxh * ezh * pi4i).v;
        SK(K::XRX, c) = (roh * (vxh * vxh) + prh + pi8i * (byh * byh - bxh * bxh)).v;
        SK(K::YRX, c) = (roh * vxh * vyh - pi4i * bxh * byh).v;
        SK(K::XRY, c) = (roh * vyh * vxh - pi4i * byh * bxh).v;
        SK(K::YRY, c) = (roh * (vyh * vyh) + prh + pi8i * (bxh * bxh - byh * byh)).v;
      }
    } else {
#pragma unroll 1
      for (int s = 0; s < K::N; s++) SK(s, c) = 0.0;
      if constexpr (G) {
        SGK(0, c) = 0.0; SGK(1, c) = 0.0; SGK(2, c) = 0.0;
      }
    }
  }
  // artificial-viscosity face coefficients q*dxim (mlw_m3.f:325-334; the
  // product qx(i,j)*dxim(i) is the first operation mlwartv applies)
  const FT qav(ph.qav);
  for (int f = tid; f < T::NQX; f += T::NT) {
    const int fx = f % (TX + 1), r = f / (TX + 1);
    const int gi = i0 - 1 + fx, gj = j0 + r;
    double v = 0.0;
    if (gi + 1 < ix && gj < jx) {
      const int cl = fx + (r + 1) * T::CX;
      if constexpr (AVF == 0) {
        const FT q = qav * FT(ax.dm[gi]) *
                     max0(fabs_(FT(SC(C::VX, cl + 1)) - FT(SC(C::VX, cl))) - CANS_AV_EPS);
        v = (q * FT(ax.dim[gi])).v;
      } else {
        const FT d = FT(SC(C::VX, cl + 1)) - FT(SC(C::VX, cl));
        const size_t gf = (size_t)gi + (size_t)gj * ix;
        const unsigned char br = av_branch<AVF>(d.v, fabs_(d) - CANS_AV_EPS, avb + gf, nflip,
                                                fx > 0 || tile_x == 0);
        FT q(0.0);
        if (br & 1) q = qav * FT(ax.dm[gi]) * (((br & 2) ? -d : d) - CANS_AV_EPS);
        v = (q * FT(ax.dim[gi])).v;
      }
    }
    sqx[f] = v;
  }
  for (int f = tid; f < T::NQY; f += T::NT) {
    const int fx = f % TX, r = f / TX;
    const int gi = i0 + fx, gj = j0 - 1 + r;
    double v = 0.0;
    if (gi < ix && gj + 1 < jx) {
      const int cl = (fx + 1) + r * T::CX;
      if constexpr (AVF == 0) {
        const FT q = qav * FT(ay.dm[gj]) *
                     max0(fabs_(FT(SC(C::VY, cl + T::CX)) - FT(SC(C::VY, cl))) - CANS_AV_EPS);
        v = (q * FT(ay.dim[gj])).v;
      } else {
        const FT d = FT(SC(C::VY, cl + T::CX)) - FT(SC(C::VY, cl));
        const size_t gf = n + (size_t)gi + (size_t)gj * ix;
        const unsigned char br = av_branch<AVF>(d.v, fabs_(d) - CANS_AV_EPS, avb + gf, nflip,
                                                r > 0 || tile_y == 0);
        FT q(0.0);
        if (br & 1) q = qav * FT(ay.dm[gj]) * (((br & 2) ? -d : d) - CANS_AV_EPS);
        v = (q * FT(ay.dim[gj])).v;
      }
    }
    sqy[f] = v;
  }
  __syncthreads();

  // ---------------- phase 3: full step on the tile's own cells -------------
  double dmin = __longlong_as_double(0x7ff0000000000000LL);  // +inf
  bool bad = false;  // a cell of the new state the CFL cannot use
  const int lx = tid % TX + 1;
#pragma unroll 1
  for (int rr = 0; rr < RPT; rr++) {
    const int ly = tid / TX + 1 + rr * (TY / RPT);
    const int gi = i0 - 1 + lx, gj = j0 - 1 + ly;
    if (gi > ix - 2 || gj > jx - 2) continue;
    const int c = lx + ly * T::CX;
    const int cE = c + 1, cW = c - 1, cN = c + T::CX, cS = c - T::CX;
    // corners around the cell: (i-1,j-1) (i,j-1) (i-1,j) (i,j)
    const int kSW = (lx - 1) + (ly - 1) * T::KX, kSE = kSW + 1;
    const int kNW = kSW + T::KX, kNE = kNW + 1;
    const FT hdt = 0.5 * dt;
    const FT hdx = 0.5 * FT(ax.di[gi]), hdy = 0.5 * FT(ay.di[gj]);
    const FT dxi(ax.di[gi]), dyi(ay.di[gj]);
    const FT ux0(ax.u0[gi]), ux1(ax.u1[gi]), uy0(ay.u0[gj]), uy1(ay.u1[gj]);
    const FT qxe(sqx[lx + (ly - 1) * (TX + 1)]), qxw(sqx[lx - 1 + (ly - 1) * (TX + 1)]);
    const FT qyn(sqy[(lx - 1) + ly * TX]), qys(sqy[(lx - 1) + (ly - 1) * TX]);

    // du for one conserved variable: half-step central difference,
    // corrector and artificial viscosity, in the reference order.
    auto dstep = [&](int su, int sfx, bool negx, int sfy, bool negy, int kfx,
                     bool nkx, int kfy, bool nky, int gs) -> FT {
      FT du(0.0);
      // mlwhalf part 1 (mlwhalf.f:36-41)
      if (sfx != NOFLUX) {
        FT fe(SC(sfx, cE)), fw(SC(sfx, cW));
        if (negx) { fe = -fe; fw = -fw; }
        du = du - hdt * (hdx * (fe - fw));
      }
      if (sfy != NOFLUX) {
        FT fn(SC(sfy, cN)), fs(SC(sfy, cS));
        if (negy) { fn = -fn; fs = -fs; }
        du = du - hdt * (hdy * (fn - fs));
      }
      // mlwsrch part 1: du += dt/2 * s (gravity)
      if (G && gs >= 0) du = du + hdt * FT(SGC(gs, c));
      // mlwfull (mlwfull.f:136-146)
      if (kfx != NOFLUX) {
        FT sw(SK(kfx, kSW)), se(SK(kfx, kSE)), nw(SK(kfx, kNW)), ne(SK(kfx, kNE));
        if (nkx) { sw = -sw; se = -se; nw = -nw; ne = -ne; }
        const FT dfdx = dxi * (uy0 * (se - sw) + uy1 * (ne - nw));
        du = du - hdt * dfdx;
      }
      if (kfy != NOFLUX) {
        FT sw(SK(kfy, kSW)), se(SK(kfy, kSE)), nw(SK(kfy, kNW)), ne(SK(kfy, kNE));
        if (nky) { sw = -sw; se = -se; nw = -nw; ne = -ne; }
        const FT dfdy = dyi * (ux0 * (nw - sw) + ux1 * (ne - se));
        du = du - hdt * dfdy;
      }
      // mlwsrcf: du += dt/2 * (corner sources weighted to the cell)
      if (G && gs >= 0) {
        const FT sh = uy0 * (ux0 * FT(SGK(gs, kSW)) + ux1 * FT(SGK(gs, kSE))) +
                      uy1 * (ux0 * FT(SGK(gs, kNW)) + ux1 * FT(SGK(gs, kNE)));
        du = du + hdt * sh;
      }
      // mlwartv (mlwartv.f:225-233)
      const FT u(SC(su, c));
      du = du + dt * (dxi * (qxe * (FT(SC(su, cE)) - u) - qxw * (u - FT(SC(su, cW))))) +
           dt * (dyi * (qyn * (FT(SC(su, cN)) - u) - qys * (u - FT(SC(su, cS)))));
      return u + du;
    };

    // Fast policy: the new value of each conserved variable is a linear
    // combination of 17 stencil values with per-cell coefficients, so it is
    // evaluated as one chain of FMAs (mathematically the same update).
    const double fcx = (hdt * hdx).v, fcy = (hdt * hdy).v;
    const double fx0 = (hdt * dxi * uy0).v, fx1 = (hdt * dxi * uy1).v;
    const double fy0 = (hdt * dyi * ux0).v, fy1 = (hdt * dyi * ux1).v;
    const double ae = (dt * dxi * qxe).v, aw = (dt * dxi * qxw).v;
    const double an = (dt * dyi * qyn).v, as = (dt * dyi * qys).v;
    const double a1 = 1.0 - ((ae + aw) + (an + as));
    auto fstep = [&](int su, int sfx, bool negx, int sfy, bool negy, int kfx,
                     bool nkx, int kfy, bool nky, int gs) -> FT {
      double r = a1 * SC(su, c);
      if (G && gs >= 0) {
        r = fma(hdt.v, SGC(gs, c), r);
        const double w0 = (hdt * uy0).v, w1 = (hdt * uy1).v;
        r = fma(w0, fma(ux0.v, SGK(gs, kSW), ux1.v * SGK(gs, kSE)), r);
        r = fma(w1, fma(ux0.v, SGK(gs, kNW), ux1.v * SGK(gs, kNE)), r);
      }
      r = fma(ae, SC(su, cE), r);
      r = fma(aw, SC(su, cW), r);
      r = fma(an, SC(su, cN), r);
      r = fma(as, SC(su, cS), r);
      if (sfx != NOFLUX) {
        const double d = SC(sfx, cE) - SC(sfx, cW);
        r = fma(negx ? fcx : -fcx, d, r);
      }
      if (sfy != NOFLUX) {
        const double d = SC(sfy, cN) - SC(sfy, cS);
        r = fma(negy ? fcy : -fcy, d, r);
      }
      if (kfx != NOFLUX) {
        const double d0 = SK(kfx, kSE) - SK(kfx, kSW), d1 = SK(kfx, kNE) - SK(kfx, kNW);
        r = fma(nkx ? fx0 : -fx0, d0, r);
        r = fma(nkx ? fx1 : -fx1, d1, r);
      }
      if (kfy != NOFLUX) {
        const double d0 = SK(kfy, kNW) - SK(kfy, kSW), d1 = SK(kfy, kNE) - SK(kfy, kSE);
        r = fma(nky ? fy0 : -fy0, d0, r);
        r = fma(nky ? fy1 : -fy1, d1, r);
      }
      return FT(r);
    };
    auto step_var = [&](int su, int sfx, bool negx, int sfy, bool negy, int kfx,
                        bool nkx, int kfy, bool nky, int gs = -1) -> FT {
      if constexpr (E) return dstep(su, sfx, negx, sfy, negy, kfx, nkx, kfy, nky, gs);
      else return fstep(su, sfx, negx, sfy, negy, kfx, nkx, kfy, nky, gs);
    };
    const FT ro = step_var(C::RO, C::RX, false, C::RY, false, K::XRO, false, K::YRO, false);
    const FT ee = step_var(C::EE, C::FXE, false, C::FYE, false, K::XEE, false, K::YEE, false, 0);
    const FT rx =
        step_var(C::RX, C::FXRX, false, C::FYRX, false, K::XRX, false, K::YRX, false, 1);
    const FT ry =
        step_var(C::RY, C::FXRY, false, C::FYRY, false, K::XRY, false, K::YRY, false, 2);
    const FT bx = step_var(C::BX, NOFLUX, false, C::EZ, false, NOFLUX, false, K::EZ, false);
    const FT by = step_var(C::BY, C::EZ, true, NOFLUX, false, K::EZ, true, NOFLUX, false);
    FT rz(0.0), bz(0.0);
    if constexpr (M3) {
      rz = step_var(C::RZ, C::FXRZ, false, C::FYRZ, false, K::XRZ, false, K::YRZ, false);
      bz = step_var(C::BZ, C::EY, false, C::EX, true, K::EY, false, K::EX, true);
    }
    // vector potential: mlwsrch part 1 + mlwsrcf with s = -ez, -ezh
    const size_t g = (size_t)gi + (size_t)gj * ix;
    FT az;
    if constexpr (E) {
      FT daz(0.0);
      daz = daz + hdt * (-FT(SC(C::EZ, c)));
      const FT ssw = -FT(SK(K::EZ, kSW)), sse = -FT(SK(K::EZ, kSE));
      const FT snw = -FT(SK(K::EZ, kNW)), sne = -FT(SK(K::EZ, kNE));
      const FT sh = uy0 * (ux0 * ssw + ux1 * sse) + uy1 * (ux0 * snw + ux1 * sne);
      daz = daz + hdt * sh;
      az = FT(A[P::AZ * n + g]) + daz;
    } else {
      const double w0 = (hdt * uy0).v, w1 = (hdt * uy1).v;
      double s = fma(ux0.v, SK(K::EZ, kSW), ux1.v * SK(K::EZ, kSE)) * w0;
      s = fma(fma(ux0.v, SK(K::EZ, kNW), ux1.v * SK(K::EZ, kNE)), w1, s);
      s = fma(hdt.v, SC(C::EZ, c), s);
      az = FT(A[P::AZ * n + g] - s);
    }

    // back to primitives (mlw_m3.f:365-374)
    FT vx, vy, vz(0.0);
    if constexpr (E) {
      vx = rx / ro;
      vy = ry / ro;
      if constexpr (M3) vz = rz / ro;
    } else {
      const FT rinv(1.0 / ro.v);
      vx = rx * rinv;
      vy = ry * rinv;
      if constexpr (M3) vz = rz * rinv;
    }
    FT vv, bb;
    if constexpr (M3) {
      vv = vx * vx + vy * vy + vz * vz;
      bb = bx * bx + by * by + bz * bz;
    } else {
      vv = vx * vx + vy * vy;
      bb = bx * bx + by * by;
    }
    const FT pr = gm1 * (ee - 0.5 * ro * vv - pi8i * bb);
    B[P::RO * n + g] = ro.v;
    B[P::PR * n + g] = pr.v;
    B[P::VX * n + g] = vx.v;
    B[P::VY * n + g] = vy.v;
    B[P::BX * n + g] = bx.v;
    B[P::BY * n + g] = by.v;
    B[P::AZ * n + g] = az.v;
    if constexpr (M3) {
      B[P::VZ * n + g] = vz.v;
      B[P::BZ * n + g] = bz.v;
    }
    // CFL of the new state (cfl_m3.f:46-55 / cfl_m.f:46-55)
    if (cfl_out != nullptr && gi >= box.lo[0] && gi <= box.hi[0] &&
        gj >= box.lo[1] && gj <= box.hi[1]) {
      FT b2, v2;
      if constexpr (M3) {
        b2 = bx * bx + by * by + bz * bz;
        v2 = vx * vx + vy * vy + vz * vz;
      } else {
        b2 = bx * bx + by * by;
        v2 = vx * vx + vy * vy;
      }
      if constexpr (E) {
        const FT ca2 = b2 * pi4i / ro;
        const FT cs2 = gm * pr / ro;
        const FT dtcfl = fmin_(FT(ax.d[gi]), FT(ay.d[gj])) / fsqrt(v2 + cs2 + ca2);
        const double dtq = (FT(safety) * dtcfl).v;
        if (dtq < dmin) dmin = dtq;
        bad |= bad_cell(ro.v, pr.v, dtq);
      } else {
        // min over cells of min(dx,dy)/sqrt(S) is 1/sqrt(max of
        // S*max(1/dx^2, 1/dy^2)): no division or root per cell.  dmin holds
        // minus the largest key; the block converts it once.
        const double rinv = 1.0 / ro.v;  // folded with the one above
        const double s = v2.v + fma(gm.v, pr.v, pi4i.v * b2.v) * rinv;
        const double kk = s * fmax(dxi.v * dxi.v, dyi.v * dyi.v);
        if (-kk < dmin) dmin = -kk;
        bad |= bad_cell(ro.v, pr.v, kk);
      }
    }
  }

  // ghost cells of the output keep their input values, as in the reference;
  // each ghost cell is copied by the tile that owns its nearest interior cell
  if (tile_x == 0 || tile_y == 0 || tile_x == ntiles_x - 1 || tile_y == ntiles_y - 1) {
    for (int c = tid; c < T::NC; c += T::NT) {
      const int hx = c % T::CX, hy = c / T::CX;
      const int gi = i0 - 1 + hx, gj = j0 - 1 + hy;
      if (gi >= ix || gj >= jx) continue;
      if (gi != 0 && gi != ix - 1 && gj != 0 && gj != jx - 1) continue;
      const int ci = min(max(gi, 1), ix - 2), cj = min(max(gj, 1), jx - 2);
      if (ci < i0 || ci >= i0 + TX || cj < j0 || cj >= j0 + TY) continue;
      const size_t g = (size_t)gi + (size_t)gj * ix;
#pragma unroll
      for (int v = 0; v < P::N; v++) B[v * n + g] = A[v * n + g];
    }
  }
  if (cfl_out != nullptr) {
    if (bad_out != nullptr) count_bad_block(bad, bad_out, tid);
    if constexpr (E) {
      block_min_to(cfl_out, dmin, sred, tid, T::NT);
    } else {
      const double m = block_min(dmin, sred, tid, T::NT);  // -(largest key)
      if (tid == 0 && m < 0.0) atomic_min_pos(cfl_out, safety / sqrt(-m));
    }
  }
#undef SC
#undef SK
#undef SGC
#undef SGK
}

}  // namespace cans
