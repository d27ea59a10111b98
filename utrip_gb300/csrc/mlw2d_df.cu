// Fused 2-D mLW step, mlw_m3 (cans2d/hdmlw/mlw_m3.f:64-374), in the
// double-float policy: the arithmetic of the three tile phases runs in
// double-float (df64.cuh) on the FP32 pipes, and the conserved variables are
// accumulated in FP64 (u_new = u + du, du in double-float).
//
// The phases are those of the FP64 tile (mlw2d_tile.cuh) with the same
// algebra as its fast policy, rearranged where the algebra allows fewer
// operations:
//   - the momentum flux tensor is symmetric, so fx(ry) = fy(rx) is formed
//     once at the cells and once at the corners (the reference forms
//     ro vy vx - by bx/4pi and ro vx vy - bx by/4pi separately);
//   - the total pressure p + B^2/8pi is formed once, and the diagonal
//     fluxes are rho v v + p_T - B B/4pi (the reference's
//     pi8i (by^2 + bz^2 - bx^2) is the same quantity);
//   - the corner x and y mass fluxes are the half-step momenta themselves
//     (roh vxh with vxh = rxh/roh).
// State layout, tiles, CFL fusion and ghost handling are those of k_mlw2d.
//
// Precision: 48-bit significands (2^-48 per conversion, a few 2^-48 per
// operation).  The run holds the fast policy's bar against the oracle (the
// tests hold it to a relative 1e-10 per variable after 100 steps); the exact
// policy remains the bit-for-bit path.
#include <cuda_runtime.h>

#include <mutex>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "df64.cuh"

namespace cans {

namespace {

using df::D;

// cell slots: conserved, cell fluxes (fxy = fx(ry) = fy(rx)), E, velocities
enum {
  CRO = 0, CEE, CRX, CRY, CRZ, CBX, CBY, CBZ,
  CFXE, CFXRX, CFXY, CFXRZ, CFYE, CFYRY, CFYRZ,
  CEX, CEY, CEZ, CVX, CVY, NCS
};
// corner slots: half-step fluxes (xy = x(ry) = y(rx)) and E
enum { KXRO = 0, KXEE, KXRX, KXY, KXRZ, KYRO, KYEE, KYRY, KYRZ, KEX, KEY, KEZ, NKS };
constexpr int NOF = -1;

template <int TX, int TY, int RPT>
struct TileD {
  static constexpr int CX = TX + 2, CY = TY + 2, NC = CX * CY;
  static constexpr int KX = TX + 1, KY = TY + 1, NK = KX * KY;
  static constexpr int NQX = (TX + 1) * TY, NQY = TX * (TY + 1);
  static constexpr int NT = TX * TY / RPT;
  static constexpr size_t smem_bytes =
      sizeof(D) * ((size_t)NCS * NC + (size_t)NKS * NK + NQX + NQY) + sizeof(double) * 32;
};

// the state's primitive order (mlw_m3)
enum { PRO = 0, PPR, PVX, PVY, PVZ, PBX, PBY, PBZ, PAZ, NPV };

struct PhysD {
  D gm, gm1, gm1i, ggm1, pi4i, pi8i, qav;
};

__device__ __forceinline__ PhysD phys_d(const Phys &ph) {
  return {df::from_double(ph.gm),  df::from_double(ph.gm1),  df::from_double(ph.gm1i),
          df::from_double(ph.ggm1), df::from_double(ph.pi4i), df::from_double(ph.pi8i),
          df::from_double(ph.qav)};
}

// a cell of the new state the CFL cannot use (see bad_cell): ro or pr not
// positive or not finite, or a key that is not a number
__device__ __forceinline__ bool bad_cell_d(double ro, double pr, D key) {
  constexpr long long kInf = 0x7ff0000000000000LL;
  const long long a = __double_as_longlong(ro), b = __double_as_longlong(pr);
  const bool knan = (__float_as_uint(key.h) & 0x7fffffffu) > 0x7f800000u;
  return a <= 0 || a > kInf || b <= 0 || b > kInf || knan;
}

// warp maximum of a double-float key (h, l compared lexicographically)
__device__ __forceinline__ D warp_max_d(D v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    D w;
    w.h = __shfl_xor_sync(0xffffffffu, v.h, o);
    w.l = __shfl_xor_sync(0xffffffffu, v.l, o);
    if (df::gt(w, v) || v.h != v.h) v = w;
  }
  return v;
}

template <int TX, int TY, int RPT>
__device__ __forceinline__ void tile_step_df(const double *__restrict__ A,
                                             double *__restrict__ B, int ix, int jx,
                                             const Axis &ax, const Axis &ay, const Phys &ph,
                                             double dtv, double safety,
                                             unsigned long long *cfl_out, const Box3 &box,
                                             int tile_x, int tile_y, int ntiles_x,
                                             int ntiles_y, D *smem, int *bad_out) {
  using T = TileD<TX, TY, RPT>;
  D *sc = smem;                            // cells   [NCS][NC]
  D *sk = sc + (size_t)NCS * T::NC;        // corners [NKS][NK]
  D *sqx = sk + (size_t)NKS * T::NK;       // q dxim  [TY][TX+1]
  D *sqy = sqx + T::NQX;                   // q dyim  [TY+1][TX]
  double *sred = reinterpret_cast<double *>(sqy + T::NQY);  // 32

  const size_t n = (size_t)ix * (size_t)jx;
  const int i0 = 1 + tile_x * TX, j0 = 1 + tile_y * TY;
  const int tid = threadIdx.x;
  const PhysD P = phys_d(ph);
  const D dt = df::from_double(dtv);

#define SC(s, c) sc[(size_t)(s) * T::NC + (c)]
#define SK(s, c) sk[(size_t)(s) * T::NK + (c)]

  // ---------------- phase 1: cells of the halo tile ------------------------
  for (int c = tid; c < T::NC; c += T::NT) {
    const int lx = c % T::CX, ly = c / T::CX;
    const int gi = i0 - 1 + lx, gj = j0 - 1 + ly;
    if (gi < ix && gj < jx) {
      const size_t g = (size_t)gi + (size_t)gj * ix;
      const D ro = df::from_double(A[PRO * n + g]), pr = df::from_double(A[PPR * n + g]);
      const D vx = df::from_double(A[PVX * n + g]), vy = df::from_double(A[PVY * n + g]);
      const D vz = df::from_double(A[PVZ * n + g]);
      const D bx = df::from_double(A[PBX * n + g]), by = df::from_double(A[PBY * n + g]);
      const D bz = df::from_double(A[PBZ * n + g]);
      const D vv = df::mad(vz, vz, df::mad(vy, vy, df::sqr(vx)));
      const D bb = df::mad(bz, bz, df::mad(by, by, df::sqr(bx)));
      const D ek = df::mul(df::scale(ro, 0.5f), vv);
      const D ee = df::mad(pr, P.gm1i, df::mad(P.pi8i, bb, ek));  // mlw_m3.f:111
      const D ep = df::mad(pr, P.ggm1, ek);                        // :141
      const D rx = df::mul(ro, vx), ry = df::mul(ro, vy), rz = df::mul(ro, vz);
      const D ex = df::mad(vz, by, df::neg(df::mul(vy, bz)));     // :119-121
      const D ey = df::mad(vx, bz, df::neg(df::mul(vz, bx)));
      const D ez = df::mad(vy, bx, df::neg(df::mul(vx, by)));
      const D pt = df::mad(P.pi8i, bb, pr);
      const D pbx = df::mul(P.pi4i, bx), pby = df::mul(P.pi4i, by);
      SC(CRO, c) = ro; SC(CEE, c) = ee; SC(CRX, c) = rx; SC(CRY, c) = ry; SC(CRZ, c) = rz;
      SC(CBX, c) = bx; SC(CBY, c) = by; SC(CBZ, c) = bz;
      SC(CEX, c) = ex; SC(CEY, c) = ey; SC(CEZ, c) = ez; SC(CVX, c) = vx; SC(CVY, c) = vy;
      // energy fluxes (:141-143)
      SC(CFXE, c) = df::mad(df::mad(bz, ey, df::neg(df::mul(by, ez))), P.pi4i, df::mul(ep, vx));
      SC(CFYE, c) = df::mad(df::mad(bx, ez, df::neg(df::mul(bz, ex))), P.pi4i, df::mul(ep, vy));
      // momentum fluxes (:151-172)
      SC(CFXRX, c) = df::mad(rx, vx, df::mad(df::neg(pbx), bx, pt));
      SC(CFYRY, c) = df::mad(ry, vy, df::mad(df::neg(pby), by, pt));
      SC(CFXY, c) = df::mad(rx, vy, df::neg(df::mul(pbx, by)));
      SC(CFXRZ, c) = df::mad(rz, vx, df::neg(df::mul(pbx, bz)));
      SC(CFYRZ, c) = df::mad(rz, vy, df::neg(df::mul(pby, bz)));
    } else {
#pragma unroll 1
      for (int s = 0; s < NCS; s++) SC(s, c) = df::mk(0.0f);
    }
  }
  __syncthreads();

  // ---------------- phase 2: corners and viscosity faces -------------------
  for (int c = tid; c < T::NK; c += T::NT) {
    const int kx = c % T::KX, ky = c / T::KX;
    const int gi = i0 - 1 + kx, gj = j0 - 1 + ky;  // lower-left cell of the corner
    if (gi <= ix - 2 && gj <= jx - 2) {
      const int a = kx + ky * T::CX, b = a + 1, cc = a + 1 + T::CX, d = a + T::CX;
      // mlwhalf part 2 (mlwhalf.f:45-52): un = avg4(u) - dt dxim/2 dxF - dt dyim/2 dyF
      const D cxk = df::scale(df::mul(dt, df::from_double(ax.dim[gi])), 0.5f);
      const D cyk = df::scale(df::mul(dt, df::from_double(ay.dim[gj])), 0.5f);
      auto pred = [&](int su, int sfx, int sfy, bool negx, bool negy) -> D {
        D r = df::scale(df::add(df::add(SC(su, b), SC(su, a)), df::add(SC(su, cc), SC(su, d))),
                        0.25f);
        if (sfx != NOF) {
          const D s = df::add(df::sub(SC(sfx, b), SC(sfx, a)), df::sub(SC(sfx, cc), SC(sfx, d)));
          r = df::mad(negx ? cxk : df::neg(cxk), s, r);
        }
        if (sfy != NOF) {
          const D s = df::add(df::sub(SC(sfy, d), SC(sfy, a)), df::sub(SC(sfy, cc), SC(sfy, b)));
          r = df::mad(negy ? cyk : df::neg(cyk), s, r);
        }
        return r;
      };
      const D roh = pred(CRO, CRX, CRY, false, false);
      const D eeh = pred(CEE, CFXE, CFYE, false, false);
      const D rxh = pred(CRX, CFXRX, CFXY, false, false);
      const D ryh = pred(CRY, CFXY, CFYRY, false, false);
      const D rzh = pred(CRZ, CFXRZ, CFYRZ, false, false);
      const D bxh = pred(CBX, NOF, CEZ, false, false);
      const D byh = pred(CBY, CEZ, NOF, true, false);
      const D bzh = pred(CBZ, CEY, CEX, false, true);
      // half-step primitives (mlw_m3.f:214-230)
      const D rinv = df::rcp(roh);
      const D vxh = df::mul(rxh, rinv), vyh = df::mul(ryh, rinv), vzh = df::mul(rzh, rinv);
      const D vv = df::mad(vzh, vzh, df::mad(vyh, vyh, df::sqr(vxh)));
      const D bb = df::mad(bzh, bzh, df::mad(byh, byh, df::sqr(bxh)));
      const D ek = df::mul(df::scale(roh, 0.5f), vv);
      const D prh = df::mul(P.gm1, df::sub(df::sub(eeh, ek), df::mul(P.pi8i, bb)));
      const D ep = df::mad(prh, P.ggm1, ek);
      const D exh = df::mad(vzh, byh, df::neg(df::mul(vyh, bzh)));
      const D eyh = df::mad(vxh, bzh, df::neg(df::mul(vzh, bxh)));
      const D ezh = df::mad(vyh, bxh, df::neg(df::mul(vxh, byh)));
      const D pt = df::mad(P.pi8i, bb, prh);
      const D pbx = df::mul(P.pi4i, bxh), pby = df::mul(P.pi4i, byh);
      SK(KXRO, c) = rxh;
      SK(KYRO, c) = ryh;
      SK(KEX, c) = exh; SK(KEY, c) = eyh; SK(KEZ, c) = ezh;
      SK(KXEE, c) = df::mad(df::mad(bzh, eyh, df::neg(df::mul(byh, ezh))), P.pi4i,
                            df::mul(ep, vxh));
      SK(KYEE, c) = df::mad(df::mad(bxh, ezh, df::neg(df::mul(bzh, exh))), P.pi4i,
                            df::mul(ep, vyh));
      SK(KXRX, c) = df::mad(rxh, vxh, df::mad(df::neg(pbx), bxh, pt));
      SK(KYRY, c) = df::mad(ryh, vyh, df::mad(df::neg(pby), byh, pt));
      SK(KXY, c) = df::mad(rxh, vyh, df::neg(df::mul(pbx, byh)));
      SK(KXRZ, c) = df::mad(rzh, vxh, df::neg(df::mul(pbx, bzh)));
      SK(KYRZ, c) = df::mad(rzh, vyh, df::neg(df::mul(pby, bzh)));
    } else {
#pragma unroll 1
      for (int s = 0; s < NKS; s++) SK(s, c) = df::mk(0.0f);
    }
  }
  // artificial-viscosity face coefficients q dxim (mlw_m3.f:325-334): the
  // real*4 threshold 1.0e-4 is a float
  for (int f = tid; f < T::NQX; f += T::NT) {
    const int fx = f % (TX + 1), r = f / (TX + 1);
    const int gi = i0 - 1 + fx, gj = j0 + r;
    D v = df::mk(0.0f);
    if (gi + 1 < ix && gj < jx) {
      const int cl = fx + (r + 1) * T::CX;
      const D q = df::addf(df::absd(df::sub(SC(CVX, cl + 1), SC(CVX, cl))), -1.0e-4f);
      if (df::pos(q))
        v = df::mul(df::mul(df::mul(P.qav, df::from_double(ax.dm[gi])), q),
                    df::from_double(ax.dim[gi]));
    }
    sqx[f] = v;
  }
  for (int f = tid; f < T::NQY; f += T::NT) {
    const int fx = f % TX, r = f / TX;
    const int gi = i0 + fx, gj = j0 - 1 + r;
    D v = df::mk(0.0f);
    if (gi < ix && gj + 1 < jx) {
      const int cl = (fx + 1) + r * T::CX;
      const D q = df::addf(df::absd(df::sub(SC(CVY, cl + T::CX), SC(CVY, cl))), -1.0e-4f);
      if (df::pos(q))
        v = df::mul(df::mul(df::mul(P.qav, df::from_double(ay.dm[gj])), q),
                    df::from_double(ay.dim[gj]));
    }
    sqy[f] = v;
  }
  __syncthreads();

  // ---------------- phase 3: full step on the tile's own cells -------------
  D kmax = df::mk(0.0f);  // largest CFL key of the thread's cells
  bool bad = false;
  const int lx = tid % TX + 1;
#pragma unroll 1
  for (int rr = 0; rr < RPT; rr++) {
    const int ly = tid / TX + 1 + rr * (TY / RPT);
    const int gi = i0 - 1 + lx, gj = j0 - 1 + ly;
    if (gi > ix - 2 || gj > jx - 2) continue;
    const int c = lx + ly * T::CX;
    const int cE = c + 1, cW = c - 1, cN = c + T::CX, cS = c - T::CX;
    const int kSW = (lx - 1) + (ly - 1) * T::KX, kSE = kSW + 1;
    const int kNW = kSW + T::KX, kNE = kNW + 1;
    const D hdt = df::scale(dt, 0.5f);
    const D dxi = df::from_double(ax.di[gi]), dyi = df::from_double(ay.di[gj]);
    const D ux0 = df::from_double(ax.u0[gi]), ux1 = df::from_double(ax.u1[gi]);
    const D uy0 = df::from_double(ay.u0[gj]), uy1 = df::from_double(ay.u1[gj]);
    const D hdx = df::mul(hdt, dxi), hdy = df::mul(hdt, dyi);
    // du = -hdt/2 dxi (F_E - F_W) ... (mlwhalf part 1), -hdt dxi (uy0 (K_SE - K_SW)
    // + uy1 (K_NE - K_NW)) ... (mlwfull), dt dxi (q_e (u_E - u) - q_w (u - u_W)) ...
    // (mlwartv): the coefficients of each difference
    const D fcx = df::scale(hdx, 0.5f), fcy = df::scale(hdy, 0.5f);
    const D fx0 = df::mul(hdx, uy0), fx1 = df::mul(hdx, uy1);
    const D fy0 = df::mul(hdy, ux0), fy1 = df::mul(hdy, ux1);
    const D dtx = df::mul(dt, dxi), dty = df::mul(dt, dyi);
    const D ae = df::mul(dtx, sqx[lx + (ly - 1) * (TX + 1)]);
    const D aw = df::mul(dtx, sqx[lx - 1 + (ly - 1) * (TX + 1)]);
    const D an = df::mul(dty, sqy[(lx - 1) + ly * TX]);
    const D as = df::mul(dty, sqy[(lx - 1) + (ly - 1) * TX]);
    auto dvar = [&](int su, int sfx, bool negx, int sfy, bool negy, int kfx, bool nkx, int kfy,
                    bool nky) -> D {
      const D u = SC(su, c);
      D du = df::mul(ae, df::sub(SC(su, cE), u));
      du = df::mad(aw, df::sub(SC(su, cW), u), du);
      du = df::mad(an, df::sub(SC(su, cN), u), du);
      du = df::mad(as, df::sub(SC(su, cS), u), du);
      if (sfx != NOF) du = df::mad(negx ? fcx : df::neg(fcx), df::sub(SC(sfx, cE), SC(sfx, cW)), du);
      if (sfy != NOF) du = df::mad(negy ? fcy : df::neg(fcy), df::sub(SC(sfy, cN), SC(sfy, cS)), du);
      if (kfx != NOF) {
        du = df::mad(nkx ? fx0 : df::neg(fx0), df::sub(SK(kfx, kSE), SK(kfx, kSW)), du);
        du = df::mad(nkx ? fx1 : df::neg(fx1), df::sub(SK(kfx, kNE), SK(kfx, kNW)), du);
      }
      if (kfy != NOF) {
        du = df::mad(nky ? fy0 : df::neg(fy0), df::sub(SK(kfy, kNW), SK(kfy, kSW)), du);
        du = df::mad(nky ? fy1 : df::neg(fy1), df::sub(SK(kfy, kNE), SK(kfy, kSE)), du);
      }
      return du;
    };
    const size_t g = (size_t)gi + (size_t)gj * ix;
    // conserved u + du, accumulated in FP64: ro and B are primitives, so the
    // input doubles carry them; ee and the momenta are rebuilt from the input
    // primitives in double-float (their values in the cell slots)
    const double ro_new = A[PRO * n + g] +
                          df::to_double(dvar(CRO, CRX, false, CRY, false, KXRO, false, KYRO, false));
    const double bx_new = A[PBX * n + g] +
                          df::to_double(dvar(CBX, NOF, false, CEZ, false, NOF, false, KEZ, false));
    const double by_new = A[PBY * n + g] +
                          df::to_double(dvar(CBY, CEZ, true, NOF, false, KEZ, true, NOF, false));
    const double bz_new = A[PBZ * n + g] +
                          df::to_double(dvar(CBZ, CEY, false, CEX, true, KEY, false, KEX, true));
    const D ee = df::add(SC(CEE, c), dvar(CEE, CFXE, false, CFYE, false, KXEE, false, KYEE, false));
    const D rx = df::add(SC(CRX, c), dvar(CRX, CFXRX, false, CFXY, false, KXRX, false, KXY, false));
    const D ry = df::add(SC(CRY, c), dvar(CRY, CFXY, false, CFYRY, false, KXY, false, KYRY, false));
    const D rz = df::add(SC(CRZ, c), dvar(CRZ, CFXRZ, false, CFYRZ, false, KXRZ, false, KYRZ, false));
    // vector potential: mlwsrch part 1 + mlwsrcf with s = -ez, -ezh
    {
      D s = df::mul(ux0, SK(KEZ, kSW));
      s = df::mad(ux1, SK(KEZ, kSE), s);
      D t = df::mul(ux0, SK(KEZ, kNW));
      t = df::mad(ux1, SK(KEZ, kNE), t);
      s = df::mad(uy1, t, df::mul(uy0, s));
      s = df::mad(hdt, SC(CEZ, c), df::mul(hdt, s));
      B[PAZ * n + g] = A[PAZ * n + g] - df::to_double(s);
    }
    // back to primitives (mlw_m3.f:365-374)
    const D ro = df::from_double(ro_new);
    const D bx = df::from_double(bx_new), by = df::from_double(by_new);
    const D bz = df::from_double(bz_new);
    const D rinv = df::rcp(ro);
    const D vx = df::mul(rx, rinv), vy = df::mul(ry, rinv), vz = df::mul(rz, rinv);
    const D vv = df::mad(vz, vz, df::mad(vy, vy, df::sqr(vx)));
    const D bb = df::mad(bz, bz, df::mad(by, by, df::sqr(bx)));
    const D pr = df::mul(P.gm1, df::sub(df::sub(ee, df::mul(df::scale(ro, 0.5f), vv)),
                                        df::mul(P.pi8i, bb)));
    const double prd = df::to_double(pr);
    B[PRO * n + g] = ro_new;
    B[PPR * n + g] = prd;
    B[PVX * n + g] = df::to_double(vx);
    B[PVY * n + g] = df::to_double(vy);
    B[PVZ * n + g] = df::to_double(vz);
    B[PBX * n + g] = bx_new;
    B[PBY * n + g] = by_new;
    B[PBZ * n + g] = bz_new;
    // CFL key of the new state: (v^2 + (gm p + B^2/4pi)/ro) max(1/dx^2, 1/dy^2)
    // (cfl_m3.f:46-55 without the per-cell division and root)
    if (cfl_out != nullptr && gi >= box.lo[0] && gi <= box.hi[0] && gj >= box.lo[1] &&
        gj <= box.hi[1]) {
      const D s = df::mad(df::mad(P.gm, pr, df::mul(P.pi4i, bb)), rinv, vv);
      const D ix2 = df::sqr(dxi), iy2 = df::sqr(dyi);
      const D key = df::mul(s, df::gt(ix2, iy2) ? ix2 : iy2);
      if (key.h == key.h && df::gt(key, kmax)) kmax = key;  // a NaN is never the maximum
      bad |= bad_cell_d(ro_new, prd, key);
    }
  }

  // ghost cells of the output keep their input values (as in k_mlw2d)
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
      for (int v = 0; v < NPV; v++) B[v * n + g] = A[v * n + g];
    }
  }
  if (cfl_out != nullptr) {
    if (bad_out != nullptr) count_bad_block(bad, bad_out, tid);
    // min over cells of min(dx,dy)/sqrt(S) = 1/sqrt(max key): the block's
    // largest key, then one conversion, root and division per block
    kmax = warp_max_d(kmax);
    const int lane = tid & 31, w = tid >> 5;
    if (lane == 0) sred[w] = df::to_double(kmax);
    __syncthreads();
    if (w == 0) {
      double x = lane < (T::NT + 31) / 32 ? sred[lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_xor_sync(0xffffffffu, x, o);
        x = (y > x || x != x) ? y : x;
      }
      if (lane == 0 && x > 0.0) atomic_min_pos(cfl_out, safety / sqrt(x));
    }
  }
#undef SC
#undef SK
}

// ---------------------------------------------------------------------------
// The same step with the tile marching in y.  A block owns a strip of 32
// interior columns and a segment of `seg` interior rows, which it takes in
// chunks of CH rows; between chunks it keeps the last two cell rows and the
// last corner row instead of recomputing them, so the halo work is that of
// a 32 x seg tile, while its shared memory is that of a 32 x CH tile.  A
// block has 34 CH threads (rounded up to whole warps): one per cell of a
// chunk's new rows (phase 1), one per corner (phase 2) and one per updated
// cell (phase 3, 32 CH of them).
// Number operations of the marching kernel, which is written once for
// both: DFN, double-float on the FP32 pipes (the double-float policy), and
// F64N, FP64 with FMA contraction (the fast policy).
struct DFN {
  using V = df::D;
  static __device__ __forceinline__ V in(double x) { return df::from_double(x); }
  static __device__ __forceinline__ double out(V x) { return df::to_double(x); }
  static __device__ __forceinline__ V zero() { return df::mk(0.0f); }
  static __device__ __forceinline__ V mad(V a, V b, V c) { return df::mad(a, b, c); }
  static __device__ __forceinline__ V mul(V a, V b) { return df::mul(a, b); }
  static __device__ __forceinline__ V add(V a, V b) { return df::add(a, b); }
  static __device__ __forceinline__ V sub(V a, V b) { return df::sub(a, b); }
  static __device__ __forceinline__ V neg(V a) { return df::neg(a); }
  static __device__ __forceinline__ V scale(V a, float p2) { return df::scale(a, p2); }
  static __device__ __forceinline__ V sqr(V a) { return df::sqr(a); }
  static __device__ __forceinline__ V rcp(V a) { return df::rcp(a); }
  static __device__ __forceinline__ V addf(V a, float b) { return df::addf(a, b); }
  static __device__ __forceinline__ V absd(V a) { return df::absd(a); }
  static __device__ __forceinline__ bool pos(V a) { return df::pos(a); }
  static __device__ __forceinline__ bool gt(V a, V b) { return df::gt(a, b); }
  static __device__ __forceinline__ bool isnan(V a) { return a.h != a.h; }
  static __device__ __forceinline__ V nan_probe(V a) { return a; }
  static __device__ __forceinline__ V warp_max(V v) { return warp_max_d(v); }
};
struct F64N {
  using V = double;
  static __device__ __forceinline__ V in(double x) { return x; }
  static __device__ __forceinline__ double out(V x) { return x; }
  static __device__ __forceinline__ V zero() { return 0.0; }
  static __device__ __forceinline__ V mad(V a, V b, V c) { return fma(a, b, c); }
  static __device__ __forceinline__ V mul(V a, V b) { return a * b; }
  static __device__ __forceinline__ V add(V a, V b) { return a + b; }
  static __device__ __forceinline__ V sub(V a, V b) { return a - b; }
  static __device__ __forceinline__ V neg(V a) { return -a; }
  static __device__ __forceinline__ V scale(V a, float p2) { return a * (double)p2; }
  static __device__ __forceinline__ V sqr(V a) { return a * a; }
  static __device__ __forceinline__ V rcp(V a) { return 1.0 / a; }
  static __device__ __forceinline__ V addf(V a, float b) { return a + (double)b; }
  static __device__ __forceinline__ V absd(V a) { return fabs(a); }
  static __device__ __forceinline__ bool pos(V a) { return a > 0.0; }
  static __device__ __forceinline__ bool gt(V a, V b) { return a > b; }
  static __device__ __forceinline__ bool isnan(V a) { return a != a; }
  // a float whose NaN-ness is the key's, for bad_cell_d
  static __device__ __forceinline__ df::D nan_probe(V a) {
    return {a != a ? __int_as_float(0x7fc00000) : 0.0f, 0.0f};
  }
  static __device__ __forceinline__ V warp_max(V v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double w = __shfl_xor_sync(0xffffffffu, v, o);
      if (w > v || v != v) v = w;
    }
    return v;
  }
};
template <class N> struct PhysN {
  typename N::V gm, gm1, gm1i, ggm1, pi4i, pi8i, qav;
};
template <class N> __device__ __forceinline__ PhysN<N> phys_n(const Phys &ph) {
  return {N::in(ph.gm),   N::in(ph.gm1),  N::in(ph.gm1i), N::in(ph.ggm1),
          N::in(ph.pi4i), N::in(ph.pi8i), N::in(ph.qav)};
}

template <int CH>
struct MarchD {
  static constexpr int TX = 32, CX = TX + 2, KX = TX + 1;
  static constexpr int CR = CH + 2, KR = CH + 1;       // cell rows, corner rows
  static constexpr int NC = CX * CR, NK = KX * KR;
  static constexpr int NQX = KX * CH, NQY = TX * KR;
  // 34 CH threads rounded up to whole warps: the warp-level reductions at the
  // end take every lane of a warp
  static constexpr int NT = (CX * CH + 31) / 32 * 32;
  static constexpr size_t smem_bytes =
      sizeof(double) * ((size_t)NCS * NC + (size_t)NKS * NK + NQX + NQY) + sizeof(double) * 32;
};

// Cell values of one cell (phase 1 of the tile).
template <class N, int NCc>
__device__ __forceinline__ void cell_m(const double *__restrict__ A, size_t n, size_t g,
                                        typename N::V *sc, int c, const PhysN<N> &P) {
  using V = typename N::V;
#define SC(s, c) sc[(size_t)(s) * NCc + (c)]
  const V ro = N::in(A[PRO * n + g]), pr = N::in(A[PPR * n + g]);
  const V vx = N::in(A[PVX * n + g]), vy = N::in(A[PVY * n + g]);
  const V vz = N::in(A[PVZ * n + g]);
  const V bx = N::in(A[PBX * n + g]), by = N::in(A[PBY * n + g]);
  const V bz = N::in(A[PBZ * n + g]);
  const V vv = N::mad(vz, vz, N::mad(vy, vy, N::sqr(vx)));
  const V bb = N::mad(bz, bz, N::mad(by, by, N::sqr(bx)));
  const V ek = N::mul(N::scale(ro, 0.5f), vv);
  const V ee = N::mad(pr, P.gm1i, N::mad(P.pi8i, bb, ek));
  const V ep = N::mad(pr, P.ggm1, ek);
  const V rx = N::mul(ro, vx), ry = N::mul(ro, vy), rz = N::mul(ro, vz);
  const V ex = N::mad(vz, by, N::neg(N::mul(vy, bz)));
  const V ey = N::mad(vx, bz, N::neg(N::mul(vz, bx)));
  const V ez = N::mad(vy, bx, N::neg(N::mul(vx, by)));
  const V pt = N::mad(P.pi8i, bb, pr);
  const V pbx = N::mul(P.pi4i, bx), pby = N::mul(P.pi4i, by);
  SC(CRO, c) = ro; SC(CEE, c) = ee; SC(CRX, c) = rx; SC(CRY, c) = ry; SC(CRZ, c) = rz;
  SC(CBX, c) = bx; SC(CBY, c) = by; SC(CBZ, c) = bz;
  SC(CEX, c) = ex; SC(CEY, c) = ey; SC(CEZ, c) = ez; SC(CVX, c) = vx; SC(CVY, c) = vy;
  SC(CFXE, c) = N::mad(N::mad(bz, ey, N::neg(N::mul(by, ez))), P.pi4i, N::mul(ep, vx));
  SC(CFYE, c) = N::mad(N::mad(bx, ez, N::neg(N::mul(bz, ex))), P.pi4i, N::mul(ep, vy));
  SC(CFXRX, c) = N::mad(rx, vx, N::mad(N::neg(pbx), bx, pt));
  SC(CFYRY, c) = N::mad(ry, vy, N::mad(N::neg(pby), by, pt));
  SC(CFXY, c) = N::mad(rx, vy, N::neg(N::mul(pbx, by)));
  SC(CFXRZ, c) = N::mad(rz, vx, N::neg(N::mul(pbx, bz)));
  SC(CFYRZ, c) = N::mad(rz, vy, N::neg(N::mul(pby, bz)));
#undef SC
}

// Half-step values of one corner from its four cells a, b (x+1), cc (x+1,
// y+1), d (y+1) (phase 2 of the tile).
template <class N, int NCc, int NKc>
__device__ __forceinline__ void corner_m(const typename N::V *sc, typename N::V *sk, int a,
                                         int b, int cc, int d, int k, typename N::V cxk,
                                         typename N::V cyk, const PhysN<N> &P) {
  using V = typename N::V;
#define SC(s, c) sc[(size_t)(s) * NCc + (c)]
#define SK(s, c) sk[(size_t)(s) * NKc + (c)]
  auto pred = [&](int su, int sfx, int sfy, bool negx, bool negy) -> V {
    V r = N::scale(N::add(N::add(SC(su, b), SC(su, a)), N::add(SC(su, cc), SC(su, d))),
                    0.25f);
    if (sfx != NOF) {
      const V s = N::add(N::sub(SC(sfx, b), SC(sfx, a)), N::sub(SC(sfx, cc), SC(sfx, d)));
      r = N::mad(negx ? cxk : N::neg(cxk), s, r);
    }
    if (sfy != NOF) {
      const V s = N::add(N::sub(SC(sfy, d), SC(sfy, a)), N::sub(SC(sfy, cc), SC(sfy, b)));
      r = N::mad(negy ? cyk : N::neg(cyk), s, r);
    }
    return r;
  };
  const V roh = pred(CRO, CRX, CRY, false, false);
  const V eeh = pred(CEE, CFXE, CFYE, false, false);
  const V rxh = pred(CRX, CFXRX, CFXY, false, false);
  const V ryh = pred(CRY, CFXY, CFYRY, false, false);
  const V rzh = pred(CRZ, CFXRZ, CFYRZ, false, false);
  const V bxh = pred(CBX, NOF, CEZ, false, false);
  const V byh = pred(CBY, CEZ, NOF, true, false);
  const V bzh = pred(CBZ, CEY, CEX, false, true);
  const V rinv = N::rcp(roh);
  const V vxh = N::mul(rxh, rinv), vyh = N::mul(ryh, rinv), vzh = N::mul(rzh, rinv);
  const V vv = N::mad(vzh, vzh, N::mad(vyh, vyh, N::sqr(vxh)));
  const V bb = N::mad(bzh, bzh, N::mad(byh, byh, N::sqr(bxh)));
  const V ek = N::mul(N::scale(roh, 0.5f), vv);
  const V prh = N::mul(P.gm1, N::sub(N::sub(eeh, ek), N::mul(P.pi8i, bb)));
  const V ep = N::mad(prh, P.ggm1, ek);
  const V exh = N::mad(vzh, byh, N::neg(N::mul(vyh, bzh)));
  const V eyh = N::mad(vxh, bzh, N::neg(N::mul(vzh, bxh)));
  const V ezh = N::mad(vyh, bxh, N::neg(N::mul(vxh, byh)));
  const V pt = N::mad(P.pi8i, bb, prh);
  const V pbx = N::mul(P.pi4i, bxh), pby = N::mul(P.pi4i, byh);
  SK(KXRO, k) = rxh;
  SK(KYRO, k) = ryh;
  SK(KEX, k) = exh; SK(KEY, k) = eyh; SK(KEZ, k) = ezh;
  SK(KXEE, k) = N::mad(N::mad(bzh, eyh, N::neg(N::mul(byh, ezh))), P.pi4i, N::mul(ep, vxh));
  SK(KYEE, k) = N::mad(N::mad(bxh, ezh, N::neg(N::mul(bzh, exh))), P.pi4i, N::mul(ep, vyh));
  SK(KXRX, k) = N::mad(rxh, vxh, N::mad(N::neg(pbx), bxh, pt));
  SK(KYRY, k) = N::mad(ryh, vyh, N::mad(N::neg(pby), byh, pt));
  SK(KXY, k) = N::mad(rxh, vyh, N::neg(N::mul(pbx, byh)));
  SK(KXRZ, k) = N::mad(rzh, vxh, N::neg(N::mul(pbx, bzh)));
  SK(KYRZ, k) = N::mad(rzh, vyh, N::neg(N::mul(pby, bzh)));
#undef SC
#undef SK
}

template <class N, int CH>
__global__ void __launch_bounds__(MarchD<CH>::NT, 2)
    k_mlw2d_march(const double *__restrict__ A, double *__restrict__ B, int ix, int jx,
                     Axis ax, Axis ay, Phys ph, double dt_arg, Ctl *__restrict__ ctl, Box3 box,
                     int seg) {
  using T = MarchD<CH>;
  using V = typename N::V;
  extern __shared__ double smem_m_raw[];
  V *sc = reinterpret_cast<V *>(smem_m_raw);                          // cells   [NCS][CR][CX]
  V *sk = sc + (size_t)NCS * T::NC;        // corners [NKS][KR][KX]
  V *sqx = sk + (size_t)NKS * T::NK;       // q dxim  [CH][KX]
  V *sqy = sqx + T::NQX;                   // q dyim  [KR][TX]
  double *sred = reinterpret_cast<double *>(sqy + T::NQY);
  double dtv = dt_arg, safety = 0.0;
  unsigned long long *cfl_out = nullptr;
  if (ctl != nullptr) {
    if (ctl->done | ctl->pause) return;
    A = ctl->buf[ctl->cur];
    B = ctl->buf[ctl->cur ^ 1];
    dtv = ctl->dt;
    safety = ctl->safety;
    cfl_out = &ctl->cfl_bits;
  }
#define SC(s, c) sc[(size_t)(s) * T::NC + (c)]
#define SK(s, c) sk[(size_t)(s) * T::NK + (c)]
  const size_t n = (size_t)ix * (size_t)jx;
  const int tid = threadIdx.x;
  const int i0 = 1 + blockIdx.x * T::TX;
  const int jb = 1 + blockIdx.y * seg;                 // first interior row of the segment
  const int je = min(jx - 2, jb + seg - 1);            // last
  const PhysN<N> P = phys_n<N>(ph);
  const V dt = N::in(dtv);
  const V hdt = N::scale(dt, 0.5f);
  const bool edge_x = blockIdx.x == 0 || blockIdx.x == gridDim.x - 1;
  V kmax = N::zero();
  bool bad = false;

  for (int j0 = jb; j0 <= je; j0 += CH) {
    const bool first = j0 == jb;
    if (!first) {
      // keep the chunk's last two cell rows and last corner row
      for (int e = tid; e < NCS * 2 * T::CX; e += T::NT) {
        const int s = e / (2 * T::CX), r = e % (2 * T::CX);
        SC(s, r) = SC(s, CH * T::CX + r);
      }
      for (int e = tid; e < NKS * T::KX; e += T::NT) {
        const int s = e / T::KX, r = e % T::KX;
        SK(s, r) = SK(s, CH * T::KX + r);
      }
      __syncthreads();
    }
    // ---- phase 1: new cell rows (all CH + 2 of the first chunk) ----
    const int last_row = min(CH + 1, je + 1 - (j0 - 1));  // rows past je+1 are not read
    for (int c = (first ? 0 : 2 * T::CX) + tid; c < (last_row + 1) * T::CX; c += T::NT) {
      const int lx = c % T::CX, ly = c / T::CX;
      const int gi = i0 - 1 + lx, gj = j0 - 1 + ly;
      if (gi < ix && gj < jx) {
        cell_m<N, T::NC>(A, n, (size_t)gi + (size_t)gj * ix, sc, c, P);
      } else {
#pragma unroll 1
        for (int s = 0; s < NCS; s++) SC(s, c) = N::zero();
      }
    }
    __syncthreads();
    // ---- phase 2: new corner rows, and the viscosity faces ----
    for (int k = (first ? 0 : T::KX) + tid; k < last_row * T::KX; k += T::NT) {
      const int kx = k % T::KX, ky = k / T::KX;
      const int gi = i0 - 1 + kx, gj = j0 - 1 + ky;
      if (gi <= ix - 2 && gj <= jx - 2) {
        const int a = kx + ky * T::CX;
        const V cxk = N::scale(N::mul(dt, N::in(ax.dim[gi])), 0.5f);
        const V cyk = N::scale(N::mul(dt, N::in(ay.dim[gj])), 0.5f);
        corner_m<N, T::NC, T::NK>(sc, sk, a, a + 1, a + 1 + T::CX, a + T::CX, k, cxk, cyk, P);
      } else {
#pragma unroll 1
        for (int s = 0; s < NKS; s++) SK(s, k) = N::zero();
      }
    }
    for (int f = tid; f < T::NQX; f += T::NT) {
      const int fx = f % T::KX, r = f / T::KX;
      const int gi = i0 - 1 + fx, gj = j0 + r;
      V v = N::zero();
      if (gi + 1 < ix && gj < jx) {
        const int cl = fx + (r + 1) * T::CX;
        const V q = N::addf(N::absd(N::sub(SC(CVX, cl + 1), SC(CVX, cl))), -1.0e-4f);
        if (N::pos(q))
          v = N::mul(N::mul(N::mul(P.qav, N::in(ax.dm[gi])), q),
                      N::in(ax.dim[gi]));
      }
      sqx[f] = v;
    }
    for (int f = tid; f < T::NQY; f += T::NT) {
      const int fx = f % T::TX, r = f / T::TX;
      const int gi = i0 + fx, gj = j0 - 1 + r;
      V v = N::zero();
      if (gi < ix && gj + 1 < jx) {
        const int cl = (fx + 1) + r * T::CX;
        const V q = N::addf(N::absd(N::sub(SC(CVY, cl + T::CX), SC(CVY, cl))), -1.0e-4f);
        if (N::pos(q))
          v = N::mul(N::mul(N::mul(P.qav, N::in(ay.dm[gj])), q),
                      N::in(ay.dim[gj]));
      }
      sqy[f] = v;
    }
    __syncthreads();
    // ---- phase 3: the chunk's own cells ----
    if (tid < T::TX * CH) {
      const int lx = tid % T::TX + 1, ly = tid / T::TX + 1;
      const int gi = i0 - 1 + lx, gj = j0 - 1 + ly;
      if (gi <= ix - 2 && gj <= je) {
        const size_t g = (size_t)gi + (size_t)gj * ix;
        // the doubles the update adds to, loaded ahead of the arithmetic
        const double ro0 = A[PRO * n + g], bx0 = A[PBX * n + g], by0 = A[PBY * n + g];
        const double bz0 = A[PBZ * n + g], az0 = A[PAZ * n + g];
        const int c = lx + ly * T::CX;
        const int cE = c + 1, cW = c - 1, cN = c + T::CX, cS = c - T::CX;
        const int kSW = (lx - 1) + (ly - 1) * T::KX, kSE = kSW + 1;
        const int kNW = kSW + T::KX, kNE = kNW + 1;
        const V dxi = N::in(ax.di[gi]), dyi = N::in(ay.di[gj]);
        const V ux0 = N::in(ax.u0[gi]), ux1 = N::in(ax.u1[gi]);
        const V uy0 = N::in(ay.u0[gj]), uy1 = N::in(ay.u1[gj]);
        const V hdx = N::mul(hdt, dxi), hdy = N::mul(hdt, dyi);
        const V fcx = N::scale(hdx, 0.5f), fcy = N::scale(hdy, 0.5f);
        const V fx0 = N::mul(hdx, uy0), fx1 = N::mul(hdx, uy1);
        const V fy0 = N::mul(hdy, ux0), fy1 = N::mul(hdy, ux1);
        const V dtx = N::mul(dt, dxi), dty = N::mul(dt, dyi);
        const V ae = N::mul(dtx, sqx[lx + (ly - 1) * T::KX]);
        const V aw = N::mul(dtx, sqx[lx - 1 + (ly - 1) * T::KX]);
        const V an = N::mul(dty, sqy[(lx - 1) + ly * T::TX]);
        const V as = N::mul(dty, sqy[(lx - 1) + (ly - 1) * T::TX]);
        auto dvar = [&](int su, int sfx, bool negx, int sfy, bool negy, int kfx, bool nkx,
                        int kfy, bool nky) -> V {
          const V u = SC(su, c);
          V du = N::mul(ae, N::sub(SC(su, cE), u));
          du = N::mad(aw, N::sub(SC(su, cW), u), du);
          du = N::mad(an, N::sub(SC(su, cN), u), du);
          du = N::mad(as, N::sub(SC(su, cS), u), du);
          if (sfx != NOF)
            du = N::mad(negx ? fcx : N::neg(fcx), N::sub(SC(sfx, cE), SC(sfx, cW)), du);
          if (sfy != NOF)
            du = N::mad(negy ? fcy : N::neg(fcy), N::sub(SC(sfy, cN), SC(sfy, cS)), du);
          if (kfx != NOF) {
            du = N::mad(nkx ? fx0 : N::neg(fx0), N::sub(SK(kfx, kSE), SK(kfx, kSW)), du);
            du = N::mad(nkx ? fx1 : N::neg(fx1), N::sub(SK(kfx, kNE), SK(kfx, kNW)), du);
          }
          if (kfy != NOF) {
            du = N::mad(nky ? fy0 : N::neg(fy0), N::sub(SK(kfy, kNW), SK(kfy, kSW)), du);
            du = N::mad(nky ? fy1 : N::neg(fy1), N::sub(SK(kfy, kNE), SK(kfy, kSE)), du);
          }
          return du;
        };
        const double ro_new =
            ro0 + N::out(dvar(CRO, CRX, false, CRY, false, KXRO, false, KYRO, false));
        const double bx_new =
            bx0 + N::out(dvar(CBX, NOF, false, CEZ, false, NOF, false, KEZ, false));
        const double by_new =
            by0 + N::out(dvar(CBY, CEZ, true, NOF, false, KEZ, true, NOF, false));
        const double bz_new =
            bz0 + N::out(dvar(CBZ, CEY, false, CEX, true, KEY, false, KEX, true));
        const V ee =
            N::add(SC(CEE, c), dvar(CEE, CFXE, false, CFYE, false, KXEE, false, KYEE, false));
        const V rx =
            N::add(SC(CRX, c), dvar(CRX, CFXRX, false, CFXY, false, KXRX, false, KXY, false));
        const V ry =
            N::add(SC(CRY, c), dvar(CRY, CFXY, false, CFYRY, false, KXY, false, KYRY, false));
        const V rz =
            N::add(SC(CRZ, c), dvar(CRZ, CFXRZ, false, CFYRZ, false, KXRZ, false, KYRZ, false));
        {
          V s = N::mul(ux0, SK(KEZ, kSW));
          s = N::mad(ux1, SK(KEZ, kSE), s);
          V t = N::mul(ux0, SK(KEZ, kNW));
          t = N::mad(ux1, SK(KEZ, kNE), t);
          s = N::mad(uy1, t, N::mul(uy0, s));
          s = N::mad(hdt, SC(CEZ, c), N::mul(hdt, s));
          B[PAZ * n + g] = az0 - N::out(s);
        }
        const V ro = N::in(ro_new);
        const V bx = N::in(bx_new), by = N::in(by_new);
        const V bz = N::in(bz_new);
        const V rinv = N::rcp(ro);
        const V vx = N::mul(rx, rinv), vy = N::mul(ry, rinv), vz = N::mul(rz, rinv);
        const V vv = N::mad(vz, vz, N::mad(vy, vy, N::sqr(vx)));
        const V bb = N::mad(bz, bz, N::mad(by, by, N::sqr(bx)));
        const V pr = N::mul(P.gm1, N::sub(N::sub(ee, N::mul(N::scale(ro, 0.5f), vv)),
                                            N::mul(P.pi8i, bb)));
        const double prd = N::out(pr);
        B[PRO * n + g] = ro_new;
        B[PPR * n + g] = prd;
        B[PVX * n + g] = N::out(vx);
        B[PVY * n + g] = N::out(vy);
        B[PVZ * n + g] = N::out(vz);
        B[PBX * n + g] = bx_new;
        B[PBY * n + g] = by_new;
        B[PBZ * n + g] = bz_new;
        if (cfl_out != nullptr && gi >= box.lo[0] && gi <= box.hi[0] && gj >= box.lo[1] &&
            gj <= box.hi[1]) {
          const V sk2 = N::mad(N::mad(P.gm, pr, N::mul(P.pi4i, bb)), rinv, vv);
          const V ix2 = N::sqr(dxi), iy2 = N::sqr(dyi);
          const V key = N::mul(sk2, N::gt(ix2, iy2) ? ix2 : iy2);
          if (!N::isnan(key) && N::gt(key, kmax)) kmax = key;
          bad |= bad_cell_d(ro_new, prd, N::nan_probe(key));
        }
      }
    }
    // ghost cells of the output keep their input values; each is copied by
    // the chunk owning its nearest interior cell
    if (edge_x || j0 == 1 || j0 + CH - 1 >= jx - 2) {
      for (int c = tid; c < T::NC; c += T::NT) {
        const int hx = c % T::CX, hy = c / T::CX;
        const int gi = i0 - 1 + hx, gj = j0 - 1 + hy;
        if (gi >= ix || gj >= jx) continue;
        if (gi != 0 && gi != ix - 1 && gj != 0 && gj != jx - 1) continue;
        const int ci = min(max(gi, 1), ix - 2), cj = min(max(gj, 1), jx - 2);
        if (ci < i0 || ci >= i0 + T::TX || cj < j0 || cj >= j0 + CH || cj > je) continue;
        const size_t g = (size_t)gi + (size_t)gj * ix;
#pragma unroll
        for (int v = 0; v < NPV; v++) B[v * n + g] = A[v * n + g];
      }
    }
    __syncthreads();
  }
#undef SC
#undef SK
  if (cfl_out != nullptr) {
    if (ctl != nullptr) count_bad_block(bad, &ctl->nonfinite, tid);
    kmax = N::warp_max(kmax);
    const int lane = tid & 31, w = tid >> 5;
    if (lane == 0) sred[w] = N::out(kmax);
    __syncthreads();
    if (w == 0) {
      double x = lane < (T::NT + 31) / 32 ? sred[lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_xor_sync(0xffffffffu, x, o);
        x = (y > x || x != x) ? y : x;
      }
      if (lane == 0 && x > 0.0) atomic_min_pos(cfl_out, safety / sqrt(x));
    }
  }
}

// Rows per block of the marching kernel.  The step is bound by the
// arithmetic pipes, so a launch takes as long as its busiest SM: the blocks
// an SM gets (all blocks spread evenly over the SMs) times the rows a block
// computes -- its segment, the two-row prologue and one row's worth of
// barriers per chunk.  A segment need not be a whole number of chunks (its
// last chunk may be short, as at the end of the grid).
inline int balance_seg(int strips, int rows, int ch, int sms) {
  int best = rows;
  long long best_cost = -1;
  for (int seg = ch > 1 ? ch / 2 : 1; seg <= rows; seg++) {
    const long long blocks = (long long)strips * ((rows + seg - 1) / seg);
    const long long per_sm = (blocks + sms - 1) / sms;
    const long long cost = per_sm * (seg + 2 + (seg + ch - 1) / ch);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = seg;
    }
  }
  return best;
}
// The same with whole chunks per block, balanced by waves of resident
// blocks (slots = SMs x resident blocks per SM): for a step that is bound by
// latency more than by one pipe, fewer and longer blocks can win.
inline int balance_seg_waves(int strips, int rows, int ch, int slots) {
  int best = ch, best_cost = -1;
  for (int seg = ch; seg <= rows + ch - 1; seg += ch) {
    const int blocks = strips * ((rows + seg - 1) / seg);
    const int waves = (blocks + slots - 1) / slots;
    const int cost = waves * (seg + 2);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = seg;
    }
  }
  return best;
}

template <int TX, int TY, int RPT>
__global__ void __launch_bounds__(TX *TY / RPT, 1)
    k_mlw2d_df(const double *__restrict__ A, double *__restrict__ B, int ix, int jx, Axis ax,
               Axis ay, Phys ph, double dt_arg, Ctl *__restrict__ ctl, Box3 box) {
  extern __shared__ D smem_d[];
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
  tile_step_df<TX, TY, RPT>(A, B, ix, jx, ax, ay, ph, dt, safety, cfl, box, blockIdx.x,
                            blockIdx.y, gridDim.x, gridDim.y, smem_d,
                            ctl ? &ctl->nonfinite : nullptr);
}

template <int TX, int TY, int RPT>
cudaError_t launch_df(const double *A, double *B, int ix, int jx, const Axis &ax,
                      const Axis &ay, const Phys &ph, double dt, Ctl *ctl, Box3 box,
                      cudaStream_t s) {
  using T = TileD<TX, TY, RPT>;
  cudaError_t e = cudaFuncSetAttribute(k_mlw2d_df<TX, TY, RPT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)T::smem_bytes);
  if (e != cudaSuccess) return e;
  dim3 grid((ix - 2 + TX - 1) / TX, (jx - 2 + TY - 1) / TY);
  k_mlw2d_df<TX, TY, RPT><<<grid, T::NT, T::smem_bytes, s>>>(A, B, ix, jx, ax, ay, ph, dt,
                                                             ctl, box);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

namespace {
template <class N, int CH>
cudaError_t launch_march(const double *A, double *B, int ix, int jx, const Axis &ax,
                         const Axis &ay, const Phys &ph, double dt, Ctl *ctl, Box3 box,
                         cudaStream_t s, bool waves = false) {
  using T = MarchD<CH>;
  static std::mutex mu;
  static int sms_of[64] = {}, slots_of[64] = {};
  int dev = 0, sms = 0, slots = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!sms_of[dev]) {
      e = cudaFuncSetAttribute(k_mlw2d_march<N, CH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)T::smem_bytes);
      if (e != cudaSuccess) return e;
      int m = 0, per_sm = 0;
      if ((e = cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return e;
      if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mlw2d_march<N, CH>,
                                                             T::NT, T::smem_bytes)) !=
          cudaSuccess)
        return e;
      sms_of[dev] = m > 0 ? m : 1;
      slots_of[dev] = sms_of[dev] * (per_sm > 0 ? per_sm : 1);
    }
    sms = sms_of[dev];
    slots = slots_of[dev];
  }
  const int strips = (ix - 2 + T::TX - 1) / T::TX, rows = jx - 2;
  const int seg = waves ? balance_seg_waves(strips, rows, CH, slots)
                        : balance_seg(strips, rows, CH, sms);
  dim3 grid(strips, (rows + seg - 1) / seg);
  k_mlw2d_march<N, CH><<<grid, T::NT, T::smem_bytes, s>>>(A, B, ix, jx, ax, ay, ph, dt, ctl,
                                                         box, seg);
  count_launch();
  return cudaGetLastError();
}
}  // namespace

int mlw2d_df_tile_count() { return 7; }

// The fast policy's mlw_m3 step with the y-marching tile (FP64, F64N).
cudaError_t launch_mlw2d_march_fast(const double *A, double *B, int ix, int jx,
                                    const Axis &ax, const Axis &ay, const Phys &ph, double dt,
                                    Ctl *ctl, Box3 box, cudaStream_t s, bool waves) {
  if (ix < 3 || jx < 3) return cudaErrorInvalidValue;
  return launch_march<F64N, 8>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s, waves);
}

cudaError_t launch_mlw2d_df(int tile, const double *A, double *B, int ix, int jx,
                            const Axis &ax, const Axis &ay, const Phys &ph, double dt,
                            Ctl *ctl, Box3 box, cudaStream_t s) {
  if (ix < 3 || jx < 3) return cudaErrorInvalidValue;
  switch (tile) {
    case 4: return launch_march<DFN, 8>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
    case 5: return launch_march<DFN, 6>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
    case 6: return launch_march<DFN, 8>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s, true);
    case 1: return launch_df<32, 9, 1>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
    case 2: return launch_df<16, 16, 2>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
    case 3: return launch_df<32, 16, 2>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
    default: return launch_df<32, 8, 2>(A, B, ix, jx, ax, ay, ph, dt, ctl, box, s);
  }
}

}  // namespace cans
