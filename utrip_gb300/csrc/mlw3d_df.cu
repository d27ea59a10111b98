// Fused 3-D mLW step, mlw_m (cans3d/hdmlw/mlw_m.f:2-453), in the double-float
// policy (df64.cuh): the arithmetic runs as pairs of floats on the FP32
// pipes and the density and field are accumulated in FP64, as in the 2-D
// double-float step (mlw2d_df.cu).
//
// The block structure is that of k_mlw3d (mlw3d.cu): a TX x TY column of
// cells marching along z over a chunk of planes, one thread per cell of the
// halo tile, two-plane rings of cell values and of corner (half-step) fluxes
// in shared memory, the own column's plane k-1 in registers.  The algebra is
// the fast policy's, with the momentum flux tensor formed once per pair
// (fx(ry) = fy(rx), fx(rz) = fz(rx), fy(rz) = fz(ry)) and the total
// pressure formed once, at the cells and the corners: 23 cell and 15 corner
// fields instead of 26 and 18.
#include <cuda_runtime.h>

#include <mutex>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "cfl3.cuh"
#include "df64.cuh"

namespace cans {

namespace {

using df::D;

// cell fields of one ring slot
enum {
  C_RO = 0, C_EE, C_RX, C_RY, C_RZ, C_BX, C_BY, C_BZ,
  C_FXE, C_FYE, C_FZE, C_FXX, C_FYY, C_FZZ, C_FXY, C_FXZ, C_FYZ,
  C_EX, C_EY, C_EZ, C_VX, C_VY, C_VZ, NC3
};
// corner fields of one ring slot (the mass fluxes are the half-step momenta)
enum {
  K_XRO = 0, K_YRO, K_ZRO, K_XEE, K_YEE, K_ZEE, K_XX, K_YY, K_ZZ, K_XY, K_XZ, K_YZ,
  K_EX, K_EY, K_EZ, NK3
};
constexpr int NOF3 = -1;

// Flux field of conserved variable v (ro ee rx ry rz bx by bz) along dir
// (x y z) at the cells and at the corners, and whether it enters negated.
__device__ __forceinline__ void flux_cell(int v, int dir, int &f, bool &neg) {
  neg = false;
  switch (v) {
    case 0: f = dir == 0 ? C_RX : dir == 1 ? C_RY : C_RZ; break;
    case 1: f = dir == 0 ? C_FXE : dir == 1 ? C_FYE : C_FZE; break;
    case 2: f = dir == 0 ? C_FXX : dir == 1 ? C_FXY : C_FXZ; break;
    case 3: f = dir == 0 ? C_FXY : dir == 1 ? C_FYY : C_FYZ; break;
    case 4: f = dir == 0 ? C_FXZ : dir == 1 ? C_FYZ : C_FZZ; break;
    case 5: f = dir == 0 ? NOF3 : dir == 1 ? C_EZ : C_EY; neg = (dir == 2); break;
    case 6: f = dir == 0 ? C_EZ : dir == 1 ? NOF3 : C_EX; neg = (dir == 0); break;
    default: f = dir == 0 ? C_EY : dir == 1 ? C_EX : NOF3; neg = (dir == 1); break;
  }
}
__device__ __forceinline__ void flux_corner(int v, int dir, int &f, bool &neg) {
  neg = false;
  switch (v) {
    case 0: f = dir == 0 ? K_XRO : dir == 1 ? K_YRO : K_ZRO; break;
    case 1: f = dir == 0 ? K_XEE : dir == 1 ? K_YEE : K_ZEE; break;
    case 2: f = dir == 0 ? K_XX : dir == 1 ? K_XY : K_XZ; break;
    case 3: f = dir == 0 ? K_XY : dir == 1 ? K_YY : K_YZ; break;
    case 4: f = dir == 0 ? K_XZ : dir == 1 ? K_YZ : K_ZZ; break;
    case 5: f = dir == 0 ? NOF3 : dir == 1 ? K_EZ : K_EY; neg = (dir == 2); break;
    case 6: f = dir == 0 ? K_EZ : dir == 1 ? NOF3 : K_EX; neg = (dir == 0); break;
    default: f = dir == 0 ? K_EY : dir == 1 ? K_EX : NOF3; neg = (dir == 1); break;
  }
}

template <int TX, int TY> struct Tile3D {
  static constexpr int CX = TX + 2, CY = TY + 2, NC = CX * CY;
  static constexpr int KX = TX + 1, KY = TY + 1, NK = KX * KY;
  static constexpr int NQX = (TX + 1) * TY, NQY = TX * (TY + 1);
  static constexpr int NT = (NC + 31) / 32 * 32;
  static constexpr size_t smem_bytes =
      sizeof(D) * (2 * (size_t)NC3 * NC + 2 * (size_t)NK3 * NK + NQX + NQY) +
      sizeof(double) * 32;
  // blocks per SM the registers are budgeted for: two of the narrow tile
  // fit in shared memory
  static constexpr int MINB = TX * TY <= 128 ? 2 : 1;
};

struct PhysD3 {
  D gm, gm1, gm1i, ggm1, pi4i, pi8i, qav, pi4i_cfl;
};

// the fluxes of one state (cell or corner): E = -v x B, the energy flux
// ep v + (B x E)/4pi and the momentum flux rho v v + p_T - B B/4pi
struct Flux3 {
  D ex, ey, ez, fxe, fye, fze, fxx, fyy, fzz, fxy, fxz, fyz;
};
__device__ __forceinline__ Flux3 fluxes3(D rx, D ry, D rz, D vx, D vy, D vz, D bx, D by, D bz,
                                         D ep, D pt, const PhysD3 &P) {
  Flux3 o;
  o.ex = df::mad(vz, by, df::neg(df::mul(vy, bz)));
  o.ey = df::mad(vx, bz, df::neg(df::mul(vz, bx)));
  o.ez = df::mad(vy, bx, df::neg(df::mul(vx, by)));
  o.fxe = df::mad(df::mad(bz, o.ey, df::neg(df::mul(by, o.ez))), P.pi4i, df::mul(ep, vx));
  o.fye = df::mad(df::mad(bx, o.ez, df::neg(df::mul(bz, o.ex))), P.pi4i, df::mul(ep, vy));
  o.fze = df::mad(df::mad(by, o.ex, df::neg(df::mul(bx, o.ey))), P.pi4i, df::mul(ep, vz));
  const D pbx = df::mul(P.pi4i, bx), pby = df::mul(P.pi4i, by), pbz = df::mul(P.pi4i, bz);
  o.fxx = df::mad(rx, vx, df::mad(df::neg(pbx), bx, pt));
  o.fyy = df::mad(ry, vy, df::mad(df::neg(pby), by, pt));
  o.fzz = df::mad(rz, vz, df::mad(df::neg(pbz), bz, pt));
  o.fxy = df::mad(rx, vy, df::neg(df::mul(pbx, by)));
  o.fxz = df::mad(rx, vz, df::neg(df::mul(pbx, bz)));
  o.fyz = df::mad(ry, vz, df::neg(df::mul(pby, bz)));
  return o;
}

template <int TX, int TY>
__global__ void __launch_bounds__(Tile3D<TX, TY>::NT, Tile3D<TX, TY>::MINB)
    k_mlw3d_df(const double *__restrict__ A, double *__restrict__ B, int ix, int jx, int kx,
               Axis ax, Axis ay, Axis az, Phys ph, double dt_arg, Ctl *__restrict__ ctl,
               Box3 box, int kchunk) {
  using T = Tile3D<TX, TY>;
  extern __shared__ D smem3[];
  D *scell = smem3;                                  // [2][NC3][NC]
  D *scorn = scell + 2 * (size_t)NC3 * T::NC;        // [2][NK3][NK]
  D *sqx = scorn + 2 * (size_t)NK3 * T::NK;          // q dxim of plane k
  D *sqy = sqx + T::NQX;                             // q dyim of plane k
  double *sred = reinterpret_cast<double *>(sqy + T::NQY);

  if (ctl != nullptr) {
    if (ctl->done | ctl->pause) return;
    A = ctl->buf[ctl->cur];
    B = ctl->buf[ctl->cur ^ 1];
  }
  const double dtv = (ctl != nullptr) ? ctl->dt : dt_arg;
  const size_t n = (size_t)ix * jx * kx;
  const size_t plane = (size_t)ix * jx;
  const int tid = threadIdx.x;
  const bool cell = tid < T::NC;
  const int hx = tid % T::CX, hy = tid / T::CX;
  const int i0 = 1 + blockIdx.x * TX, j0 = 1 + blockIdx.y * TY;
  const int gi = i0 - 1 + hx, gj = j0 - 1 + hy;
  const bool in_arr = cell && gi < ix && gj < jx;
  const bool interior = cell && hx >= 1 && hx <= TX && hy >= 1 && hy <= TY &&
                        gi <= ix - 2 && gj <= jx - 2;
  const int kb = 1 + blockIdx.z * kchunk;
  const int ke = min(kx - 2, kb + kchunk - 1);
  if (kb > ke) return;
  const PhysD3 P = {df::from_double(ph.gm),   df::from_double(ph.gm1),
                    df::from_double(ph.gm1i), df::from_double(ph.ggm1),
                    df::from_double(ph.pi4i), df::from_double(ph.pi8i),
                    df::from_double(ph.qav),  df::from_double(ph.pi4i_cfl)};
  const D dt = df::from_double(dtv);
  const D hdt = df::scale(dt, 0.5f);

  auto cslot = [&](int k) { return scell + (size_t)(k & 1) * NC3 * T::NC; };
  auto kslot = [&](int k) { return scorn + (size_t)(k & 1) * NK3 * T::NK; };

  // cells of plane k (mlw_m.f:74-202)
  auto load_plane = [&](int k) {
    D *sl = cslot(k);
#define S(f) sl[(size_t)(f) * T::NC + tid]
    if (in_arr) {
      const size_t g = (size_t)gi + (size_t)gj * ix + (size_t)k * plane;
      const D ro = df::from_double(A[P3::RO * n + g]), pr = df::from_double(A[P3::PR * n + g]);
      const D vx = df::from_double(A[P3::VX * n + g]), vy = df::from_double(A[P3::VY * n + g]);
      const D vz = df::from_double(A[P3::VZ * n + g]);
      const D bx = df::from_double(A[P3::BX * n + g]), by = df::from_double(A[P3::BY * n + g]);
      const D bz = df::from_double(A[P3::BZ * n + g]);
      const D vv = df::mad(vz, vz, df::mad(vy, vy, df::sqr(vx)));
      const D bb = df::mad(bz, bz, df::mad(by, by, df::sqr(bx)));
      const D ek = df::mul(df::scale(ro, 0.5f), vv);
      const D rx = df::mul(ro, vx), ry = df::mul(ro, vy), rz = df::mul(ro, vz);
      const Flux3 fl = fluxes3(rx, ry, rz, vx, vy, vz, bx, by, bz, df::mad(pr, P.ggm1, ek),
                               df::mad(P.pi8i, bb, pr), P);
      S(C_RO) = ro; S(C_EE) = df::mad(pr, P.gm1i, df::mad(P.pi8i, bb, ek));
      S(C_RX) = rx; S(C_RY) = ry; S(C_RZ) = rz;
      S(C_BX) = bx; S(C_BY) = by; S(C_BZ) = bz;
      S(C_VX) = vx; S(C_VY) = vy; S(C_VZ) = vz;
      S(C_EX) = fl.ex; S(C_EY) = fl.ey; S(C_EZ) = fl.ez;
      S(C_FXE) = fl.fxe; S(C_FYE) = fl.fye; S(C_FZE) = fl.fze;
      S(C_FXX) = fl.fxx; S(C_FYY) = fl.fyy; S(C_FZZ) = fl.fzz;
      S(C_FXY) = fl.fxy; S(C_FXZ) = fl.fxz; S(C_FYZ) = fl.fyz;
    } else if (cell) {
#pragma unroll 1
      for (int f = 0; f < NC3; f++) S(f) = df::mk(0.0f);
    }
#undef S
  };

  // corner plane k+1/2 from cell planes k (lower) and k+1 (upper)
  // (mlwhalf part 2, then the half-step primitives and fluxes, :206-330)
  auto corner_plane = [&](int k) {
    if (tid >= T::NK) return;
    const int cx = tid % T::KX, cy = tid / T::KX;
    const int a = i0 - 1 + cx, b = j0 - 1 + cy;  // lower corner cell
    D *ks = kslot(k);
#define KS(f) ks[(size_t)(f) * T::NK + tid]
    if (a > ix - 2 || b > jx - 2) {
#pragma unroll 1
      for (int f = 0; f < NK3; f++) KS(f) = df::mk(0.0f);
      return;
    }
    const D *L = cslot(k), *U = cslot(k + 1);
    const int p00 = cx + cy * T::CX, p10 = p00 + 1, p01 = p00 + T::CX, p11 = p01 + 1;
    const D cxk = df::scale(df::mul(dt, df::from_double(ax.dim[a])), 0.25f);
    const D cyk = df::scale(df::mul(dt, df::from_double(ay.dim[b])), 0.25f);
    const D czk = df::scale(df::mul(dt, df::from_double(az.dim[k])), 0.25f);
    D un[8];
#pragma unroll 1
    for (int v = 0; v < 8; v++) {
      const D *Lv = L + (size_t)v * T::NC, *Uv = U + (size_t)v * T::NC;
      D r = df::scale(df::add(df::add(df::add(Lv[p10], Lv[p00]), df::add(Lv[p11], Lv[p01])),
                              df::add(df::add(Uv[p10], Uv[p00]), df::add(Uv[p11], Uv[p01]))),
                      0.125f);
      int f;
      bool ng;
      flux_cell(v, 0, f, ng);
      if (f != NOF3) {
        const D *l = L + (size_t)f * T::NC, *u = U + (size_t)f * T::NC;
        const D s = df::add(df::add(df::sub(l[p10], l[p00]), df::sub(l[p11], l[p01])),
                            df::add(df::sub(u[p10], u[p00]), df::sub(u[p11], u[p01])));
        r = df::mad(ng ? cxk : df::neg(cxk), s, r);
      }
      flux_cell(v, 1, f, ng);
      if (f != NOF3) {
        const D *l = L + (size_t)f * T::NC, *u = U + (size_t)f * T::NC;
        const D s = df::add(df::add(df::sub(l[p01], l[p00]), df::sub(l[p11], l[p10])),
                            df::add(df::sub(u[p01], u[p00]), df::sub(u[p11], u[p10])));
        r = df::mad(ng ? cyk : df::neg(cyk), s, r);
      }
      flux_cell(v, 2, f, ng);
      if (f != NOF3) {
        const D *l = L + (size_t)f * T::NC, *u = U + (size_t)f * T::NC;
        const D s = df::add(df::add(df::sub(u[p00], l[p00]), df::sub(u[p10], l[p10])),
                            df::add(df::sub(u[p01], l[p01]), df::sub(u[p11], l[p11])));
        r = df::mad(ng ? czk : df::neg(czk), s, r);
      }
      un[v] = r;
    }
    const D roh = un[0], eeh = un[1], rxh = un[2], ryh = un[3], rzh = un[4];
    const D bxh = un[5], byh = un[6], bzh = un[7];
    const D rinv = df::rcp(roh);
    const D vxh = df::mul(rxh, rinv), vyh = df::mul(ryh, rinv), vzh = df::mul(rzh, rinv);
    const D vv = df::mad(vzh, vzh, df::mad(vyh, vyh, df::sqr(vxh)));
    const D bb = df::mad(bzh, bzh, df::mad(byh, byh, df::sqr(bxh)));
    const D ek = df::mul(df::scale(roh, 0.5f), vv);
    const D prh = df::mul(P.gm1, df::sub(df::sub(eeh, ek), df::mul(P.pi8i, bb)));
    const Flux3 fl = fluxes3(rxh, ryh, rzh, vxh, vyh, vzh, bxh, byh, bzh,
                             df::mad(prh, P.ggm1, ek), df::mad(P.pi8i, bb, prh), P);
    KS(K_XRO) = rxh; KS(K_YRO) = ryh; KS(K_ZRO) = rzh;
    KS(K_XEE) = fl.fxe; KS(K_YEE) = fl.fye; KS(K_ZEE) = fl.fze;
    KS(K_XX) = fl.fxx; KS(K_YY) = fl.fyy; KS(K_ZZ) = fl.fzz;
    KS(K_XY) = fl.fxy; KS(K_XZ) = fl.fxz; KS(K_YZ) = fl.fyz;
    KS(K_EX) = fl.ex; KS(K_EY) = fl.ey; KS(K_EZ) = fl.ez;
#undef KS
  };

  // own-column data of plane k-1 kept for the z terms of plane k
  D pu[8], pfz[8], pvz = df::mk(0.0f);
  auto save_prev = [&](int k) {
    const D *sl = cslot(k);
#pragma unroll
    for (int v = 0; v < 8; v++) {
      pu[v] = sl[(size_t)v * T::NC + tid];
      int f;
      bool ng;
      flux_cell(v, 2, f, ng);
      const D x = (f != NOF3) ? sl[(size_t)f * T::NC + tid] : df::mk(0.0f);
      pfz[v] = ng ? df::neg(x) : x;
    }
    pvz = sl[(size_t)C_VZ * T::NC + tid];
  };

  load_plane(kb - 1);
  load_plane(kb);
  __syncthreads();
  if (interior) save_prev(kb - 1);
  corner_plane(kb - 1);
  __syncthreads();

  D kmax = df::mk(0.0f);
  bool bad = false;
  for (int k = kb; k <= ke; k++) {
    load_plane(k + 1);
    __syncthreads();
    corner_plane(k);
    {
      const D *sl = cslot(k);
      for (int f = tid; f < T::NQX; f += T::NT) {
        const int fx = f % (TX + 1), r = f / (TX + 1);
        const int a = i0 - 1 + fx, b = j0 + r;
        D v = df::mk(0.0f);
        if (a + 1 < ix && b < jx) {
          const int cl = fx + (r + 1) * T::CX;
          const D q = df::addf(
              df::absd(df::sub(sl[(size_t)C_VX * T::NC + cl + 1], sl[(size_t)C_VX * T::NC + cl])),
              -1.0e-4f);
          if (df::pos(q))
            v = df::mul(df::mul(df::mul(P.qav, df::from_double(ax.dm[a])), q),
                        df::from_double(ax.dim[a]));
        }
        sqx[f] = v;
      }
      for (int f = tid; f < T::NQY; f += T::NT) {
        const int fx = f % TX, r = f / TX;
        const int a = i0 + fx, b = j0 - 1 + r;
        D v = df::mk(0.0f);
        if (a < ix && b + 1 < jx) {
          const int cl = (fx + 1) + r * T::CX;
          const D q = df::addf(df::absd(df::sub(sl[(size_t)C_VY * T::NC + cl + T::CX],
                                                sl[(size_t)C_VY * T::NC + cl])),
                               -1.0e-4f);
          if (df::pos(q))
            v = df::mul(df::mul(df::mul(P.qav, df::from_double(ay.dm[b])), q),
                        df::from_double(ay.dim[b]));
        }
        sqy[f] = v;
      }
    }
    __syncthreads();
    if (interior) {
      const D *S0 = cslot(k), *S1 = cslot(k + 1);
      const D *KL = kslot(k - 1), *KU = kslot(k);
      const size_t g = (size_t)gi + (size_t)gj * ix + (size_t)k * plane;
      const double ro0 = A[P3::RO * n + g], bx0 = A[P3::BX * n + g];
      const double by0 = A[P3::BY * n + g], bz0 = A[P3::BZ * n + g];
      const int c = tid, cE = c + 1, cW = c - 1, cN = c + T::CX, cS = c - T::CX;
      const int kSW = (hx - 1) + (hy - 1) * T::KX, kSE = kSW + 1;
      const int kNW = kSW + T::KX, kNE = kNW + 1;
      const D dxi = df::from_double(ax.di[gi]), dyi = df::from_double(ay.di[gj]);
      const D dzi = df::from_double(az.di[k]);
      const D ux0 = df::from_double(ax.u0[gi]), ux1 = df::from_double(ax.u1[gi]);
      const D uy0 = df::from_double(ay.u0[gj]), uy1 = df::from_double(ay.u1[gj]);
      const D uz0 = df::from_double(az.u0[k]), uz1 = df::from_double(az.u1[k]);
      const D hx_ = df::mul(hdt, dxi), hy_ = df::mul(hdt, dyi), hz_ = df::mul(hdt, dzi);
      const D fcx = df::scale(hx_, 0.5f), fcy = df::scale(hy_, 0.5f), fcz = df::scale(hz_, 0.5f);
      const D hxz0 = df::mul(hx_, uz0), hxz1 = df::mul(hx_, uz1);
      const D wxL0 = df::mul(hxz0, uy0), wxL1 = df::mul(hxz0, uy1);
      const D wxU0 = df::mul(hxz1, uy0), wxU1 = df::mul(hxz1, uy1);
      const D hyx0 = df::mul(hy_, ux0), hyx1 = df::mul(hy_, ux1);
      const D wyL0 = df::mul(hyx0, uz0), wyU0 = df::mul(hyx0, uz1);
      const D wyL1 = df::mul(hyx1, uz0), wyU1 = df::mul(hyx1, uz1);
      const D hzy0 = df::mul(hz_, uy0), hzy1 = df::mul(hz_, uy1);
      const D wzSW = df::mul(hzy0, ux0), wzSE = df::mul(hzy0, ux1);
      const D wzNW = df::mul(hzy1, ux0), wzNE = df::mul(hzy1, ux1);
      const D dtx = df::mul(dt, dxi), dty = df::mul(dt, dyi), dtz = df::mul(dt, dzi);
      const D ae = df::mul(dtx, sqx[hx + (hy - 1) * (TX + 1)]);
      const D aw = df::mul(dtx, sqx[hx - 1 + (hy - 1) * (TX + 1)]);
      const D an = df::mul(dty, sqy[(hx - 1) + hy * TX]);
      const D as = df::mul(dty, sqy[(hx - 1) + (hy - 1) * TX]);
      const D vz0 = S0[(size_t)C_VZ * T::NC + c], vz1 = S1[(size_t)C_VZ * T::NC + c];
      D au = df::mk(0.0f), ad = df::mk(0.0f);
      {
        const D qu = df::addf(df::absd(df::sub(vz1, vz0)), -1.0e-4f);
        if (df::pos(qu))
          au = df::mul(dtz, df::mul(df::mul(df::mul(P.qav, df::from_double(az.dm[k])), qu),
                                    df::from_double(az.dim[k])));
        const D qd = df::addf(df::absd(df::sub(vz0, pvz)), -1.0e-4f);
        if (df::pos(qd))
          ad = df::mul(dtz, df::mul(df::mul(df::mul(P.qav, df::from_double(az.dm[k - 1])), qd),
                                    df::from_double(az.dim[k - 1])));
      }
      // the eight variables in a rolled loop: unrolled, the kernel's code
      // outgrows the instruction cache (ncu: "no instruction" stalls)
      D du[8];
#pragma unroll 1
      for (int v = 0; v < 8; v++) {
        const D *Sv = S0 + (size_t)v * T::NC;
        const D u = Sv[c];
        D r = df::mul(ae, df::sub(Sv[cE], u));
        r = df::mad(aw, df::sub(Sv[cW], u), r);
        r = df::mad(an, df::sub(Sv[cN], u), r);
        r = df::mad(as, df::sub(Sv[cS], u), r);
        r = df::mad(au, df::sub(S1[(size_t)v * T::NC + c], u), r);
        r = df::mad(ad, df::sub(pu[v], u), r);
        int f;
        bool ng;
        flux_cell(v, 0, f, ng);
        if (f != NOF3)
          r = df::mad(ng ? fcx : df::neg(fcx),
                      df::sub(S0[(size_t)f * T::NC + cE], S0[(size_t)f * T::NC + cW]), r);
        flux_cell(v, 1, f, ng);
        if (f != NOF3)
          r = df::mad(ng ? fcy : df::neg(fcy),
                      df::sub(S0[(size_t)f * T::NC + cN], S0[(size_t)f * T::NC + cS]), r);
        flux_cell(v, 2, f, ng);
        if (f != NOF3) {
          const D up = S1[(size_t)f * T::NC + c];
          r = df::mad(df::neg(fcz), df::sub(ng ? df::neg(up) : up, pfz[v]), r);
        }
        flux_corner(v, 0, f, ng);
        if (f != NOF3) {
          const D *L = KL + (size_t)f * T::NK, *U = KU + (size_t)f * T::NK;
          r = df::mad(ng ? wxL0 : df::neg(wxL0), df::sub(L[kSE], L[kSW]), r);
          r = df::mad(ng ? wxL1 : df::neg(wxL1), df::sub(L[kNE], L[kNW]), r);
          r = df::mad(ng ? wxU0 : df::neg(wxU0), df::sub(U[kSE], U[kSW]), r);
          r = df::mad(ng ? wxU1 : df::neg(wxU1), df::sub(U[kNE], U[kNW]), r);
        }
        flux_corner(v, 1, f, ng);
        if (f != NOF3) {
          const D *L = KL + (size_t)f * T::NK, *U = KU + (size_t)f * T::NK;
          r = df::mad(ng ? wyL0 : df::neg(wyL0), df::sub(L[kNW], L[kSW]), r);
          r = df::mad(ng ? wyU0 : df::neg(wyU0), df::sub(U[kNW], U[kSW]), r);
          r = df::mad(ng ? wyL1 : df::neg(wyL1), df::sub(L[kNE], L[kSE]), r);
          r = df::mad(ng ? wyU1 : df::neg(wyU1), df::sub(U[kNE], U[kSE]), r);
        }
        flux_corner(v, 2, f, ng);
        if (f != NOF3) {
          const D *L = KL + (size_t)f * T::NK, *U = KU + (size_t)f * T::NK;
          r = df::mad(ng ? wzSW : df::neg(wzSW), df::sub(U[kSW], L[kSW]), r);
          r = df::mad(ng ? wzSE : df::neg(wzSE), df::sub(U[kSE], L[kSE]), r);
          r = df::mad(ng ? wzNW : df::neg(wzNW), df::sub(U[kNW], L[kNW]), r);
          r = df::mad(ng ? wzNE : df::neg(wzNE), df::sub(U[kNE], L[kNE]), r);
        }
        du[v] = r;
      }
      // conserved u + du: ro and B in FP64 on the input doubles, the energy
      // and momenta in double-float on their cell values
      const double ro_new = ro0 + df::to_double(du[0]);
      const double bx_new = bx0 + df::to_double(du[5]);
      const double by_new = by0 + df::to_double(du[6]);
      const double bz_new = bz0 + df::to_double(du[7]);
      const D ee = df::add(S0[(size_t)C_EE * T::NC + c], du[1]);
      const D rx = df::add(S0[(size_t)C_RX * T::NC + c], du[2]);
      const D ry = df::add(S0[(size_t)C_RY * T::NC + c], du[3]);
      const D rz = df::add(S0[(size_t)C_RZ * T::NC + c], du[4]);
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
      B[P3::RO * n + g] = ro_new;
      B[P3::PR * n + g] = prd;
      B[P3::VX * n + g] = df::to_double(vx);
      B[P3::VY * n + g] = df::to_double(vy);
      B[P3::VZ * n + g] = df::to_double(vz);
      B[P3::BX * n + g] = bx_new;
      B[P3::BY * n + g] = by_new;
      B[P3::BZ * n + g] = bz_new;
      if (ctl != nullptr && gi >= box.lo[0] && gi <= box.hi[0] && gj >= box.lo[1] &&
          gj <= box.hi[1] && k >= box.lo[2] && k <= box.hi[2]) {
        // cans3d/common/cfl_m.f:52-59 (pi in single precision), as the
        // largest S max(1/dx^2, 1/dy^2, 1/dz^2)
        const D s = df::mad(df::mad(P.gm, pr, df::mul(P.pi4i_cfl, bb)), rinv, vv);
        const D x2 = df::sqr(dxi), y2 = df::sqr(dyi), z2 = df::sqr(dzi);
        D m2 = df::gt(x2, y2) ? x2 : y2;
        if (df::gt(z2, m2)) m2 = z2;
        const D key = df::mul(s, m2);
        if (key.h == key.h && df::gt(key, kmax)) kmax = key;
        constexpr long long kInf = 0x7ff0000000000000LL;
        const long long ra = __double_as_longlong(ro_new), pa = __double_as_longlong(prd);
        bad |= ra <= 0 || ra > kInf || pa <= 0 || pa > kInf ||
               (__float_as_uint(key.h) & 0x7fffffffu) > 0x7f800000u;
      }
      save_prev(k);
    }
    // ghost cells keep their input values; each is copied by the block owning
    // its nearest interior cell, plane by plane, plus the z ghost planes at
    // the chunk ends
    if (in_arr) {
      const int ci = min(max(gi, 1), ix - 2), cj = min(max(gj, 1), jx - 2);
      if (ci >= i0 && ci < i0 + TX && cj >= j0 && cj < j0 + TY) {
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
    // largest key of the block, one conversion, root and division
    D m = kmax;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      D w;
      w.h = __shfl_xor_sync(0xffffffffu, m.h, o);
      w.l = __shfl_xor_sync(0xffffffffu, m.l, o);
      if (df::gt(w, m)) m = w;
    }
    const int lane = tid & 31, w = tid >> 5;
    if (lane == 0) sred[w] = df::to_double(m);
    __syncthreads();
    if (w == 0) {
      double x = lane < T::NT / 32 ? sred[lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_xor_sync(0xffffffffu, x, o);
        x = y > x ? y : x;
      }
      if (lane == 0 && x > 0.0) atomic_min_pos(&ctl->cfl_bits, ctl->safety / sqrt(x));
    }
  }
}

// The z chunk with the fewest waves x (planes + 1), as for the FP64 step.
int balance_kchunk_df(long long bxy, int nz, int kmax, int slots) {
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

template <int TX, int TY>
cudaError_t launch3df(const double *A, double *B, int ix, int jx, int kx, const Axis &ax,
                      const Axis &ay, const Axis &az, const Phys &ph, double dt, Ctl *ctl,
                      Box3 box, int kchunk, cudaStream_t s) {
  using T = Tile3D<TX, TY>;
  static std::mutex mu;
  static int slots_of[64] = {};
  int dev = 0, slots = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!slots_of[dev]) {
      e = cudaFuncSetAttribute(k_mlw3d_df<TX, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)T::smem_bytes);
      if (e != cudaSuccess) return e;
      int sms = 0, per_sm = 0;
      if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return e;
      if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mlw3d_df<TX, TY>, T::NT,
                                                             T::smem_bytes)) != cudaSuccess)
        return e;
      slots_of[dev] = sms * (per_sm > 0 ? per_sm : 1);
    }
    slots = slots_of[dev];
  }
  const int bx = (ix - 2 + TX - 1) / TX, by = (jx - 2 + TY - 1) / TY;
  kchunk = balance_kchunk_df((long long)bx * by, kx - 2, kchunk, slots);
  dim3 grid(bx, by, (kx - 2 + kchunk - 1) / kchunk);
  k_mlw3d_df<TX, TY><<<grid, T::NT, T::smem_bytes, s>>>(A, B, ix, jx, kx, ax, ay, az, ph, dt,
                                                       ctl, box, kchunk);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

int mlw3d_df_tile_count() { return 2; }

cudaError_t launch_mlw3d_df(int tile, const double *A, double *B, int ix, int jx, int kx,
                            const Axis &ax, const Axis &ay, const Axis &az, const Phys &ph,
                            double dt, Ctl *ctl, Box3 box, cudaStream_t s) {
  if (ix < 3 || jx < 3 || kx < 3) return cudaErrorInvalidValue;
  // tile 0: 16 x 16 columns, tile 1: 16 x 8 (z chunks of at most 64 planes)
  if (tile == 1)
    return launch3df<16, 8>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl, box, 64, s);
  return launch3df<16, 16>(A, B, ix, jx, kx, ax, ay, az, ph, dt, ctl, box, 64, s);
}

}  // namespace cans
