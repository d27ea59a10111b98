// Discrete adjoint of the 2.5-D mLW step (cans2d/hdmlw/mlw_m3.f:2-377) and of
// the boundary fill, by hand: the transpose of the linearised step, applied to
// an adjoint state lambda (one array per primitive variable), on the device.
//
// Forward step, in the stage form the reverse follows (1-based indices,
// interior = 2..n-1 in both axes, dt frozen):
//   (1) cell values of the input primitives P: conserved U, fluxes FX, FY
//       (mlw_m3.f:107-202);
//   (2) du = -0.25 dt (dxi (FX(i+1)-FX(i-1)) + dyi (FY(j+1)-FY(j-1)))   interior
//       Uh(corner) = avg4(U) - dt dxim/2 (dx FX) - dt dyim/2 (dy FY)  (mlwhalf.f)
//   (3) corner primitives Ph = prim(Uh), corner fluxes GX, GY (:214-310)
//   (4) du -= 0.5 dt (dxi sum_uy (dx GX) + dyi sum_ux (dy GY))         (mlwfull.f)
//   (5) q = qav dxm max(0, |dv| - 1e-4) on faces; du += dt dxi (q dxim dU - ...)
//       for the 8 conserved variables (mlwartv.f, :324-345)
//   (6) P' = prim(U + du) on the interior; other cells keep P (:349-374)
// az is updated by sources of its own and feeds back into nothing, and the
// objective does not read it, so its adjoint is identically zero.
//
// Reverse, given lambda' for P' after the boundary fill (bc_transpose first):
//   k_adj_cells   a' = (dP'/dU')^T lambda' on the interior (= adjoint of du),
//                 plus the cell values U, FX, FY of P for the kernels below
//   k_adj_corners adjoint of GX, GY gathered from the four cells that read each
//                 corner (transpose of (4)), then of Uh through (3)
//   k_adj_gather  adjoint of U, FX, FY of every cell gathered from its corners
//                 (transpose of the predictor), its neighbours (transpose of
//                 the half step and of the viscosity in U), the adjoint of q
//                 on its two faces per axis, then (dU,FX,FY/dP)^T; cells
//                 outside the interior pass lambda' through unchanged.
// Every transpose is a gather: no atomics, deterministic results.
#include <cuda_runtime.h>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "df64.cuh"

namespace cans {

namespace {

constexpr int kT = 128;
// four resident blocks per SM (at most 128 registers a thread): a 258^2
// grid's 520 blocks then fit in one wave of 152 x 4 slots, where three
// blocks per SM (the registers the reverse kernels would otherwise take)
// need two waves, the second nearly empty
constexpr int kMinBlocks = 4;
// primitive slots of the state (mlw_m3 order) and conserved slots
enum { P_RO = 0, P_PR, P_VX, P_VY, P_VZ, P_BX, P_BY, P_BZ, P_AZ };
enum { C_RO = 0, C_EE, C_RX, C_RY, C_RZ, C_BX, C_BY, C_BZ };

struct G2 {
  int ix, jx;
  size_t n;
};

__device__ __forceinline__ bool interior(const G2 &g, int i, int j) {
  return i >= 1 && i <= g.ix - 2 && j >= 1 && j <= g.jx - 2;  // 0-based
}

// The reverse kernels are written once for a number type R: double (FP64
// pipe) or df::DF (double-float on the FP32 pipes, about 2^-46 per
// operation; see df64.cuh).  The gradient is checked to 1e-6 relative, so the
// reverse sweep may run in double-float; the forward steps it linearises
// about are the run's own FP64 steps in either case.  Scratch arrays between
// the kernels hold R values (num_ld / num_st); the states read and the
// adjoint written are doubles (num_in / num_out).
template <class R> struct PhysR {
  R gm1, gm1i, ggm1, pi8i, pi4i, qav;
};
template <class R> __device__ __forceinline__ PhysR<R> phys_r(const Phys &ph) {
  return {num_in<R>(ph.gm1), num_in<R>(ph.gm1i), num_in<R>(ph.ggm1), num_in<R>(ph.pi8i),
          num_in<R>(ph.pi4i), num_in<R>(ph.qav)};
}

// (1): conserved values and fluxes of one primitive state (mlw_m3.f:107-202)
template <class R> struct CellF {
  R U[8], FX[8], FY[8];
};
template <class R>
__device__ __forceinline__ void cell_forward(const R *p, const PhysR<R> &ph, CellF<R> &o) {
  const R ro = p[P_RO], pr = p[P_PR], vx = p[P_VX], vy = p[P_VY], vz = p[P_VZ];
  const R bx = p[P_BX], by = p[P_BY], bz = p[P_BZ];
  const R vv = vx * vx + vy * vy + vz * vz, bb = bx * bx + by * by + bz * bz;
  const R ex = -vy * bz + vz * by, ey = -vz * bx + vx * bz, ez = -vx * by + vy * bx;
  const R ep = pr * ph.ggm1 + 0.5f * ro * vv;
  o.U[C_RO] = ro;
  o.U[C_EE] = pr * ph.gm1i + 0.5f * ro * vv + ph.pi8i * bb;
  o.U[C_RX] = ro * vx;
  o.U[C_RY] = ro * vy;
  o.U[C_RZ] = ro * vz;
  o.U[C_BX] = bx;
  o.U[C_BY] = by;
  o.U[C_BZ] = bz;
  o.FX[C_RO] = ro * vx;
  o.FY[C_RO] = ro * vy;
  o.FX[C_EE] = ep * vx + (bz * ey - by * ez) * ph.pi4i;
  o.FY[C_EE] = ep * vy + (bx * ez - bz * ex) * ph.pi4i;
  o.FX[C_RX] = ro * vx * vx + pr + ph.pi8i * (by * by + bz * bz - bx * bx);
  o.FY[C_RX] = ro * vx * vy - ph.pi4i * bx * by;
  o.FX[C_RY] = ro * vy * vx - ph.pi4i * by * bx;
  o.FY[C_RY] = ro * vy * vy + pr + ph.pi8i * (bx * bx + bz * bz - by * by);
  o.FX[C_RZ] = ro * vz * vx - ph.pi4i * bz * bx;
  o.FY[C_RZ] = ro * vz * vy - ph.pi4i * bz * by;
  o.FX[C_BX] = R(0.0f);
  o.FY[C_BX] = ez;
  o.FX[C_BY] = -ez;
  o.FY[C_BY] = R(0.0f);
  o.FX[C_BZ] = ey;
  o.FY[C_BZ] = -ex;
}

// primitives of a conserved state (mlw_m3.f:214-223, 365-374)
template <class R>
__device__ __forceinline__ void prim_forward(const R *u, const PhysR<R> &ph, R *p) {
  const R ro = u[C_RO];
  const R ri = R(1.0f) / ro;
  const R vx = u[C_RX] * ri, vy = u[C_RY] * ri, vz = u[C_RZ] * ri;
  const R vv = vx * vx + vy * vy + vz * vz;
  const R bb = u[C_BX] * u[C_BX] + u[C_BY] * u[C_BY] + u[C_BZ] * u[C_BZ];
  p[P_RO] = ro;
  p[P_PR] = ph.gm1 * (u[C_EE] - 0.5f * ro * vv - ph.pi8i * bb);
  p[P_VX] = vx;
  p[P_VY] = vy;
  p[P_VZ] = vz;
  p[P_BX] = u[C_BX];
  p[P_BY] = u[C_BY];
  p[P_BZ] = u[C_BZ];
}

// Transpose of (1): given the adjoints aU, aX, aY of U, FX, FY at the point
// p, add (d(U,FX,FY)/dP)^T (aU, aX, aY) to ap.
template <class R>
__device__ __forceinline__ void cell_reverse(const R *p, const PhysR<R> &ph, const R *aU,
                                             const R *aX, const R *aY, R *ap) {
  const R ro = p[P_RO], pr = p[P_PR], vx = p[P_VX], vy = p[P_VY], vz = p[P_VZ];
  const R bx = p[P_BX], by = p[P_BY], bz = p[P_BZ];
  const R vv = vx * vx + vy * vy + vz * vz;
  const R ex = -vy * bz + vz * by, ey = -vz * bx + vx * bz, ez = -vx * by + vy * bx;
  const R ep = pr * ph.ggm1 + 0.5f * ro * vv;
  const R p4 = ph.pi4i, p8 = ph.pi8i;
  R aro(0.0f), apr(0.0f), avx(0.0f), avy(0.0f), avz(0.0f), abx(0.0f), aby(0.0f),
      abz(0.0f);
  R aep(0.0f), aex(0.0f), aey(0.0f), aez(0.0f), avv(0.0f), abb(0.0f);
  // U
  aro += aU[C_RO];
  apr += aU[C_EE] * ph.gm1i;
  aro += aU[C_EE] * 0.5f * vv;
  avv += aU[C_EE] * 0.5f * ro;
  abb += aU[C_EE] * p8;
  aro += aU[C_RX] * vx + aU[C_RY] * vy + aU[C_RZ] * vz;
  avx += aU[C_RX] * ro;
  avy += aU[C_RY] * ro;
  avz += aU[C_RZ] * ro;
  abx += aU[C_BX];
  aby += aU[C_BY];
  abz += aU[C_BZ];
  // FX
  aro += aX[C_RO] * vx;
  avx += aX[C_RO] * ro;
  aep += aX[C_EE] * vx;
  avx += aX[C_EE] * ep;
  abz += aX[C_EE] * p4 * ey;
  aey += aX[C_EE] * p4 * bz;
  aby -= aX[C_EE] * p4 * ez;
  aez -= aX[C_EE] * p4 * by;
  aro += aX[C_RX] * vx * vx;
  avx += aX[C_RX] * 2.0f * ro * vx;
  apr += aX[C_RX];
  aby += aX[C_RX] * p8 * 2.0f * by;
  abz += aX[C_RX] * p8 * 2.0f * bz;
  abx -= aX[C_RX] * p8 * 2.0f * bx;
  aro += aX[C_RY] * vy * vx;
  avy += aX[C_RY] * ro * vx;
  avx += aX[C_RY] * ro * vy;
  aby -= aX[C_RY] * p4 * bx;
  abx -= aX[C_RY] * p4 * by;
  aro += aX[C_RZ] * vz * vx;
  avz += aX[C_RZ] * ro * vx;
  avx += aX[C_RZ] * ro * vz;
  abz -= aX[C_RZ] * p4 * bx;
  abx -= aX[C_RZ] * p4 * bz;
  aez -= aX[C_BY];
  aey += aX[C_BZ];
  // FY
  aro += aY[C_RO] * vy;
  avy += aY[C_RO] * ro;
  aep += aY[C_EE] * vy;
  avy += aY[C_EE] * ep;
  abx += aY[C_EE] * p4 * ez;
  aez += aY[C_EE] * p4 * bx;
  abz -= aY[C_EE] * p4 * ex;
  aex -= aY[C_EE] * p4 * bz;
  aro += aY[C_RX] * vx * vy;
  avx += aY[C_RX] * ro * vy;
  avy += aY[C_RX] * ro * vx;
  abx -= aY[C_RX] * p4 * by;
  aby -= aY[C_RX] * p4 * bx;
  aro += aY[C_RY] * vy * vy;
  avy += aY[C_RY] * 2.0f * ro * vy;
  apr += aY[C_RY];
  abx += aY[C_RY] * p8 * 2.0f * bx;
  abz += aY[C_RY] * p8 * 2.0f * bz;
  aby -= aY[C_RY] * p8 * 2.0f * by;
  aro += aY[C_RZ] * vz * vy;
  avz += aY[C_RZ] * ro * vy;
  avy += aY[C_RZ] * ro * vz;
  abz -= aY[C_RZ] * p4 * by;
  aby -= aY[C_RZ] * p4 * bz;
  aez += aY[C_BX];
  aex -= aY[C_BZ];
  // ep, E, |v|^2, |B|^2
  apr += aep * ph.ggm1;
  aro += aep * 0.5f * vv;
  avv += aep * 0.5f * ro;
  avy -= aex * bz;
  abz -= aex * vy;
  avz += aex * by;
  aby += aex * vz;
  avz -= aey * bx;
  abx -= aey * vz;
  avx += aey * bz;
  abz += aey * vx;
  avx -= aez * by;
  aby -= aez * vx;
  avy += aez * bx;
  abx += aez * vy;
  avx += 2.0f * vx * avv;
  avy += 2.0f * vy * avv;
  avz += 2.0f * vz * avv;
  abx += 2.0f * bx * abb;
  aby += 2.0f * by * abb;
  abz += 2.0f * bz * abb;
  ap[P_RO] += aro;
  ap[P_PR] += apr;
  ap[P_VX] += avx;
  ap[P_VY] += avy;
  ap[P_VZ] += avz;
  ap[P_BX] += abx;
  ap[P_BY] += aby;
  ap[P_BZ] += abz;
}

// Transpose of prim_forward at the point whose primitives are p: given ap,
// return au = (dP/dU)^T ap.
template <class R>
__device__ __forceinline__ void prim_reverse(const R *p, const PhysR<R> &ph, const R *ap,
                                             R *au) {
  const R ro = p[P_RO], vx = p[P_VX], vy = p[P_VY], vz = p[P_VZ];
  const R vv = vx * vx + vy * vy + vz * vz;
  const R apr = ap[P_PR];
  const R avv = -ph.gm1 * 0.5f * ro * apr;
  const R abb = -ph.gm1 * ph.pi8i * apr;
  const R ri = R(1.0f) / ro;
  const R avx = ap[P_VX] + 2.0f * vx * avv, avy = ap[P_VY] + 2.0f * vy * avv,
          avz = ap[P_VZ] + 2.0f * vz * avv;
  au[C_EE] = ph.gm1 * apr;
  au[C_RX] = avx * ri;
  au[C_RY] = avy * ri;
  au[C_RZ] = avz * ri;
  au[C_RO] = ap[P_RO] - ph.gm1 * 0.5f * vv * apr - (avx * vx + avy * vy + avz * vz) * ri;
  au[C_BX] = ap[P_BX] + 2.0f * p[P_BX] * abb;
  au[C_BY] = ap[P_BY] + 2.0f * p[P_BY] * abb;
  au[C_BZ] = ap[P_BZ] + 2.0f * p[P_BZ] * abb;
}

template <class R>
__device__ __forceinline__ void load_prim(const double *S, size_t n, size_t c, R *p) {
#pragma unroll
  for (int v = 0; v < 8; v++) p[v] = num_in<R>(S[v * n + c]);
}

// a' on the interior, the cell values U, FX, FY of P everywhere
template <class R>
__global__ void __launch_bounds__(kT, kMinBlocks)
    k_adj_cells(const double *__restrict__ P, const double *__restrict__ Rw,
                const double *__restrict__ lam, double *__restrict__ A1,
                double *__restrict__ CU, G2 g, Phys ph_) {
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= g.n) return;
  const PhysR<R> ph = phys_r<R>(ph_);
  const int i = (int)(c % g.ix), j = (int)(c / g.ix);
  R p[8];
  load_prim(P, g.n, c, p);
  CellF<R> f;
  cell_forward(p, ph, f);
#pragma unroll
  for (int v = 0; v < 8; v++) {
    num_st(CU + v * g.n + c, f.U[v]);
    num_st(CU + (8 + v) * g.n + c, f.FX[v]);
    num_st(CU + (16 + v) * g.n + c, f.FY[v]);
  }
  R au[8];
#pragma unroll
  for (int v = 0; v < 8; v++) au[v] = R(0.0f);
  if (interior(g, i, j)) {
    R r[8], ap[8];
    load_prim(Rw, g.n, c, r);
    load_prim(lam, g.n, c, ap);
    prim_reverse(r, ph, ap, au);
  }
#pragma unroll
  for (int v = 0; v < 8; v++) num_st(A1 + v * g.n + c, au[v]);
}

// corners (p+1/2, q+1/2), p = 0..ix-2, q = 0..jx-2 (0-based), stored at p+q*ix
template <class R>
__global__ void __launch_bounds__(kT, kMinBlocks)
    k_adj_corners(const double *__restrict__ CU, const double *__restrict__ A1,
                  double *__restrict__ A2, G2 g, Axis ax, Axis ay, Phys ph_,
                  double dt_) {
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= g.n) return;
  const PhysR<R> ph = phys_r<R>(ph_);
  const R dt = num_in<R>(dt_);
  const int p = (int)(c % g.ix), q = (int)(c / g.ix);
  R out[8];
#pragma unroll
  for (int v = 0; v < 8; v++) out[v] = R(0.0f);
  if (p <= g.ix - 2 && q <= g.jx - 2) {
    const size_t c00 = c, c10 = c + 1, c01 = c + g.ix, c11 = c + g.ix + 1;
    // forward corner state (mlwhalf.f part 2)
    const R hdxim = 0.5f * num_in<R>(ax.dim[p]), hdyim = 0.5f * num_in<R>(ay.dim[q]);
    R uh[8];
#pragma unroll
    for (int v = 0; v < 8; v++) {
      const double *U = CU + v * g.n, *FX = CU + (8 + v) * g.n, *FY = CU + (16 + v) * g.n;
      const R avg = 0.25f * (num_ld<R>(U + c10) + num_ld<R>(U + c00) + num_ld<R>(U + c11) +
                             num_ld<R>(U + c01));
      const R dfdx = hdxim * (num_ld<R>(FX + c10) - num_ld<R>(FX + c00) +
                              num_ld<R>(FX + c11) - num_ld<R>(FX + c01));
      const R dfdy = hdyim * (num_ld<R>(FY + c01) - num_ld<R>(FY + c00) +
                              num_ld<R>(FY + c11) - num_ld<R>(FY + c10));
      uh[v] = avg - dt * dfdx - dt * dfdy;
    }
    R ph8[8];
    prim_forward(uh, ph, ph8);
    // adjoint of GX, GY at this corner: the cells (p,q), (p+1,q), (p,q+1),
    // (p+1,q+1) that read it in mlwfull (0-based cell indices)
    const bool i00 = interior(g, p, q), i10 = interior(g, p + 1, q),
               i01 = interior(g, p, q + 1), i11 = interior(g, p + 1, q + 1);
    const R hx0 = 0.5f * dt * num_in<R>(ax.di[p]), hx1 = 0.5f * dt * num_in<R>(ax.di[p + 1]);
    const R hy0 = 0.5f * dt * num_in<R>(ay.di[q]), hy1 = 0.5f * dt * num_in<R>(ay.di[q + 1]);
    const R uy1q = num_in<R>(ay.u1[q]), uy0q1 = num_in<R>(ay.u0[q + 1]);
    const R ux1p = num_in<R>(ax.u1[p]), ux0p1 = num_in<R>(ax.u0[p + 1]);
    R aX[8], aY[8];
#pragma unroll
    for (int v = 0; v < 8; v++) {
      const double *a = A1 + v * g.n;
      const R l00 = i00 ? num_ld<R>(a + c00) : R(0.0f), l10 = i10 ? num_ld<R>(a + c10) : R(0.0f);
      const R l01 = i01 ? num_ld<R>(a + c01) : R(0.0f), l11 = i11 ? num_ld<R>(a + c11) : R(0.0f);
      aX[v] = -hx0 * uy1q * l00 + hx1 * uy1q * l10 - hx0 * uy0q1 * l01 + hx1 * uy0q1 * l11;
      aY[v] = -hy0 * ux1p * l00 - hy0 * ux0p1 * l10 + hy1 * ux1p * l01 + hy1 * ux0p1 * l11;
    }
    R aP[8], zero8[8];
#pragma unroll
    for (int v = 0; v < 8; v++) {
      aP[v] = R(0.0f);
      zero8[v] = R(0.0f);
    }
    cell_reverse(ph8, ph, zero8, aX, aY, aP);
    prim_reverse(ph8, ph, aP, out);
  }
#pragma unroll
  for (int v = 0; v < 8; v++) num_st(A2 + v * g.n + c, out[v]);
}

// adjoint of P for every cell
template <class R>
__global__ void __launch_bounds__(kT, kMinBlocks)
    k_adj_gather(const double *__restrict__ P, const double *__restrict__ CU,
                 const double *__restrict__ A1, const double *__restrict__ A2,
                 const double *__restrict__ lam, double *__restrict__ out, G2 g,
                 Axis ax, Axis ay, Phys ph_, double dt_) {
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= g.n) return;
  const PhysR<R> ph = phys_r<R>(ph_);
  const R dt = num_in<R>(dt_);
  const int i = (int)(c % g.ix), j = (int)(c / g.ix);
  const size_t n = g.n, sx = 1, sy = (size_t)g.ix;
  R p[8];
  load_prim(P, n, c, p);
  const bool in_c = interior(g, i, j);
  const bool in_xm = interior(g, i - 1, j), in_xp = interior(g, i + 1, j);
  const bool in_ym = interior(g, i, j - 1), in_yp = interior(g, i, j + 1);
  // corners around the cell: (i-1+1/2, j-1+1/2) .. (i+1/2, j+1/2)
  const bool k_mm = i >= 1 && j >= 1, k_pm = i <= g.ix - 2 && j >= 1;
  const bool k_mp = i >= 1 && j <= g.jx - 2, k_pp = i <= g.ix - 2 && j <= g.jx - 2;
  // metrics the coefficients below read
  const R zero(0.0f);
  const R dim_xm = i >= 1 ? num_in<R>(ax.dim[i - 1]) : zero, dim_x = num_in<R>(ax.dim[i]);
  const R dim_ym = j >= 1 ? num_in<R>(ay.dim[j - 1]) : zero, dim_y = num_in<R>(ay.dim[j]);
  const R di_x = num_in<R>(ax.di[i]), di_y = num_in<R>(ay.di[j]);
  const R di_xm = i >= 1 ? num_in<R>(ax.di[i - 1]) : zero;
  const R di_xp = i <= g.ix - 2 ? num_in<R>(ax.di[i + 1]) : zero;
  const R di_ym = j >= 1 ? num_in<R>(ay.di[j - 1]) : zero;
  const R di_yp = j <= g.jx - 2 ? num_in<R>(ay.di[j + 1]) : zero;
  // artificial-viscosity coefficients of the four faces (mlw_m3.f:324-334)
  // and their derivatives in dv: q = qav dxm max(0, |dv| - eps)
  const double *VX = P + P_VX * n, *VY = P + P_VY * n;
  R qxm = zero, qxp = zero, qym = zero, qyp = zero, gxm = zero, gxp = zero, gym = zero,
    gyp = zero;
  const float eps = 1.0e-4f;  // the real*4 literal of the reference
  if (i >= 1) {
    const R d = num_in<R>(VX[c]) - num_in<R>(VX[c - sx]);
    const R e = fabs(d) - eps;
    const R qd = ph.qav * num_in<R>(ax.dm[i - 1]);
    qxm = e > 0.0f ? qd * e : zero;
    gxm = e > 0.0f ? (d > 0.0f ? qd : -qd) : zero;
  }
  if (i <= g.ix - 2) {
    const R d = num_in<R>(VX[c + sx]) - num_in<R>(VX[c]);
    const R e = fabs(d) - eps;
    const R qd = ph.qav * num_in<R>(ax.dm[i]);
    qxp = e > 0.0f ? qd * e : zero;
    gxp = e > 0.0f ? (d > 0.0f ? qd : -qd) : zero;
  }
  if (j >= 1) {
    const R d = num_in<R>(VY[c]) - num_in<R>(VY[c - sy]);
    const R e = fabs(d) - eps;
    const R qd = ph.qav * num_in<R>(ay.dm[j - 1]);
    qym = e > 0.0f ? qd * e : zero;
    gym = e > 0.0f ? (d > 0.0f ? qd : -qd) : zero;
  }
  if (j <= g.jx - 2) {
    const R d = num_in<R>(VY[c + sy]) - num_in<R>(VY[c]);
    const R e = fabs(d) - eps;
    const R qd = ph.qav * num_in<R>(ay.dm[j]);
    qyp = e > 0.0f ? qd * e : zero;
    gyp = e > 0.0f ? (d > 0.0f ? qd : -qd) : zero;
  }
  const bool aqxm_on = qxm != 0.0f, aqxp_on = qxp != 0.0f;
  const bool aqym_on = qym != 0.0f, aqyp_on = qyp != 0.0f;
  // coefficients shared by the 8 variables: viscosity in U (mlwartv.f),
  // half-step differences (mlwhalf.f part 1), corner predictor (part 2),
  // viscosity in q; zero where the reading cell is not updated
  const R cxm = in_xm ? dt * di_xm * qxm * dim_xm : zero;
  const R cxp = in_xp ? dt * di_xp * qxp * dim_x : zero;
  const R cym = in_ym ? dt * di_ym * qym * dim_ym : zero;
  const R cyp = in_yp ? dt * di_yp * qyp * dim_y : zero;
  const R c0 = in_c ? dt * (di_x * (qxp * dim_x + qxm * dim_xm) +
                            di_y * (qyp * dim_y + qym * dim_ym))
                    : zero;
  const bool av = aqxm_on | aqxp_on | aqym_on | aqyp_on;
  const R hxm = i >= 1 ? 0.25f * dt * di_xm : zero;
  const R hxp = i <= g.ix - 2 ? 0.25f * dt * di_xp : zero;
  const R hym = j >= 1 ? 0.25f * dt * di_ym : zero;
  const R hyp = j <= g.jx - 2 ? 0.25f * dt * di_yp : zero;
  const R pxm = i >= 1 ? 0.5f * dt * dim_xm : zero;
  const R pxp = i <= g.ix - 2 ? 0.5f * dt * dim_x : zero;
  const R pym = j >= 1 ? 0.5f * dt * dim_ym : zero;
  const R pyp = j <= g.jx - 2 ? 0.5f * dt * dim_y : zero;
  // d(du(o))/dq(face) per unit dU: the cell below the face gains, the cell
  // above loses (in_* already folded in)
  const R wxm_a = in_xm ? dt * dim_xm * di_xm : zero;
  const R wxm_b = (in_c && i >= 1) ? dt * dim_xm * di_x : zero;
  const R wxp_a = in_c ? dt * dim_x * di_x : zero;
  const R wxp_b = in_xp ? dt * dim_x * di_xp : zero;
  const R wym_a = in_ym ? dt * dim_ym * di_ym : zero;
  const R wym_b = (in_c && j >= 1) ? dt * dim_ym * di_y : zero;
  const R wyp_a = in_c ? dt * dim_y * di_y : zero;
  const R wyp_b = in_yp ? dt * dim_y * di_yp : zero;
  R aU[8], aX[8], aY[8];
  R aqxm = zero, aqxp = zero, aqym = zero, aqyp = zero;
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const double *a = A1 + v * n, *h = A2 + v * n;
    const R l0 = in_c ? num_ld<R>(a + c) : zero;
    const R lxm = in_xm ? num_ld<R>(a + c - sx) : zero, lxp = in_xp ? num_ld<R>(a + c + sx) : zero;
    const R lym = in_ym ? num_ld<R>(a + c - sy) : zero, lyp = in_yp ? num_ld<R>(a + c + sy) : zero;
    const R hmm = k_mm ? num_ld<R>(h + c - sx - sy) : zero, hpm = k_pm ? num_ld<R>(h + c - sy) : zero;
    const R hmp = k_mp ? num_ld<R>(h + c - sx) : zero, hpp = k_pp ? num_ld<R>(h + c) : zero;
    const R ylo = hmm + hpm, yhi = hmp + hpp;  // corners below / above
    // U' = U + du on the interior; 0.25 of each surrounding corner
    R au = fma(R(0.25f), ylo + yhi, l0);
    if (av) au += cxm * lxm + cxp * lxp + cym * lym + cyp * lyp - c0 * l0;
    aU[v] = au;
    aX[v] = hxp * lxp - hxm * lxm + pxp * (hpm + hpp) - pxm * (hmm + hmp);
    aY[v] = hyp * lyp - hym * lym + pyp * yhi - pym * ylo;
    if (av) {
      const double *U = CU + v * n;
      const R u0 = num_ld<R>(U + c);
      if (aqxm_on) aqxm += (u0 - num_ld<R>(U + c - sx)) * (wxm_a * lxm - wxm_b * l0);
      if (aqxp_on) aqxp += (num_ld<R>(U + c + sx) - u0) * (wxp_a * l0 - wxp_b * lxp);
      if (aqym_on) aqym += (u0 - num_ld<R>(U + c - sy)) * (wym_a * lym - wym_b * l0);
      if (aqyp_on) aqyp += (num_ld<R>(U + c + sy) - u0) * (wyp_a * l0 - wyp_b * lyp);
    }
  }
  R ap[8];
#pragma unroll
  for (int v = 0; v < 8; v++) ap[v] = zero;
  cell_reverse(p, ph, aU, aX, aY, ap);
  // q(face) = qav dxm max(0, |v(+) - v(-)| - eps): the cell is (+) of the
  // lower face and (-) of the upper face
  ap[P_VX] += aqxm * gxm - aqxp * gxp;
  ap[P_VY] += aqym * gym - aqyp * gyp;
  // cells the step does not update pass the adjoint through
  if (!in_c) {
#pragma unroll
    for (int v = 0; v < 8; v++) ap[v] += num_in<R>(lam[v * n + c]);
  }
#pragma unroll
  for (int v = 0; v < 8; v++) out[v * n + c] = num_out(ap[v]);
  out[P_AZ * n + c] = 0.0;
}

// Transpose of the boundary program of one axis on one line, over all
// variables: the rules of bd_line (bc_line.cuh) in reverse order, each
// assignment dst = s*src turned into a(src) += s*a(dst), a(dst) = 0.
__device__ void bd_line_t(int kind, int mbnd, int m, double *q, int n, size_t st,
                          const double *dxm) {
#define QL(l) q[(size_t)((l)-1) * st]
  if (kind == BD_PER) {
    const int b0 = 1 + m, b1 = n - m;
    if (mbnd == 0)
      for (int i = m; i >= 1; i--) { QL(b1 + 1 - i) += QL(b0 - i); QL(b0 - i) = 0.0; }
    else
      for (int i = m; i >= 1; i--) { QL(b0 - 1 + i) += QL(b1 + i); QL(b1 + i) = 0.0; }
    return;
  }
  if (mbnd == 0) {
    const int b = 1 + m;
    switch (kind) {
      case BD_SPP: for (int i = m; i >= 1; i--) { QL(b - 1 + i) += QL(b - i); QL(b - i) = 0.0; } break;
      case BD_SPN: for (int i = m; i >= 1; i--) { QL(b - 1 + i) -= QL(b - i); QL(b - i) = 0.0; } break;
      case BD_SMP: for (int i = m; i >= 1; i--) { QL(b + i) += QL(b - i); QL(b - i) = 0.0; } break;
      case BD_SMN:
        QL(b) = 0.0;
        for (int i = m; i >= 1; i--) { QL(b + i) -= QL(b - i); QL(b - i) = 0.0; }
        break;
      case BD_FRE: for (int i = m; i >= 1; i--) { QL(b) += QL(b - i); QL(b - i) = 0.0; } break;
      case BD_CNS: for (int i = m; i >= 1; i--) QL(b - i) = 0.0; break;
      case BD_FRD: {
        double adq = 0.0;  // q(b-i) = q(b-i+1) - dqq dxm(b-i), dqq = (q(b+1)-q(b))/dxm(b)
        for (int i = m; i >= 1; i--) {
          QL(b - i + 1) += QL(b - i);
          adq -= QL(b - i) * dxm[b - i - 1];
          QL(b - i) = 0.0;
        }
        QL(b + 1) += adq / dxm[b - 1];
        QL(b) -= adq / dxm[b - 1];
        break;
      }
      default: break;
    }
  } else {
    const int b = n - m;
    switch (kind) {
      case BD_SPP: for (int i = m; i >= 1; i--) { QL(b + 1 - i) += QL(b + i); QL(b + i) = 0.0; } break;
      case BD_SPN: for (int i = m; i >= 1; i--) { QL(b + 1 - i) -= QL(b + i); QL(b + i) = 0.0; } break;
      case BD_SMP: for (int i = m; i >= 1; i--) { QL(b - i) += QL(b + i); QL(b + i) = 0.0; } break;
      case BD_SMN:
        QL(b) = 0.0;
        for (int i = m; i >= 1; i--) { QL(b - i) -= QL(b + i); QL(b + i) = 0.0; }
        break;
      case BD_FRE: for (int i = m; i >= 1; i--) { QL(b) += QL(b + i); QL(b + i) = 0.0; } break;
      case BD_CNS: for (int i = m; i >= 1; i--) QL(b + i) = 0.0; break;
      case BD_FRD: {
        double adq = 0.0;  // q(b+i) = q(b+i-1) + dqq dxm(b+i-1), dqq = (q(b)-q(b-1))/dxm(b-1)
        for (int i = m; i >= 1; i--) {
          QL(b + i - 1) += QL(b + i);
          adq += QL(b + i) * dxm[b + i - 2];
          QL(b + i) = 0.0;
        }
        QL(b) += adq / dxm[b - 2];
        QL(b - 1) -= adq / dxm[b - 2];
        break;
      }
      default: break;
    }
  }
#undef QL
}

__global__ void k_bc2d_t(int nvar, double *L, int ix, int jx, int axis, BcTable bc,
                         const double *dxm) {
  const int n = axis == 0 ? ix : jx;
  const size_t st = axis == 0 ? 1 : (size_t)ix;
  const long long nlines = axis == 0 ? jx : ix;
  const size_t nall = (size_t)ix * jx;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nlines * nvar;
       t += (long long)gridDim.x * blockDim.x) {
    const int v = (int)(t / nlines);
    const long long line = t % nlines;
    double *q = L + (size_t)v * nall + (axis == 0 ? (size_t)line * ix : (size_t)line);
    const int klo = bc.kind[v][2 * axis], khi = bc.kind[v][2 * axis + 1];
    // the forward applies the lower then the upper rule: reverse order here
    if (khi >= 0) bd_line_t(khi, 1, bc.margin, q, n, st, dxm);
    if (klo >= 0) bd_line_t(klo, 0, bc.margin, q, n, st, dxm);
  }
}

// Error-free sum of two doubles (Knuth's TwoSum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}
// (s, c) += (t, d): a compensated partial sum, the rounding errors of every
// addition carried in c (the cascaded summation of Ogita, Rump and Oishi,
// "Accurate sum and dot product", 2005), so that J is the exact sum of its
// terms to about one rounding -- a finite difference of J then sees the
// state's rounding, not that of a 65k-term sum.
__device__ __forceinline__ void comp_add(double &s, double &c, double t, double d) {
  double e;
  two_sum(s, t, s, e);
  c = __dadd_rn(c, __dadd_rn(d, e));
}

// J = sum over the interior of (bx^2+by^2+bz^2)/(8 pi) dx dy (compensated
// block partial sums, reduced in a fixed order by k_sum_final) and its
// gradient
__global__ void __launch_bounds__(256)
    k_objective(const double *__restrict__ P, double *__restrict__ lam,
                double *__restrict__ part, G2 g, Axis ax, Axis ay, Phys ph) {
  __shared__ double red[2][256];
  double s = 0.0, c = 0.0;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < g.n;
       k += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(k % g.ix), j = (int)(k / g.ix);
    const double bx = P[P_BX * g.n + k], by = P[P_BY * g.n + k], bz = P[P_BZ * g.n + k];
    const bool in = interior(g, i, j);
    const double w = in ? ax.d[i] * ay.d[j] : 0.0;
    comp_add(s, c, (bx * bx + by * by + bz * bz) * ph.pi8i * w, 0.0);
    if (lam) {
#pragma unroll
      for (int v = 0; v < 9; v++) lam[v * g.n + k] = 0.0;
      lam[P_BX * g.n + k] = 2.0 * ph.pi8i * w * bx;
      lam[P_BY * g.n + k] = 2.0 * ph.pi8i * w * by;
      lam[P_BZ * g.n + k] = 2.0 * ph.pi8i * w * bz;
    }
  }
  red[0][threadIdx.x] = s;
  red[1][threadIdx.x] = c;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      double a = red[0][threadIdx.x], b = red[1][threadIdx.x];
      comp_add(a, b, red[0][threadIdx.x + o], red[1][threadIdx.x + o]);
      red[0][threadIdx.x] = a;
      red[1][threadIdx.x] = b;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = red[0][0];
    part[2 * blockIdx.x + 1] = red[1][0];
  }
}

__global__ void k_sum_final(const double *part, int nb, double *out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0, c = 0.0;
    for (int b = 0; b < nb; b++) comp_add(s, c, part[2 * b], part[2 * b + 1]);
    *out = __dadd_rn(s, c);
  }
}

}  // namespace

size_t adj2d_scratch_doubles(size_t ncells) { return 40 * ncells + 1024; }

cudaError_t launch_adj2d_step(const double *P, const double *R, const double *lam_in,
                              double *lam_out, double *scratch, int ix, int jx,
                              const Axis &ax, const Axis &ay, const Phys &ph,
                              double dt, bool df, cudaStream_t s) {
  G2 g{ix, jx, (size_t)ix * jx};
  double *A1 = scratch, *A2 = scratch + 8 * g.n, *CU = scratch + 16 * g.n;
  const unsigned blocks = (unsigned)((g.n + kT - 1) / kT);
  if (df) {
    k_adj_cells<df::DF><<<blocks, kT, 0, s>>>(P, R, lam_in, A1, CU, g, ph);
    k_adj_corners<df::DF><<<blocks, kT, 0, s>>>(CU, A1, A2, g, ax, ay, ph, dt);
    k_adj_gather<df::DF><<<blocks, kT, 0, s>>>(P, CU, A1, A2, lam_in, lam_out, g, ax, ay, ph,
                                               dt);
  } else {
    k_adj_cells<double><<<blocks, kT, 0, s>>>(P, R, lam_in, A1, CU, g, ph);
    k_adj_corners<double><<<blocks, kT, 0, s>>>(CU, A1, A2, g, ax, ay, ph, dt);
    k_adj_gather<double><<<blocks, kT, 0, s>>>(P, CU, A1, A2, lam_in, lam_out, g, ax, ay, ph,
                                               dt);
  }
  count_launch(3);
  return cudaGetLastError();
}

cudaError_t launch_bc2d_transpose(int nvar, double *lam, int ix, int jx,
                                  const Axis &ax, const Axis &ay, const BcTable &bc,
                                  cudaStream_t s) {
  // the forward fills x, then y: transpose y first
  for (int axis = 1; axis >= 0; axis--) {
    const long long total = (long long)(axis == 0 ? jx : ix) * nvar;
    int blocks = (int)((total + 127) / 128);
    if (blocks < 1) blocks = 1;
    k_bc2d_t<<<blocks, 128, 0, s>>>(nvar, lam, ix, jx, axis, bc, axis == 0 ? ax.dm : ay.dm);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Raw output of a step rebuilt from the two filled states around it: the
// step writes every cell but the outer layer, which it copies from its input,
// and a boundary program of margin 1 without bdsmn* rules then rewrites only
// that layer.  So R = P_next inside, P_cur on the outer layer.
__global__ void k_adj_merge(const double *__restrict__ P_next,
                            const double *__restrict__ P_cur, double *__restrict__ R,
                            int nvar, int ix, int jx) {
  const size_t n = (size_t)ix * jx;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n * nvar;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t c = t % n;
    const int i = (int)(c % ix), j = (int)(c / ix);
    const bool edge = i == 0 || i == ix - 1 || j == 0 || j == jx - 1;
    R[t] = edge ? P_cur[t] : P_next[t];
  }
}

cudaError_t launch_adj2d_merge(const double *P_next, const double *P_cur, double *R,
                               int nvar, int ix, int jx, cudaStream_t s) {
  const size_t total = (size_t)ix * jx * nvar;
  size_t blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_adj_merge<<<(unsigned)blocks, 256, 0, s>>>(P_next, P_cur, R, nvar, ix, jx);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_adj2d_objective(const double *P, double *lam, double *J,
                                   double *scratch, int ix, int jx, const Axis &ax,
                                   const Axis &ay, const Phys &ph, cudaStream_t s) {
  G2 g{ix, jx, (size_t)ix * jx};
  const int nb = 256;
  double *part = scratch;
  k_objective<<<nb, 256, 0, s>>>(P, lam, part, g, ax, ay, ph);
  k_sum_final<<<1, 32, 0, s>>>(part, nb, J);
  count_launch(2);
  return cudaGetLastError();
}

}  // namespace cans
