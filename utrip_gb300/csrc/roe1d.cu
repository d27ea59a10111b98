// 1-D Roe-MUSCL step (sm_103a, FP64): cans1d/hdroe/roe_m.f:2-136 with its
// two-component Roe flux cans1d/hdroe/roeflux_m.f:2-245 and the minmod
// reconstruction cans1d/hdroe/tvdminmod.f:2-43, as four kernels over one
// thread per face or cell:
//
//   k_r1_flux1  first-order fluxes of the faces 1..ix-1 (roe_m.f:31-46)
//   k_r1_half   dt/2 update of the cells 2..ix-1 and their primitives
//               (roe_m.f:48-65)
//   k_r1_flux2  minmod states of the half-step primitives and the fluxes of
//               the faces 2..ix-2 (roe_m.f:66-73)
//   k_r1_full   dt update and primitives of the cells 3..ix-2, copy of the
//               others (roe_m.f:75-89)
//
// bx is a fixed profile: the faces take bxm on both sides (roe_m.f:35,41),
// the cells bx in the energy.  As in the 2-D and 3-D steps, the half-step
// primitives the reference leaves unset on the end cells (1 and ix) hold the
// input primitives; only the cells 3 and ix-2, boundary cells at margin 3
// (md_mhdshktb/hdroe/main.f:5), depend on them.
//
// The flux is written once, in the reference's order of operations, for
// both arithmetic policies: the exact policy rounds every operation as the
// Fortran does, the fast policy lets the compiler contract.  A 1-D grid of
// ~10^3 cells is launch-bound, not FP64-bound.
#include <cuda_runtime.h>

#include <cmath>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "roe_flux.cuh"

namespace cans {

namespace {

constexpr int kR1Threads = 128;
// primitive / conserved slots: ro pr vx vy by / ro ee rx ry by
enum { Q_RO = 0, Q_PR = 1, Q_VX = 2, Q_VY = 3, Q_BY = 4, NQ = 5 };

// roeflux_m.f:15-236 for one face.  L, R: (ro, pr, vx, vy, bx, by) of the two
// sides; f: (fro, fee, frx, fry, fby).
template <bool E>
__device__ __forceinline__ void roe_flux1d(const RoeK &K, const double *L,
                                           const double *R, double *f) {
  using T = F<E>;
  const T gm(K.gm), gm1(K.gm1), gm2(K.gm2), pi4(K.pi4), pi4i(K.pi4i), pi8i(K.pi8i);
  const T one(1.0), half(0.5), zero(0.0);
  const T rhol(L[0]), prl(L[1]), vxl(L[2]), vyl(L[3]), byl(L[5]);
  const T rhor(R[0]), prr(R[1]), vxr(R[2]), vyr(R[3]), bxr(R[4]), byr(R[5]);
  const T bxl(L[4]);
  // roe's averages (:30-40)
  const T sr0 = fsqrt(rhol), sr1 = fsqrt(rhor);
  const T sri = one / (sr0 + sr1);
  const T rhobar = sr0 * sr1;
  const T vxbar = (sr0 * vxl + sr1 * vxr) * sri;
  const T vybar = (sr0 * vyl + sr1 * vyr) * sri;
  const T bxbar = (sr0 * bxr + sr1 * bxl) * sri;
  const T bybar = (sr0 * byr + sr1 * byl) * sri;
  const T hl = half * (vxl * vxl + vyl * vyl) + gm * prl / (gm1 * rhol) +
               (bxbar * bxbar + byl * byl) / (pi4 * rhol);
  const T hr = half * (vxr * vxr + vyr * vyr) + gm * prr / (gm1 * rhor) +
               (bxbar * bxbar + byr * byr) / (pi4 * rhor);
  const T hbar = (sr0 * hl + sr1 * hr) * sri;
  const T byave = (byl + byr) / T(2.0);
  const T dby = byr - byl;
  const T delb2 = T(K.gm21) * (dby * dby) * (sri * sri) * pi8i;
  const T v2bar = vxbar * vxbar + vybar * vybar;
  const T b2bar = bxbar * bxbar + bybar * bybar;
  const T cs2 = gm1 * (hbar - half * v2bar - delb2 - b2bar * pi4i / rhobar);
  const T astar2 = gm1 * (hbar - half * v2bar - delb2) - gm2 * b2bar * pi4i / rhobar;
  const T ca2 = bxbar * bxbar / (pi4 * rhobar);
  const T cbr2 = (bybar * bybar) * pi4i / rhobar;
  const T dca = cs2 - ca2;
  const T cfast2 = half * (astar2 + fsqrt(cbr2 * (astar2 + cs2 + ca2) + dca * dca));
  const T cslow2 = cs2 * ca2 / cfast2;
  const T cfast = fsqrt(cfast2), cslow = fsqrt(cslow2), ca = fsqrt(ca2), cs = fsqrt(cs2);
  // eigenvector normalisations (:49-65)
  const T sgr = bybar * bybar - T(1.0e-12);
  const T sp = half + fsign_(half, sgr);
  const T sqh(K.sqh);
  const T betay = sp * bybar * fsqrt(one / (bybar * bybar + one - sp)) + sqh * (one - sp);
  const T betaz = sqh * (one - sp);
  const T sgr2 = (bybar * bybar) / (pi4 * rhobar) + fabs_(ca2 - cs2) - T(1.0e-12);
  const T sp2 = half + fsign_(half, sgr2);
  const T cfca = fmax_(zero, cfast2 - ca2);
  const T cfcs = fmax_(zero, cfast2 - cslow2);
  const T cfa = fmax_(zero, cfast2 - cs2);
  const T alphf = sp2 * fsqrt(cfca / (cfcs + one - sp2)) + one - sp2;
  const T alphs = sp2 * fsqrt(cfa / (cfcs + one - sp2));
  const T sgnbx = fsign_(one, bxbar);
  // eigenvalues with the entropy floor (:67-74)
  const T dvx = vxr - vxl;
  const T eeps = (dvx + fabs_(dvx)) * T(2.5e-1);
  const T elpf = -fmax_(fabs_(vxbar + cfast), eeps);
  const T elmf = -fmax_(fabs_(vxbar - cfast), eeps);
  const T elps = -fmax_(fabs_(vxbar + cslow), eeps);
  const T elms = -fmax_(fabs_(vxbar - cslow), eeps);
  const T elpa = -fmax_(fabs_(vxbar + ca), eeps);
  const T elma = -fmax_(fabs_(vxbar - ca), eeps);
  const T elze = -fmax_(fabs_(vxbar), eeps);
  // wave strengths (:75-103)
  const T drho = rhor - rhol;
  const T du21 = rhobar * (vxr - vxl);
  const T du31 = rhobar * (vyr - vyl);
  const T du41 = zero, du5 = zero;
  const T du6 = byr - byl;
  const T t1 = betay * du6 + betaz * du5;
  const T t2 = (prr - prl + (byave * du6) * pi4i + gm2 * (bybar * du6) * pi4i) / gm1;
  const T t3 = betaz * du6 - betay * du5;
  const T s1 = du21;
  const T s2 = betay * du31 + betaz * du41;
  const T s3 = betaz * du31 - betay * du41;
  const T sq4r = fsqrt(pi4 / rhobar);
  const T p11 = alphs * cfast * sq4r;
  const T p12 = -(alphf * cs2 / cfast * sq4r);
  const T cg = cs2 * gm2 / gm1;
  const T p21 = alphf * (cfast2 - cg);
  const T p22 = alphs * (cslow2 - cg);
  const T q11 = alphf * cfast;
  const T q12 = alphs * cslow;
  const T q21 = -(alphs * ca * sgnbx);
  const T q22 = alphf * cs * sgnbx;
  const T detp = p11 * p22 - p12 * p21;
  const T detq = q11 * q22 - q12 * q21;
  const T ap = (p22 * t1 - p12 * t2) / detp, aq = (q22 * s1 - q12 * s2) / detq;
  const T bp = (-(p21 * t1) + p11 * t2) / detp, bq = (-(q21 * s1) + q11 * s2) / detq;
  const T wpf = half * (ap + aq), wmf = half * (ap - aq);
  const T wps = half * (bp + bq), wms = half * (bp - bq);
  const T sra = fsqrt(rhobar * pi4i);
  const T wpa = half * (sra * t3 - sgnbx * s3);
  const T wma = half * (sra * t3 + sgnbx * s3);
  const T wze = drho - alphf * (wpf + wmf) - alphs * (wps + wms);
  // physical fluxes of the two sides (:104-115)
  const T fluxlro = rhol * vxl;
  const T fluxlrx = rhol * vxl * vxl + prl + (-(bxbar * bxbar) + byl * byl) * pi8i;
  const T fluxlry = rhol * vxl * vyl - bxbar * byl * pi4i;
  const T fluxlby = vxl * byl - vyl * bxbar;
  const T fluxlee = rhol * vxl * hl - bxbar * (bxbar * vxl + byl * vyl) * pi4i;
  const T fluxrro = rhor * vxr;
  const T fluxrrx = rhor * vxr * vxr + prr + (-(bxbar * bxbar) + byr * byr) * pi8i;
  const T fluxrry = rhor * vxr * vyr - bxbar * byr * pi4i;
  const T fluxrby = vxr * byr - vyr * bxbar;
  const T fluxree = rhor * vxr * hr - bxbar * (bxbar * vxr + byr * vyr) * pi4i;
  // right eigenvectors (:116-183)
  const T vh = half * v2bar;
  const T ff = (cfast2 - cs2) * gm2 / gm1, fs = (cslow2 - cs2) * gm2 / gm1;
  const T rpfro = alphf;
  const T rpfrx = alphf * (vxbar + cfast);
  const T rpfry = alphf * vybar - alphs * betay * ca * sgnbx;
  const T rpfby = alphs * betay * cfast * sq4r;
  const T rpfee = alphf * (vh + delb2 + cfast * vxbar + cfast2 / gm1 + ff) -
                  alphs * ca * (betay * vybar) * sgnbx;
  const T rmfro = alphf;
  const T rmfrx = alphf * (vxbar - cfast);
  const T rmfry = alphf * vybar + alphs * betay * ca * sgnbx;
  const T rmfby = rpfby;
  const T rmfee = alphf * (vh + delb2 - cfast * vxbar + cfast2 / gm1 + ff) +
                  alphs * ca * (betay * vybar) * sgnbx;
  const T rpsro = alphs;
  const T rpsrx = alphs * (vxbar + cslow);
  const T rpsry = alphs * vybar + cs * sgnbx * alphf * betay;
  const T rpsby = -(sq4r * cs2 * alphf * betay / cfast);
  const T rpsee = alphs * (vh + delb2 + cslow * vxbar + cslow2 / gm1 + fs) +
                  alphf * cs * (betay * vybar) * sgnbx;
  const T rmsro = alphs;
  const T rmsrx = alphs * (vxbar - cslow);
  const T rmsry = alphs * vybar - cs * sgnbx * alphf * betay;
  const T rmsby = rpsby;
  const T rmsee = alphs * (vh + delb2 - cslow * vxbar + cslow2 / gm1 + fs) -
                  alphf * cs * (betay * vybar) * sgnbx;
  const T rparo = zero, rparx = zero;
  const T rpary = -(sgnbx * betaz);
  const T rpaby = sq4r * betaz;
  const T rpaee = -((betaz * vybar) * sgnbx);
  const T rmaro = zero, rmarx = zero;
  const T rmary = -rpary;
  const T rmaby = rpaby;
  const T rmaee = -rpaee;
  const T rzero = one, rzerx = vxbar, rzery = vybar, rzeby = zero;
  const T rzeee = vh + delb2;
  // f(i+1/2) (:185-212), summed left to right as the Fortran does
  const T pf = elpf * wpf, mf = elmf * wmf, ps = elps * wps, ms = elms * wms;
  const T pa = elpa * wpa, ma = elma * wma, ze = elze * wze;
  auto sum = [&](T fl, T fr, T rpf, T rmf, T rps, T rms, T rpa, T rma, T rze) {
    return half * (fl + fr + pf * rpf + mf * rmf + ps * rps + ms * rms + pa * rpa +
                   ma * rma + ze * rze);
  };
  f[0] = sum(fluxlro, fluxrro, rpfro, rmfro, rpsro, rmsro, rparo, rmaro, rzero).v;
  f[1] = sum(fluxlee, fluxree, rpfee, rmfee, rpsee, rmsee, rpaee, rmaee, rzeee).v;
  f[2] = sum(fluxlrx, fluxrrx, rpfrx, rmfrx, rpsrx, rmsrx, rparx, rmarx, rzerx).v;
  f[3] = sum(fluxlry, fluxrry, rpfry, rmfry, rpsry, rmsry, rpary, rmary, rzery).v;
  f[4] = sum(fluxlby, fluxrby, rpfby, rmfby, rpsby, rmsby, rpaby, rmaby, rzeby).v;
}

// primitives (ro pr vx vy by) and face field bx of a side
__device__ __forceinline__ void side(const double *q, double bxf, double *w) {
  w[0] = q[Q_RO];
  w[1] = q[Q_PR];
  w[2] = q[Q_VX];
  w[3] = q[Q_VY];
  w[4] = bxf;
  w[5] = q[Q_BY];
}

template <bool E>
__global__ void __launch_bounds__(kR1Threads)
    k_r1_flux1(const double *__restrict__ A, const double *__restrict__ bxm,
               double *__restrict__ Fl, int ix, RoeK K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // face (i, i+1), 0-based
  if (i >= ix - 1) return;
  double a[NQ], b[NQ], L[6], R[6], f[5];
#pragma unroll
  for (int v = 0; v < NQ; v++) {
    a[v] = A[(size_t)v * ix + i];
    b[v] = A[(size_t)v * ix + i + 1];
  }
  side(a, bxm[i], L);
  side(b, bxm[i], R);
  roe_flux1d<E>(K, L, R, f);
#pragma unroll
  for (int v = 0; v < NQ; v++) Fl[(size_t)v * ix + i] = f[v];
}

// conserved variables of cell i (roe_m.f:23-29): ro ee rx ry by
template <bool E>
__device__ __forceinline__ void conserved(const RoeK &K, const double *q, double bx,
                                          F<E> *u) {
  using T = F<E>;
  const T ro(q[Q_RO]), pr(q[Q_PR]), vx(q[Q_VX]), vy(q[Q_VY]), by(q[Q_BY]), b(bx);
  const T v2 = vx * vx + vy * vy;
  const T b2 = b * b + by * by;
  u[0] = ro;
  u[1] = pr / T(K.gm1) + T(0.5) * ro * v2 + T(K.pi8i) * b2;
  u[2] = ro * vx;
  u[3] = ro * vy;
  u[4] = by;
}

// primitives of conserved u with the cell's bx (roe_m.f:60-64, 84-88)
template <bool E>
__device__ __forceinline__ void primitive(const RoeK &K, const F<E> *u, double bx,
                                          double *q) {
  using T = F<E>;
  const T vx = u[2] / u[0], vy = u[3] / u[0];
  const T v2 = vx * vx + vy * vy;
  const T b(bx);
  const T b2 = b * b + u[4] * u[4];
  const T pr = T(K.gm1) * (u[1] - T(0.5) * u[0] * v2 - T(K.pi8i) * b2);
  q[Q_RO] = u[0].v;
  q[Q_PR] = pr.v;
  q[Q_VX] = vx.v;
  q[Q_VY] = vy.v;
  q[Q_BY] = u[4].v;
}

template <bool E>
__global__ void __launch_bounds__(kR1Threads)
    k_r1_half(const double *__restrict__ A, const double *__restrict__ Fl,
              const double *__restrict__ bx, const double *__restrict__ dx,
              double *__restrict__ H, int ix, RoeK K, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ix) return;
  double q[NQ];
#pragma unroll
  for (int v = 0; v < NQ; v++) q[v] = A[(size_t)v * ix + i];
  if (i >= 1 && i <= ix - 2) {
    using T = F<E>;
    T u[NQ];
    conserved<E>(K, q, bx[i], u);
    const T hdt = T(0.5) * T(dt), d(dx[i]);
#pragma unroll
    for (int v = 0; v < NQ; v++)
      u[v] = u[v] + hdt * ((T(Fl[(size_t)v * ix + i - 1]) - T(Fl[(size_t)v * ix + i])) / d);
    primitive<E>(K, u, bx[i], q);
  }
#pragma unroll
  for (int v = 0; v < NQ; v++) H[(size_t)v * ix + i] = q[v];
}

template <bool E>
__global__ void __launch_bounds__(kR1Threads)
    k_r1_flux2(const double *__restrict__ H, const double *__restrict__ bxm,
               double *__restrict__ Fl, int ix, RoeK K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // faces 2..ix-2, 1-based
  if (i < 1 || i > ix - 3) return;
  using T = F<E>;
  double wl[NQ], wr[NQ], L[6], R[6], f[5];
#pragma unroll
  for (int v = 0; v < NQ; v++) {
    const double *h = H + (size_t)v * ix + i;
    const T dm(h[-1]), d0(h[0]), d1(h[1]), d2(h[2]);
    // tvdminmod.f:14-17
    wl[v] = (d0 + T(0.5) * flmt(d1 - d0, d0 - dm)).v;
    wr[v] = (d1 - T(0.5) * flmt(d1 - d0, d2 - d1)).v;
  }
  side(wl, bxm[i], L);
  side(wr, bxm[i], R);
  roe_flux1d<E>(K, L, R, f);
#pragma unroll
  for (int v = 0; v < NQ; v++) Fl[(size_t)v * ix + i] = f[v];
}

template <bool E>
__global__ void __launch_bounds__(kR1Threads)
    k_r1_full(const double *__restrict__ A, const double *__restrict__ Fl,
              const double *__restrict__ bx, const double *__restrict__ dx,
              double *__restrict__ B, int ix, RoeK K, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ix) return;
  double q[NQ];
#pragma unroll
  for (int v = 0; v < NQ; v++) q[v] = A[(size_t)v * ix + i];
  if (i >= 2 && i <= ix - 3) {
    using T = F<E>;
    T u[NQ];
    conserved<E>(K, q, bx[i], u);
    const T d(dx[i]), tdt(dt);
#pragma unroll
    for (int v = 0; v < NQ; v++)
      u[v] = u[v] + tdt * ((T(Fl[(size_t)v * ix + i - 1]) - T(Fl[(size_t)v * ix + i])) / d);
    primitive<E>(K, u, bx[i], q);
  }
#pragma unroll
  for (int v = 0; v < NQ; v++) B[(size_t)v * ix + i] = q[v];
}

template <bool E>
cudaError_t launch_r1(const double *A, double *B, double *scratch, const double *bx,
                      const double *bxm, const double *dx, int ix, const RoeK &K,
                      double dt, cudaStream_t s) {
  const unsigned blocks = (unsigned)((ix + kR1Threads - 1) / kR1Threads);
  double *H = scratch, *Fl = scratch + (size_t)NQ * ix;
  k_r1_flux1<E><<<blocks, kR1Threads, 0, s>>>(A, bxm, Fl, ix, K);
  k_r1_half<E><<<blocks, kR1Threads, 0, s>>>(A, Fl, bx, dx, H, ix, K, dt);
  k_r1_flux2<E><<<blocks, kR1Threads, 0, s>>>(H, bxm, Fl, ix, K);
  k_r1_full<E><<<blocks, kR1Threads, 0, s>>>(A, Fl, bx, dx, B, ix, K, dt);
  count_launch(4);
  return cudaGetLastError();
}

}  // namespace

size_t roe1d_scratch_doubles(size_t ncells) { return 2 * (size_t)NQ * ncells; }

cudaError_t launch_roe1d(bool exact, const double *A, double *B, double *scratch,
                         const double *bx, const double *bxm, const double *dx,
                         int ix, double gm, double dt, cudaStream_t s) {
  if (ix < 5) return cudaErrorInvalidValue;
  RoeK K{};
  const double pi = std::acos(-1.0);
  K.gm = gm;
  K.gm1 = gm - 1.0;
  K.gm2 = gm - 2.0;
  K.gm21 = (gm - 2.0) / (gm - 1.0);
  K.pi4 = 4.0 * pi;
  K.pi4i = 1.0 / K.pi4;
  K.pi8i = 5.0e-1 * K.pi4i;
  K.sqh = std::sqrt(0.5);
  return exact ? launch_r1<true>(A, B, scratch, bx, bxm, dx, ix, K, dt, s)
               : launch_r1<false>(A, B, scratch, bx, bxm, dx, ix, K, dt, s);
}

}  // namespace cans
