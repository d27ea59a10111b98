// Roe flux of one face and the minmod MUSCL state of one side, on the device.
//
//   roe_flux   cans3d/hdroe/roeflux_m.f:29-263 (one face of the loop)
//   flmt       cans3d/hdroe/tvdminmod.f:15
//
// The face states are given in the frame of the face normal: (ro, pr, vn,
// vt1, vt2, bn, bt1, bt2); the flux comes back as (ro, ee, rn, rt1, rt2,
// bt1, bt2).  roe_m.f:96,146,196 rotates (x,y,z) -> (y,z,x) -> (z,x,y) for
// the y and z faces, a cyclic rotation, so one routine serves all axes.
//
// FIX selects the slow-wave normalisation: cans3d/hdroe/roeflux_m.f:79 (the
// 2006 fix) has alphs = sp2 sqrt(cfa/(cfcs+1-sp2)) + 1 - sp2; the 1-D and
// 2-D roeflux_m3.f:77 keep alphs = sp2 sqrt(cfa/(cfcs+1-sp2)).  Otherwise the
// three routines evaluate the same expressions.
//
// Policy E=true evaluates every expression in the order the Fortran does,
// with separately rounded operations (bit-identical to a -ffp-contract=off
// build of the same expressions).  E=false is the fast policy: the same
// algebra with one reciprocal per repeated divisor and FMA contraction.
#pragma once
#include <type_traits>
#include "cans_common.cuh"
#include "df64.cuh"

namespace cans {

// Constants of roeflux_m.f:21-24 and the gamma terms it uses, computed on the
// host with the expressions of the reference.
struct RoeK {
  double gm, gm1, gm2;   // gm, gm-1, gm-2
  double gm21;           // (gm-2)/(gm-1), the leading factor of delb2
  double pi4, pi4i, pi8i;
  double sqh;            // sqrt(0.5)
  double gm1i, ggm1;     // fast policy: 1/(gm-1), gm/(gm-1)
  double sq4pi, sq4pii;  // fast policy: sqrt(4 pi), sqrt(1/(4 pi))
};

// Fortran max/min on doubles as the oracle evaluates them: max(a,b) is
// (a > b ? a : b), min(a,b) is (a < b ? a : b).
template <bool E> __device__ __forceinline__ F<E> fmax_(F<E> a, F<E> b) {
  return F<E>(a.v > b.v ? a.v : b.v);
}
// Fortran sign(a, b): |a| with the sign of b.
template <bool E> __device__ __forceinline__ F<E> fsign_(F<E> a, F<E> b) {
  return F<E>(copysign(fabs(a.v), b.v));
}

// tvdminmod.f:15  flmt(a,b) = max(0, min(b*sign(1,a), |a|)) * sign(1,a)
template <bool E> __device__ __forceinline__ F<E> flmt(F<E> a, F<E> b) {
  const F<E> s = fsign_(F<E>(1.0), a);
  return fmax_(F<E>(0.0), fmin_(b * s, fabs_(a))) * s;
}

template <bool E, bool FIX = true>
__device__ __forceinline__ void roe_flux_ref(const RoeK &K, const double *L,
                                             const double *R, double *f) {
  using T = F<E>;
  const T gm(K.gm), gm1(K.gm1), gm2(K.gm2), pi4(K.pi4), pi4i(K.pi4i),
      pi8i(K.pi8i);
  const T rhol(L[0]), prl(L[1]), vxl(L[2]), vyl(L[3]), vzl(L[4]), byl(L[6]),
      bzl(L[7]);
  const T rhor(R[0]), prr(R[1]), vxr(R[2]), vyr(R[3]), vzr(R[4]), byr(R[6]),
      bzr(R[7]);
  const T bxl(L[5]), bxr(R[5]);
  // roe's variable (:47-61)
  const T sr0 = fsqrt(rhol), sr1 = fsqrt(rhor);
  const T sri = T(1.0) / (sr0 + sr1);
  const T rhobar = sr0 * sr1;
  const T vxbar = (sr0 * vxl + sr1 * vxr) * sri;
  const T vybar = (sr0 * vyl + sr1 * vyr) * sri;
  const T vzbar = (sr0 * vzl + sr1 * vzr) * sri;
  const T bxbar = (sr0 * bxr + sr1 * bxl) * sri;
  const T bybar = (sr0 * byr + sr1 * byl) * sri;
  const T bzbar = (sr0 * bzr + sr1 * bzl) * sri;
  const T hl = T(0.5) * (vxl * vxl + vyl * vyl + vzl * vzl) + gm * prl / (gm1 * rhol) +
               (bxbar * bxbar + byl * byl + bzl * bzl) / (pi4 * rhol);
  const T hr = T(0.5) * (vxr * vxr + vyr * vyr + vzr * vzr) + gm * prr / (gm1 * rhor) +
               (bxbar * bxbar + byr * byr + bzr * bzr) / (pi4 * rhor);
  const T hbar = (sr0 * hl + sr1 * hr) * sri;
  // average (:64-65)
  const T byave = (byl + byr) / T(2.0);
  const T bzave = (bzl + bzr) / T(2.0);
  // characteristic speed (:68-82)
  const T delb2 = T(K.gm21) * ((byr - byl) * (byr - byl) + (bzr - bzl) * (bzr - bzl)) *
                  (sri * sri) * pi8i;
  const T vb2 = vxbar * vxbar + vybar * vybar + vzbar * vzbar;
  const T bt2 = bybar * bybar + bzbar * bzbar;
  const T bb2 = bxbar * bxbar + bybar * bybar + bzbar * bzbar;
  const T cs2 = gm1 * (hbar - T(0.5) * vb2 - delb2 - bb2 * pi4i / rhobar);
  const T astar2 = gm1 * (hbar - T(0.5) * vb2 - delb2) - gm2 * bb2 * pi4i / rhobar;
  const T ca2 = bxbar * bxbar / (pi4 * rhobar);
  const T cbr2 = bt2 * pi4i / rhobar;
  const T cfast2 =
      T(0.5) * (astar2 + fsqrt(cbr2 * (astar2 + cs2 + ca2) + (cs2 - ca2) * (cs2 - ca2)));
  const T cslow2 = cs2 * ca2 / cfast2;
  const T cfast = fsqrt(cfast2), cslow = fsqrt(cslow2);
  const T ca = fsqrt(ca2), cs = fsqrt(cs2);
  // for singular points (:85-100)
  const T sgr = bt2 - T(1.0e-12);
  const T sp = T(0.5) + fsign_(T(0.5), sgr);
  const T rbt = fsqrt(T(1.0) / (bt2 + T(1.0) - sp));
  const T betay = sp * bybar * rbt + T(K.sqh) * (T(1.0) - sp);
  const T betaz = sp * bzbar * rbt + T(K.sqh) * (T(1.0) - sp);
  const T sgr2 = bt2 / (pi4 * rhobar) + fabs_(ca2 - cs2) - T(1.0e-12);
  const T sp2 = T(0.5) + fsign_(T(0.5), sgr2);
  const T cfca = fmax_(T(0.0), cfast2 - ca2);
  const T cfcs = fmax_(T(0.0), cfast2 - cslow2);
  const T cfa = fmax_(T(0.0), cfast2 - cs2);
  const T alphf = sp2 * fsqrt(cfca / (cfcs + T(1.0) - sp2)) + T(1.0) - sp2;
  T alphs = sp2 * fsqrt(cfa / (cfcs + T(1.0) - sp2));
  if constexpr (FIX) alphs = alphs + T(1.0) - sp2;
  const T sgnbx = fsign_(T(1.0), bxbar);
  // eigen value & entropy condition (:103-110)
  const T eeps = (vxr - vxl + fabs_(vxr - vxl)) * T(2.5e-1);
  const T elpf = -fmax_(fabs_(vxbar + cfast), eeps);
  const T elmf = -fmax_(fabs_(vxbar - cfast), eeps);
  const T elps = -fmax_(fabs_(vxbar + cslow), eeps);
  const T elms = -fmax_(fabs_(vxbar - cslow), eeps);
  const T elpa = -fmax_(fabs_(vxbar + ca), eeps);
  const T elma = -fmax_(fabs_(vxbar - ca), eeps);
  const T elze = -fmax_(fabs_(vxbar), eeps);
  // amplitude; w's (:113-142)
  const T drho = rhor - rhol;
  const T du21 = rhobar * (vxr - vxl);
  const T du31 = rhobar * (vyr - vyl);
  const T du41 = rhobar * (vzr - vzl);
  const T du6 = byr - byl, du5 = bzr - bzl;
  const T t1 = betay * du6 + betaz * du5;
  const T t2 = (prr - prl + (byave * du6 + bzave * du5) * pi4i +
                gm2 * (bybar * du6 + bzbar * du5) * pi4i) / gm1;
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
  const T q11 = alphf * cfast, q12 = alphs * cslow;
  const T q21 = -(alphs * ca * sgnbx), q22 = alphf * cs * sgnbx;
  const T detp = p11 * p22 - p12 * p21;
  const T detq = q11 * q22 - q12 * q21;
  const T ap = (p22 * t1 - p12 * t2) / detp, aq = (q22 * s1 - q12 * s2) / detq;
  const T bp = (-(p21 * t1) + p11 * t2) / detp, bq = (-(q21 * s1) + q11 * s2) / detq;
  const T wpf = T(0.5) * (ap + aq), wmf = T(0.5) * (ap - aq);
  const T wps = T(0.5) * (bp + bq), wms = T(0.5) * (bp - bq);
  const T sqr4 = fsqrt(rhobar * pi4i);
  const T wpa = T(0.5) * (sqr4 * t3 - sgnbx * s3);
  const T wma = T(0.5) * (sqr4 * t3 + sgnbx * s3);
  const T wze = drho - alphf * (wpf + wmf) - alphs * (wps + wms);
  // physical fluxes of both sides (:145-158)
  const T bx2 = bxbar * bxbar;
  const T fllro = rhol * vxl;
  const T fllrx = rhol * vxl * vxl + prl + (-bx2 + byl * byl + bzl * bzl) * pi8i;
  const T fllry = rhol * vxl * vyl - bxbar * byl * pi4i;
  const T fllrz = rhol * vxl * vzl - bxbar * bzl * pi4i;
  const T fllby = vxl * byl - vyl * bxbar;
  const T fllbz = vxl * bzl - vzl * bxbar;
  const T fllee = rhol * vxl * hl - bxbar * (bxbar * vxl + byl * vyl + bzl * vzl) * pi4i;
  const T flrro = rhor * vxr;
  const T flrrx = rhor * vxr * vxr + prr + (-bx2 + byr * byr + bzr * bzr) * pi8i;
  const T flrry = rhor * vxr * vyr - bxbar * byr * pi4i;
  const T flrrz = rhor * vxr * vzr - bxbar * bzr * pi4i;
  const T flrby = vxr * byr - vyr * bxbar;
  const T flrbz = vxr * bzr - vzr * bxbar;
  const T flree = rhor * vxr * hr - bxbar * (bxbar * vxr + byr * vyr + bzr * vzr) * pi4i;
  // right eigenvectors (:161-227)
  const T bv = betay * vybar + betaz * vzbar;
  const T hv = T(0.5) * vb2 + delb2;
  const T rpfro = alphf;
  const T rpfrx = alphf * (vxbar + cfast);
  const T rpfry = alphf * vybar - alphs * betay * ca * sgnbx;
  const T rpfrz = alphf * vzbar - alphs * betaz * ca * sgnbx;
  const T rpfby = alphs * betay * cfast * sq4r;
  const T rpfbz = alphs * betaz * cfast * sq4r;
  const T rpfee = alphf * (hv + cfast * vxbar + cfast2 / gm1 + (cfast2 - cs2) * gm2 / gm1) -
                  alphs * ca * bv * sgnbx;
  const T rmfro = alphf;
  const T rmfrx = alphf * (vxbar - cfast);
  const T rmfry = alphf * vybar + alphs * betay * ca * sgnbx;
  const T rmfrz = alphf * vzbar + alphs * betaz * ca * sgnbx;
  const T rmfby = rpfby, rmfbz = rpfbz;
  const T rmfee = alphf * (hv - cfast * vxbar + cfast2 / gm1 + (cfast2 - cs2) * gm2 / gm1) +
                  alphs * ca * bv * sgnbx;
  const T rpsro = alphs;
  const T rpsrx = alphs * (vxbar + cslow);
  const T rpsry = alphs * vybar + cs * sgnbx * alphf * betay;
  const T rpsrz = alphs * vzbar + cs * sgnbx * alphf * betaz;
  const T rpsby = -(sq4r * cs2 * alphf * betay / cfast);
  const T rpsbz = -(sq4r * cs2 * alphf * betaz / cfast);
  const T rpsee = alphs * (hv + cslow * vxbar + cslow2 / gm1 + (cslow2 - cs2) * gm2 / gm1) +
                  alphf * cs * bv * sgnbx;
  const T rmsro = alphs;
  const T rmsrx = alphs * (vxbar - cslow);
  const T rmsry = alphs * vybar - cs * sgnbx * alphf * betay;
  const T rmsrz = alphs * vzbar - cs * sgnbx * alphf * betaz;
  const T rmsby = rpsby, rmsbz = rpsbz;
  const T rmsee = alphs * (hv - cslow * vxbar + cslow2 / gm1 + (cslow2 - cs2) * gm2 / gm1) -
                  alphf * cs * bv * sgnbx;
  const T rparo(0.0), rparx(0.0);
  const T rpary = -(sgnbx * betaz), rparz = sgnbx * betay;
  const T rpaby = sq4r * betaz, rpabz = -(sq4r * betay);
  const T rpaee = -((betaz * vybar - betay * vzbar) * sgnbx);
  const T rmaro(0.0), rmarx(0.0);
  const T rmary = -rpary, rmarz = -rparz;
  const T rmaby = rpaby, rmabz = rpabz, rmaee = -rpaee;
  const T rzero(1.0), rzerx = vxbar, rzery = vybar, rzerz = vzbar;
  const T rzeby(0.0), rzebz(0.0);
  const T rzeee = hv;
  // f(i+1/2) (:230-263)
  const T pf = elpf * wpf, mf = elmf * wmf, ps = elps * wps, ms = elms * wms;
  const T pa = elpa * wpa, ma = elma * wma, ze = elze * wze;
#define CANS_ROE_SUM(FL, FR, P, M, PS, MS, PA, MA, Z)                              \
  (T(0.5) * (FL + FR + pf * P + mf * M + ps * PS + ms * MS + pa * PA + ma * MA + ze * Z)).v
  f[0] = CANS_ROE_SUM(fllro, flrro, rpfro, rmfro, rpsro, rmsro, rparo, rmaro, rzero);
  f[1] = CANS_ROE_SUM(fllee, flree, rpfee, rmfee, rpsee, rmsee, rpaee, rmaee, rzeee);
  f[2] = CANS_ROE_SUM(fllrx, flrrx, rpfrx, rmfrx, rpsrx, rmsrx, rparx, rmarx, rzerx);
  f[3] = CANS_ROE_SUM(fllry, flrry, rpfry, rmfry, rpsry, rmsry, rpary, rmary, rzery);
  f[4] = CANS_ROE_SUM(fllrz, flrrz, rpfrz, rmfrz, rpsrz, rmsrz, rparz, rmarz, rzerz);
  f[5] = CANS_ROE_SUM(fllby, flrby, rpfby, rmfby, rpsby, rmsby, rpaby, rmaby, rzeby);
  f[6] = CANS_ROE_SUM(fllbz, flrbz, rpfbz, rmfbz, rpsbz, rmsbz, rpabz, rmabz, rzebz);
#undef CANS_ROE_SUM
}

// ---------------------------------------------------------------------------
// Fast policy.  The same flux with the algebra rearranged for the FP64 pipe:
//  - square roots and divisions become reciprocal square roots and
//    reciprocals that are reused: 1/rho and sqrt(rho) of both sides from one
//    rsqrt each, 1/rhobar = 1/(sqrt(rhol) sqrt(rhor)), cfast and 1/cfast from
//    one rsqrt(cfast2), ca = |bxbar| / sqrt(4 pi rhobar), cslow = cs ca/cfast;
//  - the eigenvector sum  sum_k lambda_k w_k r_k  is factored by wave pairs
//    (r+f and r-f share all but the sign of the cfast terms, and so on), and
//    wpf+wmf = ap, wps+wms = bp are used directly;
//  - the switches keep the reference's own rounding where it matters:
//    sqrt(1/((bt2+1)-sp)) and (sp2 sqrt(..)+1)-sp2 are evaluated as written.
// Results agree with the exact policy to rounding, not bit for bit.

__device__ __forceinline__ double rcp_(double x) { return __drcp_rn(x); }
__device__ __forceinline__ double rsq_(double x) { return rsqrt(x); }
// sqrt from rsqrt; x = 0 gives 0 (x * rsqrt(x) alone would give NaN)
__device__ __forceinline__ double sqrt_(double x) {
  return x == 0.0 ? 0.0 : x * rsq_(x);
}
__device__ __forceinline__ double max_(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double sign1_(double x) { return copysign(1.0, x); }
__device__ __forceinline__ bool ge0_(double x) { return x >= 0.0; }

// The same helpers in double-float (df64.cuh): the reciprocal square root is
// one Newton step on the correctly rounded float one, with x r^2 formed in
// double-float (about 2^-46).
__device__ __forceinline__ df::DF rcp_(df::DF x) { return df::DF(df::rcp(x.d)); }
__device__ __forceinline__ df::DF rsq_(df::DF x) {
  const float r = __frsqrt_rn(x.d.h);
  const df::D q = df::mulf(df::mulf(x.d, r), r);
  const float e = __fsub_rn(__fsub_rn(1.0f, q.h), q.l);  // 1 - q.h is exact
  return df::DF(df::fast_two_sum(r, __fmul_rn(__fmul_rn(0.5f, r), e)));
}
__device__ __forceinline__ df::DF sqrt_(df::DF x) {
  return x.d.h == 0.0f ? df::DF(0.0f) : x * rsq_(x);
}
__device__ __forceinline__ df::DF max_(df::DF a, df::DF b) { return df::gt(a.d, b.d) ? a : b; }
__device__ __forceinline__ df::DF sign1_(df::DF x) {
  return df::DF(copysignf(1.0f, x.d.h));
}
__device__ __forceinline__ bool ge0_(df::DF x) { return !(x.d.h < 0.0f); }

// The constants of the fast flux in its number type.
template <class R> struct RoeKR {
  R gm1, gm2, gm21, pi4i, pi8i, sqh, gm1i, ggm1, sq4pi, sq4pii, eps12;
};
template <class R> __device__ __forceinline__ RoeKR<R> roe_k(const RoeK &K) {
  return {num_in<R>(K.gm1),  num_in<R>(K.gm2),  num_in<R>(K.gm21),  num_in<R>(K.pi4i),
          num_in<R>(K.pi8i), num_in<R>(K.sqh),  num_in<R>(K.gm1i),  num_in<R>(K.ggm1),
          num_in<R>(K.sq4pi), num_in<R>(K.sq4pii), num_in<R>(1.0e-12)};
}

// The fast flux, written once for a number type R (double: the fast policy;
// df::DF: the double-float policy).  Literal constants are floats: exact in
// both types.
// Where the double-float flux hands a face to the FP64 one: the normalised
// eigenvector weights alphf = sqrt(cf^2 - ca^2) / sqrt(cf^2 - cs_slow^2) and
// alphs = sqrt(cf^2 - cs^2) / ... are square roots of differences of nearly
// equal squares near the c_f = c_a and c_f = c_s degeneracies, where their
// absolute error grows as the rounding unit / sqrt(difference / cf^2).  Below
// kIllCond the 48-bit significand of double-float would leave it 32 times the
// FP64 flux's; there the face is evaluated in FP64.
constexpr float kIllCond = 1.0e-3f;

template <class R, bool FIX>
__device__ __forceinline__ void roe_flux_fast_r(const RoeKR<R> &K, const R *L, const R *Rs,
                                                R *f, bool *ill = nullptr) {
  const R rl = L[0], pl = L[1], ul = L[2], vl = L[3], wl = L[4];
  const R bxl = L[5], byl = L[6], bzl = L[7];
  const R rr = Rs[0], pr = Rs[1], ur = Rs[2], vr = Rs[3], wr = Rs[4];
  const R bxr = Rs[5], byr = Rs[6], bzr = Rs[7];
  const R pi4i = K.pi4i, pi8i = K.pi8i;
  const R one(1.0f), half(0.5f), zero(0.0f);
  // Roe averages
  const R q0 = rsq_(rl), q1 = rsq_(rr);
  const R sr0 = rl * q0, sr1 = rr * q1;
  const R irl = q0 * q0, irr = q1 * q1;
  const R sri = rcp_(sr0 + sr1);
  const R rhobar = sr0 * sr1, irb = q0 * q1;
  const R w0 = sr0 * sri, w1 = sr1 * sri;
  const R ub = fma(w0, ul, w1 * ur), vb = fma(w0, vl, w1 * vr), wb = fma(w0, wl, w1 * wr);
  const R bxb = fma(w0, bxr, w1 * bxl), byb = fma(w0, byr, w1 * byl),
          bzb = fma(w0, bzr, w1 * bzl);
  const R bx2 = bxb * bxb;
  const R btl = fma(byl, byl, bzl * bzl), btr = fma(byr, byr, bzr * bzr);
  const R v2l = fma(ul, ul, fma(vl, vl, wl * wl));
  const R v2r = fma(ur, ur, fma(vr, vr, wr * wr));
  const R hl = fma(half, v2l, irl * fma(K.ggm1, pl, pi4i * (bx2 + btl)));
  const R hr = fma(half, v2r, irr * fma(K.ggm1, pr, pi4i * (bx2 + btr)));
  const R hbar = fma(w0, hl, w1 * hr);
  const R dby = byr - byl, dbz = bzr - bzl;
  const R byave = half * (byl + byr), bzave = half * (bzl + bzr);
  const R delb2 = K.gm21 * fma(dby, dby, dbz * dbz) * (sri * sri) * pi8i;
  const R vb2 = fma(ub, ub, fma(vb, vb, wb * wb));
  const R bt2 = fma(byb, byb, bzb * bzb);
  const R pib = pi4i * irb;
  const R bbr = (bx2 + bt2) * pib;
  const R hv = fma(half, vb2, delb2);
  const R qh = hbar - hv;
  const R cs2 = K.gm1 * (qh - bbr);
  const R astar2 = fma(K.gm1, qh, -K.gm2 * bbr);
  const R ca2 = bx2 * pib, cbr2 = bt2 * pib;
  const R dcs = cs2 - ca2;
  const R cfast2 = half * (astar2 + sqrt_(fma(cbr2, astar2 + cs2 + ca2, dcs * dcs)));
  const R rcf = rsq_(cfast2);
  const R cfast = cfast2 * rcf;
  const R rrb = rsq_(rhobar);
  const R cs = sqrt_(cs2);
  const R ca = fabs(bxb) * K.sq4pii * rrb;
  const R cslow2 = cs2 * ca2 * (rcf * rcf);
  const R cslow = cs * ca * rcf;
  // singular points
  const bool spb = ge0_(bt2 - K.eps12);
  const R sp = spb ? one : zero;
  const R rbt = rsq_(bt2 + one - sp);
  const R betay = spb ? byb * rbt : K.sqh;
  const R betaz = spb ? bzb * rbt : K.sqh;
  const bool sp2b = ge0_(fma(bt2, pib, fabs(ca2 - cs2)) - K.eps12);
  const R sp2 = sp2b ? one : zero;
  const R cfca = max_(zero, cfast2 - ca2);
  const R cfcs = max_(zero, cfast2 - cslow2);
  const R cfa = max_(zero, cfast2 - cs2);
  if constexpr (std::is_same<R, df::DF>::value) {
    if (ill != nullptr) {
      const float lim = kIllCond * cfast2.d.h;
      *ill = !(cfca.d.h >= lim && cfa.d.h >= lim);
      if (*ill) return;  // the caller evaluates the face in FP64
    }
  }
  const R rden = rsq_(cfcs + one - sp2);
  const R alphf = sp2 * (sqrt_(cfca) * rden) + one - sp2;
  const R alphs = FIX ? sp2 * (sqrt_(cfa) * rden) + one - sp2 : sp2 * (sqrt_(cfa) * rden);
  const R sg = sign1_(bxb);
  // eigenvalues with the entropy floor
  const R du = ur - ul;
  const R eeps = half * max_(du, zero);
  const R elpf = -max_(fabs(ub + cfast), eeps), elmf = -max_(fabs(ub - cfast), eeps);
  const R elps = -max_(fabs(ub + cslow), eeps), elms = -max_(fabs(ub - cslow), eeps);
  const R elpa = -max_(fabs(ub + ca), eeps), elma = -max_(fabs(ub - ca), eeps);
  const R elze = -max_(fabs(ub), eeps);
  // wave amplitudes
  const R t1 = fma(betay, dby, betaz * dbz);
  const R t2 = (pr - pl + pi4i * fma(byave, dby, bzave * dbz) +
                K.gm2 * pi4i * fma(byb, dby, bzb * dbz)) * K.gm1i;
  const R t3 = fma(betaz, dby, -betay * dbz);
  const R s1 = rhobar * du;
  const R dv = rhobar * (vr - vl), dw = rhobar * (wr - wl);
  const R s2 = fma(betay, dv, betaz * dw), s3 = fma(betaz, dv, -betay * dw);
  const R sq4r = K.sq4pi * rrb;
  const R sqr4 = K.sq4pii * rhobar * rrb;
  const R cg = cs2 * K.gm21;
  const R p11 = alphs * cfast * sq4r, p12 = -alphf * cs2 * rcf * sq4r;
  const R p21 = alphf * (cfast2 - cg), p22 = alphs * (cslow2 - cg);
  const R q11 = alphf * cfast, q12 = alphs * cslow;
  const R q21 = -alphs * ca * sg, q22 = alphf * cs * sg;
  const R rdp = rcp_(fma(p11, p22, -p12 * p21));
  const R rdq = rcp_(fma(q11, q22, -q12 * q21));
  const R ap = fma(p22, t1, -p12 * t2) * rdp, aq = fma(q22, s1, -q12 * s2) * rdq;
  const R bp = fma(p11, t2, -p21 * t1) * rdp, bq = fma(q11, s2, -q21 * s1) * rdq;
  const R PF = elpf * half * (ap + aq), MF = elmf * half * (ap - aq);
  const R PS = elps * half * (bp + bq), MS = elms * half * (bp - bq);
  const R PA = elpa * half * fma(sqr4, t3, -sg * s3);
  const R MA = elma * half * fma(sqr4, t3, sg * s3);
  const R ZE = elze * (rr - rl - alphf * ap - alphs * bp);
  // wave-pair sums
  const R fS = PF + MF, fD = PF - MF, sS = PS + MS, sD = PS - MS;
  const R aS = PA + MA, aD = PA - MA;
  const R dro = fma(alphf, fS, fma(alphs, sS, ZE));
  const R tcf = fma(-alphs * ca, fD, alphf * cs * sD) * sg;  // shared by ry, rz
  const R tb = sq4r * fma(alphs * cfast, fS, -cs2 * rcf * alphf * sS);
  const R bv = fma(betay, vb, betaz * wb);
  const R cfg = fma(cfast2 - cs2, K.gm2, cfast2) * K.gm1i;
  const R csg = fma(cslow2 - cs2, K.gm2, cslow2) * K.gm1i;
  const R dee =
      alphf * fma(hv + cfg, fS, cfast * ub * fD) + alphs * fma(hv + csg, sS, cslow * ub * sD) +
      bv * sg * fma(-alphs * ca, fD, alphf * cs * sD) -
      fma(betaz, vb, -betay * wb) * sg * aD + hv * ZE;
  // physical fluxes of both sides
  const R ml = rl * ul, mr = rr * ur;
  const R fro = ml + mr;
  const R frx = fma(ml, ul, pl) + fma(mr, ur, pr) + (btl + btr - 2.0f * bx2) * pi8i;
  const R fry = fma(ml, vl, mr * vr) - bxb * (byl + byr) * pi4i;
  const R frz = fma(ml, wl, mr * wr) - bxb * (bzl + bzr) * pi4i;
  const R fby = fma(ul, byl, -vl * bxb) + fma(ur, byr, -vr * bxb);
  const R fbz = fma(ul, bzl, -wl * bxb) + fma(ur, bzr, -wr * bxb);
  const R fee = fma(ml, hl, mr * hr) -
                bxb * pi4i * (fma(bxb, ul, fma(byl, vl, bzl * wl)) +
                              fma(bxb, ur, fma(byr, vr, bzr * wr)));
  f[0] = half * (fro + dro);
  f[1] = half * (fee + dee);
  f[2] = half * (frx + fma(ub, dro, fma(alphf * cfast, fD, alphs * cslow * sD)));
  f[3] = half * (fry + fma(vb, dro, fma(betay, tcf, -sg * betaz * aD)));
  f[4] = half * (frz + fma(wb, dro, fma(betaz, tcf, sg * betay * aD)));
  f[5] = half * (fby + fma(betay, tb, sq4r * betaz * aS));
  f[6] = half * (fbz + fma(betaz, tb, -sq4r * betay * aS));
}

template <bool FIX = true>
__device__ __forceinline__ void roe_flux_fast(const RoeK &K, const double *L,
                                              const double *R, double *f) {
  roe_flux_fast_r<double, FIX>(roe_k<double>(K), L, R, f);
}

// The double-float policy: the fast flux on the FP32 pipes, states and
// fluxes converted once.
// A face whose flux is ill-conditioned for double-float (kIllCond) is
// evaluated again by the FP64 fast flux.
// The forecast of such a face, before any double-float work: the field of
// both face states within about 1/32 of the face normal (judged on the
// exponent fields with integer operations), where c_f meets c_a or c_s.
// When every active lane of a warp forecasts it (a field along the axis, as
// on the faces of that axis), the warp takes the FP64 flux directly; a warp
// with any other face takes the double-float flux with its own test, so
// that no warp pays for both paths on a forecast alone.
__device__ __forceinline__ int roe_exp_field(double x) {
  return (__double2hiint(x) >> 20) & 0x7ff;
}
__device__ __forceinline__ bool roe_near_degenerate(const double *L, const double *R) {
  const int en = min(roe_exp_field(L[5]), roe_exp_field(R[5]));
  const int et = max(max(roe_exp_field(L[6]), roe_exp_field(L[7])),
                     max(roe_exp_field(R[6]), roe_exp_field(R[7])));
  return en > 0 && et + 6 <= en;
}

template <bool FIX = true>
__device__ __forceinline__ void roe_flux_df(const RoeK &K, const double *L,
                                            const double *R, double *f) {
  if (__all_sync(__activemask(), roe_near_degenerate(L, R))) {
    roe_flux_fast_r<double, FIX>(roe_k<double>(K), L, R, f);
    return;
  }
  df::DF l[8], r[8], o[7];
#pragma unroll
  for (int v = 0; v < 8; v++) {
    l[v] = num_in<df::DF>(L[v]);
    r[v] = num_in<df::DF>(R[v]);
  }
  bool ill = false;
  roe_flux_fast_r<df::DF, FIX>(roe_k<df::DF>(K), l, r, o, &ill);
  if (ill) {
    roe_flux_fast_r<double, FIX>(roe_k<double>(K), L, R, f);
    return;
  }
#pragma unroll
  for (int v = 0; v < 7; v++) f[v] = num_out(o[v]);
}

}  // namespace cans
