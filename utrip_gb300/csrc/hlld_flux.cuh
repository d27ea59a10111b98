// HLLD flux of one face on the device:
// cansxx-nosupport/hdhlld/hlld_flux.f90:148-480 (Miyoshi & Kusano, J. Comput.
// Phys. 208, 315 (2005)), Heaviside units (pb = B^2/2).
//
// Face states in the frame of the face normal: (ro, pr, vn, vt1, vt2, bn,
// bt1, bt2) with bn unused -- the normal field is the face value bxs; the
// flux comes back as (ro, ee, rn, rt1, rt2, bt1, bt2).
//
// The flux is written once for its number type T:
//   F<true>   the exact policy: the expressions in the Fortran order with
//             separately rounded operations;
//   F<false>  the fast policy: the same expressions with FMA contraction and
//             reciprocals in place of the repeated divisions;
//   df::DF    the double-float policy: the fast policy's algebra on the FP32
//             pipes (df64.cuh), face states and fluxes converted once.
#pragma once
#include <type_traits>

#include "cans_common.cuh"
#include "df64.cuh"
#include "roe_flux.cuh"  // fmax_, fsign_, the double-float rcp_ and sqrt_

namespace cans {

struct HlldK {
  double gm, gm1;   // gm, gm-1
  double zfloor;    // hlld_mh.f:34
  double gm1i;      // fast policy: 1/(gm-1)
};

// What the flux needs of its number type beyond the arithmetic operators:
// conversion from and to the caller's doubles, the sign tests of its
// branches and the reciprocal of the fast algebra.
template <class T> struct HNum;
template <bool E> struct HNum<F<E>> {
  static constexpr bool exact = E;
  static __device__ __forceinline__ F<E> in(double x) { return F<E>(x); }
  static __device__ __forceinline__ double out(F<E> x) { return x.v; }
  static __device__ __forceinline__ bool ge0(F<E> x) { return x.v >= 0.0; }
  static __device__ __forceinline__ bool gt0(F<E> x) { return x.v > 0.0; }
  static __device__ __forceinline__ bool le0(F<E> x) { return x.v <= 0.0; }
  static __device__ __forceinline__ F<E> rcp(F<E> x) { return F<E>(1.0) / x; }
};
// a normalised double-float carries its sign in the head (a zero head has a
// zero tail)
template <> struct HNum<df::DF> {
  static constexpr bool exact = false;
  static __device__ __forceinline__ df::DF in(double x) { return num_in<df::DF>(x); }
  static __device__ __forceinline__ double out(df::DF x) { return num_out(x); }
  static __device__ __forceinline__ bool ge0(df::DF x) { return !(x.d.h < 0.0f); }
  static __device__ __forceinline__ bool gt0(df::DF x) { return x.d.h > 0.0f; }
  static __device__ __forceinline__ bool le0(df::DF x) { return !(x.d.h > 0.0f); }
  static __device__ __forceinline__ df::DF rcp(df::DF x) { return rcp_(x); }
};
// Fortran max, min, sign, abs and sqrt of double-floats, in the forms the
// F<E> versions take
__device__ __forceinline__ df::DF fmax_(df::DF a, df::DF b) {
  return df::gt(a.d, b.d) ? a : b;
}
__device__ __forceinline__ df::DF fmin_(df::DF a, df::DF b) {
  return df::gt(b.d, a.d) ? a : b;
}
__device__ __forceinline__ df::DF fsign_(df::DF a, df::DF b) {
  const df::D m = df::absd(a.d);
  return df::DF(signbit(b.d.h) ? df::neg(m) : m);
}
__device__ __forceinline__ df::DF fabs_(df::DF a) { return df::DF(df::absd(a.d)); }
__device__ __forceinline__ df::DF fsqrt(df::DF a) { return sqrt_(a); }

// ill (double-float instance): set when a subsonic face's star state is
// ill-conditioned for double-float -- its denominator
// ro (S - vn)(S - S_M) - bn^2 a difference of nearly equal terms, below
// kIllCond of them, where the star state's error grows as the rounding unit
// over that ratio -- so that the caller evaluates the face in FP64.
template <class T>
__device__ __forceinline__ void hlld_flux_t(const HlldK &K, const double *L,
                                            const double *R, double bxv,
                                            double *f, bool *ill = nullptr) {
  using N = HNum<T>;
  constexpr bool E = N::exact;
  const T gm = N::in(K.gm), gm1 = N::in(K.gm1), zf = N::in(K.zfloor);
  const T bxs = N::in(bxv);
  const T bxsq = bxs * bxs;
  // left and right states (:152-191)
  const T rol = N::in(L[0]), prl = N::in(L[1]), vxl = N::in(L[2]), vyl = N::in(L[3]),
          vzl = N::in(L[4]), byl = N::in(L[6]), bzl = N::in(L[7]);
  const T ror = N::in(R[0]), prr = N::in(R[1]), vxr = N::in(R[2]), vyr = N::in(R[3]),
          vzr = N::in(R[4]), byr = N::in(R[6]), bzr = N::in(R[7]);
  const T pbl = T(0.5) * (bxs * bxs + byl * byl + bzl * bzl);
  const T ptl = prl + pbl;
  T eel, eer;
  if constexpr (E) {
    eel = prl / gm1 + T(0.5) * rol * (vxl * vxl + vyl * vyl + vzl * vzl) + pbl;
  } else {
    eel = prl * N::in(K.gm1i) + T(0.5) * rol * (vxl * vxl + vyl * vyl + vzl * vzl) + pbl;
  }
  const T rxl = rol * vxl, ryl = rol * vyl, rzl = rol * vzl;
  const T pbr = T(0.5) * (bxs * bxs + byr * byr + bzr * bzr);
  const T ptr = prr + pbr;
  if constexpr (E) {
    eer = prr / gm1 + T(0.5) * (ror * (vxr * vxr + vyr * vyr + vzr * vzr)) + pbr;
  } else {
    eer = prr * N::in(K.gm1i) + T(0.5) * (ror * (vxr * vxr + vyr * vyr + vzr * vzr)) + pbr;
  }
  const T rxr = ror * vxr, ryr = ror * vyr, rzr = ror * vzr;
  // wave speeds (:197-207)
  const T gmpl = gm * prl, gmpr = gm * prr;
  const T gpbl = gmpl + T(2.0) * pbl, gpbr = gmpr + T(2.0) * pbr;
  const T cfl = fsqrt((gpbl + fsqrt(gpbl * gpbl - T(4.0) * gmpl * bxsq)) / (T(2.0) * rol));
  const T cfr = fsqrt((gpbr + fsqrt(gpbr * gpbr - T(4.0) * gmpr * bxsq)) / (T(2.0) * ror));
  const T cfm = fmax_(cfl, cfr);
  const T sl = fmin_(vxl, vxr) - cfm;
  const T sr = fmax_(vxl, vxr) + cfm;
  // physical fluxes (:214-229)
  const T frol = rxl;
  const T frxl = rxl * vxl + ptl - bxsq;
  const T fryl = rol * vxl * vyl - bxs * byl;
  const T frzl = rol * vxl * vzl - bxs * bzl;
  const T feel = vxl * (eel + ptl - bxsq) - bxs * (vyl * byl + vzl * bzl);
  const T fbyl = byl * vxl - bxs * vyl;
  const T fbzl = bzl * vxl - bxs * vzl;
  const T fror = rxr;
  const T frxr = rxr * vxr + ptr - bxsq;
  const T fryr = ror * vxr * vyr - bxs * byr;
  const T frzr = ror * vxr * vzr - bxs * bzr;
  const T feer = vxr * (eer + ptr - bxsq) - bxs * (vyr * byr + vzr * bzr);
  const T fbyr = byr * vxr - bxs * vyr;
  const T fbzr = bzr * vxr - bxs * vzr;
  // The double-float instance runs one straight-line path: its instruction
  // footprint, not its arithmetic, bounds it, so the branches below become
  // selects (SL: the face takes a one-sided state; the supersonic cases keep
  // the physical flux of their side).
  constexpr bool SL = std::is_same<T, df::DF>::value;
  // supersonic cases (:235-255)
  if (!SL && N::ge0(sl)) {
    f[0] = N::out(frol); f[1] = N::out(feel); f[2] = N::out(frxl); f[3] = N::out(fryl);
    f[4] = N::out(frzl); f[5] = N::out(fbyl); f[6] = N::out(fbzl);
    return;
  }
  if (!SL && N::le0(sr)) {
    f[0] = N::out(fror); f[1] = N::out(feer); f[2] = N::out(frxr); f[3] = N::out(fryr);
    f[4] = N::out(frzr); f[5] = N::out(fbyr); f[6] = N::out(fbzr);
    return;
  }
  // contact speed and star total pressure (:260-275)
  const T sdl = sl - vxl, sdr = sr - vxr;
  const T den = sdr * ror - sdl * rol;
  T sm, ptst;
  if constexpr (E) {
    sm = (sdr * ror * vxr - sdl * rol * vxl - ptr + ptl) / den;
    ptst = (sdr * ror * ptl - sdl * rol * ptr + rol * ror * sdr * sdl * (vxr - vxl)) / den;
  } else {
    const T di = N::rcp(den);
    sm = (sdr * ror * vxr - sdl * rol * vxl - ptr + ptl) * di;
    ptst = (sdr * ror * ptl - sdl * rol * ptr + rol * ror * sdr * sdl * (vxr - vxl)) * di;
  }
  const T sdml = sl - sm, sdmr = sr - sm;
  // one-sided star state (:281-342); side 0 left, 1 right
  T rost[2], rxst[2], ryst[2], rzst[2], vyst[2], vzst[2], byst[2], bzst[2], eest[2];
  T vdbst[2];
  // the star states' denominators first: where one is ill-conditioned for
  // double-float the caller evaluates the face in FP64, and the double-float
  // instance stops before the rest of the star states
  T temp_fst[2];
  bool illv = false;
#pragma unroll
  for (int s = 0; s < 2; s++) {
    const T ro = s ? ror : rol, sd = s ? sdr : sdl, sdm = s ? sdmr : sdml;
    temp_fst[s] = ro * sd * sdm - bxsq;
    if constexpr (std::is_same<T, df::DF>::value) {
      if (ill != nullptr) {
        const float big = fabsf(ro.d.h * sd.d.h * sdm.d.h) + bxsq.d.h;
        if (!(fabsf(temp_fst[s].d.h) >= kIllCond * big)) illv = true;
      }
    }
  }
  if constexpr (SL) {
    if (ill != nullptr && illv && !(N::ge0(sl) || N::le0(sr))) {
      *ill = true;  // the caller evaluates the face in FP64
      return;
    }
  }
#pragma unroll
  for (int s = 0; s < 2; s++) {
    const T ro = s ? ror : rol, vx = s ? vxr : vxl, vy = s ? vyr : vyl, vz = s ? vzr : vzl;
    const T by = s ? byr : byl, bz = s ? bzr : bzl, pt = s ? ptr : ptl, ee = s ? eer : eel;
    const T sd = s ? sdr : sdl, sdm = s ? sdmr : sdml;
    const T s3 = fsign_(T(1.0), temp_fst[s] + zf) * fsign_(T(1.0), temp_fst[s] - zf);
    const T mx = fmax_(T(0.0), s3), mn = fmin_(T(0.0), s3);
    const T dd = temp_fst[s] + mn;
    T tmp, tmp2, rsd, esd;
    if constexpr (E) {
      tmp = bxs * (sd - sdm) / dd;
      tmp2 = (ro * (sd * sd) - bxsq) / dd;
      rsd = ro * sd / sdm;
    } else {
      const T ddi = N::rcp(dd);
      tmp = bxs * (sd - sdm) * ddi;
      tmp2 = (ro * (sd * sd) - bxsq) * ddi;
      rsd = ro * sd * N::rcp(sdm);
    }
    rost[s] = mx * rsd - mn * ro;
    const T vxst = mx * sm - mn * vx;
    rxst[s] = rost[s] * vxst;
    vyst[s] = mx * (vy - by * tmp) - mn * vy;
    ryst[s] = rost[s] * vyst[s];
    vzst[s] = mx * (vz - bz * tmp) - mn * vz;
    rzst[s] = rost[s] * vzst[s];
    byst[s] = mx * (by * tmp2) - mn * by;
    bzst[s] = mx * (bz * tmp2) - mn * bz;
    vdbst[s] = vxst * bxs + vyst[s] * byst[s] + vzst[s] * bzst[s];
    const T num = sd * ee - pt * vx + ptst * sm + bxs * (vx * bxs + vy * by + vz * bz - vdbst[s]);
    if constexpr (E) esd = num / sdm;
    else esd = num * N::rcp(sdm);
    eest[s] = mx * esd - mn * ee;
  }
  // double-star states (:347-414)
  const T sqrtrol = fsqrt(rost[0]), sqrtror = fsqrt(rost[1]);
  T slst, srst;
  if constexpr (E) {
    slst = sm - fabs_(bxs) / sqrtrol;
    srst = sm + fabs_(bxs) / sqrtror;
  } else {
    slst = sm - fabs_(bxs) * N::rcp(sqrtrol);
    srst = sm + fabs_(bxs) * N::rcp(sqrtror);
  }
  T ryd[2], rzd[2], byd, bzd, eed[2];
  if (!SL && bxv == 0.0) {
    ryd[0] = ryst[0]; ryd[1] = ryst[1];
    rzd[0] = rzst[0]; rzd[1] = rzst[1];
    eed[0] = eest[0]; eed[1] = eest[1];
    byd = byst[0];  // unused: the flux takes byst of each side below
    bzd = bzst[0];
  } else {
    const T invsumro = N::rcp(sqrtrol + sqrtror);
    const T signbx = fsign_(T(1.0), bxs);
    const T vyd = invsumro * (sqrtrol * vyst[0] + sqrtror * vyst[1] + signbx * (byst[1] - byst[0]));
    ryd[0] = rost[0] * vyd;
    ryd[1] = rost[1] * vyd;
    const T vzd = invsumro * (sqrtrol * vzst[0] + sqrtror * vzst[1] + signbx * (bzst[1] - bzst[0]));
    rzd[0] = rost[0] * vzd;
    rzd[1] = rost[1] * vzd;
    byd = invsumro * (sqrtrol * byst[1] + sqrtror * byst[0] +
                      signbx * sqrtrol * sqrtror * (vyst[1] - vyst[0]));
    bzd = invsumro * (sqrtrol * bzst[1] + sqrtror * bzst[0] +
                      signbx * sqrtrol * sqrtror * (vzst[1] - vzst[0]));
    const T temp = sm * bxs + vyd * byd + vzd * bzd;
    eed[0] = eest[0] - sqrtrol * signbx * (vdbst[0] - temp);
    eed[1] = eest[1] + sqrtror * signbx * (vdbst[1] - temp);
  }
  const bool zb = bxv == 0.0;
  // flux (:446-480)
  if constexpr (SL) {
    // one side s and f = F_s + c1 (U*_s - U_s) + c2 (U**_s - U*_s): c1 = sl or
    // sr, c2 = slst or srst in the inner fans, 0 in the outer ones (the
    // branches of the reference, rearranged); the supersonic cases select the
    // physical flux.  With bx = 0 the double-star state is the star state.
    const bool right = !N::ge0(sm), sup = N::ge0(sl) || N::le0(sr);
    if (ill != nullptr) *ill = illv && !sup;
    const bool supr = N::le0(sr) && !N::ge0(sl);
    const bool inner = right ? N::gt0(srst) : !N::ge0(slst);
    const T c1 = right ? sr : sl;
    const T c2 = inner ? (right ? srst : slst) : T(0.0f);
    auto put = [&](int v, T fl, T fr, T ul, T ur, T usv, T udv) {
      const T fv = (right ? fr : fl) + c1 * (usv - (right ? ur : ul)) + c2 * (udv - usv);
      f[v] = N::out(sup ? (supr ? fr : fl) : fv);
    };
    // the star and double-star values of side s, picked by selects (an index
    // into the two-element arrays would place them in local memory)
    auto pick = [&](const T *x) { return right ? x[1] : x[0]; };
    const T ro_s = pick(rost), ee_s = pick(eest), ry_s = pick(ryst), rz_s = pick(rzst);
    const T by_s = pick(byst), bz_s = pick(bzst);
    put(0, frol, fror, rol, ror, ro_s, ro_s);
    put(1, feel, feer, eel, eer, ee_s, zb ? ee_s : pick(eed));
    put(2, frxl, frxr, rxl, rxr, pick(rxst), pick(rxst));
    put(3, fryl, fryr, ryl, ryr, ry_s, zb ? ry_s : pick(ryd));
    put(4, frzl, frzr, rzl, rzr, rz_s, zb ? rz_s : pick(rzd));
    put(5, fbyl, fbyr, byl, byr, by_s, zb ? by_s : byd);
    put(6, fbzl, fbzr, bzl, bzr, bz_s, zb ? bz_s : bzd);
  } else if (N::ge0(slst)) {
    f[0] = N::out(frol + sl * (rost[0] - rol));
    f[2] = N::out(frxl + sl * (rxst[0] - rxl));
    f[3] = N::out(fryl + sl * (ryst[0] - ryl));
    f[4] = N::out(frzl + sl * (rzst[0] - rzl));
    f[1] = N::out(feel + sl * (eest[0] - eel));
    f[5] = N::out(fbyl + sl * (byst[0] - byl));
    f[6] = N::out(fbzl + sl * (bzst[0] - bzl));
  } else if (N::ge0(sm)) {
    const T temp = slst - sl;
    const T byd0 = zb ? byst[0] : byd, bzd0 = zb ? bzst[0] : bzd;
    f[0] = N::out(frol - sl * rol - temp * rost[0] + slst * rost[0]);
    f[2] = N::out(frxl - sl * rxl - temp * rxst[0] + slst * rxst[0]);
    f[3] = N::out(fryl - sl * ryl - temp * ryst[0] + slst * ryd[0]);
    f[4] = N::out(frzl - sl * rzl - temp * rzst[0] + slst * rzd[0]);
    f[1] = N::out(feel - sl * eel - temp * eest[0] + slst * eed[0]);
    f[5] = N::out(fbyl - sl * byl - temp * byst[0] + slst * byd0);
    f[6] = N::out(fbzl - sl * bzl - temp * bzst[0] + slst * bzd0);
  } else if (N::gt0(srst)) {
    const T temp = srst - sr;
    const T byd1 = zb ? byst[1] : byd, bzd1 = zb ? bzst[1] : bzd;
    f[0] = N::out(fror - sr * ror - temp * rost[1] + srst * rost[1]);
    f[2] = N::out(frxr - sr * rxr - temp * rxst[1] + srst * rxst[1]);
    f[3] = N::out(fryr - sr * ryr - temp * ryst[1] + srst * ryd[1]);
    f[4] = N::out(frzr - sr * rzr - temp * rzst[1] + srst * rzd[1]);
    f[1] = N::out(feer - sr * eer - temp * eest[1] + srst * eed[1]);
    f[5] = N::out(fbyr - sr * byr - temp * byst[1] + srst * byd1);
    f[6] = N::out(fbzr - sr * bzr - temp * bzst[1] + srst * bzd1);
  } else {
    f[0] = N::out(fror + sr * (rost[1] - ror));
    f[2] = N::out(frxr + sr * (rxst[1] - rxr));
    f[3] = N::out(fryr + sr * (ryst[1] - ryr));
    f[4] = N::out(frzr + sr * (rzst[1] - rzr));
    f[1] = N::out(feer + sr * (eest[1] - eer));
    f[5] = N::out(fbyr + sr * (byst[1] - byr));
    f[6] = N::out(fbzr + sr * (bzst[1] - bzr));
  }
}

template <bool E>
__device__ __forceinline__ void hlld_flux(const HlldK &K, const double *L,
                                          const double *R, double bxv,
                                          double *f) {
  hlld_flux_t<F<E>>(K, L, R, bxv, f);
}

}  // namespace cans
