// HLLD flux of one face on the device:
// cansxx-nosupport/hdhlld/hlld_flux.f90:148-480 (Miyoshi & Kusano, J. Comput.
// Phys. 208, 315 (2005)), Heaviside units (pb = B^2/2).
//
// Face states in the frame of the face normal: (ro, pr, vn, vt1, vt2, bn,
// bt1, bt2) with bn unused -- the normal field is the face value bxs; the
// flux comes back as (ro, ee, rn, rt1, rt2, bt1, bt2).
//
// E=true evaluates the expressions in the Fortran order with separately
// rounded operations.  E=false uses the same expressions with FMA
// contraction and reciprocals in place of the repeated divisions.
#pragma once
#include "cans_common.cuh"
#include "roe_flux.cuh"  // fmax_, fsign_

namespace cans {

struct HlldK {
  double gm, gm1;   // gm, gm-1
  double zfloor;    // hlld_mh.f:34
  double gm1i;      // fast policy: 1/(gm-1)
};

template <bool E>
__device__ __forceinline__ void hlld_flux(const HlldK &K, const double *L,
                                          const double *R, double bxv,
                                          double *f) {
  using T = F<E>;
  const T gm(K.gm), gm1(K.gm1), zf(K.zfloor);
  const T bxs(bxv);
  const T bxsq = bxs * bxs;
  // left and right states (:152-191)
  const T rol(L[0]), prl(L[1]), vxl(L[2]), vyl(L[3]), vzl(L[4]), byl(L[6]), bzl(L[7]);
  const T ror(R[0]), prr(R[1]), vxr(R[2]), vyr(R[3]), vzr(R[4]), byr(R[6]), bzr(R[7]);
  const T pbl = T(0.5) * (bxs * bxs + byl * byl + bzl * bzl);
  const T ptl = prl + pbl;
  T eel, eer;
  if constexpr (E) {
    eel = prl / gm1 + T(0.5) * rol * (vxl * vxl + vyl * vyl + vzl * vzl) + pbl;
  } else {
    eel = prl * T(K.gm1i) + T(0.5) * rol * (vxl * vxl + vyl * vyl + vzl * vzl) + pbl;
  }
  const T rxl = rol * vxl, ryl = rol * vyl, rzl = rol * vzl;
  const T pbr = T(0.5) * (bxs * bxs + byr * byr + bzr * bzr);
  const T ptr = prr + pbr;
  if constexpr (E) {
    eer = prr / gm1 + T(0.5) * (ror * (vxr * vxr + vyr * vyr + vzr * vzr)) + pbr;
  } else {
    eer = prr * T(K.gm1i) + T(0.5) * (ror * (vxr * vxr + vyr * vyr + vzr * vzr)) + pbr;
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
  // supersonic cases (:235-255)
  if (sl.v >= 0.0) {
    f[0] = frol.v; f[1] = feel.v; f[2] = frxl.v; f[3] = fryl.v; f[4] = frzl.v;
    f[5] = fbyl.v; f[6] = fbzl.v;
    return;
  }
  if (sr.v <= 0.0) {
    f[0] = fror.v; f[1] = feer.v; f[2] = frxr.v; f[3] = fryr.v; f[4] = frzr.v;
    f[5] = fbyr.v; f[6] = fbzr.v;
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
    const T di = T(1.0) / den;
    sm = (sdr * ror * vxr - sdl * rol * vxl - ptr + ptl) * di;
    ptst = (sdr * ror * ptl - sdl * rol * ptr + rol * ror * sdr * sdl * (vxr - vxl)) * di;
  }
  const T sdml = sl - sm, sdmr = sr - sm;
  // one-sided star state (:281-342); side 0 left, 1 right
  T rost[2], rxst[2], ryst[2], rzst[2], vyst[2], vzst[2], byst[2], bzst[2], eest[2];
  T vdbst[2];
#pragma unroll
  for (int s = 0; s < 2; s++) {
    const T ro = s ? ror : rol, vx = s ? vxr : vxl, vy = s ? vyr : vyl, vz = s ? vzr : vzl;
    const T by = s ? byr : byl, bz = s ? bzr : bzl, pt = s ? ptr : ptl, ee = s ? eer : eel;
    const T sd = s ? sdr : sdl, sdm = s ? sdmr : sdml;
    const T temp_fst = ro * sd * sdm - bxsq;
    const T s3 = fsign_(T(1.0), temp_fst + zf) * fsign_(T(1.0), temp_fst - zf);
    const T mx = fmax_(T(0.0), s3), mn = fmin_(T(0.0), s3);
    const T dd = temp_fst + mn;
    T tmp, tmp2, rsd, esd;
    if constexpr (E) {
      tmp = bxs * (sd - sdm) / dd;
      tmp2 = (ro * (sd * sd) - bxsq) / dd;
      rsd = ro * sd / sdm;
    } else {
      const T ddi = T(1.0) / dd;
      tmp = bxs * (sd - sdm) * ddi;
      tmp2 = (ro * (sd * sd) - bxsq) * ddi;
      rsd = ro * sd * (T(1.0) / sdm);
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
    else esd = num * (T(1.0) / sdm);
    eest[s] = mx * esd - mn * ee;
  }
  // double-star states (:347-414)
  const T sqrtrol = fsqrt(rost[0]), sqrtror = fsqrt(rost[1]);
  T slst, srst;
  if constexpr (E) {
    slst = sm - fabs_(bxs) / sqrtrol;
    srst = sm + fabs_(bxs) / sqrtror;
  } else {
    slst = sm - fabs_(bxs) * (T(1.0) / sqrtrol);
    srst = sm + fabs_(bxs) * (T(1.0) / sqrtror);
  }
  T ryd[2], rzd[2], byd, bzd, eed[2];
  if (bxv == 0.0) {
    ryd[0] = ryst[0]; ryd[1] = ryst[1];
    rzd[0] = rzst[0]; rzd[1] = rzst[1];
    eed[0] = eest[0]; eed[1] = eest[1];
    byd = byst[0];  // unused: the flux takes byst of each side below
    bzd = bzst[0];
  } else {
    const T invsumro = T(1.0) / (sqrtrol + sqrtror);
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
  if (slst.v >= 0.0) {
    f[0] = (frol + sl * (rost[0] - rol)).v;
    f[2] = (frxl + sl * (rxst[0] - rxl)).v;
    f[3] = (fryl + sl * (ryst[0] - ryl)).v;
    f[4] = (frzl + sl * (rzst[0] - rzl)).v;
    f[1] = (feel + sl * (eest[0] - eel)).v;
    f[5] = (fbyl + sl * (byst[0] - byl)).v;
    f[6] = (fbzl + sl * (bzst[0] - bzl)).v;
  } else if (sm.v >= 0.0) {
    const T temp = slst - sl;
    const T byd0 = zb ? byst[0] : byd, bzd0 = zb ? bzst[0] : bzd;
    f[0] = (frol - sl * rol - temp * rost[0] + slst * rost[0]).v;
    f[2] = (frxl - sl * rxl - temp * rxst[0] + slst * rxst[0]).v;
    f[3] = (fryl - sl * ryl - temp * ryst[0] + slst * ryd[0]).v;
    f[4] = (frzl - sl * rzl - temp * rzst[0] + slst * rzd[0]).v;
    f[1] = (feel - sl * eel - temp * eest[0] + slst * eed[0]).v;
    f[5] = (fbyl - sl * byl - temp * byst[0] + slst * byd0).v;
    f[6] = (fbzl - sl * bzl - temp * bzst[0] + slst * bzd0).v;
  } else if (srst.v > 0.0) {
    const T temp = srst - sr;
    const T byd1 = zb ? byst[1] : byd, bzd1 = zb ? bzst[1] : bzd;
    f[0] = (fror - sr * ror - temp * rost[1] + srst * rost[1]).v;
    f[2] = (frxr - sr * rxr - temp * rxst[1] + srst * rxst[1]).v;
    f[3] = (fryr - sr * ryr - temp * ryst[1] + srst * ryd[1]).v;
    f[4] = (frzr - sr * rzr - temp * rzst[1] + srst * rzd[1]).v;
    f[1] = (feer - sr * eer - temp * eest[1] + srst * eed[1]).v;
    f[5] = (fbyr - sr * byr - temp * byst[1] + srst * byd1).v;
    f[6] = (fbzr - sr * bzr - temp * bzst[1] + srst * bzd1).v;
  } else {
    f[0] = (fror + sr * (rost[1] - ror)).v;
    f[2] = (frxr + sr * (rxst[1] - rxr)).v;
    f[3] = (fryr + sr * (ryst[1] - ryr)).v;
    f[4] = (frzr + sr * (rzst[1] - rzr)).v;
    f[1] = (feer + sr * (eest[1] - eer)).v;
    f[5] = (fbyr + sr * (byst[1] - byr)).v;
    f[6] = (fbzr + sr * (bzst[1] - bzr)).v;
  }
}

}  // namespace cans
