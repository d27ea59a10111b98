/*
 * 3-D Roe-MUSCL step: line-faithful C restatement of the CANS Fortran
 * (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 *   roe_m      cans3d/hdroe/roe_m.f:2-340      two-stage driver
 *   roeflux_m  cans3d/hdroe/roeflux_m.f:6-270  Roe flux of one face
 *   tvdminmod  cans3d/hdroe/tvdminmod.f:4-58   minmod MUSCL reconstruction
 *
 * The reference keeps the half-step primitives prh, vxh, vyh, vzh unset on
 * the outer layer of cells (an index equal to 1 or n; roe_m.f:222-233 only
 * fills 2..n-1), and tvdminmod reads that layer for the faces 2 and n-2
 * (tvdminmod.f:22-25).  Those faces feed only the cells with an index 3 or
 * n-2, which are boundary cells when margin = 3 (hdroe main.f:5) and are
 * rewritten by the boundary fill after every step.  This restatement gives
 * the unset values a definite content -- the input primitives of the same
 * cell -- so that every cell of its output is reproducible; cells away from
 * that layer do not depend on the choice.
 *
 * roeflux_m evaluates every face of the box 1..n-1 in all three indices; the
 * corrector here evaluates the faces that tvdminmod reconstructs (2..n-2 in
 * all three indices, tvdminmod.f:19-21), which contain every face the
 * updates of roe_m.f:253-321 read.  The predictor evaluates the box of the
 * reference.
 */
#include "oracle.h"
#include "oracle_common.h"

static oracle_arena arena_roe;

#define A(a, i, j, k) a[I3(i, j, k)]

/* Fortran sign(a, b) for a >= 0: |a| carrying the sign of b. */
static inline double fsign(double a, double b) { return copysign(fabs(a), b); }

/* roeflux_m.f:29-263 for one face.  L and R hold (ro, pr, vn, vt1, vt2, bn,
 * bt1, bt2) of the two sides in the frame of the face normal; f receives
 * (fro, fee, frn, frt1, frt2, fbt1, fbt2).  fix = 1 is the 3-D routine;
 * fix = 0 is roeflux_m3.f of cans1d/cans2d, whose slow-wave normalisation
 * lacks the "+ 1 - sp2" of roeflux_m.f:79 (cans2d/hdroe/roeflux_m3.f:77). */
void oracle_roe_face(double gm, const double *L, const double *R, double *f, int fix) {
  const double pi = acos(-1.0);
  const double pi4 = 4.0 * pi;
  const double pi4i = 1.0 / pi4;
  const double pi8i = 5.0e-1 * pi4i;
  const double rhol = L[0], prl = L[1], vxl = L[2], vyl = L[3], vzl = L[4];
  const double bxl = L[5], byl = L[6], bzl = L[7];
  const double rhor = R[0], prr = R[1], vxr = R[2], vyr = R[3], vzr = R[4];
  const double bxr = R[5], byr = R[6], bzr = R[7];

  /* roe's variable (:47-61) */
  double sr0 = sqrt(rhol);
  double sr1 = sqrt(rhor);
  double sri = 1.0 / (sr0 + sr1);
  double rhobar = sr0 * sr1;
  double vxbar = (sr0 * vxl + sr1 * vxr) * sri;
  double vybar = (sr0 * vyl + sr1 * vyr) * sri;
  double vzbar = (sr0 * vzl + sr1 * vzr) * sri;
  double bxbar = (sr0 * bxr + sr1 * bxl) * sri;
  double bybar = (sr0 * byr + sr1 * byl) * sri;
  double bzbar = (sr0 * bzr + sr1 * bzl) * sri;
  double hl = 0.5 * (vxl * vxl + vyl * vyl + vzl * vzl) + gm * prl / ((gm - 1.0) * rhol) +
              (bxbar * bxbar + byl * byl + bzl * bzl) / (pi4 * rhol);
  double hr = 0.5 * (vxr * vxr + vyr * vyr + vzr * vzr) + gm * prr / ((gm - 1.0) * rhor) +
              (bxbar * bxbar + byr * byr + bzr * bzr) / (pi4 * rhor);
  double hbar = (sr0 * hl + sr1 * hr) * sri;

  /* average (:64-65) */
  double byave = (byl + byr) / 2.0;
  double bzave = (bzl + bzr) / 2.0;

  /* characteristic speed (:68-82) */
  double delb2 = (gm - 2.0) / (gm - 1.0) *
                 ((byr - byl) * (byr - byl) + (bzr - bzl) * (bzr - bzl)) * (sri * sri) * pi8i;
  double vb2 = vxbar * vxbar + vybar * vybar + vzbar * vzbar;
  double bb2 = bxbar * bxbar + bybar * bybar + bzbar * bzbar;
  double cs2 = (gm - 1.0) * (hbar - 0.5 * vb2 - delb2 - bb2 * pi4i / rhobar);
  double astar2 = (gm - 1.0) * (hbar - 0.5 * vb2 - delb2) - (gm - 2.0) * bb2 * pi4i / rhobar;
  double ca2 = bxbar * bxbar / (pi4 * rhobar);
  double cbr2 = (bybar * bybar + bzbar * bzbar) * pi4i / rhobar;
  double cfast2 = 0.5 * (astar2 + sqrt(cbr2 * (astar2 + cs2 + ca2) + (cs2 - ca2) * (cs2 - ca2)));
  double cslow2 = cs2 * ca2 / cfast2;
  double cfast = sqrt(cfast2);
  double cslow = sqrt(cslow2);
  double ca = sqrt(ca2);
  double cs = sqrt(cs2);

  /* for singular points (:85-100) */
  double epsi = 1.0e-12;
  double sgr = bybar * bybar + bzbar * bzbar - epsi;
  double sp = 0.5 + fsign(0.5, sgr);
  double betay = sp * bybar * sqrt(1.0 / (bybar * bybar + bzbar * bzbar + 1.0 - sp)) +
                 sqrt(0.5) * (1.0 - sp);
  double betaz = sp * bzbar * sqrt(1.0 / (bybar * bybar + bzbar * bzbar + 1.0 - sp)) +
                 sqrt(0.5) * (1.0 - sp);
  double eps2 = 1.0e-12;
  double sgr2 = (bybar * bybar + bzbar * bzbar) / (pi4 * rhobar) + fabs(ca2 - cs2) - eps2;
  double sp2 = 0.5 + fsign(0.5, sgr2);
  double cfca = fmax2(0.0, cfast2 - ca2);
  double cfcs = fmax2(0.0, cfast2 - cslow2);
  double cfa = fmax2(0.0, cfast2 - cs2);
  double alphf = sp2 * sqrt(cfca / (cfcs + 1.0 - sp2)) + 1.0 - sp2;
  double alphs = sp2 * sqrt(cfa / (cfcs + 1.0 - sp2));
  if (fix) alphs = alphs + 1.0 - sp2;
  double sgnbx = fsign(1.0, bxbar);

  /* eigen value & entropy condition (:103-110) */
  double eeps = (vxr - vxl + fabs(vxr - vxl)) * 2.5e-1;
  double elpf = -fmax2(fabs(vxbar + cfast), eeps);
  double elmf = -fmax2(fabs(vxbar - cfast), eeps);
  double elps = -fmax2(fabs(vxbar + cslow), eeps);
  double elms = -fmax2(fabs(vxbar - cslow), eeps);
  double elpa = -fmax2(fabs(vxbar + ca), eeps);
  double elma = -fmax2(fabs(vxbar - ca), eeps);
  double elze = -fmax2(fabs(vxbar), eeps);

  /* amplitude; w's (:113-142) */
  double drho = rhor - rhol;
  double du21 = rhobar * (vxr - vxl);
  double du31 = rhobar * (vyr - vyl);
  double du41 = rhobar * (vzr - vzl);
  double du6 = byr - byl;
  double du5 = bzr - bzl;
  double t1 = betay * du6 + betaz * du5;
  double t2 = (prr - prl + (byave * du6 + bzave * du5) * pi4i +
               (gm - 2.0) * (bybar * du6 + bzbar * du5) * pi4i) /
              (gm - 1.0);
  double t3 = betaz * du6 - betay * du5;
  double s1 = du21;
  double s2 = betay * du31 + betaz * du41;
  double s3 = betaz * du31 - betay * du41;
  double sq4r = sqrt(pi4 / rhobar);
  double p11 = alphs * cfast * sq4r;
  double p12 = -(alphf * cs2 / cfast * sq4r);
  double p21 = alphf * (cfast2 - cs2 * (gm - 2.0) / (gm - 1.0));
  double p22 = alphs * (cslow2 - cs2 * (gm - 2.0) / (gm - 1.0));
  double q11 = alphf * cfast;
  double q12 = alphs * cslow;
  double q21 = -(alphs * ca * sgnbx);
  double q22 = alphf * cs * sgnbx;
  double detp = p11 * p22 - p12 * p21;
  double detq = q11 * q22 - q12 * q21;
  double wpf = 0.5 * ((p22 * t1 - p12 * t2) / detp + (q22 * s1 - q12 * s2) / detq);
  double wmf = 0.5 * ((p22 * t1 - p12 * t2) / detp - (q22 * s1 - q12 * s2) / detq);
  double wps = 0.5 * ((-(p21 * t1) + p11 * t2) / detp + (-(q21 * s1) + q11 * s2) / detq);
  double wms = 0.5 * ((-(p21 * t1) + p11 * t2) / detp - (-(q21 * s1) + q11 * s2) / detq);
  double wpa = 0.5 * (sqrt(rhobar * pi4i) * t3 - sgnbx * s3);
  double wma = 0.5 * (sqrt(rhobar * pi4i) * t3 + sgnbx * s3);
  double wze = drho - alphf * (wpf + wmf) - alphs * (wps + wms);

  /* physical fluxes of both sides (:145-158) */
  double fluxlro = rhol * vxl;
  double fluxlrx = rhol * vxl * vxl + prl + (-(bxbar * bxbar) + byl * byl + bzl * bzl) * pi8i;
  double fluxlry = rhol * vxl * vyl - bxbar * byl * pi4i;
  double fluxlrz = rhol * vxl * vzl - bxbar * bzl * pi4i;
  double fluxlby = vxl * byl - vyl * bxbar;
  double fluxlbz = vxl * bzl - vzl * bxbar;
  double fluxlee = rhol * vxl * hl - bxbar * (bxbar * vxl + byl * vyl + bzl * vzl) * pi4i;
  double fluxrro = rhor * vxr;
  double fluxrrx = rhor * vxr * vxr + prr + (-(bxbar * bxbar) + byr * byr + bzr * bzr) * pi8i;
  double fluxrry = rhor * vxr * vyr - bxbar * byr * pi4i;
  double fluxrrz = rhor * vxr * vzr - bxbar * bzr * pi4i;
  double fluxrby = vxr * byr - vyr * bxbar;
  double fluxrbz = vxr * bzr - vzr * bxbar;
  double fluxree = rhor * vxr * hr - bxbar * (bxbar * vxr + byr * vyr + bzr * vzr) * pi4i;

  /* right eigenvectors (:161-227) */
  double bv = betay * vybar + betaz * vzbar;
  double rpfro = alphf;
  double rpfrx = alphf * (vxbar + cfast);
  double rpfry = alphf * vybar - alphs * betay * ca * sgnbx;
  double rpfrz = alphf * vzbar - alphs * betaz * ca * sgnbx;
  double rpfby = alphs * betay * cfast * sq4r;
  double rpfbz = alphs * betaz * cfast * sq4r;
  double rpfee = alphf * (0.5 * vb2 + delb2 + cfast * vxbar + cfast2 / (gm - 1.0) +
                          (cfast2 - cs2) * (gm - 2.0) / (gm - 1.0)) -
                 alphs * ca * bv * sgnbx;
  double rmfro = alphf;
  double rmfrx = alphf * (vxbar - cfast);
  double rmfry = alphf * vybar + alphs * betay * ca * sgnbx;
  double rmfrz = alphf * vzbar + alphs * betaz * ca * sgnbx;
  double rmfby = rpfby;
  double rmfbz = rpfbz;
  double rmfee = alphf * (0.5 * vb2 + delb2 - cfast * vxbar + cfast2 / (gm - 1.0) +
                          (cfast2 - cs2) * (gm - 2.0) / (gm - 1.0)) +
                 alphs * ca * bv * sgnbx;
  double rpsro = alphs;
  double rpsrx = alphs * (vxbar + cslow);
  double rpsry = alphs * vybar + cs * sgnbx * alphf * betay;
  double rpsrz = alphs * vzbar + cs * sgnbx * alphf * betaz;
  double rpsby = -(sq4r * cs2 * alphf * betay / cfast);
  double rpsbz = -(sq4r * cs2 * alphf * betaz / cfast);
  double rpsee = alphs * (0.5 * vb2 + delb2 + cslow * vxbar + cslow2 / (gm - 1.0) +
                          (cslow2 - cs2) * (gm - 2.0) / (gm - 1.0)) +
                 alphf * cs * bv * sgnbx;
  double rmsro = alphs;
  double rmsrx = alphs * (vxbar - cslow);
  double rmsry = alphs * vybar - cs * sgnbx * alphf * betay;
  double rmsrz = alphs * vzbar - cs * sgnbx * alphf * betaz;
  double rmsby = rpsby;
  double rmsbz = rpsbz;
  double rmsee = alphs * (0.5 * vb2 + delb2 - cslow * vxbar + cslow2 / (gm - 1.0) +
                          (cslow2 - cs2) * (gm - 2.0) / (gm - 1.0)) -
                 alphf * cs * bv * sgnbx;
  double rparo = 0.0;
  double rparx = 0.0;
  double rpary = -(sgnbx * betaz);
  double rparz = sgnbx * betay;
  double rpaby = sq4r * betaz;
  double rpabz = -(sq4r * betay);
  double rpaee = -((betaz * vybar - betay * vzbar) * sgnbx);
  double rmaro = 0.0;
  double rmarx = 0.0;
  double rmary = -rpary;
  double rmarz = -rparz;
  double rmaby = rpaby;
  double rmabz = rpabz;
  double rmaee = -rpaee;
  double rzero = 1.0;
  double rzerx = vxbar;
  double rzery = vybar;
  double rzerz = vzbar;
  double rzeby = 0.0;
  double rzebz = 0.0;
  double rzeee = 0.5 * vb2 + delb2;

  /* f(i+1/2) (:230-263) */
  double pf = elpf * wpf, mf = elmf * wmf, ps = elps * wps, ms = elms * wms;
  double pa = elpa * wpa, ma = elma * wma, ze = elze * wze;
#define ROE_SUM(FL, FR, P, M, PS, MS, PA, MA, Z)                                 \
  (0.5 * (FL + FR + pf * P + mf * M + ps * PS + ms * MS + pa * PA + ma * MA + ze * Z))
  f[0] = ROE_SUM(fluxlro, fluxrro, rpfro, rmfro, rpsro, rmsro, rparo, rmaro, rzero);
  f[1] = ROE_SUM(fluxlee, fluxree, rpfee, rmfee, rpsee, rmsee, rpaee, rmaee, rzeee);
  f[2] = ROE_SUM(fluxlrx, fluxrrx, rpfrx, rmfrx, rpsrx, rmsrx, rparx, rmarx, rzerx);
  f[3] = ROE_SUM(fluxlry, fluxrry, rpfry, rmfry, rpsry, rmsry, rpary, rmary, rzery);
  f[4] = ROE_SUM(fluxlrz, fluxrrz, rpfrz, rmfrz, rpsrz, rmsrz, rparz, rmarz, rzerz);
  f[5] = ROE_SUM(fluxlby, fluxrby, rpfby, rmfby, rpsby, rmsby, rpaby, rmaby, rzeby);
  f[6] = ROE_SUM(fluxlbz, fluxrbz, rpfbz, rmfbz, rpsbz, rmsbz, rpabz, rmabz, rzebz);
#undef ROE_SUM
}

/* Variable order of the state and of the reconstructed face states:
 * ro, pr, vx, vy, vz, bx, by, bz.  Flux order: ro, ee, rx, ry, rz, bx, by,
 * bz (the normal-B flux of an axis is never written). */
enum { V_RO, V_PR, V_VX, V_VY, V_VZ, V_BX, V_BY, V_BZ };
enum { F_RO, F_EE, F_RX, F_RY, F_RZ, F_BX, F_BY, F_BZ };

/* Rotation of roe_m.f:96,146,196: the normal, first and second tangential
 * components of an axis. */
static const int rot[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};

/* Roe fluxes of the faces (c, c + e_axis) for c in [lo, hi] per index.
 * wl / wr give the 8 variables of the left / right face states at c. */
static void roeflux_axis(double *const *fl, double gm, const double *const *wl,
                         const double *const *wr, int axis, const int lo[3],
                         const int hi[3], int ix, int jx, int kx) {
  const int *r = rot[axis];
  OMP_FOR
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        const size_t c = I3(i, j, k);
        double L[8], R[8], f[7];
        L[0] = wl[V_RO][c];
        L[1] = wl[V_PR][c];
        R[0] = wr[V_RO][c];
        R[1] = wr[V_PR][c];
        for (int m = 0; m < 3; m++) {
          L[2 + m] = wl[V_VX + r[m]][c];
          L[5 + m] = wl[V_BX + r[m]][c];
          R[2 + m] = wr[V_VX + r[m]][c];
          R[5 + m] = wr[V_BX + r[m]][c];
        }
        oracle_roe_face(gm, L, R, f, 1);
        fl[F_RO][c] = f[0];
        fl[F_EE][c] = f[1];
        for (int m = 0; m < 3; m++) fl[F_RX + r[m]][c] = f[2 + m];
        fl[F_BX + r[1]][c] = f[5];
        fl[F_BX + r[2]][c] = f[6];
      }
}

/* tvdminmod.f:15 */
static inline double flmt(double a, double b) {
  const double s = fsign(1.0, a);
  return fmax2(0.0, fmin2(b * s, fabs(a))) * s;
}

/* tvdminmod.f:18-55 on one variable: left / right states of the faces
 * (c, c + e_axis) for c in 2..n-2 in every index. */
static void tvdminmod3(int axis, const double *da, double *dl, double *dr, int ix,
                       int jx, int kx) {
  const size_t st = axis == 0 ? 1 : (axis == 1 ? (size_t)ix : (size_t)ix * jx);
  OMP_FOR
  for (int k = 2; k <= kx - 2; k++)
    for (int j = 2; j <= jx - 2; j++)
      for (int i = 2; i <= ix - 2; i++) {
        const size_t c = I3(i, j, k);
        const double dm = da[c - st], d0 = da[c], d1 = da[c + st], d2 = da[c + 2 * st];
        dl[c] = d0 + 0.5 * flmt(d0 - dm, d1 - d0);
        dr[c] = d1 - 0.5 * flmt(d2 - d1, d1 - d0);
      }
}

void oracle_roe_m_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                     double *bx, double *by, double *bz, double dt, double gm,
                     const double *dx, int ix, const double *dy, int jx,
                     const double *dz, int kx) {
  const size_t n = (size_t)ix * jx * kx;
  /* arena: ee rx ry rz | 8 conserved half | 8 primitive half | 8 fluxes |
   * 8 left + 8 right face states */
  double *w = arena_get(&arena_roe, n * 44);
  double *ee = w, *rx = w + n, *ry = w + 2 * n, *rz = w + 3 * n;
  double *cons_h = w + 4 * n;  /* roh eeh rxh ryh rzh bxh byh bzh */
  double *prim_h = w + 12 * n; /* roh prh vxh vyh vzh bxh byh bzh */
  double *flx = w + 20 * n;
  double *wl = w + 28 * n, *wr = w + 36 * n;
  double *P[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  double *Fl[8], *Wl[8], *Wr[8], *Hc[8], *Hp[8];
  for (int v = 0; v < 8; v++) {
    Fl[v] = flx + v * n;
    Wl[v] = wl + v * n;
    Wr[v] = wr + v * n;
    Hc[v] = cons_h + v * n;
    Hp[v] = prim_h + v * n;
  }
  const double pi = acos(-1.0);
  const double pi4 = 4.0 * pi;
  const double pi4i = 1.0 / pi4;
  const double pi8i = 5.0e-1 * pi4i;
  const double *dd[3] = {dx, dy, dz};
  const size_t st[3] = {1, (size_t)ix, (size_t)ix * jx};

  /* conservative variables (roe_m.f:39-50) and the half-step copies (:55-68) */
  OMP_FOR
  for (size_t c = 0; c < n; c++) {
    rx[c] = ro[c] * vx[c];
    ry[c] = ro[c] * vy[c];
    rz[c] = ro[c] * vz[c];
    double v2 = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
    double b2 = bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c];
    ee[c] = pr[c] / (gm - 1.0) + 0.5 * ro[c] * v2 + pi8i * b2;
    Hc[F_RO][c] = ro[c];
    Hc[F_EE][c] = ee[c];
    Hc[F_RX][c] = rx[c];
    Hc[F_RY][c] = ry[c];
    Hc[F_RZ][c] = rz[c];
    Hc[F_BX][c] = bx[c];
    Hc[F_BY][c] = by[c];
    Hc[F_BZ][c] = bz[c];
  }

  /* predictor: first-order fluxes and the dt/2 update (roe_m.f:73-218) */
  const int lo1[3] = {1, 1, 1}, hi1[3] = {ix - 1, jx - 1, kx - 1};
  for (int a = 0; a < 3; a++) {
    const size_t nf = n - st[a];
    for (int v = 0; v < 8; v++) {  /* L = cell c, R = cell c + e_a */
      OMP_FOR
      for (size_t c = 0; c < nf; c++) {
        Wl[v][c] = P[v][c];
        Wr[v][c] = P[v][c + st[a]];
      }
    }
    roeflux_axis(Fl, gm, (const double *const *)Wl, (const double *const *)Wr, a,
                 lo1, hi1, ix, jx, kx);
    OMP_FOR
    for (int k = 2; k <= kx - 1; k++)
      for (int j = 2; j <= jx - 1; j++)
        for (int i = 2; i <= ix - 1; i++) {
          const size_t c = I3(i, j, k);
          const int ic[3] = {i, j, k};
          const double h = dd[a][I1(ic[a])];
          for (int v = 0; v < 8; v++) {
            if (v == F_BX + a) continue;
            Hc[v][c] = Hc[v][c] + 0.5 * dt * ((Fl[v][c - st[a]] - Fl[v][c]) / h);
          }
        }
  }

  /* primitives of the half step (:222-233); the outer layer keeps the input
   * primitives (see the header) */
  OMP_FOR
  for (int k = 1; k <= kx; k++)
    for (int j = 1; j <= jx; j++)
      for (int i = 1; i <= ix; i++) {
        const size_t c = I3(i, j, k);
        Hp[V_RO][c] = Hc[F_RO][c];
        Hp[V_BX][c] = Hc[F_BX][c];
        Hp[V_BY][c] = Hc[F_BY][c];
        Hp[V_BZ][c] = Hc[F_BZ][c];
        if (i == 1 || i == ix || j == 1 || j == jx || k == 1 || k == kx) {
          Hp[V_PR][c] = pr[c];
          Hp[V_VX][c] = vx[c];
          Hp[V_VY][c] = vy[c];
          Hp[V_VZ][c] = vz[c];
          continue;
        }
        double vxh = Hc[F_RX][c] / Hc[F_RO][c];
        double vyh = Hc[F_RY][c] / Hc[F_RO][c];
        double vzh = Hc[F_RZ][c] / Hc[F_RO][c];
        double v2 = vxh * vxh + vyh * vyh + vzh * vzh;
        double b2 = Hc[F_BX][c] * Hc[F_BX][c] + Hc[F_BY][c] * Hc[F_BY][c] +
                    Hc[F_BZ][c] * Hc[F_BZ][c];
        Hp[V_VX][c] = vxh;
        Hp[V_VY][c] = vyh;
        Hp[V_VZ][c] = vzh;
        Hp[V_PR][c] = (gm - 1.0) * (Hc[F_EE][c] - 0.5 * Hc[F_RO][c] * v2 - pi8i * b2);
      }

  /* corrector: minmod states, Roe fluxes and the dt update (:241-321) */
  double *U[8] = {ro, ee, rx, ry, rz, bx, by, bz};
  const int lo2[3] = {2, 2, 2}, hi2[3] = {ix - 2, jx - 2, kx - 2};
  for (int a = 0; a < 3; a++) {
    for (int v = 0; v < 8; v++) tvdminmod3(a, Hp[v], Wl[v], Wr[v], ix, jx, kx);
    roeflux_axis(Fl, gm, (const double *const *)Wl, (const double *const *)Wr, a,
                 lo2, hi2, ix, jx, kx);
    OMP_FOR
    for (int k = 3; k <= kx - 2; k++)
      for (int j = 3; j <= jx - 2; j++)
        for (int i = 3; i <= ix - 2; i++) {
          const size_t c = I3(i, j, k);
          const int ic[3] = {i, j, k};
          const double h = dd[a][I1(ic[a])];
          for (int v = 0; v < 8; v++) {
            if (v == F_BX + a) continue;
            U[v][c] = U[v][c] + dt * ((Fl[v][c - st[a]] - Fl[v][c]) / h);
          }
        }
  }

  /* primitives of the full step (:325-336) */
  OMP_FOR
  for (int k = 3; k <= kx - 2; k++)
    for (int j = 3; j <= jx - 2; j++)
      for (int i = 3; i <= ix - 2; i++) {
        const size_t c = I3(i, j, k);
        vx[c] = rx[c] / ro[c];
        vy[c] = ry[c] / ro[c];
        vz[c] = rz[c] / ro[c];
        double v2 = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
        double b2 = bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c];
        pr[c] = (gm - 1.0) * (ee[c] - 0.5 * ro[c] * v2 - pi8i * b2);
      }
}
