/*
 * 1-D Roe-MUSCL step: line-faithful C restatement of the CANS Fortran
 * (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 *   roe_m      cans1d/hdroe/roe_m.f:2-136        two-stage driver
 *   roeflux_m  cans1d/hdroe/roeflux_m.f:2-245    two-component Roe flux
 *   tvdminmod  cans1d/hdroe/tvdminmod.f:2-43     minmod MUSCL reconstruction
 *
 * The half-step primitives the reference leaves unset on the end cells
 * (roe_m.f:57-64 fills 2..ix-1) hold the input primitives here; only the
 * cells 3 and ix-2 (boundary cells at margin 3) depend on them.  The
 * corrector evaluates the faces tvdminmod reconstructs (2..ix-2), which are
 * every face the update of roe_m.f:75-81 reads.
 */
#include "oracle.h"
#include "oracle_common.h"

static oracle_arena arena_roe1;

static inline double fsign1(double a, double b) { return copysign(fabs(a), b); }

/* roeflux_m.f:15-236 for one face: L, R = (ro, pr, vx, vy, bx, by);
 * f = (fro, fee, frx, fry, fby) */
static void roe_face1(double gm, const double *L, const double *R, double *f) {
  const double pi = acos(-1.0);
  const double pi4 = 4.0 * pi;
  const double pi4i = 1.0 / pi4;
  const double pi8i = 5.0e-1 * pi4i;
  const double rhol = L[0], prl = L[1], vxl = L[2], vyl = L[3], bxl = L[4], byl = L[5];
  const double rhor = R[0], prr = R[1], vxr = R[2], vyr = R[3], bxr = R[4], byr = R[5];
  double sr0 = sqrt(rhol);
  double sr1 = sqrt(rhor);
  double sri = 1.0 / (sr0 + sr1);
  double rhobar = sr0 * sr1;
  double vxbar = (sr0 * vxl + sr1 * vxr) * sri;
  double vybar = (sr0 * vyl + sr1 * vyr) * sri;
  double bxbar = (sr0 * bxr + sr1 * bxl) * sri;
  double bybar = (sr0 * byr + sr1 * byl) * sri;
  double hl = 0.5 * (vxl * vxl + vyl * vyl) + gm * prl / ((gm - 1.0) * rhol) +
              (bxbar * bxbar + byl * byl) / (pi4 * rhol);
  double hr = 0.5 * (vxr * vxr + vyr * vyr) + gm * prr / ((gm - 1.0) * rhor) +
              (bxbar * bxbar + byr * byr) / (pi4 * rhor);
  double hbar = (sr0 * hl + sr1 * hr) * sri;
  double byave = (byl + byr) / 2.0;
  double delb2 = (gm - 2.0) / (gm - 1.0) * ((byr - byl) * (byr - byl)) * (sri * sri) * pi8i;
  double cs2 = (gm - 1.0) * (hbar - 0.5 * (vxbar * vxbar + vybar * vybar) - delb2 -
                             (bxbar * bxbar + bybar * bybar) * pi4i / rhobar);
  double astar2 = (gm - 1.0) * (hbar - 0.5 * (vxbar * vxbar + vybar * vybar) - delb2) -
                  (gm - 2.0) * (bxbar * bxbar + bybar * bybar) * pi4i / rhobar;
  double ca2 = bxbar * bxbar / (pi4 * rhobar);
  double cbr2 = (bybar * bybar) * pi4i / rhobar;
  double cfast2 = 0.5 * (astar2 + sqrt(cbr2 * (astar2 + cs2 + ca2) + (cs2 - ca2) * (cs2 - ca2)));
  double cslow2 = cs2 * ca2 / cfast2;
  double cfast = sqrt(cfast2);
  double cslow = sqrt(cslow2);
  double ca = sqrt(ca2);
  double cs = sqrt(cs2);
  double epsi = 1.0e-12;
  double sgr = bybar * bybar - epsi;
  double sp = 0.5 + fsign1(0.5, sgr);
  double betay = sp * bybar * sqrt(1.0 / (bybar * bybar + 1.0 - sp)) + sqrt(0.5) * (1.0 - sp);
  double betaz = sqrt(0.5) * (1.0 - sp);
  double eps2 = 1.0e-12;
  double sgr2 = (bybar * bybar) / (pi4 * rhobar) + fabs(ca2 - cs2) - eps2;
  double sp2 = 0.5 + fsign1(0.5, sgr2);
  double cfca = fmax2(0.0, cfast2 - ca2);
  double cfcs = fmax2(0.0, cfast2 - cslow2);
  double cfa = fmax2(0.0, cfast2 - cs2);
  double alphf = sp2 * sqrt(cfca / (cfcs + 1.0 - sp2)) + 1.0 - sp2;
  double alphs = sp2 * sqrt(cfa / (cfcs + 1.0 - sp2));
  double sgnbx = fsign1(1.0, bxbar);
  double eeps = (vxr - vxl + fabs(vxr - vxl)) * 2.5e-1;
  double elpf = -fmax2(fabs(vxbar + cfast), eeps);
  double elmf = -fmax2(fabs(vxbar - cfast), eeps);
  double elps = -fmax2(fabs(vxbar + cslow), eeps);
  double elms = -fmax2(fabs(vxbar - cslow), eeps);
  double elpa = -fmax2(fabs(vxbar + ca), eeps);
  double elma = -fmax2(fabs(vxbar - ca), eeps);
  double elze = -fmax2(fabs(vxbar), eeps);
  double drho = rhor - rhol;
  double du21 = rhobar * (vxr - vxl);
  double du31 = rhobar * (vyr - vyl);
  double du41 = 0;
  double du6 = byr - byl;
  double du5 = 0.;
  double t1 = betay * du6 + betaz * du5;
  double t2 = (prr - prl + (byave * du6) * pi4i + (gm - 2.0) * (bybar * du6) * pi4i) / (gm - 1.0);
  double t3 = betaz * du6 - betay * du5;
  double s1 = du21;
  double s2 = betay * du31 + betaz * du41;
  double s3 = betaz * du31 - betay * du41;
  double p11 = alphs * cfast * sqrt(pi4 / rhobar);
  double p12 = -(alphf * cs2 / cfast * sqrt(pi4 / rhobar));
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
  double fluxlro = rhol * vxl;
  double fluxlrx = rhol * vxl * vxl + prl + (-(bxbar * bxbar) + byl * byl) * pi8i;
  double fluxlry = rhol * vxl * vyl - bxbar * byl * pi4i;
  double fluxlby = vxl * byl - vyl * bxbar;
  double fluxlee = rhol * vxl * hl - bxbar * (bxbar * vxl + byl * vyl) * pi4i;
  double fluxrro = rhor * vxr;
  double fluxrrx = rhor * vxr * vxr + prr + (-(bxbar * bxbar) + byr * byr) * pi8i;
  double fluxrry = rhor * vxr * vyr - bxbar * byr * pi4i;
  double fluxrby = vxr * byr - vyr * bxbar;
  double fluxree = rhor * vxr * hr - bxbar * (bxbar * vxr + byr * vyr) * pi4i;
  double vh = 0.5 * (vxbar * vxbar + vybar * vybar);
  double rpfro = alphf;
  double rpfrx = alphf * (vxbar + cfast);
  double rpfry = alphf * vybar - alphs * betay * ca * sgnbx;
  double rpfby = alphs * betay * cfast * sqrt(pi4 / rhobar);
  double rpfee = alphf * (vh + delb2 + cfast * vxbar + cfast2 / (gm - 1.0) +
                          (cfast2 - cs2) * (gm - 2.0) / (gm - 1.0)) -
                 alphs * ca * (betay * vybar) * sgnbx;
  double rmfro = alphf;
  double rmfrx = alphf * (vxbar - cfast);
  double rmfry = alphf * vybar + alphs * betay * ca * sgnbx;
  double rmfby = rpfby;
  double rmfee = alphf * (vh + delb2 - cfast * vxbar + cfast2 / (gm - 1.0) +
                          (cfast2 - cs2) * (gm - 2.0) / (gm - 1.0)) +
                 alphs * ca * (betay * vybar) * sgnbx;
  double rpsro = alphs;
  double rpsrx = alphs * (vxbar + cslow);
  double rpsry = alphs * vybar + cs * sgnbx * alphf * betay;
  double rpsby = -(sqrt(pi4 / rhobar) * cs2 * alphf * betay / cfast);
  double rpsee = alphs * (vh + delb2 + cslow * vxbar + cslow2 / (gm - 1.0) +
                          (cslow2 - cs2) * (gm - 2.0) / (gm - 1.0)) +
                 alphf * cs * (betay * vybar) * sgnbx;
  double rmsro = alphs;
  double rmsrx = alphs * (vxbar - cslow);
  double rmsry = alphs * vybar - cs * sgnbx * alphf * betay;
  double rmsby = rpsby;
  double rmsee = alphs * (vh + delb2 - cslow * vxbar + cslow2 / (gm - 1.0) +
                          (cslow2 - cs2) * (gm - 2.0) / (gm - 1.0)) -
                 alphf * cs * (betay * vybar) * sgnbx;
  double rparo = 0.0, rparx = 0.0;
  double rpary = -(sgnbx * betaz);
  double rpaby = sqrt(pi4 / rhobar) * betaz;
  double rpaee = -((betaz * vybar) * sgnbx);
  double rmaro = 0.0, rmarx = 0.0;
  double rmary = -rpary;
  double rmaby = rpaby;
  double rmaee = -rpaee;
  double rzero = 1.0, rzerx = vxbar, rzery = vybar, rzeby = 0.0;
  double rzeee = vh + delb2;
  double pf = elpf * wpf, mf = elmf * wmf, ps = elps * wps, ms = elms * wms;
  double pa = elpa * wpa, ma = elma * wma, ze = elze * wze;
#define ROE1_SUM(FL, FR, P, M, PS, MS, PA, MA, Z)                                \
  (0.5 * (FL + FR + pf * P + mf * M + ps * PS + ms * MS + pa * PA + ma * MA + ze * Z))
  f[0] = ROE1_SUM(fluxlro, fluxrro, rpfro, rmfro, rpsro, rmsro, rparo, rmaro, rzero);
  f[1] = ROE1_SUM(fluxlee, fluxree, rpfee, rmfee, rpsee, rmsee, rpaee, rmaee, rzeee);
  f[2] = ROE1_SUM(fluxlrx, fluxrrx, rpfrx, rmfrx, rpsrx, rmsrx, rparx, rmarx, rzerx);
  f[3] = ROE1_SUM(fluxlry, fluxrry, rpfry, rmfry, rpsry, rmsry, rpary, rmary, rzery);
  f[4] = ROE1_SUM(fluxlby, fluxrby, rpfby, rmfby, rpsby, rmsby, rpaby, rmaby, rzeby);
#undef ROE1_SUM
}

/* cans1d/hdroe/tvdminmod.f:8 */
static inline double flmt1(double a, double b) {
  const double s = fsign1(1.0, a);
  return fmax2(0.0, fmin2(b * s, fabs(a))) * s;
}

/* cans1d/hdroe/roe_m.f:2-136 */
void oracle_roe_m_1d(double *ro, double *pr, double *vx, double *vy, double *by,
                     const double *bx, const double *bxm, double dt, double gm,
                     const double *dx, int ix) {
  double *w = arena_get(&arena_roe1, (size_t)ix * 13);
  double *ee = w, *rx = w + ix, *ry = w + 2 * ix;
  double *fl[5], *hp[5];
  for (int v = 0; v < 5; v++) {
    fl[v] = w + (3 + v) * (size_t)ix;
    hp[v] = w + (8 + v) * (size_t)ix;
  }
  const double pi = acos(-1.0);
  const double pi4 = 4.0 * pi;
  const double pi4i = 1.0 / pi4;
  const double pi8i = 5.0e-1 * pi4i;
  double *P[5] = {ro, pr, vx, vy, by};
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    rx[c] = ro[c] * vx[c];
    ry[c] = ro[c] * vy[c];
    double v2 = vx[c] * vx[c] + vy[c] * vy[c];
    double b2 = bx[c] * bx[c] + by[c] * by[c];
    ee[c] = pr[c] / (gm - 1.0) + 0.5 * ro[c] * v2 + pi8i * b2;
  }
  /* :31-46 first-order states and fluxes */
  for (int i = 1; i <= ix - 1; i++) {
    size_t c = I1(i);
    double L[6] = {ro[c], pr[c], vx[c], vy[c], bxm[c], by[c]};
    double R[6] = {ro[c + 1], pr[c + 1], vx[c + 1], vy[c + 1], bxm[c], by[c + 1]};
    double f[5];
    roe_face1(gm, L, R, f);
    for (int v = 0; v < 5; v++) fl[v][c] = f[v];
  }
  /* :48-54 dt/2 update; :57-64 half-step primitives (the end cells keep the
   * input primitives, see the header) */
  for (int v = 0; v < 5; v++) {
    hp[v][0] = P[v][0];
    hp[v][ix - 1] = P[v][ix - 1];
  }
  for (int i = 2; i <= ix - 1; i++) {
    size_t c = I1(i);
    double roh = ro[c] + 0.5 * dt * ((fl[0][c - 1] - fl[0][c]) / dx[c]);
    double eeh = ee[c] + 0.5 * dt * ((fl[1][c - 1] - fl[1][c]) / dx[c]);
    double rxh = rx[c] + 0.5 * dt * ((fl[2][c - 1] - fl[2][c]) / dx[c]);
    double ryh = ry[c] + 0.5 * dt * ((fl[3][c - 1] - fl[3][c]) / dx[c]);
    double byh = by[c] + 0.5 * dt * ((fl[4][c - 1] - fl[4][c]) / dx[c]);
    double vxh = rxh / roh;
    double vyh = ryh / roh;
    double v2 = vxh * vxh + vyh * vyh;
    double b2 = bx[c] * bx[c] + byh * byh;
    hp[0][c] = roh;
    hp[1][c] = (gm - 1.0) * (eeh - 0.5 * roh * v2 - pi8i * b2);
    hp[2][c] = vxh;
    hp[3][c] = vyh;
    hp[4][c] = byh;
  }
  /* :66-73 minmod states and fluxes of the faces 2..ix-2 */
  for (int i = 2; i <= ix - 2; i++) {
    size_t c = I1(i);
    double L[6], R[6], f[5];
    double ql[5], qr[5];
    for (int v = 0; v < 5; v++) {
      const double dm = hp[v][c - 1], d0 = hp[v][c], d1 = hp[v][c + 1], d2 = hp[v][c + 2];
      ql[v] = d0 + 0.5 * flmt1(d1 - d0, d0 - dm);
      qr[v] = d1 - 0.5 * flmt1(d1 - d0, d2 - d1);
    }
    L[0] = ql[0]; L[1] = ql[1]; L[2] = ql[2]; L[3] = ql[3]; L[4] = bxm[c]; L[5] = ql[4];
    R[0] = qr[0]; R[1] = qr[1]; R[2] = qr[2]; R[3] = qr[3]; R[4] = bxm[c]; R[5] = qr[4];
    roe_face1(gm, L, R, f);
    for (int v = 0; v < 5; v++) fl[v][c] = f[v];
  }
  /* :75-89 full update and primitives */
  for (int i = 3; i <= ix - 2; i++) {
    size_t c = I1(i);
    ro[c] = ro[c] + dt * ((fl[0][c - 1] - fl[0][c]) / dx[c]);
    ee[c] = ee[c] + dt * ((fl[1][c - 1] - fl[1][c]) / dx[c]);
    rx[c] = rx[c] + dt * ((fl[2][c - 1] - fl[2][c]) / dx[c]);
    ry[c] = ry[c] + dt * ((fl[3][c - 1] - fl[3][c]) / dx[c]);
    by[c] = by[c] + dt * ((fl[4][c - 1] - fl[4][c]) / dx[c]);
  }
  for (int i = 3; i <= ix - 2; i++) {
    size_t c = I1(i);
    vx[c] = rx[c] / ro[c];
    vy[c] = ry[c] / ro[c];
    double v2 = vx[c] * vx[c] + vy[c] * vy[c];
    double b2 = bx[c] * bx[c] + by[c] * by[c];
    pr[c] = (gm - 1.0) * (ee[c] - 0.5 * ro[c] * v2 - pi8i * b2);
  }
}
