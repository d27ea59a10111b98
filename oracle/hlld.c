/*
 * HLLD step of the cansxx engine: line-faithful C restatement of the CANS
 * Fortran (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 *   engine         cansxx-nosupport/md_mhdshktb/hdhlld-x/engine.f:2-73
 *   hlld_mh        cansxx-nosupport/hdhlld/hlld_mh.f:2-127
 *   hlld_flux      cansxx-nosupport/hdhlld/hlld_flux.f90:2-484
 *                  (Miyoshi & Kusano, J. Comput. Phys. 208, 315 (2005))
 *   inp_const      cansxx-nosupport/interpolation/inp_const.f
 *   inp_tvdminmod  cansxx-nosupport/interpolation/inp_tvdminmod.f
 *   adddfdx        cansxx-nosupport/common/adddfdx.f:1-49
 *   vvtorv, pr2eh, eh2ee, rvtovv, ee2eh, eh2pr, daupdate
 *                  cansxx-nosupport/common/{vvtorv,pr2eh,...}.f
 *   roereset       cansxx-nosupport/hdroe/roereset.f
 *
 * Units are Heaviside with permeability mu (pb = B^2/2, eh2ee.f).
 *
 * Two places where the reference reads memory it never wrote get a
 * definite meaning here:
 *  - hlld_flux evaluates the face n of every axis from face states that
 *    inp_const / inp_tvdminmod never set; adddfdx never reads that face, and
 *    it is not evaluated here;
 *  - hlld_mh zeroes the normal-field flux only for i = 1..ix-1
 *    (hlld_mh.f:88-94, 105-111), so for the y and z axes the column i = ix
 *    keeps the tangential flux of the previous axis and adddfdx applies it to
 *    that column.  Here the normal-field flux is zero everywhere, so the
 *    normal field component of an axis never changes in that axis's pass.
 *    Only the boundary column i = ix can differ, and the boundary fill
 *    rewrites it after every step.
 */
#include "oracle.h"
#include "oracle_common.h"

static oracle_arena arena_hlld;

static inline double fsign(double a, double b) { return copysign(fabs(a), b); }

/* hlld_flux.f90:148-480 for one face: L and R hold (ro, pr, vn, vt1, vt2,
 * bn, bt1, bt2) (bn unused), bxs the face normal field; f receives (fro,
 * fee, frn, frt1, frt2, fbt1, fbt2). */
static void hlld_face(double gm, double zfloor, const double *L, const double *R,
                      double bxs, double *f) {
  const double bxsq = bxs * bxs;
  /* left state (:152-169) */
  const double rol = L[0], vxl = L[2], vyl = L[3], vzl = L[4], byl = L[6], bzl = L[7];
  const double pbl = 0.5 * (bxs * bxs + byl * byl + bzl * bzl);
  const double prl = L[1];
  const double ptl = prl + pbl;
  const double eel = prl / (gm - 1.0) + 0.5 * rol * (vxl * vxl + vyl * vyl + vzl * vzl) + pbl;
  const double rxl = rol * vxl, ryl = rol * vyl, rzl = rol * vzl;
  /* right state (:173-191) */
  const double ror = R[0], vxr = R[2], vyr = R[3], vzr = R[4], byr = R[6], bzr = R[7];
  const double pbr = 0.5 * (bxs * bxs + byr * byr + bzr * bzr);
  const double prr = R[1];
  const double ptr = prr + pbr;
  const double eer = prr / (gm - 1.0) + 0.5 * (ror * (vxr * vxr + vyr * vyr + vzr * vzr)) + pbr;
  const double rxr = ror * vxr, ryr = ror * vyr, rzr = ror * vzr;
  /* wave speeds (:197-207) */
  const double gmpl = gm * prl, gmpr = gm * prr;
  const double gpbl = gmpl + 2.0 * pbl, gpbr = gmpr + 2.0 * pbr;
  const double cfl = sqrt((gpbl + sqrt(gpbl * gpbl - 4.0 * gmpl * bxsq)) / (2.0 * rol));
  const double cfr = sqrt((gpbr + sqrt(gpbr * gpbr - 4.0 * gmpr * bxsq)) / (2.0 * ror));
  const double sl = fmin2(vxl, vxr) - fmax2(cfl, cfr);
  const double sr = fmax2(vxl, vxr) + fmax2(cfl, cfr);
  /* physical fluxes (:214-229) */
  const double frol = rxl;
  const double frxl = rxl * vxl + ptl - bxsq;
  const double fryl = rol * vxl * vyl - bxs * byl;
  const double frzl = rol * vxl * vzl - bxs * bzl;
  const double feel = vxl * (eel + ptl - bxsq) - bxs * (vyl * byl + vzl * bzl);
  const double fbyl = byl * vxl - bxs * vyl;
  const double fbzl = bzl * vxl - bxs * vzl;
  const double fror = rxr;
  const double frxr = rxr * vxr + ptr - bxsq;
  const double fryr = ror * vxr * vyr - bxs * byr;
  const double frzr = ror * vxr * vzr - bxs * bzr;
  const double feer = vxr * (eer + ptr - bxsq) - bxs * (vyr * byr + vzr * bzr);
  const double fbyr = byr * vxr - bxs * vyr;
  const double fbzr = bzr * vxr - bxs * vzr;
  /* upwind cases (:235-255) */
  if (sl >= 0.0) {
    f[0] = frol; f[1] = feel; f[2] = frxl; f[3] = fryl; f[4] = frzl; f[5] = fbyl; f[6] = fbzl;
    return;
  }
  if (sr <= 0.0) {
    f[0] = fror; f[1] = feer; f[2] = frxr; f[3] = fryr; f[4] = frzr; f[5] = fbyr; f[6] = fbzr;
    return;
  }
  /* middle wave (:260-267) */
  const double sdl = sl - vxl, sdr = sr - vxr;
  const double sm = (sdr * ror * vxr - sdl * rol * vxl - ptr + ptl) / (sdr * ror - sdl * rol);
  const double sdml = sl - sm, sdmr = sr - sm;
  /* total pressure of the star states (:274-275) */
  const double ptst = (sdr * ror * ptl - sdl * rol * ptr + rol * ror * sdr * sdl * (vxr - vxl)) /
                      (sdr * ror - sdl * rol);
  /* Ul* (:281-308) */
  double temp_fst = rol * sdl * sdml - bxsq;
  double s3 = fsign(1.0, temp_fst + zfloor) * fsign(1.0, temp_fst - zfloor);
  double mx = fmax2(0.0, s3), mn = fmin2(0.0, s3);
  double tmp = bxs * (sdl - sdml) / (temp_fst + mn);
  const double rolst = mx * (rol * sdl / sdml) - mn * rol;
  const double vxlst = mx * sm - mn * vxl;
  const double rxlst = rolst * vxlst;
  const double vylst = mx * (vyl - byl * tmp) - mn * vyl;
  const double rylst = rolst * vylst;
  const double vzlst = mx * (vzl - bzl * tmp) - mn * vzl;
  const double rzlst = rolst * vzlst;
  tmp = (rol * (sdl * sdl) - bxsq) / (temp_fst + mn);
  const double bylst = mx * (byl * tmp) - mn * byl;
  const double bzlst = mx * (bzl * tmp) - mn * bzl;
  const double vdbstl = vxlst * bxs + vylst * bylst + vzlst * bzlst;
  const double eelst =
      mx * ((sdl * eel - ptl * vxl + ptst * sm + bxs * (vxl * bxs + vyl * byl + vzl * bzl - vdbstl)) /
            sdml) -
      mn * eel;
  /* Ur* (:314-342) */
  temp_fst = ror * sdr * sdmr - bxsq;
  s3 = fsign(1.0, temp_fst + zfloor) * fsign(1.0, temp_fst - zfloor);
  mx = fmax2(0.0, s3);
  mn = fmin2(0.0, s3);
  tmp = bxs * (sdr - sdmr) / (temp_fst + mn);
  const double rorst = mx * (ror * sdr / sdmr) - mn * ror;
  const double vxrst = mx * sm - mn * vxr;
  const double rxrst = rorst * vxrst;
  const double vyrst = mx * (vyr - byr * tmp) - mn * vyr;
  const double ryrst = rorst * vyrst;
  const double vzrst = mx * (vzr - bzr * tmp) - mn * vzr;
  const double rzrst = rorst * vzrst;
  tmp = (ror * (sdr * sdr) - bxsq) / (temp_fst + mn);
  const double byrst = mx * (byr * tmp) - mn * byr;
  const double bzrst = mx * (bzr * tmp) - mn * bzr;
  const double vdbstr = vxrst * bxs + vyrst * byrst + vzrst * bzrst;
  const double eerst =
      mx * ((sdr * eer - ptr * vxr + ptst * sm + bxs * (vxr * bxs + vyr * byr + vzr * bzr - vdbstr)) /
            sdmr) -
      mn * eer;
  /* Ul**, Ur** (:347-414) */
  const double sqrtrol = sqrt(rolst), sqrtror = sqrt(rorst);
  const double slst = sm - fabs(bxs) / sqrtrol;
  const double srst = sm + fabs(bxs) / sqrtror;
  double roldst, rxldst, ryldst, rzldst, eeldst, byldst, bzldst;
  double rordst, rxrdst, ryrdst, rzrdst, eerdst, byrdst, bzrdst;
  if (bxs == 0.0) {
    roldst = rolst; rxldst = rxlst; ryldst = rylst; rzldst = rzlst;
    eeldst = eelst; byldst = bylst; bzldst = bzlst;
    rordst = rorst; rxrdst = rxrst; ryrdst = ryrst; rzrdst = rzrst;
    eerdst = eerst; byrdst = byrst; bzrdst = bzrst;
  } else {
    const double invsumro = 1.0 / (sqrtrol + sqrtror);
    const double signbx = fsign(1.0, bxs);
    roldst = rolst;
    rordst = rorst;
    rxldst = rxlst;
    rxrdst = rxrst;
    double temp = invsumro * (sqrtrol * vylst + sqrtror * vyrst + signbx * (byrst - bylst));
    const double vyd = temp;
    ryldst = roldst * temp;
    ryrdst = rordst * temp;
    temp = invsumro * (sqrtrol * vzlst + sqrtror * vzrst + signbx * (bzrst - bzlst));
    const double vzd = temp;
    rzldst = roldst * temp;
    rzrdst = rordst * temp;
    temp = invsumro * (sqrtrol * byrst + sqrtror * bylst + signbx * sqrtrol * sqrtror * (vyrst - vylst));
    byldst = temp;
    byrdst = temp;
    temp = invsumro * (sqrtrol * bzrst + sqrtror * bzlst + signbx * sqrtrol * sqrtror * (vzrst - vzlst));
    bzldst = temp;
    bzrdst = temp;
    temp = sm * bxs + vyd * byldst + vzd * bzldst;
    eeldst = eelst - sqrtrol * signbx * (vdbstl - temp);
    eerdst = eerst + sqrtror * signbx * (vdbstr - temp);
  }
  /* flux (:446-480), written in the order fro, fee, frx, fry, frz, fby, fbz */
  if (slst >= 0.0) {
    f[0] = frol + sl * (rolst - rol);
    f[2] = frxl + sl * (rxlst - rxl);
    f[3] = fryl + sl * (rylst - ryl);
    f[4] = frzl + sl * (rzlst - rzl);
    f[1] = feel + sl * (eelst - eel);
    f[5] = fbyl + sl * (bylst - byl);
    f[6] = fbzl + sl * (bzlst - bzl);
  } else if (sm >= 0.0) {
    const double temp = slst - sl;
    f[0] = frol - sl * rol - temp * rolst + slst * roldst;
    f[2] = frxl - sl * rxl - temp * rxlst + slst * rxldst;
    f[3] = fryl - sl * ryl - temp * rylst + slst * ryldst;
    f[4] = frzl - sl * rzl - temp * rzlst + slst * rzldst;
    f[1] = feel - sl * eel - temp * eelst + slst * eeldst;
    f[5] = fbyl - sl * byl - temp * bylst + slst * byldst;
    f[6] = fbzl - sl * bzl - temp * bzlst + slst * bzldst;
  } else if (srst > 0.0) {
    const double temp = srst - sr;
    f[0] = fror - sr * ror - temp * rorst + srst * rordst;
    f[2] = frxr - sr * rxr - temp * rxrst + srst * rxrdst;
    f[3] = fryr - sr * ryr - temp * ryrst + srst * ryrdst;
    f[4] = frzr - sr * rzr - temp * rzrst + srst * rzrdst;
    f[1] = feer - sr * eer - temp * eerst + srst * eerdst;
    f[5] = fbyr - sr * byr - temp * byrst + srst * byrdst;
    f[6] = fbzr - sr * bzr - temp * bzrst + srst * bzrdst;
  } else {
    f[0] = fror + sr * (rorst - ror);
    f[2] = frxr + sr * (rxrst - rxr);
    f[3] = fryr + sr * (ryrst - ryr);
    f[4] = frzr + sr * (rzrst - rzr);
    f[1] = feer + sr * (eerst - eer);
    f[5] = fbyr + sr * (byrst - byr);
    f[6] = fbzr + sr * (bzrst - bzr);
  }
}

/* variable order: prims ro pr vx vy vz bx by bz; conserved ro ee rx ry rz bx by bz */
enum { V_RO, V_PR, V_VX, V_VY, V_VZ, V_BX, V_BY, V_BZ };
enum { F_RO, F_EE, F_RX, F_RY, F_RZ, F_BX, F_BY, F_BZ };
static const int rot[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};

/* inp_tvdminmod.f:118 */
static inline double flmt(double a, double b) {
  const double s = fsign(1.0, a);
  return fmax2(0.0, fmin2(b * s, fabs(a))) * s;
}

/* hlld_mh.f:36-124: one stage over the active axes.  P are the primitives the
 * stage reads, U the conserved variables it updates in place. */
static void hlld_stage(double *const *P, double *const *U, double gm, double dt,
                       const double *const *dd, const int *nn, const size_t *st,
                       const int *mfdim, int mstage, double *F) {
  const double zfloor = 1.0e-10;
  const int ix = nn[0], jx = nn[1], kx = nn[2];
  const size_t n = (size_t)ix * jx * kx;
  double *Fl[8];
  for (int v = 0; v < 8; v++) Fl[v] = F + v * n;
  for (int a = 0; a < 3; a++) {
    if (mfdim[a] != 1) continue;
    const int *r = rot[a];
    const int na = nn[a];
    /* faces (c, c + e_a) for c_a = 1..n_a-1, every transverse cell */
    OMP_FOR
    for (int k = 1; k <= kx; k++)
      for (int j = 1; j <= jx; j++)
        for (int i = 1; i <= ix; i++) {
          const int ic[3] = {i, j, k};
          const int ca = ic[a];
          if (ca > na - 1) continue;
          const size_t c = I3(i, j, k), s = st[a];
          double w[2][8];
          for (int v = 0; v < 8; v++) {
            const double *q = P[v];
            if (mstage == 1 || ca == 1 || ca == na - 1) { /* inp_const, ends of inp_tvdminmod */
              w[0][v] = q[c];
              w[1][v] = q[c + s];
            } else {
              w[0][v] = q[c] + 0.5 * flmt(q[c] - q[c - s], q[c + s] - q[c]);
              w[1][v] = q[c + s] - 0.5 * flmt(q[c + 2 * s] - q[c + s], q[c + s] - q[c]);
            }
          }
          double L[8], R[8], f[7];
          L[0] = w[0][V_RO];
          L[1] = w[0][V_PR];
          R[0] = w[1][V_RO];
          R[1] = w[1][V_PR];
          for (int m = 0; m < 3; m++) {
            L[2 + m] = w[0][V_VX + r[m]];
            L[5 + m] = w[0][V_BX + r[m]];
            R[2 + m] = w[1][V_VX + r[m]];
            R[5 + m] = w[1][V_BX + r[m]];
          }
          /* bb: the cell-centred normal field averaged onto the face */
          const double bb = (P[V_BX + a][c] + P[V_BX + a][c + s]) / 2.0;
          hlld_face(gm, zfloor, L, R, bb, f);
          Fl[F_RO][c] = f[0];
          Fl[F_EE][c] = f[1];
          for (int m = 0; m < 3; m++) Fl[F_RX + r[m]][c] = f[2 + m];
          Fl[F_BX + r[1]][c] = f[5];
          Fl[F_BX + r[2]][c] = f[6];
        }
    /* adddfdx: cells 2..n_a-1 along a, every transverse cell */
    OMP_FOR
    for (int k = 1; k <= kx; k++)
      for (int j = 1; j <= jx; j++)
        for (int i = 1; i <= ix; i++) {
          const int ic[3] = {i, j, k};
          const int ca = ic[a];
          if (ca < 2 || ca > na - 1) continue;
          const size_t c = I3(i, j, k);
          const double h = dd[a][I1(ca)];
          for (int v = 0; v < 8; v++) {
            if (v == F_BX + a) continue; /* zero normal-field flux */
            U[v][c] = U[v][c] - dt * ((Fl[v][c] - Fl[v][c - st[a]]) / h);
          }
        }
  }
}

/* rvtovv + ee2eh + eh2pr (engine.f:50-52, 68-70) */
static void to_primitive(double *const *U, double *const *P, double gm, double mu, size_t n) {
  OMP_FOR
  for (size_t c = 0; c < n; c++) {
    const double ro = U[F_RO][c];
    const double vx = U[F_RX][c] / ro, vy = U[F_RY][c] / ro, vz = U[F_RZ][c] / ro;
    const double bx = U[F_BX][c], by = U[F_BY][c], bz = U[F_BZ][c];
    const double ek = (vx * vx + vy * vy + vz * vz) * ro / 2.0;
    const double em = (bx * bx + by * by + bz * bz) / (2.0 * mu);
    const double eh = U[F_EE][c] - ek - em;
    P[V_RO][c] = ro;
    P[V_VX][c] = vx;
    P[V_VY][c] = vy;
    P[V_VZ][c] = vz;
    P[V_BX][c] = bx;
    P[V_BY][c] = by;
    P[V_BZ][c] = bz;
    P[V_PR][c] = (gm - 1.0) * eh;
  }
}

void oracle_hlld_engine_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                           double *bx, double *by, double *bz, double gm, double mu,
                           double dt, const double *dx, int ix, const double *dy, int jx,
                           const double *dz, int kx, const int *mfdim) {
  const size_t n = (size_t)ix * jx * kx;
  /* arena: U (8) | Uh (8) | U2 (8) | Ph (8) | fluxes (8) */
  double *w = arena_get(&arena_hlld, n * 40);
  double *U[8], *Uh[8], *U2[8], *Ph[8];
  for (int v = 0; v < 8; v++) {
    U[v] = w + v * n;
    Uh[v] = w + (8 + v) * n;
    U2[v] = w + (16 + v) * n;
    Ph[v] = w + (24 + v) * n;
  }
  double *F = w + 32 * n;
  double *P[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  const double *dd[3] = {dx, dy, dz};
  const int nn[3] = {ix, jx, kx};
  const size_t st[3] = {1, (size_t)ix, (size_t)ix * jx};
  /* vvtorv, pr2eh, eh2ee, roereset (engine.f:32-43) */
  OMP_FOR
  for (size_t c = 0; c < n; c++) {
    const double rxv = vx[c] * ro[c], ryv = vy[c] * ro[c], rzv = vz[c] * ro[c];
    const double eh = pr[c] / (gm - 1.0);
    const double ek = (vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c]) * ro[c] / 2.0;
    const double em = (bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c]) / (2.0 * mu);
    const double u[8] = {ro[c], eh + ek + em, rxv, ryv, rzv, bx[c], by[c], bz[c]};
    for (int v = 0; v < 8; v++) U[v][c] = Uh[v][c] = U2[v][c] = u[v];
  }
  /* stage 1: first order, dt/2 (engine.f:45-48) */
  const double dth = 0.5 * dt;
  hlld_stage(P, Uh, gm, dth, dd, nn, st, mfdim, 1, F);
  to_primitive(Uh, Ph, gm, mu, n);
  /* stage 2: minmod, dt (engine.f:54-57) */
  hlld_stage(Ph, U2, gm, dt, dd, nn, st, mfdim, 2, F);
  /* daupdate and the primitives of the new state (engine.f:59-70) */
  to_primitive(U2, P, gm, mu, n);
  (void)U;
}
