/*
 * 1-D mLW step and CFL: line-faithful C restatement of the CANS Fortran
 * (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 *   mlwhalf   cans1d/hdmlw/mlwhalf.f:33-46
 *   mlwfull   cans1d/hdmlw/mlwfull.f:30-33
 *   mlwartv   cans1d/hdmlw/mlwartv.f:31-34
 *   mlw_m     cans1d/hdmlw/mlw_m.f:2-215 (ro,pr,vx,vy,by; bx, bxm constant)
 *   cfl_m     cans1d/common/cfl_m.f:42-71
 */
#include "oracle.h"
#include "oracle_common.h"

static oracle_arena arena1d;

/* cans1d/hdmlw/mlwhalf.f */
static void mlwhalf1(const double *u, double *un, double *du, double dt,
                     const double *f, const double *dxi, const double *dxim,
                     int ix) {
  for (int i = 2; i <= ix - 1; i++)
    du[I1(i)] = du[I1(i)] - 0.5 * dt * (0.5 * dxi[I1(i)] * (f[I1(i + 1)] - f[I1(i - 1)]));
  for (int i = 1; i <= ix - 1; i++) {
    double uh = 0.5 * (u[I1(i + 1)] + u[I1(i)]);
    double dfdx = dxim[I1(i)] * (f[I1(i + 1)] - f[I1(i)]);
    un[I1(i)] = uh - dt * dfdx;
  }
}

/* cans1d/hdmlw/mlwfull.f */
static void mlwfull1(double *du, double dt, const double *f, const double *dxi,
                     int ix) {
  for (int i = 2; i <= ix - 1; i++) {
    double dfdx = dxi[I1(i)] * (f[I1(i)] - f[I1(i - 1)]);
    du[I1(i)] = du[I1(i)] - 0.5 * dt * dfdx;
  }
}

/* cans1d/hdmlw/mlwartv.f */
static void mlwartv1(const double *u, double *du, double dt, const double *qx,
                     const double *dxi, const double *dxim, int ix) {
  for (int i = 2; i <= ix - 1; i++)
    du[I1(i)] = du[I1(i)] +
                dt * (dxi[I1(i)] *
                      (qx[I1(i)] * dxim[I1(i)] * (u[I1(i + 1)] - u[I1(i)]) -
                       qx[I1(i - 1)] * dxim[I1(i - 1)] * (u[I1(i)] - u[I1(i - 1)])));
}

/* cans1d/hdmlw/mlw_m.f:2-215 */
void oracle_mlw_m_1d(double *ro, double *pr, double *vx, double *vy, double *by,
                     const double *bx, const double *bxm, double dt, double qav,
                     double gm, const double *dx, const double *dxm, int ix) {
  enum { NT = 24 };
  double *w = arena_get(&arena1d, (size_t)NT * ix);
  double *t[NT];
  for (int a = 0; a < NT; a++) t[a] = w + (size_t)a * ix;
  double *dxi = t[0], *dxim = t[1], *ee = t[2], *rx = t[3], *ry = t[4];
  double *ez = t[5], *roh = t[6], *eeh = t[7], *rxh = t[8], *ryh = t[9];
  double *byh = t[10], *prh = t[11], *vxh = t[12], *vyh = t[13], *ezh = t[14];
  double *dro = t[15], *dee = t[16], *drx = t[17], *dry = t[18], *dby = t[19];
  double *fx = t[20], *qx = t[21];

  const double pi = acos(-1.0);
  const double pi8i = 1. / pi / 8.;
  const double pi4i = 1. / pi / 4.;
  for (int i = 1; i <= ix; i++) {
    dxim[I1(i)] = 1.0 / dxm[I1(i)];
    dxi[I1(i)] = 1.0 / dx[I1(i)];
  }
  for (int i = 1; i <= ix; i++) {
    dro[I1(i)] = 0.0; dee[I1(i)] = 0.0; drx[I1(i)] = 0.0;
    dry[I1(i)] = 0.0; dby[I1(i)] = 0.0;
  }
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    double vv = vx[c] * vx[c] + vy[c] * vy[c];
    double bb = by[c] * by[c];
    ee[c] = pr[c] / (gm - 1) + 0.5 * ro[c] * vv + pi8i * bb;
    rx[c] = ro[c] * vx[c];
    ry[c] = ro[c] * vy[c];
  }
  for (int i = 1; i <= ix; i++) ez[I1(i)] = -vx[I1(i)] * by[I1(i)] + vy[I1(i)] * bx[I1(i)];
  for (int i = 1; i <= ix; i++) fx[I1(i)] = ro[I1(i)] * vx[I1(i)];
  mlwhalf1(ro, roh, dro, dt, fx, dxi, dxim, ix);
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    double vv = vx[c] * vx[c] + vy[c] * vy[c];
    double ep = pr[c] * gm / (gm - 1.) + 0.5 * ro[c] * vv;
    fx[c] = ep * vx[c] - by[c] * ez[c] * pi4i;
  }
  mlwhalf1(ee, eeh, dee, dt, fx, dxi, dxim, ix);
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    double bbm = by[c] * by[c];
    fx[c] = ro[c] * (vx[c] * vx[c]) + pr[c] + bbm * pi8i;
  }
  mlwhalf1(rx, rxh, drx, dt, fx, dxi, dxim, ix);
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    fx[c] = ro[c] * vx[c] * vy[c] - bx[c] * by[c] * pi4i;
  }
  mlwhalf1(ry, ryh, dry, dt, fx, dxi, dxim, ix);
  for (int i = 1; i <= ix; i++) fx[I1(i)] = -ez[I1(i)];
  mlwhalf1(by, byh, dby, dt, fx, dxi, dxim, ix);

  for (int i = 1; i <= ix - 1; i++) {
    size_t c = I1(i);
    vxh[c] = rxh[c] / roh[c];
    vyh[c] = ryh[c] / roh[c];
    double vv = vxh[c] * vxh[c] + vyh[c] * vyh[c];
    double bb = byh[c] * byh[c];
    prh[c] = (gm - 1) * (eeh[c] - 0.5 * roh[c] * vv - pi8i * bb);
  }
  for (int i = 1; i <= ix; i++)
    ezh[I1(i)] = -vxh[I1(i)] * byh[I1(i)] + vyh[I1(i)] * bxm[I1(i)];
  for (int i = 1; i <= ix - 1; i++) fx[I1(i)] = roh[I1(i)] * vxh[I1(i)];
  mlwfull1(dro, dt, fx, dxi, ix);
  for (int i = 1; i <= ix - 1; i++) {
    size_t c = I1(i);
    double vv = vxh[c] * vxh[c] + vyh[c] * vyh[c];
    double eph = prh[c] * gm / (gm - 1.) + 0.5 * roh[c] * vv;
    fx[c] = eph * vxh[c] - byh[c] * ezh[c] * pi4i;
  }
  mlwfull1(dee, dt, fx, dxi, ix);
  for (int i = 1; i <= ix - 1; i++) {
    size_t c = I1(i);
    double bbm = byh[c] * byh[c];
    fx[c] = roh[c] * (vxh[c] * vxh[c]) + prh[c] + bbm * pi8i;
  }
  mlwfull1(drx, dt, fx, dxi, ix);
  for (int i = 1; i <= ix - 1; i++) {
    size_t c = I1(i);
    fx[c] = roh[c] * vxh[c] * vyh[c] - bxm[c] * byh[c] * pi4i;
  }
  mlwfull1(dry, dt, fx, dxi, ix);
  for (int i = 1; i <= ix - 1; i++) fx[I1(i)] = -ezh[I1(i)];
  mlwfull1(dby, dt, fx, dxi, ix);

  const double zero = 0.0;
  for (int i = 1; i <= ix - 1; i++)
    qx[I1(i)] = qav * dxm[I1(i)] *
                fmax2(zero, fabs(vx[I1(i + 1)] - vx[I1(i)]) - R4_1EM4);
  mlwartv1(ro, dro, dt, qx, dxi, dxim, ix);
  mlwartv1(ee, dee, dt, qx, dxi, dxim, ix);
  mlwartv1(rx, drx, dt, qx, dxi, dxim, ix);
  mlwartv1(ry, dry, dt, qx, dxi, dxim, ix);
  mlwartv1(by, dby, dt, qx, dxi, dxim, ix);
  for (int i = 2; i <= ix - 1; i++) {
    size_t c = I1(i);
    ro[c] = ro[c] + dro[c];
    rx[c] = rx[c] + drx[c];
    ry[c] = ry[c] + dry[c];
    by[c] = by[c] + dby[c];
    ee[c] = ee[c] + dee[c];
  }
  for (int i = 2; i <= ix - 1; i++) {
    size_t c = I1(i);
    vx[c] = rx[c] / ro[c];
    vy[c] = ry[c] / ro[c];
    double vv = vx[c] * vx[c] + vy[c] * vy[c];
    double bb = by[c] * by[c];
    pr[c] = (gm - 1) * (ee[c] - 0.5 * ro[c] * vv - pi8i * bb);
  }
}

/* cans1d/common/cfl_m.f:42-71 (interior cells only, |vx| + fast speed) */
void oracle_cfl_m_1d(double *dt, double safety, double dtmin, int *merr,
                     double gm, const double *bx, const double *ro,
                     const double *pr, const double *vx, const double *vy,
                     const double *by, const double *dx, int ix) {
  (void)vy;
  const double pi = acos(-1.0);
  const double pi4i = 0.25 / pi;
  double dmin = R4_1E20;
  for (int i = 2; i <= ix - 1; i++) {
    size_t c = I1(i);
    double onero = 1.0 / ro[c];
    double ca2 = (bx[c] * bx[c] + by[c] * by[c]) * pi4i * onero;
    double cs2 = gm * pr[c] * onero;
    double dtcfl = dx[c] / (fabs(vx[c]) + sqrt(cs2 + ca2));
    double dtq = safety * dtcfl;
    if (dtq < dmin) dmin = dtq;
  }
  *dt = dmin;
  *merr = 0;
  if (*dt < dtmin) *merr = 9001;
}
