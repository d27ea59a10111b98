/*
 * 1-D mLW step with gravity, flux-tube cross section and rotation
 * (mlw_m_bg), the density/pressure floor (chkdav) and the spicule model's
 * random torque (trqalfven): line-faithful C restatement of the CANS Fortran
 * (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 *   mlw_m_bg   cans1d/hdmlw/mlw_m_bg.f:2-271
 *   mlwsrch    cans1d/hdmlw/mlwsrch.f (half-step source)
 *   mlwsrcf    cans1d/hdmlw/mlwsrcf.f (full-step source)
 *   chkdav     cans1d/common/chkdav.f:68-76
 *   trqalfven  cans1d/md_spicule/hdmlw/trqalfven.f:18-40
 */
#include <stdint.h>

#include "oracle.h"
#include "oracle_common.h"

static oracle_arena arena_bg;

/* cans1d/hdmlw/mlwhalf.f */
static void half(const double *u, double *un, double *du, double dt,
                 const double *f, const double *dxi, const double *dxim, int ix) {
  for (int i = 2; i <= ix - 1; i++)
    du[I1(i)] = du[I1(i)] - 0.5 * dt * (0.5 * dxi[I1(i)] * (f[I1(i + 1)] - f[I1(i - 1)]));
  for (int i = 1; i <= ix - 1; i++) {
    double uh = 0.5 * (u[I1(i + 1)] + u[I1(i)]);
    double dfdx = dxim[I1(i)] * (f[I1(i + 1)] - f[I1(i)]);
    un[I1(i)] = uh - dt * dfdx;
  }
}

/* cans1d/hdmlw/mlwsrch.f */
static void srch(double *un, double *du, double dt, const double *s, int ix) {
  for (int i = 2; i <= ix - 1; i++) du[I1(i)] = du[I1(i)] + 0.5 * dt * s[I1(i)];
  for (int i = 1; i <= ix - 1; i++) {
    double sh = 0.5 * (s[I1(i + 1)] + s[I1(i)]);
    un[I1(i)] = un[I1(i)] + dt * sh;
  }
}

/* cans1d/hdmlw/mlwfull.f */
static void full(double *du, double dt, const double *f, const double *dxi, int ix) {
  for (int i = 2; i <= ix - 1; i++) {
    double dfdx = dxi[I1(i)] * (f[I1(i)] - f[I1(i - 1)]);
    du[I1(i)] = du[I1(i)] - 0.5 * dt * dfdx;
  }
}

/* cans1d/hdmlw/mlwsrcf.f */
static void srcf(double *du, double dt, const double *s, const double *ux0,
                 const double *ux1, int ix) {
  for (int i = 2; i <= ix - 1; i++) {
    double sh = ux0[I1(i)] * s[I1(i - 1)] + ux1[I1(i)] * s[I1(i)];
    du[I1(i)] = du[I1(i)] + 0.5 * dt * sh;
  }
}

/* cans1d/hdmlw/mlwartv.f */
static void artv(const double *u, double *du, double dt, const double *qx,
                 const double *dxi, const double *dxim, int ix) {
  for (int i = 2; i <= ix - 1; i++)
    du[I1(i)] = du[I1(i)] +
                dt * (dxi[I1(i)] *
                      (qx[I1(i)] * dxim[I1(i)] * (u[I1(i + 1)] - u[I1(i)]) -
                       qx[I1(i - 1)] * dxim[I1(i - 1)] * (u[I1(i)] - u[I1(i - 1)])));
}

/* cans1d/hdmlw/mlw_m_bg.f:2-271 */
void oracle_mlw_m_bg_1d(double *ro, double *pr, double *vx, double *vy, double *by,
                        const double *bx, const double *bxm, double dt, double qav,
                        double gm, const double *gx, const double *gxm,
                        const double *sc, const double *dsc, const double *scm,
                        const double *dscm, const double *rr, const double *rrm,
                        const double *drr, const double *drrm, const double *dx,
                        const double *dxm, int ix) {
  enum { NT = 36 };
  double *w = arena_get(&arena_bg, (size_t)NT * ix);
  double *t[NT];
  for (int a = 0; a < NT; a++) t[a] = w + (size_t)a * ix;
  double *dxim = t[0], *dxi = t[1], *ux0 = t[2], *ux1 = t[3];
  double *ee = t[4], *rx = t[5], *ry = t[6], *ez = t[7];
  double *roh = t[8], *prh = t[9], *vxh = t[10], *vyh = t[11], *byh = t[12];
  double *eeh = t[13], *ezh = t[14];
  double *rosc = t[15], *eesc = t[16], *rxsc = t[17], *rysc = t[18], *bysc = t[19];
  double *rosch = t[20], *eesch = t[21], *rxsch = t[22], *rysch = t[23], *bysch = t[24];
  double *drosc = t[25], *deesc = t[26], *drxsc = t[27], *drysc = t[28], *dbysc = t[29];
  double *fx = t[30], *qx = t[31], *ss = t[32];

  const double pi = acos(-1.0);
  const double pi8i = 1. / pi / 8.;
  const double pi4i = 1. / pi / 4.;
  for (int i = 1; i <= ix; i++) {
    dxim[I1(i)] = 1.0 / dxm[I1(i)];
    dxi[I1(i)] = 1.0 / dx[I1(i)];
  }
  for (int i = 2; i <= ix - 1; i++) {
    ux1[I1(i)] = 0.5 * dxm[I1(i - 1)] / dx[I1(i)];
    ux0[I1(i)] = 0.5 * dxm[I1(i)] / dx[I1(i)];
  }
  for (int i = 1; i <= ix; i++) {
    drosc[I1(i)] = 0.0; deesc[I1(i)] = 0.0; drxsc[I1(i)] = 0.0;
    drysc[I1(i)] = 0.0; dbysc[I1(i)] = 0.0;
  }
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    double vv = vx[c] * vx[c] + vy[c] * vy[c];
    double bb = by[c] * by[c] + bx[c] * bx[c];
    ee[c] = pr[c] / (gm - 1) + 0.5 * ro[c] * vv + pi8i * bb;
    rx[c] = ro[c] * vx[c];
    ry[c] = ro[c] * vy[c];
  }
  for (int i = 1; i <= ix; i++) ez[I1(i)] = -vx[I1(i)] * by[I1(i)] + vy[I1(i)] * bx[I1(i)];
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    rosc[c] = ro[c] * sc[c];
    eesc[c] = ee[c] * sc[c];
    rxsc[c] = rx[c] * sc[c];
    rysc[c] = ry[c] * sc[c] * rr[c];
    bysc[c] = by[c] * sc[c] / rr[c];
  }
  /* density */
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    fx[c] = ro[c] * vx[c];
    fx[c] = fx[c] * sc[c];
  }
  half(rosc, rosch, drosc, dt, fx, dxi, dxim, ix);
  /* energy */
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    double vv = vx[c] * vx[c] + vy[c] * vy[c];
    double ep = pr[c] * gm / (gm - 1.) + 0.5 * ro[c] * vv;
    fx[c] = ep * vx[c] - by[c] * ez[c] * pi4i;
    fx[c] = fx[c] * sc[c];
    ss[c] = ro[c] * vx[c] * gx[c];
    ss[c] = ss[c] * sc[c];
  }
  half(eesc, eesch, deesc, dt, fx, dxi, dxim, ix);
  srch(eesch, deesc, dt, ss, ix);
  /* x-momentum */
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    double bbm = by[c] * by[c] - bx[c] * bx[c];
    double bb = by[c] * by[c] + bx[c] * bx[c];
    fx[c] = ro[c] * (vx[c] * vx[c]) + pr[c] + bbm * pi8i;
    ss[c] = ro[c] * gx[c] + (ro[c] * (vy[c] * vy[c]) - (by[c] * by[c]) * pi4i) / rr[c] * drr[c];
    fx[c] = fx[c] * sc[c];
    ss[c] = ss[c] * sc[c] + (pr[c] + bb * pi8i) * dsc[c];
  }
  half(rxsc, rxsch, drxsc, dt, fx, dxi, dxim, ix);
  srch(rxsch, drxsc, dt, ss, ix);
  /* y-momentum */
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    fx[c] = ro[c] * vx[c] * vy[c] - bx[c] * by[c] * pi4i;
    fx[c] = fx[c] * sc[c] * rr[c];
  }
  half(rysc, rysch, drysc, dt, fx, dxi, dxim, ix);
  /* y-magnetic */
  for (int i = 1; i <= ix; i++) {
    size_t c = I1(i);
    fx[c] = -ez[c];
    fx[c] = fx[c] * sc[c];
    fx[c] = fx[c] / rr[c];
  }
  half(bysc, bysch, dbysc, dt, fx, dxi, dxim, ix);

  for (int i = 1; i <= ix - 1; i++) {
    size_t c = I1(i);
    roh[c] = rosch[c] / scm[c];
    eeh[c] = eesch[c] / scm[c];
    vxh[c] = rxsch[c] / rosch[c];
    vyh[c] = rysch[c] / rosch[c] / rrm[c];
    byh[c] = bysch[c] / scm[c] * rrm[c];
    double vv = vxh[c] * vxh[c] + vyh[c] * vyh[c];
    double bb = bxm[c] * bxm[c] + byh[c] * byh[c];
    prh[c] = (gm - 1) * (eeh[c] - 0.5 * roh[c] * vv - pi8i * bb);
  }
  /* the reference loop runs to ix; entry ix is never read */
  for (int i = 1; i <= ix - 1; i++)
    ezh[I1(i)] = -vxh[I1(i)] * byh[I1(i)] + vyh[I1(i)] * bxm[I1(i)];
  /* density */
  for (int i = 1; i <= ix - 1; i++) {
    size_t c = I1(i);
    fx[c] = roh[c] * vxh[c];
    fx[c] = fx[c] * scm[c];
  }
  full(drosc, dt, fx, dxi, ix);
  /* energy */
  for (int i = 1; i <= ix - 1; i++) {
    size_t c = I1(i);
    double vv = vxh[c] * vxh[c] + vyh[c] * vyh[c];
    double eph = prh[c] * gm / (gm - 1.) + 0.5 * roh[c] * vv;
    fx[c] = eph * vxh[c] - byh[c] * ezh[c] * pi4i;
    ss[c] = roh[c] * vxh[c] * gxm[c];
    fx[c] = fx[c] * scm[c];
    ss[c] = ss[c] * scm[c];
  }
  full(deesc, dt, fx, dxi, ix);
  srcf(deesc, dt, ss, ux0, ux1, ix);
  /* x-momentum */
  for (int i = 1; i <= ix - 1; i++) {
    size_t c = I1(i);
    double bbm = byh[c] * byh[c] - bxm[c] * bxm[c];
    double bb = byh[c] * byh[c] + bxm[c] * bxm[c];
    fx[c] = roh[c] * (vxh[c] * vxh[c]) + prh[c] + bbm * pi8i;
    ss[c] = roh[c] * gxm[c] +
            (roh[c] * (vyh[c] * vyh[c]) - (byh[c] * byh[c]) * pi4i) / rrm[c] * drrm[c];
    fx[c] = fx[c] * scm[c];
    ss[c] = ss[c] * scm[c] + (prh[c] + bb * pi8i) * dscm[c];
  }
  full(drxsc, dt, fx, dxi, ix);
  srcf(drxsc, dt, ss, ux0, ux1, ix);
  /* y-momentum */
  for (int i = 1; i <= ix - 1; i++) {
    size_t c = I1(i);
    fx[c] = roh[c] * vxh[c] * vyh[c] - bxm[c] * byh[c] * pi4i;
    fx[c] = fx[c] * scm[c] * rrm[c];
  }
  full(drysc, dt, fx, dxi, ix);
  /* y-magnetic */
  for (int i = 1; i <= ix - 1; i++) {
    size_t c = I1(i);
    fx[c] = -ezh[c];
    fx[c] = fx[c] * scm[c];
    fx[c] = fx[c] / rrm[c];
  }
  full(dbysc, dt, fx, dxi, ix);

  const double zero = 0.0;
  for (int i = 1; i <= ix - 1; i++)
    qx[I1(i)] = qav * dxm[I1(i)] * fmax2(zero, fabs(vx[I1(i + 1)] - vx[I1(i)]) - R4_1EM4);
  artv(rosc, drosc, dt, qx, dxi, dxim, ix);
  artv(eesc, deesc, dt, qx, dxi, dxim, ix);
  artv(rxsc, drxsc, dt, qx, dxi, dxim, ix);
  artv(rysc, drysc, dt, qx, dxi, dxim, ix);
  artv(bysc, dbysc, dt, qx, dxi, dxim, ix);
  for (int i = 2; i <= ix - 1; i++) {
    size_t c = I1(i);
    ro[c] = (rosc[c] + drosc[c]) / sc[c];
    ee[c] = (eesc[c] + deesc[c]) / sc[c];
    rx[c] = (rxsc[c] + drxsc[c]) / sc[c];
    ry[c] = (rysc[c] + drysc[c]) / sc[c] / rr[c];
    by[c] = (bysc[c] + dbysc[c]) / sc[c] * rr[c];
  }
  for (int i = 2; i <= ix - 1; i++) {
    size_t c = I1(i);
    vx[c] = rx[c] / ro[c];
    vy[c] = ry[c] / ro[c];
    double vv = vx[c] * vx[c] + vy[c] * vy[c];
    double bb = bx[c] * bx[c] + by[c] * by[c];
    pr[c] = (gm - 1) * (ee[c] - 0.5 * ro[c] * vv - pi8i * bb);
  }
}

/* cans1d/common/chkdav.f:68-76 */
int oracle_chkdav(double *da, double *vx, double floor_, int ix) {
  int n = 0;
  for (int i = 1; i <= ix; i++) {
    if (da[I1(i)] < floor_) {
      n = n + 1;
      da[I1(i)] = floor_;
      vx[I1(i)] = 0.0;
    }
  }
  return n;
}

/* Uniform deviate in [0, 1) for cell g (0-based) of loop step ns: SplitMix64
 * (Steele, Lea and Flood, "Fast splittable pseudorandom number generators",
 * OOPSLA 2014) of the counter ns*ix + g offset by the seed, top 53 bits. */
double oracle_torque_uniform(unsigned long long seed, long long ns, int g, int ix) {
  uint64_t z = (uint64_t)seed + ((uint64_t)ns * (uint64_t)ix + (uint64_t)g + 1u) *
                          0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * 0x1.0p-53;
}

/* cans1d/md_spicule/hdmlw/trqalfven.f:18-40 with trq(ix) precomputed (the
 * host profile tanh((x-0.75)/0.075)-1 with trq(ix) = trq(ix-2)) and the
 * random number of random_number(anum) replaced by oracle_torque_uniform;
 * q(ix) = q(ix-2) as in the reference. */
void oracle_trqalfven(double *vy, double dt, const double *trq, const double *rr,
                      double trq0, unsigned long long seed, long long ns, int ix) {
  for (int i = 1; i <= ix; i++) {
    const int ic = (i == ix) ? ix - 2 : i;
    const double anum = oracle_torque_uniform(seed, ns, ic - 1, ix);
    const double q = 2 * rr[I1(ic)] * (anum - 0.5);
    vy[I1(i)] = vy[I1(i)] + dt * trq0 * q * trq[I1(i)];
  }
}

/* cans1d/md_spicule/hdmlw/main.f:160-219: the spicule time loop.  Per step:
 * cfl_m (safety, dtmin), t += dt, mlw_m_bg, trqalfven (torque != 0), the
 * boundary program (kind[v][face], lower faces then upper, margin), chkdav of
 * ro then pr (chk != 0), the loop test ns < nstop and t < tend.  The state
 * starts at (t0, ns0).  Returns merr; *t_out, *ns_out and *nev_out receive
 * the final time, step counter and chkdav event count. */
int oracle_spicule_run(double *ro, double *pr, double *vx, double *vy, double *by,
                       const double *bx, const double *bxm, double qav, double gm,
                       const double *gx, const double *gxm, const double *sc,
                       const double *dsc, const double *scm, const double *dscm,
                       const double *rr, const double *rrm, const double *drr,
                       const double *drrm, const double *dx, const double *dxm,
                       const double *trq, double trq0, unsigned long long seed,
                       int torque, double floor_, int chk, const int *kind,
                       int margin, double safety, double dtmin, long long nstop,
                       double tend, double t0, long long ns0, int ix,
                       double *t_out, long long *ns_out, long long *nev_out) {
  double *st[5] = {ro, pr, vx, vy, by};
  double t = t0;
  long long ns = ns0, nev = 0;
  int merr = 0;
  for (;;) {
    ns = ns + 1;
    double dt;
    oracle_cfl_m_1d(&dt, safety, dtmin, &merr, gm, bx, ro, pr, vx, vy, by, dx, ix);
    if (merr) break;
    t = t + dt;
    oracle_mlw_m_bg_1d(ro, pr, vx, vy, by, bx, bxm, dt, qav, gm, gx, gxm, sc, dsc, scm,
                       dscm, rr, rrm, drr, drrm, dx, dxm, ix);
    if (torque) oracle_trqalfven(vy, dt, trq, rr, trq0, seed, ns, ix);
    for (int side = 0; side < 2; side++)
      for (int v = 0; v < 5; v++)
        if (kind[2 * v + side] >= 0)
          oracle_bd_1d(kind[2 * v + side], side, margin, st[v], 0.0, dxm, ix);
    if (chk) {
      nev += oracle_chkdav(ro, vx, floor_, ix);
      nev += oracle_chkdav(pr, vx, floor_, ix);
    }
    if (!(ns < nstop && t < tend)) break;
  }
  *t_out = t;
  *ns_out = ns;
  *nev_out = nev;
  return merr;
}
