/*
 * 2-D mLW step, CFL and vector-potential set-up: line-faithful C restatement
 * of the CANS Fortran (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 *   mlwhalf   cans2d/hdmlw/mlwhalf.f:36-52
 *   mlwsrch   cans2d/hdmlw/mlwsrch.f:87-102
 *   mlwfull   cans2d/hdmlw/mlwfull.f:136-146
 *   mlwsrcf   cans2d/hdmlw/mlwsrcf.f:182-189
 *   mlwartv   cans2d/hdmlw/mlwartv.f:225-233
 *   mlw_m3    cans2d/hdmlw/mlw_m3.f:64-374   (8 conserved variables + az)
 *   mlw_m     cans2d/hdmlw/mlw_m.f           (6 conserved variables + az)
 *   mlw_m3_g, mlw_m_g  cans2d/hdmlw/mlw_m3_g.f, mlw_m_g.f (the same with gravity)
 *   mlw_m3_e, mlw_m_e  cans2d/hdmlw/mlw_m3_e.f, mlw_m_e.f (with resistivity)
 *   mlw_m3_ge, mlw_m_ge cans2d/hdmlw/mlw_m3_ge.f, mlw_m_ge.f (both)
 *   bbtocz, bbtocx, bbtocy  cans2d/common/bbtocz.f:30-41, bbtocx.f:29-33,
 *             bbtocy.f:29-33 (current density)
 *   cfl_m3_e, cfl_m_e  cans2d/common/cfl_m3_e.f:49-86, cfl_m_e.f:47-84
 *   cfl_m3    cans2d/common/cfl_m3.f:38-65
 *   cfl_m     cans2d/common/cfl_m.f:38-77
 *   bbtoaa    cans2d/common/bbtoaa.f:28-49
 */
#include <string.h>

#include "oracle.h"
#include "oracle_common.h"

static oracle_arena arena2d;

/* The artificial viscosity's branch, for the finite-difference check of the
 * adjoint (not a reference routine): mode 0 evaluates q = qav dxm
 * max(0, |dv| - 1e-4) as mlw_m3.f:325-334 does; mode 1 does the same and
 * records each face's branch (bit 0: the max takes |dv| - 1e-4, bit 1:
 * dv < 0) in av_rec, 2 ix jx bytes per step (x faces, then y faces); mode 2
 * holds every face at the recorded branch, q = qav dxm (s dv - 1e-4) on
 * active faces with s the recorded sign, 0 on the others. */
static int av_mode = 0;
static unsigned char *av_rec = NULL;

void oracle_set_av_branch(int mode, unsigned char *rec) {
  av_mode = mode;
  av_rec = rec;
}

static inline double av_coef(double d, size_t f) {
  const double a = fabs(d) - R4_1EM4;
  if (av_mode == 2) {
    const unsigned char b = av_rec[f];
    return (b & 1) ? ((b & 2) ? -d : d) - R4_1EM4 : 0.0;
  }
  if (av_mode == 1) av_rec[f] = (unsigned char)((a > 0.0) | ((d < 0.0) << 1));
  return fmax2(0.0, a);
}

/* cans2d/hdmlw/mlwhalf.f:36-52 */
static void mlwhalf2(const double *u, double *un, double *du, double dt,
                     const double *fx, const double *dxi, const double *dxim,
                     int ix, const double *fy, const double *dyi,
                     const double *dyim, int jx) {
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++)
      du[I2(i, j)] =
          du[I2(i, j)] -
          0.5 * dt * (0.5 * dxi[I1(i)] * (fx[I2(i + 1, j)] - fx[I2(i - 1, j)])) -
          0.5 * dt * (0.5 * dyi[I1(j)] * (fy[I2(i, j + 1)] - fy[I2(i, j - 1)]));
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      double uh = 0.25 * (u[I2(i + 1, j)] + u[I2(i, j)] + u[I2(i + 1, j + 1)] +
                          u[I2(i, j + 1)]);
      double dfdx = dxim[I1(i)] *
                    (fx[I2(i + 1, j)] - fx[I2(i, j)] + fx[I2(i + 1, j + 1)] -
                     fx[I2(i, j + 1)]) /
                    2;
      double dfdy = dyim[I1(j)] *
                    (fy[I2(i, j + 1)] - fy[I2(i, j)] + fy[I2(i + 1, j + 1)] -
                     fy[I2(i + 1, j)]) /
                    2;
      un[I2(i, j)] = uh - dt * dfdx - dt * dfdy;
    }
}

/* cans2d/hdmlw/mlwsrch.f:87-102 */
static void mlwsrch2(double *un, double *du, double dt, const double *s, int ix,
                     int jx) {
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++)
      du[I2(i, j)] = du[I2(i, j)] + 0.5 * dt * s[I2(i, j)];
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      double sh = (s[I2(i + 1, j)] + s[I2(i, j)] + s[I2(i + 1, j + 1)] +
                   s[I2(i, j + 1)]) /
                  4.0;
      un[I2(i, j)] = un[I2(i, j)] + dt * sh;
    }
}

/* cans2d/hdmlw/mlwfull.f:136-146 */
static void mlwfull2(double *du, double dt, const double *fx, const double *dxi,
                     const double *ux0, const double *ux1, int ix,
                     const double *fy, const double *dyi, const double *uy0,
                     const double *uy1, int jx) {
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++) {
      double dfdx =
          dxi[I1(i)] *
          (uy0[I1(j)] * (fx[I2(i, j - 1)] - fx[I2(i - 1, j - 1)]) +
           uy1[I1(j)] * (fx[I2(i, j)] - fx[I2(i - 1, j)]));
      double dfdy =
          dyi[I1(j)] *
          (ux0[I1(i)] * (fy[I2(i - 1, j)] - fy[I2(i - 1, j - 1)]) +
           ux1[I1(i)] * (fy[I2(i, j)] - fy[I2(i, j - 1)]));
      du[I2(i, j)] = du[I2(i, j)] - 0.5 * dt * dfdx - 0.5 * dt * dfdy;
    }
}

/* cans2d/hdmlw/mlwsrcf.f:182-189 */
static void mlwsrcf2(double *du, double dt, const double *s, const double *ux0,
                     const double *ux1, int ix, const double *uy0,
                     const double *uy1, int jx) {
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++) {
      double sh = uy0[I1(j)] * (ux0[I1(i)] * s[I2(i - 1, j - 1)] +
                                ux1[I1(i)] * s[I2(i, j - 1)]) +
                  uy1[I1(j)] * (ux0[I1(i)] * s[I2(i - 1, j)] +
                                ux1[I1(i)] * s[I2(i, j)]);
      du[I2(i, j)] = du[I2(i, j)] + 0.5 * dt * sh;
    }
}

/* cans2d/hdmlw/mlwartv.f:225-233 */
static void mlwartv2(const double *u, double *du, double dt, const double *qx,
                     const double *dxi, const double *dxim, int ix,
                     const double *qy, const double *dyi, const double *dyim,
                     int jx) {
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++)
      du[I2(i, j)] =
          du[I2(i, j)] +
          dt * (dxi[I1(i)] *
                (qx[I2(i, j)] * dxim[I1(i)] * (u[I2(i + 1, j)] - u[I2(i, j)]) -
                 qx[I2(i - 1, j)] * dxim[I1(i - 1)] *
                     (u[I2(i, j)] - u[I2(i - 1, j)]))) +
          dt * (dyi[I1(j)] *
                (qy[I2(i, j)] * dyim[I1(j)] * (u[I2(i, j + 1)] - u[I2(i, j)]) -
                 qy[I2(i, j - 1)] * dyim[I1(j - 1)] *
                     (u[I2(i, j)] - u[I2(i, j - 1)])));
}

/* cans2d/common/bbtocz.f:30-41: z current density at the cells (or corners)
 * 2..ix-1, 2..jx-1 from a 3x3 stencil of bx, by.  Entries outside that
 * range are not written. */
static void bbtocz2(double *cz, const double *bx, const double *by,
                    const double *dx, const double *dy, int ix, int jx) {
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++)
      cz[I2(i, j)] =
          (by[I2(i + 1, j)] - by[I2(i - 1, j)]) / dx[I1(i)] / 2.0 / 2.0 +
          (by[I2(i + 1, j + 1)] - by[I2(i - 1, j + 1)]) / dx[I1(i)] / 2.0 / 4.0 +
          (by[I2(i + 1, j - 1)] - by[I2(i - 1, j - 1)]) / dx[I1(i)] / 2.0 / 4.0 -
          (bx[I2(i, j + 1)] - bx[I2(i, j - 1)]) / dy[I1(j)] / 2.0 / 2.0 -
          (bx[I2(i + 1, j + 1)] - bx[I2(i + 1, j - 1)]) / dy[I1(j)] / 2.0 / 4.0 -
          (bx[I2(i - 1, j + 1)] - bx[I2(i - 1, j - 1)]) / dy[I1(j)] / 2.0 / 4.0;
}

/* cans2d/common/bbtocx.f:29-33 */
static void bbtocx2(double *cx, const double *bz, const double *dy, int ix,
                    int jx) {
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++)
      cx[I2(i, j)] = (bz[I2(i, j + 1)] - bz[I2(i, j - 1)]) / dy[I1(j)] / 2.0;
}

/* cans2d/common/bbtocy.f:29-33 */
static void bbtocy2(double *cy, const double *bz, const double *dx, int ix,
                    int jx) {
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++)
      cy[I2(i, j)] = -(bz[I2(i + 1, j)] - bz[I2(i - 1, j)]) / dx[I1(i)] / 2.0;
}

/* The resistive steps leave two sets of values undefined: the current
 * density on the outer ring of cells (bbtocz writes 2..ix-1 only) and the
 * half-step field at corner ix / row jx, which mlwhalf never sets but the
 * corner bbtocz reads for corner ix-1.  Both are taken as zero here; in
 * the md_recon and md_reccnd set-ups et and etm vanish there, so nothing
 * depends on them. */
static void zero_edge_corners(double *a, int ix, int jx) {
  for (int j = 1; j <= jx; j++) a[I2(ix, j)] = 0.0;
  for (int i = 1; i <= ix; i++) a[I2(i, jx)] = 0.0;
}

/* Metric set-up shared by mlw_m and mlw_m3 (mlw_m3.f:70-86). */
static void metrics2(const double *dx, const double *dxm, int ix,
                     const double *dy, const double *dym, int jx, double *dxi,
                     double *dxim, double *ux0, double *ux1, double *dyi,
                     double *dyim, double *uy0, double *uy1) {
  for (int i = 1; i <= ix; i++) {
    dxi[I1(i)] = 1.0 / dx[I1(i)];
    dxim[I1(i)] = 1.0 / dxm[I1(i)];
  }
  for (int i = 2; i <= ix - 1; i++) {
    ux1[I1(i)] = 0.5 * dxm[I1(i - 1)] / dx[I1(i)];
    ux0[I1(i)] = 0.5 * dxm[I1(i)] / dx[I1(i)];
  }
  for (int j = 1; j <= jx; j++) {
    dyi[I1(j)] = 1.0 / dy[I1(j)];
    dyim[I1(j)] = 1.0 / dym[I1(j)];
  }
  for (int j = 2; j <= jx - 1; j++) {
    uy1[I1(j)] = 0.5 * dym[I1(j - 1)] / dy[I1(j)];
    uy0[I1(j)] = 0.5 * dym[I1(j)] / dy[I1(j)];
  }
}

/* cans2d/hdmlw/mlw_m3.f:2-377 */
/* With gx != NULL this is mlw_m3_g (cans2d/hdmlw/mlw_m3_g.f:1-393): the
 * gravity sources of mlw_m3_g.f:95-121 (cells) and :194-220 (corners) are
 * added through mlwsrch / mlwsrcf to the energy and the x, y momenta. */
static void mlw_m3_core(double *ro, double *pr, double *vx, double *vy,
                        double *vz, double *bx, double *by, double *bz,
                        double *az, double dt, double qav, double gm,
                        const double *gx, const double *gxm, const double *gy,
                        const double *gym, const double *et, const double *etm,
                        const double *dx, const double *dxm,
                        int ix, const double *dy, const double *dym, int jx) {
  const size_t n = (size_t)ix * (size_t)jx;
  const size_t nm = (size_t)(ix > jx ? ix : jx);
  enum { NT = 43 };
  double *w = arena_get(&arena2d, NT * n + 8 * nm);
  double *t[NT];
  for (int a = 0; a < NT; a++) t[a] = w + a * n;
  double *ee = t[0], *rx = t[1], *ry = t[2], *rz = t[3];
  double *ex = t[4], *ey = t[5], *ez = t[6];
  double *roh = t[7], *eeh = t[8], *rxh = t[9], *ryh = t[10], *rzh = t[11];
  double *bxh = t[12], *byh = t[13], *bzh = t[14];
  double *prh = t[15], *vxh = t[16], *vyh = t[17], *vzh = t[18];
  double *exh = t[19], *eyh = t[20], *ezh = t[21], *azh = t[22];
  double *dro = t[23], *dee = t[24], *drx = t[25], *dry = t[26], *drz = t[27];
  double *dbx = t[28], *dby = t[29], *dbz = t[30], *daz = t[31];
  double *fx = t[32], *qx = t[33], *fy = t[34], *qy = t[35], *ss = t[36];
  double *cx = t[37], *cy = t[38], *cz = t[39];
  double *cxh = t[40], *cyh = t[41], *czh = t[42];
  double *m = w + NT * n;
  double *dxi = m, *dxim = m + nm, *ux0 = m + 2 * nm, *ux1 = m + 3 * nm;
  double *dyi = m + 4 * nm, *dyim = m + 5 * nm, *uy0 = m + 6 * nm,
         *uy1 = m + 7 * nm;

  const double pi = acos(-1.0);
  const double pi8i = 1. / pi / 8.;
  const double pi4i = 1. / pi / 4.;
  metrics2(dx, dxm, ix, dy, dym, jx, dxi, dxim, ux0, ux1, dyi, dyim, uy0, uy1);

  /* initialize dro etc. (:91-103) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      dro[c] = 0.0; dee[c] = 0.0; drx[c] = 0.0; dry[c] = 0.0; drz[c] = 0.0;
      dbx[c] = 0.0; dby[c] = 0.0; dbz[c] = 0.0; daz[c] = 0.0;
    }
  /* energy from pressure (:107-116) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      double vv = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
      double bb = bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c];
      ee[c] = pr[c] / (gm - 1) + 0.5 * ro[c] * vv + pi8i * bb;
      rx[c] = ro[c] * vx[c];
      ry[c] = ro[c] * vy[c];
      rz[c] = ro[c] * vz[c];
    }
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      ex[c] = -vy[c] * bz[c] + vz[c] * by[c];
      ey[c] = -vz[c] * bx[c] + vx[c] * bz[c];
      ez[c] = -vx[c] * by[c] + vy[c] * bx[c];
    }
  if (et) {  /* mlw_m3_e.f:124-132: E += et * J */
    memset(cx, 0, n * sizeof(double));
    memset(cy, 0, n * sizeof(double));
    memset(cz, 0, n * sizeof(double));
    bbtocx2(cx, bz, dy, ix, jx);
    bbtocy2(cy, bz, dx, ix, jx);
    bbtocz2(cz, bx, by, dx, dy, ix, jx);
    OMP_FOR
    for (int j = 1; j <= jx; j++)
      for (int i = 1; i <= ix; i++) {
        size_t c = I2(i, j);
        ex[c] = -vy[c] * bz[c] + vz[c] * by[c] + et[c] * cx[c];
        ey[c] = -vz[c] * bx[c] + vx[c] * bz[c] + et[c] * cy[c];
        ez[c] = -vx[c] * by[c] + vy[c] * bx[c] + et[c] * cz[c];
      }
  }

  /* density (:129-135) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = ro[c] * vx[c];
      fy[c] = ro[c] * vy[c];
    }
  mlwhalf2(ro, roh, dro, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  /* energy (:138-146) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      double vv = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
      double ep = pr[c] * gm / (gm - 1.) + 0.5 * ro[c] * vv;
      fx[c] = ep * vx[c] + (bz[c] * ey[c] - by[c] * ez[c]) * pi4i;
      fy[c] = ep * vy[c] + (bx[c] * ez[c] - bz[c] * ex[c]) * pi4i;
    }
  mlwhalf2(ee, eeh, dee, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx; j++)
      for (int i = 1; i <= ix; i++) {
        size_t c = I2(i, j);
        ss[c] = ro[c] * (vx[c] * gx[c] + vy[c] * gy[c]);
      }
    mlwsrch2(eeh, dee, dt, ss, ix, jx);
  }
  /* x-momentum (:149-156) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = ro[c] * (vx[c] * vx[c]) + pr[c] +
              pi8i * (by[c] * by[c] + bz[c] * bz[c] - bx[c] * bx[c]);
      fy[c] = ro[c] * vx[c] * vy[c] - pi4i * bx[c] * by[c];
    }
  mlwhalf2(rx, rxh, drx, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx; j++)
      for (int i = 1; i <= ix; i++) {
        size_t c = I2(i, j);
        ss[c] = ro[c] * gx[c];
      }
    mlwsrch2(rxh, drx, dt, ss, ix, jx);
  }
  /* y-momentum (:159-166) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = ro[c] * vy[c] * vx[c] - pi4i * by[c] * bx[c];
      fy[c] = ro[c] * (vy[c] * vy[c]) + pr[c] +
              pi8i * (bx[c] * bx[c] + bz[c] * bz[c] - by[c] * by[c]);
    }
  mlwhalf2(ry, ryh, dry, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx; j++)
      for (int i = 1; i <= ix; i++) {
        size_t c = I2(i, j);
        ss[c] = ro[c] * gy[c];
      }
    mlwsrch2(ryh, dry, dt, ss, ix, jx);
  }
  /* z-momentum (:169-175) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = ro[c] * vz[c] * vx[c] - pi4i * bz[c] * bx[c];
      fy[c] = ro[c] * vz[c] * vy[c] - pi4i * bz[c] * by[c];
    }
  mlwhalf2(rz, rzh, drz, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  /* x-magnetic (:178-184) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = 0.;
      fy[c] = ez[c];
    }
  mlwhalf2(bx, bxh, dbx, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  /* y-magnetic (:187-193) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = -ez[c];
      fy[c] = 0.;
    }
  mlwhalf2(by, byh, dby, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  /* z-magnetic (:196-202) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = ey[c];
      fy[c] = -ex[c];
    }
  mlwhalf2(bz, bzh, dbz, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  /* z-magnetic potential (:205-210) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) ss[I2(i, j)] = -ez[I2(i, j)];
  mlwsrch2(azh, daz, dt, ss, ix, jx);

  /* half-step primitives (:214-230) */
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      vxh[c] = rxh[c] / roh[c];
      vyh[c] = ryh[c] / roh[c];
      vzh[c] = rzh[c] / roh[c];
      double vv = vxh[c] * vxh[c] + vyh[c] * vyh[c] + vzh[c] * vzh[c];
      double bb = bxh[c] * bxh[c] + byh[c] * byh[c] + bzh[c] * bzh[c];
      prh[c] = (gm - 1) * (eeh[c] - 0.5 * roh[c] * vv - pi8i * bb);
    }
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      exh[c] = -vyh[c] * bzh[c] + vzh[c] * byh[c];
      eyh[c] = -vzh[c] * bxh[c] + vxh[c] * bzh[c];
      ezh[c] = -vxh[c] * byh[c] + vyh[c] * bxh[c];
    }
  if (et) {  /* mlw_m3_e.f:236-244: Eh += etm * Jh at the corners */
    zero_edge_corners(bxh, ix, jx);
    zero_edge_corners(byh, ix, jx);
    zero_edge_corners(bzh, ix, jx);
    memset(cxh, 0, n * sizeof(double));
    memset(cyh, 0, n * sizeof(double));
    memset(czh, 0, n * sizeof(double));
    bbtocx2(cxh, bzh, dym, ix, jx);
    bbtocy2(cyh, bzh, dxm, ix, jx);
    bbtocz2(czh, bxh, byh, dxm, dym, ix, jx);
    OMP_FOR
    for (int j = 1; j <= jx - 1; j++)
      for (int i = 1; i <= ix - 1; i++) {
        size_t c = I2(i, j);
        exh[c] = -vyh[c] * bzh[c] + vzh[c] * byh[c] + etm[c] * cxh[c];
        eyh[c] = -vzh[c] * bxh[c] + vxh[c] * bzh[c] + etm[c] * cyh[c];
        ezh[c] = -vxh[c] * byh[c] + vyh[c] * bxh[c] + etm[c] * czh[c];
      }
  }

  /* full step: density (:235-241) */
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      fx[c] = roh[c] * vxh[c];
      fy[c] = roh[c] * vyh[c];
    }
  mlwfull2(dro, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  /* energy (:244-254) */
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      double vv = vxh[c] * vxh[c] + vyh[c] * vyh[c] + vzh[c] * vzh[c];
      double ep = prh[c] * gm / (gm - 1.) + 0.5 * roh[c] * vv;
      fx[c] = ep * vxh[c] + (bzh[c] * eyh[c] - byh[c] * ezh[c]) * pi4i;
      fy[c] = ep * vyh[c] + (bxh[c] * ezh[c] - bzh[c] * exh[c]) * pi4i;
    }
  mlwfull2(dee, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx - 1; j++)
      for (int i = 1; i <= ix - 1; i++) {
        size_t c = I2(i, j);
        ss[c] = roh[c] * (vxh[c] * gxm[c] + vyh[c] * gym[c]);
      }
    mlwsrcf2(dee, dt, ss, ux0, ux1, ix, uy0, uy1, jx);
  }
  /* x-momentum (:257-264) */
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      fx[c] = roh[c] * (vxh[c] * vxh[c]) + prh[c] +
              pi8i * (byh[c] * byh[c] + bzh[c] * bzh[c] - bxh[c] * bxh[c]);
      fy[c] = roh[c] * vxh[c] * vyh[c] - pi4i * bxh[c] * byh[c];
    }
  mlwfull2(drx, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx - 1; j++)
      for (int i = 1; i <= ix - 1; i++) {
        size_t c = I2(i, j);
        ss[c] = roh[c] * gxm[c];
      }
    mlwsrcf2(drx, dt, ss, ux0, ux1, ix, uy0, uy1, jx);
  }
  /* y-momentum (:267-274) */
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      fx[c] = roh[c] * vyh[c] * vxh[c] - pi4i * byh[c] * bxh[c];
      fy[c] = roh[c] * (vyh[c] * vyh[c]) + prh[c] +
              pi8i * (bxh[c] * bxh[c] + bzh[c] * bzh[c] - byh[c] * byh[c]);
    }
  mlwfull2(dry, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx - 1; j++)
      for (int i = 1; i <= ix - 1; i++) {
        size_t c = I2(i, j);
        ss[c] = roh[c] * gym[c];
      }
    mlwsrcf2(dry, dt, ss, ux0, ux1, ix, uy0, uy1, jx);
  }
  /* z-momentum (:277-283); the reference sweeps the whole array here, the
   * extra edge entries are never read by mlwfull. */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = roh[c] * vzh[c] * vxh[c] - pi4i * bzh[c] * bxh[c];
      fy[c] = roh[c] * vzh[c] * vyh[c] - pi4i * bzh[c] * byh[c];
    }
  mlwfull2(drz, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  /* x-magnetic (:286-292) */
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      fx[c] = 0.;
      fy[c] = ezh[c];
    }
  mlwfull2(dbx, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  /* y-magnetic (:294-301) */
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      fx[c] = -ezh[c];
      fy[c] = 0.;
    }
  mlwfull2(dby, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  /* z-magnetic (:303-310) */
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      fx[c] = eyh[c];
      fy[c] = -exh[c];
    }
  mlwfull2(dbz, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  /* z-magnetic potential (:313-318) */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) ss[I2(i, j)] = -ezh[I2(i, j)];
  mlwsrcf2(daz, dt, ss, ux0, ux1, ix, uy0, uy1, jx);

  /* artificial-viscosity coefficients (:324-334) */
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++)
      qx[I2(i, j)] =
          qav * dxm[I1(i)] * av_coef(vx[I2(i + 1, j)] - vx[I2(i, j)], I2(i, j));
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix; i++)
      qy[I2(i, j)] =
          qav * dym[I1(j)] * av_coef(vy[I2(i, j + 1)] - vy[I2(i, j)], n + I2(i, j));
  /* apply artificial viscosity (:338-345) */
  mlwartv2(ro, dro, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(ee, dee, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(rx, drx, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(ry, dry, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(rz, drz, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(bx, dbx, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(by, dby, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(bz, dbz, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);

  /* update internal points (:349-361) */
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      ro[c] = ro[c] + dro[c];
      ee[c] = ee[c] + dee[c];
      rx[c] = rx[c] + drx[c];
      ry[c] = ry[c] + dry[c];
      rz[c] = rz[c] + drz[c];
      bx[c] = bx[c] + dbx[c];
      by[c] = by[c] + dby[c];
      bz[c] = bz[c] + dbz[c];
      az[c] = az[c] + daz[c];
    }
  /* total energy to pressure (:365-374) */
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      vx[c] = rx[c] / ro[c];
      vy[c] = ry[c] / ro[c];
      vz[c] = rz[c] / ro[c];
      double vv = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
      double bb = bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c];
      pr[c] = (gm - 1) * (ee[c] - 0.5 * ro[c] * vv - pi8i * bb);
    }
}

/* cans2d/hdmlw/mlw_m.f:2-324 (ro,pr,vx,vy,bx,by + az; no z components) */
/* With gx != NULL this is mlw_m_g (cans2d/hdmlw/mlw_m_g.f): gravity sources
 * of mlw_m_g.f:96-122 and :175-201 through mlwsrch / mlwsrcf. */
static void mlw_m_core(double *ro, double *pr, double *vx, double *vy,
                       double *bx, double *by, double *az, double dt, double qav,
                       double gm, const double *gx, const double *gxm,
                       const double *gy, const double *gym, const double *et,
                       const double *etm, const double *dx,
                       const double *dxm, int ix, const double *dy,
                       const double *dym, int jx) {
  const size_t n = (size_t)ix * (size_t)jx;
  const size_t nm = (size_t)(ix > jx ? ix : jx);
  enum { NT = 29 };
  double *w = arena_get(&arena2d, NT * n + 8 * nm);
  double *t[NT];
  for (int a = 0; a < NT; a++) t[a] = w + a * n;
  double *ee = t[0], *rx = t[1], *ry = t[2], *ez = t[3];
  double *roh = t[4], *eeh = t[5], *rxh = t[6], *ryh = t[7];
  double *bxh = t[8], *byh = t[9];
  double *prh = t[10], *vxh = t[11], *vyh = t[12], *ezh = t[13], *azh = t[14];
  double *dro = t[15], *dee = t[16], *drx = t[17], *dry = t[18];
  double *dbx = t[19], *dby = t[20], *daz = t[21];
  double *fx = t[22], *qx = t[23], *fy = t[24], *qy = t[25], *ss = t[26];
  double *cz = t[27], *czh = t[28];
  double *m = w + NT * n;
  double *dxi = m, *dxim = m + nm, *ux0 = m + 2 * nm, *ux1 = m + 3 * nm;
  double *dyi = m + 4 * nm, *dyim = m + 5 * nm, *uy0 = m + 6 * nm,
         *uy1 = m + 7 * nm;

  const double pi = acos(-1.0);
  const double pi8i = 1. / pi / 8.;
  const double pi4i = 1. / pi / 4.;
  metrics2(dx, dxm, ix, dy, dym, jx, dxi, dxim, ux0, ux1, dyi, dyim, uy0, uy1);

  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      dro[c] = 0.0; dee[c] = 0.0; drx[c] = 0.0; dry[c] = 0.0;
      dbx[c] = 0.0; dby[c] = 0.0; daz[c] = 0.0;
    }
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      double vv = vx[c] * vx[c] + vy[c] * vy[c];
      double bb = bx[c] * bx[c] + by[c] * by[c];
      ee[c] = pr[c] / (gm - 1) + 0.5 * ro[c] * vv + pi8i * bb;
      rx[c] = ro[c] * vx[c];
      ry[c] = ro[c] * vy[c];
    }
  if (et) {  /* mlw_m_e.f:125-129: ez += et * cz */
    memset(cz, 0, n * sizeof(double));
    bbtocz2(cz, bx, by, dx, dy, ix, jx);
  }
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      ez[c] = et ? -vx[c] * by[c] + vy[c] * bx[c] + et[c] * cz[c]
                 : -vx[c] * by[c] + vy[c] * bx[c];
    }
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = ro[c] * vx[c];
      fy[c] = ro[c] * vy[c];
    }
  mlwhalf2(ro, roh, dro, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      double vv = vx[c] * vx[c] + vy[c] * vy[c];
      double ep = pr[c] * gm / (gm - 1.) + 0.5 * ro[c] * vv;
      fx[c] = ep * vx[c] - by[c] * ez[c] * pi4i;
      fy[c] = ep * vy[c] + bx[c] * ez[c] * pi4i;
    }
  mlwhalf2(ee, eeh, dee, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx; j++)
      for (int i = 1; i <= ix; i++) {
        size_t c = I2(i, j);
        ss[c] = ro[c] * (vx[c] * gx[c] + vy[c] * gy[c]);
      }
    mlwsrch2(eeh, dee, dt, ss, ix, jx);
  }
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = ro[c] * (vx[c] * vx[c]) + pr[c] +
              pi8i * (by[c] * by[c] - bx[c] * bx[c]);
      fy[c] = ro[c] * vx[c] * vy[c] - pi4i * bx[c] * by[c];
    }
  mlwhalf2(rx, rxh, drx, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx; j++)
      for (int i = 1; i <= ix; i++) {
        size_t c = I2(i, j);
        ss[c] = ro[c] * gx[c];
      }
    mlwsrch2(rxh, drx, dt, ss, ix, jx);
  }
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = ro[c] * vy[c] * vx[c] - pi4i * by[c] * bx[c];
      fy[c] = ro[c] * (vy[c] * vy[c]) + pr[c] +
              pi8i * (bx[c] * bx[c] - by[c] * by[c]);
    }
  mlwhalf2(ry, ryh, dry, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx; j++)
      for (int i = 1; i <= ix; i++) {
        size_t c = I2(i, j);
        ss[c] = ro[c] * gy[c];
      }
    mlwsrch2(ryh, dry, dt, ss, ix, jx);
  }
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = 0.;
      fy[c] = ez[c];
    }
  mlwhalf2(bx, bxh, dbx, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      fx[c] = -ez[c];
      fy[c] = 0.;
    }
  mlwhalf2(by, byh, dby, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx);
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) ss[I2(i, j)] = -ez[I2(i, j)];
  mlwsrch2(azh, daz, dt, ss, ix, jx);

  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      vxh[c] = rxh[c] / roh[c];
      vyh[c] = ryh[c] / roh[c];
      double vv = vxh[c] * vxh[c] + vyh[c] * vyh[c];
      double bb = bxh[c] * bxh[c] + byh[c] * byh[c];
      prh[c] = (gm - 1) * (eeh[c] - 0.5 * roh[c] * vv - pi8i * bb);
    }
  if (et) {  /* mlw_m_e.f:216-220: ezh += etm * czh */
    zero_edge_corners(bxh, ix, jx);
    zero_edge_corners(byh, ix, jx);
    memset(czh, 0, n * sizeof(double));
    bbtocz2(czh, bxh, byh, dxm, dym, ix, jx);
  }
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      ezh[c] = et ? -vxh[c] * byh[c] + vyh[c] * bxh[c] + etm[c] * czh[c]
                  : -vxh[c] * byh[c] + vyh[c] * bxh[c];
    }
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      fx[c] = roh[c] * vxh[c];
      fy[c] = roh[c] * vyh[c];
    }
  mlwfull2(dro, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      double vv = vxh[c] * vxh[c] + vyh[c] * vyh[c];
      double ep = prh[c] * gm / (gm - 1.) + 0.5 * roh[c] * vv;
      fx[c] = ep * vxh[c] - byh[c] * ezh[c] * pi4i;
      fy[c] = ep * vyh[c] + bxh[c] * ezh[c] * pi4i;
    }
  mlwfull2(dee, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx - 1; j++)
      for (int i = 1; i <= ix - 1; i++) {
        size_t c = I2(i, j);
        ss[c] = roh[c] * (vxh[c] * gxm[c] + vyh[c] * gym[c]);
      }
    mlwsrcf2(dee, dt, ss, ux0, ux1, ix, uy0, uy1, jx);
  }
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      fx[c] = roh[c] * (vxh[c] * vxh[c]) + prh[c] +
              pi8i * (byh[c] * byh[c] - bxh[c] * bxh[c]);
      fy[c] = roh[c] * vxh[c] * vyh[c] - pi4i * bxh[c] * byh[c];
    }
  mlwfull2(drx, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx - 1; j++)
      for (int i = 1; i <= ix - 1; i++) {
        size_t c = I2(i, j);
        ss[c] = roh[c] * gxm[c];
      }
    mlwsrcf2(drx, dt, ss, ux0, ux1, ix, uy0, uy1, jx);
  }
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      fx[c] = roh[c] * vyh[c] * vxh[c] - pi4i * byh[c] * bxh[c];
      fy[c] = roh[c] * (vyh[c] * vyh[c]) + prh[c] +
              pi8i * (bxh[c] * bxh[c] - byh[c] * byh[c]);
    }
  mlwfull2(dry, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  if (gx) {
    OMP_FOR
    for (int j = 1; j <= jx - 1; j++)
      for (int i = 1; i <= ix - 1; i++) {
        size_t c = I2(i, j);
        ss[c] = roh[c] * gym[c];
      }
    mlwsrcf2(dry, dt, ss, ux0, ux1, ix, uy0, uy1, jx);
  }
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      fx[c] = 0.;
      fy[c] = ezh[c];
    }
  mlwfull2(dbx, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      fx[c] = -ezh[c];
      fy[c] = 0.;
    }
  mlwfull2(dby, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx);
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) ss[I2(i, j)] = -ezh[I2(i, j)];
  mlwsrcf2(daz, dt, ss, ux0, ux1, ix, uy0, uy1, jx);

  const double zero = 0.0;
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix - 1; i++)
      qx[I2(i, j)] =
          qav * dxm[I1(i)] *
          fmax2(zero, fabs(vx[I2(i + 1, j)] - vx[I2(i, j)]) - R4_1EM4);
  OMP_FOR
  for (int j = 1; j <= jx - 1; j++)
    for (int i = 1; i <= ix; i++)
      qy[I2(i, j)] =
          qav * dym[I1(j)] *
          fmax2(zero, fabs(vy[I2(i, j + 1)] - vy[I2(i, j)]) - R4_1EM4);
  mlwartv2(ro, dro, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(ee, dee, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(rx, drx, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(ry, dry, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(bx, dbx, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  mlwartv2(by, dby, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx);
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      ro[c] = ro[c] + dro[c];
      ee[c] = ee[c] + dee[c];
      rx[c] = rx[c] + drx[c];
      ry[c] = ry[c] + dry[c];
      bx[c] = bx[c] + dbx[c];
      by[c] = by[c] + dby[c];
      az[c] = az[c] + daz[c];
    }
  OMP_FOR
  for (int j = 2; j <= jx - 1; j++)
    for (int i = 2; i <= ix - 1; i++) {
      size_t c = I2(i, j);
      vx[c] = rx[c] / ro[c];
      vy[c] = ry[c] / ro[c];
      double vv = vx[c] * vx[c] + vy[c] * vy[c];
      double bb = bx[c] * bx[c] + by[c] * by[c];
      pr[c] = (gm - 1) * (ee[c] - 0.5 * ro[c] * vv - pi8i * bb);
    }
}

/* cans2d/common/cfl_m3.f:38-65.  The per-cell dtq array and the serial
 * first-minimum scan give the same value as a min-reduction: min is exact. */
void oracle_mlw_m3_2d(double *ro, double *pr, double *vx, double *vy,
                      double *vz, double *bx, double *by, double *bz,
                      double *az, double dt, double qav, double gm,
                      const double *dx, const double *dxm, int ix,
                      const double *dy, const double *dym, int jx) {
  mlw_m3_core(ro, pr, vx, vy, vz, bx, by, bz, az, dt, qav, gm, NULL, NULL, NULL, NULL,
              NULL, NULL, dx, dxm, ix, dy, dym, jx);
}

void oracle_mlw_m3_g_2d(double *ro, double *pr, double *vx, double *vy,
                        double *vz, double *bx, double *by, double *bz,
                        double *az, double dt, double qav, double gm,
                        const double *gx, const double *gxm, const double *gy,
                        const double *gym, const double *dx, const double *dxm,
                        int ix, const double *dy, const double *dym, int jx) {
  mlw_m3_core(ro, pr, vx, vy, vz, bx, by, bz, az, dt, qav, gm, gx, gxm, gy, gym,
              NULL, NULL, dx, dxm, ix, dy, dym, jx);
}

void oracle_mlw_m_2d(double *ro, double *pr, double *vx, double *vy,
                     double *bx, double *by, double *az, double dt, double qav,
                     double gm, const double *dx, const double *dxm, int ix,
                     const double *dy, const double *dym, int jx) {
  mlw_m_core(ro, pr, vx, vy, bx, by, az, dt, qav, gm, NULL, NULL, NULL, NULL, NULL,
             NULL, dx, dxm, ix, dy, dym, jx);
}

void oracle_mlw_m_g_2d(double *ro, double *pr, double *vx, double *vy,
                       double *bx, double *by, double *az, double dt, double qav,
                       double gm, const double *gx, const double *gxm,
                       const double *gy, const double *gym, const double *dx,
                       const double *dxm, int ix, const double *dy,
                       const double *dym, int jx) {
  mlw_m_core(ro, pr, vx, vy, bx, by, az, dt, qav, gm, gx, gxm, gy, gym, NULL, NULL,
             dx, dxm, ix, dy, dym, jx);
}

/* mlw_m3_e / mlw_m3_ge (cans2d/hdmlw/mlw_m3_e.f:2, mlw_m3_ge.f:2): gx NULL
 * gives the step without gravity. */
void oracle_mlw_m3_ge_2d(double *ro, double *pr, double *vx, double *vy,
                         double *vz, double *bx, double *by, double *bz,
                         double *az, double dt, double qav, double gm,
                         const double *gx, const double *gxm, const double *gy,
                         const double *gym, const double *et, const double *etm,
                         const double *dx, const double *dxm, int ix,
                         const double *dy, const double *dym, int jx) {
  mlw_m3_core(ro, pr, vx, vy, vz, bx, by, bz, az, dt, qav, gm, gx, gxm, gy, gym,
              et, etm, dx, dxm, ix, dy, dym, jx);
}

/* mlw_m_e / mlw_m_ge (cans2d/hdmlw/mlw_m_e.f:2, mlw_m_ge.f:2) */
void oracle_mlw_m_ge_2d(double *ro, double *pr, double *vx, double *vy,
                        double *bx, double *by, double *az, double dt, double qav,
                        double gm, const double *gx, const double *gxm,
                        const double *gy, const double *gym, const double *et,
                        const double *etm, const double *dx, const double *dxm,
                        int ix, const double *dy, const double *dym, int jx) {
  mlw_m_core(ro, pr, vx, vy, bx, by, az, dt, qav, gm, gx, gxm, gy, gym, et, etm,
             dx, dxm, ix, dy, dym, jx);
}

/* cfl_m3_e / cfl_m_e (cans2d/common/cfl_m3_e.f:49-86, cfl_m_e.f:47-84): the
 * wave limit of cfl_m3 / cfl_m and the diffusion limit
 * safety*0.5*dmesh**2/max(et,etmin), etmin the single-precision 1.e-5.
 * bz, vz NULL gives cfl_m_e. */
void oracle_cfl_m3_e_2d(double *dt, double safety, double dtmin, int *merr,
                        double gm, const double *ro, const double *pr,
                        const double *vx, const double *vy, const double *vz,
                        const double *bx, const double *by, const double *bz,
                        const double *et, const double *dx, int ix,
                        const double *dy, int jx) {
  const double pi = acos(-1.0);
  const double pi4i = 1. / pi / 4.;
  const double etmin = (double)1.e-5f;
  double dmin = R4_1E20;
#ifdef _OPENMP
#pragma omp parallel for reduction(min : dmin) schedule(static)
#endif
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      double dmesh = fmin2(dx[I1(i)], dy[I1(j)]);
      double b2 = bz ? bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c]
                     : bx[c] * bx[c] + by[c] * by[c];
      double ca2 = b2 * pi4i / ro[c];
      double cs2 = gm * pr[c] / ro[c];
      double v2 = vz ? vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c]
                     : vx[c] * vx[c] + vy[c] * vy[c];
      double dtcfl = dmesh / sqrt(v2 + cs2 + ca2);
      double dtwav = safety * dtcfl;
      double dtdif = safety * 0.5 * (dmesh * dmesh) / fmax2(et[c], etmin);
      double dtq = fmin2(dtwav, dtdif);
      if (dtq < dmin) dmin = dtq;
    }
  *dt = dmin;
  *merr = 0;
  if (*dt < dtmin) *merr = 9001;
}

void oracle_cfl_m3_2d(double *dt, double safety, double dtmin, int *merr,
                      double gm, const double *ro, const double *pr,
                      const double *vx, const double *vy, const double *vz,
                      const double *bx, const double *by, const double *bz,
                      const double *dx, int ix, const double *dy, int jx) {
  const double pi = acos(-1.0);
  const double pi4i = 1. / pi / 4.;
  double dmin = R4_1E20;
#ifdef _OPENMP
#pragma omp parallel for reduction(min : dmin) schedule(static)
#endif
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      double b2 = bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c];
      double ca2 = b2 * pi4i / ro[c];
      double cs2 = gm * pr[c] / ro[c];
      double v2 = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
      double dtcfl = fmin2(dx[I1(i)], dy[I1(j)]) / sqrt(v2 + cs2 + ca2);
      double dtq = safety * dtcfl;
      if (dtq < dmin) dmin = dtq;
    }
  *dt = dmin;
  *merr = 0;
  if (*dt < dtmin) *merr = 9001;
}

/* cans2d/common/cfl_m.f:38-77 */
void oracle_cfl_m_2d(double *dt, double safety, double dtmin, int *merr,
                     double gm, const double *ro, const double *pr,
                     const double *vx, const double *vy, const double *bx,
                     const double *by, const double *dx, int ix,
                     const double *dy, int jx) {
  const double pi = acos(-1.0);
  const double pi4i = 1. / pi / 4.;
  double dmin = R4_1E20;
#ifdef _OPENMP
#pragma omp parallel for reduction(min : dmin) schedule(static)
#endif
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      size_t c = I2(i, j);
      double b2 = bx[c] * bx[c] + by[c] * by[c];
      double ca2 = b2 * pi4i / ro[c];
      double cs2 = gm * pr[c] / ro[c];
      double v2 = vx[c] * vx[c] + vy[c] * vy[c];
      double dtcfl = fmin2(dx[I1(i)], dy[I1(j)]) / sqrt(v2 + cs2 + ca2);
      double dtq = safety * dtcfl;
      if (dtq < dmin) dmin = dtq;
    }
  *dt = dmin;
  *merr = 0;
  if (*dt < dtmin) *merr = 9001;
}

/* cans2d/common/bbtoaa.f:28-49 */
void oracle_bbtoaa_2d(double *az, const double *bx, const double *by,
                      const double *dxm, const double *dym, int margin, int ix,
                      int jx) {
  az[I2(margin + 1, margin + 1)] = 0.0;
  int i = margin + 1;
  for (int j = margin + 2; j <= jx; j++)
    az[I2(i, j)] = az[I2(i, j - 1)] +
                   0.5 * (bx[I2(i, j - 1)] + bx[I2(i, j)]) * dym[I1(j - 1)];
  for (int j = margin; j >= 1; j--)
    az[I2(i, j)] =
        az[I2(i, j + 1)] - 0.5 * (bx[I2(i, j)] + bx[I2(i, j + 1)]) * dym[I1(j)];
  for (int j = 1; j <= jx; j++) {
    for (int ii = margin + 2; ii <= ix; ii++)
      az[I2(ii, j)] = az[I2(ii - 1, j)] -
                      0.5 * (by[I2(ii - 1, j)] + by[I2(ii, j)]) * dxm[I1(ii - 1)];
    for (int ii = margin; ii >= 1; ii--)
      az[I2(ii, j)] =
          az[I2(ii + 1, j)] + 0.5 * (by[I2(ii, j)] + by[I2(ii + 1, j)]) * dxm[I1(ii)];
  }
}
