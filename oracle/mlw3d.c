/*
 * 3-D mLW step and CFL: line-faithful C restatement of the CANS Fortran
 * (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 *   mlwhalf   cans3d/hdmlw/mlwhalf.f:38-65
 *   mlwfull   cans3d/hdmlw/mlwfull.f:34-52
 *   mlwartv   cans3d/hdmlw/mlwartv.f
 *   mlw_m     cans3d/hdmlw/mlw_m.f:2-453
 *   mlw_m_g   cans3d/hdmlw/mlw_m_g.f:2-469 (with gravity), with
 *   mlwsrch   cans3d/hdmlw/mlwsrch.f:32-50 and mlwsrcf cans3d/hdmlw/mlwsrcf.f:35-45
 *   mlw_m_e   cans3d/hdmlw/mlw_m_e.f:2-473 (with resistivity), with
 *   bbtocx/y/z cans3d/common/bbtocx.f:29-35, bbtocy.f, bbtocz.f
 *   cfl_m_e   cans3d/common/cfl_m_e.f (diffusion limit, etmin 1.d-10)
 *   cfl_m     cans3d/common/cfl_m.f:39-85 (pi in single precision)
 */
#include <string.h>

#include "oracle.h"
#include "oracle_common.h"

static oracle_arena arena3d;

#define A(a, i, j, k) a[I3(i, j, k)]

/* cans3d/hdmlw/mlwhalf.f */
static void mlwhalf3(const double *u, double *un, double *du, double dt,
                     const double *fx, const double *dxi, const double *dxim,
                     int ix, const double *fy, const double *dyi,
                     const double *dyim, int jx, const double *fz,
                     const double *dzi, const double *dzim, int kx) {
  OMP_FOR
  for (int k = 2; k <= kx - 1; k++)
    for (int j = 2; j <= jx - 1; j++)
      for (int i = 2; i <= ix - 1; i++)
        A(du, i, j, k) =
            A(du, i, j, k) -
            0.5 * dt * (0.5 * dxi[I1(i)] * (A(fx, i + 1, j, k) - A(fx, i - 1, j, k))) -
            0.5 * dt * (0.5 * dyi[I1(j)] * (A(fy, i, j + 1, k) - A(fy, i, j - 1, k))) -
            0.5 * dt * (0.5 * dzi[I1(k)] * (A(fz, i, j, k + 1) - A(fz, i, j, k - 1)));
  OMP_FOR
  for (int k = 1; k <= kx - 1; k++)
    for (int j = 1; j <= jx - 1; j++)
      for (int i = 1; i <= ix - 1; i++) {
        double uh = (A(u, i + 1, j, k) + A(u, i, j, k) + A(u, i + 1, j + 1, k) +
                     A(u, i, j + 1, k) + A(u, i + 1, j, k + 1) + A(u, i, j, k + 1) +
                     A(u, i + 1, j + 1, k + 1) + A(u, i, j + 1, k + 1)) /
                    8;
        double dfdx = (A(fx, i + 1, j, k) - A(fx, i, j, k) + A(fx, i + 1, j + 1, k) -
                       A(fx, i, j + 1, k) + A(fx, i + 1, j, k + 1) - A(fx, i, j, k + 1) +
                       A(fx, i + 1, j + 1, k + 1) - A(fx, i, j + 1, k + 1)) /
                      4 * dxim[I1(i)];
        double dfdy = (A(fy, i, j + 1, k) - A(fy, i, j, k) + A(fy, i + 1, j + 1, k) -
                       A(fy, i + 1, j, k) + A(fy, i, j + 1, k + 1) - A(fy, i, j, k + 1) +
                       A(fy, i + 1, j + 1, k + 1) - A(fy, i + 1, j, k + 1)) /
                      4 * dyim[I1(j)];
        double dfdz = (A(fz, i, j, k + 1) - A(fz, i, j, k) + A(fz, i + 1, j, k + 1) -
                       A(fz, i + 1, j, k) + A(fz, i, j + 1, k + 1) - A(fz, i, j + 1, k) +
                       A(fz, i + 1, j + 1, k + 1) - A(fz, i + 1, j + 1, k)) /
                      4 * dzim[I1(k)];
        A(un, i, j, k) = uh - dt * dfdx - dt * dfdy - dt * dfdz;
      }
}

/* cans3d/hdmlw/mlwfull.f */
static void mlwfull3(double *du, double dt, const double *fx, const double *dxi,
                     const double *ux0, const double *ux1, int ix,
                     const double *fy, const double *dyi, const double *uy0,
                     const double *uy1, int jx, const double *fz,
                     const double *dzi, const double *uz0, const double *uz1,
                     int kx) {
  OMP_FOR
  for (int k = 2; k <= kx - 1; k++)
    for (int j = 2; j <= jx - 1; j++)
      for (int i = 2; i <= ix - 1; i++) {
        double dfdx =
            dxi[I1(i)] *
            (uz0[I1(k)] * (uy0[I1(j)] * (A(fx, i, j - 1, k - 1) - A(fx, i - 1, j - 1, k - 1)) +
                           uy1[I1(j)] * (A(fx, i, j, k - 1) - A(fx, i - 1, j, k - 1))) +
             uz1[I1(k)] * (uy0[I1(j)] * (A(fx, i, j - 1, k) - A(fx, i - 1, j - 1, k)) +
                           uy1[I1(j)] * (A(fx, i, j, k) - A(fx, i - 1, j, k))));
        double dfdy =
            dyi[I1(j)] *
            (ux0[I1(i)] * (uz0[I1(k)] * (A(fy, i - 1, j, k - 1) - A(fy, i - 1, j - 1, k - 1)) +
                           uz1[I1(k)] * (A(fy, i - 1, j, k) - A(fy, i - 1, j - 1, k))) +
             ux1[I1(i)] * (uz0[I1(k)] * (A(fy, i, j, k - 1) - A(fy, i, j - 1, k - 1)) +
                           uz1[I1(k)] * (A(fy, i, j, k) - A(fy, i, j - 1, k))));
        double dfdz =
            dzi[I1(k)] *
            (uy0[I1(j)] * (ux0[I1(i)] * (A(fz, i - 1, j - 1, k) - A(fz, i - 1, j - 1, k - 1)) +
                           ux1[I1(i)] * (A(fz, i, j - 1, k) - A(fz, i, j - 1, k - 1))) +
             uy1[I1(j)] * (ux0[I1(i)] * (A(fz, i - 1, j, k) - A(fz, i - 1, j, k - 1)) +
                           ux1[I1(i)] * (A(fz, i, j, k) - A(fz, i, j, k - 1))));
        A(du, i, j, k) = A(du, i, j, k) - 0.5 * dt * dfdx - 0.5 * dt * dfdy -
                         0.5 * dt * dfdz;
      }
}

/* cans3d/hdmlw/mlwartv.f */
static void mlwartv3(const double *u, double *du, double dt, const double *qx,
                     const double *dxi, const double *dxim, int ix,
                     const double *qy, const double *dyi, const double *dyim,
                     int jx, const double *qz, const double *dzi,
                     const double *dzim, int kx) {
  OMP_FOR
  for (int k = 2; k <= kx - 1; k++)
    for (int j = 2; j <= jx - 1; j++)
      for (int i = 2; i <= ix - 1; i++)
        A(du, i, j, k) =
            A(du, i, j, k) +
            dt * (dxi[I1(i)] *
                  (A(qx, i, j, k) * dxim[I1(i)] * (A(u, i + 1, j, k) - A(u, i, j, k)) -
                   A(qx, i - 1, j, k) * dxim[I1(i - 1)] *
                       (A(u, i, j, k) - A(u, i - 1, j, k)))) +
            dt * (dyi[I1(j)] *
                  (A(qy, i, j, k) * dyim[I1(j)] * (A(u, i, j + 1, k) - A(u, i, j, k)) -
                   A(qy, i, j - 1, k) * dyim[I1(j - 1)] *
                       (A(u, i, j, k) - A(u, i, j - 1, k)))) +
            dt * (dzi[I1(k)] *
                  (A(qz, i, j, k) * dzim[I1(k)] * (A(u, i, j, k + 1) - A(u, i, j, k)) -
                   A(qz, i, j, k - 1) * dzim[I1(k - 1)] *
                       (A(u, i, j, k) - A(u, i, j, k - 1))));
}

/* cans3d/hdmlw/mlwsrch.f:32-50 */
static void mlwsrch3(double *un, double *du, double dt, const double *s, int ix,
                     int jx, int kx) {
  OMP_FOR
  for (int k = 2; k <= kx - 1; k++)
    for (int j = 2; j <= jx - 1; j++)
      for (int i = 2; i <= ix - 1; i++)
        A(du, i, j, k) = A(du, i, j, k) + 0.5 * dt * A(s, i, j, k);
  OMP_FOR
  for (int k = 1; k <= kx - 1; k++)
    for (int j = 1; j <= jx - 1; j++)
      for (int i = 1; i <= ix - 1; i++) {
        double sh = (A(s, i + 1, j, k) + A(s, i, j, k) + A(s, i + 1, j + 1, k) +
                     A(s, i, j + 1, k) + A(s, i + 1, j, k + 1) + A(s, i, j, k + 1) +
                     A(s, i + 1, j + 1, k + 1) + A(s, i, j + 1, k + 1)) /
                    8;
        A(un, i, j, k) = A(un, i, j, k) + dt * sh;
      }
}

/* cans3d/hdmlw/mlwsrcf.f:35-45 */
static void mlwsrcf3(double *du, double dt, const double *s, const double *ux0,
                     const double *ux1, int ix, const double *uy0,
                     const double *uy1, int jx, const double *uz0,
                     const double *uz1, int kx) {
  OMP_FOR
  for (int k = 2; k <= kx - 1; k++)
    for (int j = 2; j <= jx - 1; j++)
      for (int i = 2; i <= ix - 1; i++) {
        double sh =
            uz0[I1(k)] * (uy0[I1(j)] * (ux0[I1(i)] * A(s, i - 1, j - 1, k - 1) +
                                        ux1[I1(i)] * A(s, i, j - 1, k - 1)) +
                          uy1[I1(j)] * (ux0[I1(i)] * A(s, i - 1, j, k - 1) +
                                        ux1[I1(i)] * A(s, i, j, k - 1))) +
            uz1[I1(k)] * (uy0[I1(j)] * (ux0[I1(i)] * A(s, i - 1, j - 1, k) +
                                        ux1[I1(i)] * A(s, i, j - 1, k)) +
                          uy1[I1(j)] * (ux0[I1(i)] * A(s, i - 1, j, k) +
                                        ux1[I1(i)] * A(s, i, j, k)));
        A(du, i, j, k) = A(du, i, j, k) + 0.5 * dt * sh;
      }
}

/* cans3d/common/bbtocx.f:29-35 (and bbtocy.f, bbtocz.f by cyclic
 * permutation): c = (b2(+1 along axis 1) - b2(-1)) / d1 / 2
 *                 - (b1(+1 along axis 2) - b1(-1)) / d2 / 2
 * on the cells 2..n-1 of every axis; s1, s2 are the index strides of the two
 * axes and d1, d2 their spacings at the point. */
static void bbtoc3(double *c, const double *b1, const double *b2, const double *d1,
                   int a1, const double *d2, int a2, int ix, int jx, int kx) {
  const size_t st[3] = {1, (size_t)ix, (size_t)ix * (size_t)jx};
  OMP_FOR
  for (int k = 2; k <= kx - 1; k++)
    for (int j = 2; j <= jx - 1; j++)
      for (int i = 2; i <= ix - 1; i++) {
        const int idx[3] = {i, j, k};
        const size_t g = I3(i, j, k);
        c[g] = (b2[g + st[a1]] - b2[g - st[a1]]) / d1[I1(idx[a1])] / 2.0 -
               (b1[g + st[a2]] - b1[g - st[a2]]) / d2[I1(idx[a2])] / 2.0;
      }
}

/* the half-step field of corners ix, jx or kx is never set by mlwhalf; the
 * corner currents read it for the last corner of each axis, and take zero */
static void zero_top_corners(double *a, int ix, int jx, int kx) {
  for (int k = 1; k <= kx; k++)
    for (int j = 1; j <= jx; j++)
      for (int i = 1; i <= ix; i++)
        if (i == ix || j == jx || k == kx) a[I3(i, j, k)] = 0.0;
}

#define LOOP3(k0, k1, j0, j1, i0, i1)                                          \
  OMP_FOR                                                                      \
  for (int k = k0; k <= k1; k++)                                               \
    for (int j = j0; j <= j1; j++)                                             \
      for (int i = i0; i <= i1; i++)

/* cans3d/hdmlw/mlw_m.f:2-453.  With g (gx, gxm, gy, gym, gz, gzm) this is
 * mlw_m_g (cans3d/hdmlw/mlw_m_g.f:2-469): the gravity sources of
 * mlw_m_g.f:135-196 at the cells and :289-350 at the corners enter the energy
 * and the three momenta through mlwsrch / mlwsrcf. */
static void mlw_m_3d_core(double *ro, double *pr, double *vx, double *vy, double *vz,
                          double *bx, double *by, double *bz, double dt, double qav,
                          double gm, const double *const *g, const double *et,
                          const double *etm, const double *dx,
                          const double *dxm, int ix, const double *dy,
                          const double *dym, int jx, const double *dz,
                          const double *dzm, int kx) {
  const size_t n = (size_t)ix * (size_t)jx * (size_t)kx;
  const size_t nm = (size_t)(ix > jx ? (ix > kx ? ix : kx) : (jx > kx ? jx : kx));
  enum { NT = 40 };
  double *w = arena_get(&arena3d, NT * n + 12 * nm);
  double *t[NT];
  for (int a = 0; a < NT; a++) t[a] = w + a * n;
  double *ex = t[0], *ey = t[1], *ez = t[2];
  double *ee = t[3], *rx = t[4], *ry = t[5], *rz = t[6];
  double *roh = t[7], *eeh = t[8], *rxh = t[9], *ryh = t[10], *rzh = t[11];
  double *bxh = t[12], *byh = t[13], *bzh = t[14];
  double *exh = t[15], *eyh = t[16], *ezh = t[17];
  double *prh = t[18], *vxh = t[19], *vyh = t[20], *vzh = t[21];
  double *dro = t[22], *dee = t[23], *drx = t[24], *dry = t[25], *drz = t[26];
  double *dbx = t[27], *dby = t[28], *dbz = t[29];
  double *fx = t[30], *qx = t[31], *fy = t[32], *qy = t[33], *fz = t[34],
         *qz = t[35], *ss = t[36];
  double *cx = t[37], *cy = t[38], *cz = t[39];
  double *m = w + NT * n;
  double *dxi = m, *dxim = m + nm, *ux0 = m + 2 * nm, *ux1 = m + 3 * nm;
  double *dyi = m + 4 * nm, *dyim = m + 5 * nm, *uy0 = m + 6 * nm,
         *uy1 = m + 7 * nm;
  double *dzi = m + 8 * nm, *dzim = m + 9 * nm, *uz0 = m + 10 * nm,
         *uz1 = m + 11 * nm;

  const double pi = acos(-1.0);
  const double pi8i = 1. / pi / 8.;
  const double pi4i = 1. / pi / 4.;
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
  for (int k = 1; k <= kx; k++) {
    dzi[I1(k)] = 1.0 / dz[I1(k)];
    dzim[I1(k)] = 1.0 / dzm[I1(k)];
  }
  for (int k = 2; k <= kx - 1; k++) {
    uz1[I1(k)] = 0.5 * dzm[I1(k - 1)] / dz[I1(k)];
    uz0[I1(k)] = 0.5 * dzm[I1(k)] / dz[I1(k)];
  }

  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    dro[c] = 0.0; dee[c] = 0.0; drx[c] = 0.0; dry[c] = 0.0;
    drz[c] = 0.0; dbx[c] = 0.0; dby[c] = 0.0; dbz[c] = 0.0;
  }
  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    double vv = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
    double bb = bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c];
    ee[c] = pr[c] / (gm - 1) + 0.5 * ro[c] * vv + pi8i * bb;
    rx[c] = ro[c] * vx[c];
    ry[c] = ro[c] * vy[c];
    rz[c] = ro[c] * vz[c];
  }
  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    ex[c] = -vy[c] * bz[c] + vz[c] * by[c];
    ey[c] = -vz[c] * bx[c] + vx[c] * bz[c];
    ez[c] = -vx[c] * by[c] + vy[c] * bx[c];
  }
  if (et) {  /* mlw_m_e.f:103-115: E += et * J */
    memset(cx, 0, 3 * n * sizeof(double));
    bbtoc3(cx, by, bz, dy, 1, dz, 2, ix, jx, kx);
    bbtoc3(cy, bz, bx, dz, 2, dx, 0, ix, jx, kx);
    bbtoc3(cz, bx, by, dx, 0, dy, 1, ix, jx, kx);
    LOOP3(1, kx, 1, jx, 1, ix) {
      size_t c = I3(i, j, k);
      ex[c] = -vy[c] * bz[c] + vz[c] * by[c] + et[c] * cx[c];
      ey[c] = -vz[c] * bx[c] + vx[c] * bz[c] + et[c] * cy[c];
      ez[c] = -vx[c] * by[c] + vy[c] * bx[c] + et[c] * cz[c];
    }
  }
#define HALF3(u, un, du)                                                       \
  mlwhalf3(u, un, du, dt, fx, dxi, dxim, ix, fy, dyi, dyim, jx, fz, dzi, dzim, kx)
  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    fx[c] = ro[c] * vx[c];
    fy[c] = ro[c] * vy[c];
    fz[c] = ro[c] * vz[c];
  }
  HALF3(ro, roh, dro);
  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    double vv = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
    double ep = pr[c] * gm / (gm - 1.) + 0.5 * ro[c] * vv;
    fx[c] = ep * vx[c] + (bz[c] * ey[c] - by[c] * ez[c]) * pi4i;
    fy[c] = ep * vy[c] + (bx[c] * ez[c] - bz[c] * ex[c]) * pi4i;
    fz[c] = ep * vz[c] + (by[c] * ex[c] - bx[c] * ey[c]) * pi4i;
  }
  HALF3(ee, eeh, dee);
  if (g) {  /* mlw_m_g.f:135-142 */
    LOOP3(1, kx, 1, jx, 1, ix) {
      size_t c = I3(i, j, k);
      ss[c] = ro[c] * (vx[c] * g[0][c] + vy[c] * g[2][c] + vz[c] * g[4][c]);
    }
    mlwsrch3(eeh, dee, dt, ss, ix, jx, kx);
  }
  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    fx[c] = ro[c] * (vx[c] * vx[c]) + pr[c] +
            pi8i * (by[c] * by[c] + bz[c] * bz[c] - bx[c] * bx[c]);
    fy[c] = ro[c] * vx[c] * vy[c] - pi4i * bx[c] * by[c];
    fz[c] = ro[c] * vx[c] * vz[c] - pi4i * bx[c] * bz[c];
  }
  HALF3(rx, rxh, drx);
  if (g) {  /* mlw_m_g.f:154-160 */
    LOOP3(1, kx, 1, jx, 1, ix) ss[I3(i, j, k)] = ro[I3(i, j, k)] * g[0][I3(i, j, k)];
    mlwsrch3(rxh, drx, dt, ss, ix, jx, kx);
  }
  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    fx[c] = ro[c] * vy[c] * vx[c] - pi4i * by[c] * bx[c];
    fy[c] = ro[c] * (vy[c] * vy[c]) + pr[c] +
            pi8i * (bx[c] * bx[c] + bz[c] * bz[c] - by[c] * by[c]);
    fz[c] = ro[c] * vy[c] * vz[c] - pi4i * by[c] * bz[c];
  }
  HALF3(ry, ryh, dry);
  if (g) {  /* mlw_m_g.f:172-178 */
    LOOP3(1, kx, 1, jx, 1, ix) ss[I3(i, j, k)] = ro[I3(i, j, k)] * g[2][I3(i, j, k)];
    mlwsrch3(ryh, dry, dt, ss, ix, jx, kx);
  }
  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    fx[c] = ro[c] * vz[c] * vx[c] - pi4i * bz[c] * bx[c];
    fy[c] = ro[c] * vz[c] * vy[c] - pi4i * bz[c] * by[c];
    fz[c] = ro[c] * (vz[c] * vz[c]) + pr[c] +
            pi8i * (bx[c] * bx[c] + by[c] * by[c] - bz[c] * bz[c]);
  }
  HALF3(rz, rzh, drz);
  if (g) {  /* mlw_m_g.f:190-196 */
    LOOP3(1, kx, 1, jx, 1, ix) ss[I3(i, j, k)] = ro[I3(i, j, k)] * g[4][I3(i, j, k)];
    mlwsrch3(rzh, drz, dt, ss, ix, jx, kx);
  }
  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    fx[c] = 0.;
    fy[c] = ez[c];
    fz[c] = -ey[c];
  }
  HALF3(bx, bxh, dbx);
  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    fx[c] = -ez[c];
    fy[c] = 0.;
    fz[c] = ex[c];
  }
  HALF3(by, byh, dby);
  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    fx[c] = ey[c];
    fy[c] = -ex[c];
    fz[c] = 0.;
  }
  HALF3(bz, bzh, dbz);
#undef HALF3

  LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) {
    size_t c = I3(i, j, k);
    vxh[c] = rxh[c] / roh[c];
    vyh[c] = ryh[c] / roh[c];
    vzh[c] = rzh[c] / roh[c];
    double vv = vxh[c] * vxh[c] + vyh[c] * vyh[c] + vzh[c] * vzh[c];
    double bb = bxh[c] * bxh[c] + byh[c] * byh[c] + bzh[c] * bzh[c];
    prh[c] = (gm - 1) * (eeh[c] - 0.5 * roh[c] * vv - pi8i * bb);
  }
  LOOP3(1, kx, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    exh[c] = -vyh[c] * bzh[c] + vzh[c] * byh[c];
    eyh[c] = -vzh[c] * bxh[c] + vxh[c] * bzh[c];
    ezh[c] = -vxh[c] * byh[c] + vyh[c] * bxh[c];
  }
  if (et) {  /* mlw_m_e.f:257-270: Eh += etm * Jh at the corners */
    zero_top_corners(bxh, ix, jx, kx);
    zero_top_corners(byh, ix, jx, kx);
    zero_top_corners(bzh, ix, jx, kx);
    memset(cx, 0, 3 * n * sizeof(double));
    bbtoc3(cx, byh, bzh, dym, 1, dzm, 2, ix, jx, kx);
    bbtoc3(cy, bzh, bxh, dzm, 2, dxm, 0, ix, jx, kx);
    bbtoc3(cz, bxh, byh, dxm, 0, dym, 1, ix, jx, kx);
    LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) {
      size_t c = I3(i, j, k);
      exh[c] = -vyh[c] * bzh[c] + vzh[c] * byh[c] + etm[c] * cx[c];
      eyh[c] = -vzh[c] * bxh[c] + vxh[c] * bzh[c] + etm[c] * cy[c];
      ezh[c] = -vxh[c] * byh[c] + vyh[c] * bxh[c] + etm[c] * cz[c];
    }
  }
#define FULL3(du)                                                              \
  mlwfull3(du, dt, fx, dxi, ux0, ux1, ix, fy, dyi, uy0, uy1, jx, fz, dzi, uz0, \
           uz1, kx)
  LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) {
    size_t c = I3(i, j, k);
    fx[c] = roh[c] * vxh[c];
    fy[c] = roh[c] * vyh[c];
    fz[c] = roh[c] * vzh[c];
  }
  FULL3(dro);
  LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) {
    size_t c = I3(i, j, k);
    double vv = vxh[c] * vxh[c] + vyh[c] * vyh[c] + vzh[c] * vzh[c];
    double ep = prh[c] * gm / (gm - 1.) + 0.5 * roh[c] * vv;
    fx[c] = ep * vxh[c] + (bzh[c] * eyh[c] - byh[c] * ezh[c]) * pi4i;
    fy[c] = ep * vyh[c] + (bxh[c] * ezh[c] - bzh[c] * exh[c]) * pi4i;
    fz[c] = ep * vzh[c] + (byh[c] * exh[c] - bxh[c] * eyh[c]) * pi4i;
  }
  FULL3(dee);
  if (g) {  /* mlw_m_g.f:289-296 */
    LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) {
      size_t c = I3(i, j, k);
      ss[c] = roh[c] * (vxh[c] * g[1][c] + vyh[c] * g[3][c] + vzh[c] * g[5][c]);
    }
    mlwsrcf3(dee, dt, ss, ux0, ux1, ix, uy0, uy1, jx, uz0, uz1, kx);
  }
  LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) {
    size_t c = I3(i, j, k);
    fx[c] = roh[c] * (vxh[c] * vxh[c]) + prh[c] +
            pi8i * (byh[c] * byh[c] + bzh[c] * bzh[c] - bxh[c] * bxh[c]);
    fy[c] = roh[c] * vxh[c] * vyh[c] - pi4i * bxh[c] * byh[c];
    fz[c] = roh[c] * vxh[c] * vzh[c] - pi4i * bxh[c] * bzh[c];
  }
  FULL3(drx);
  if (g) {  /* mlw_m_g.f:308-314 */
    LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) ss[I3(i, j, k)] = roh[I3(i, j, k)] * g[1][I3(i, j, k)];
    mlwsrcf3(drx, dt, ss, ux0, ux1, ix, uy0, uy1, jx, uz0, uz1, kx);
  }
  LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) {
    size_t c = I3(i, j, k);
    fx[c] = roh[c] * vyh[c] * vxh[c] - pi4i * byh[c] * bxh[c];
    fy[c] = roh[c] * (vyh[c] * vyh[c]) + prh[c] +
            pi8i * (bxh[c] * bxh[c] + bzh[c] * bzh[c] - byh[c] * byh[c]);
    fz[c] = roh[c] * vyh[c] * vzh[c] - pi4i * byh[c] * bzh[c];
  }
  FULL3(dry);
  if (g) {  /* mlw_m_g.f:326-332 */
    LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) ss[I3(i, j, k)] = roh[I3(i, j, k)] * g[3][I3(i, j, k)];
    mlwsrcf3(dry, dt, ss, ux0, ux1, ix, uy0, uy1, jx, uz0, uz1, kx);
  }
  /* the reference sweeps j and i over the full range here (:286-297) */
  LOOP3(1, kx - 1, 1, jx, 1, ix) {
    size_t c = I3(i, j, k);
    fx[c] = roh[c] * vzh[c] * vxh[c] - pi4i * bzh[c] * bxh[c];
    fy[c] = roh[c] * vzh[c] * vyh[c] - pi4i * bzh[c] * byh[c];
    fz[c] = roh[c] * (vzh[c] * vzh[c]) + prh[c] +
            pi8i * (bxh[c] * bxh[c] + byh[c] * byh[c] - bzh[c] * bzh[c]);
  }
  FULL3(drz);
  if (g) {  /* mlw_m_g.f:344-350 */
    LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) ss[I3(i, j, k)] = roh[I3(i, j, k)] * g[5][I3(i, j, k)];
    mlwsrcf3(drz, dt, ss, ux0, ux1, ix, uy0, uy1, jx, uz0, uz1, kx);
  }
  LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) {
    size_t c = I3(i, j, k);
    fx[c] = 0.;
    fy[c] = ezh[c];
    fz[c] = -eyh[c];
  }
  FULL3(dbx);
  LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) {
    size_t c = I3(i, j, k);
    fx[c] = -ezh[c];
    fy[c] = 0.;
    fz[c] = exh[c];
  }
  FULL3(dby);
  LOOP3(1, kx - 1, 1, jx - 1, 1, ix - 1) {
    size_t c = I3(i, j, k);
    fx[c] = eyh[c];
    fy[c] = -exh[c];
    fz[c] = 0.;
  }
  FULL3(dbz);
#undef FULL3

  const double zero = 0.0;
  LOOP3(1, kx, 1, jx, 1, ix - 1)
  A(qx, i, j, k) = qav * dxm[I1(i)] *
                   fmax2(zero, fabs(A(vx, i + 1, j, k) - A(vx, i, j, k)) - R4_1EM4);
  LOOP3(1, kx, 1, jx - 1, 1, ix)
  A(qy, i, j, k) = qav * dym[I1(j)] *
                   fmax2(zero, fabs(A(vy, i, j + 1, k) - A(vy, i, j, k)) - R4_1EM4);
  LOOP3(1, kx - 1, 1, jx, 1, ix)
  A(qz, i, j, k) = qav * dzm[I1(k)] *
                   fmax2(zero, fabs(A(vz, i, j, k + 1) - A(vz, i, j, k)) - R4_1EM4);
#define ARTV3(u, du)                                                           \
  mlwartv3(u, du, dt, qx, dxi, dxim, ix, qy, dyi, dyim, jx, qz, dzi, dzim, kx)
  ARTV3(ro, dro);
  ARTV3(ee, dee);
  ARTV3(rx, drx);
  ARTV3(ry, dry);
  ARTV3(rz, drz);
  ARTV3(bx, dbx);
  ARTV3(by, dby);
  ARTV3(bz, dbz);
#undef ARTV3
  LOOP3(2, kx - 1, 2, jx - 1, 2, ix - 1) {
    size_t c = I3(i, j, k);
    ro[c] = ro[c] + dro[c];
    ee[c] = ee[c] + dee[c];
    rx[c] = rx[c] + drx[c];
    ry[c] = ry[c] + dry[c];
    rz[c] = rz[c] + drz[c];
    bx[c] = bx[c] + dbx[c];
    by[c] = by[c] + dby[c];
    bz[c] = bz[c] + dbz[c];
  }
  LOOP3(2, kx - 1, 2, jx - 1, 2, ix - 1) {
    size_t c = I3(i, j, k);
    vx[c] = rx[c] / ro[c];
    vy[c] = ry[c] / ro[c];
    vz[c] = rz[c] / ro[c];
    double vv = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
    double bb = bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c];
    pr[c] = (gm - 1) * (ee[c] - 0.5 * ro[c] * vv - pi8i * bb);
  }
}

void oracle_mlw_m_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                     double *bx, double *by, double *bz, double dt, double qav,
                     double gm, const double *dx, const double *dxm, int ix,
                     const double *dy, const double *dym, int jx,
                     const double *dz, const double *dzm, int kx) {
  mlw_m_3d_core(ro, pr, vx, vy, vz, bx, by, bz, dt, qav, gm, NULL, NULL, NULL, dx, dxm, ix,
                dy, dym, jx, dz, dzm, kx);
}

/* cans3d/hdmlw/mlw_m_g.f:2-4 */
void oracle_mlw_m_g_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                       double *bx, double *by, double *bz, double dt, double qav,
                       double gm, const double *gx, const double *gxm,
                       const double *gy, const double *gym, const double *gz,
                       const double *gzm, const double *dx, const double *dxm,
                       int ix, const double *dy, const double *dym, int jx,
                       const double *dz, const double *dzm, int kx) {
  const double *g[6] = {gx, gxm, gy, gym, gz, gzm};
  mlw_m_3d_core(ro, pr, vx, vy, vz, bx, by, bz, dt, qav, gm, g, NULL, NULL, dx, dxm, ix, dy,
                dym, jx, dz, dzm, kx);
}

/* cans3d/hdmlw/mlw_m_e.f:2-3 */
void oracle_mlw_m_e_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                       double *bx, double *by, double *bz, double dt, double qav,
                       double gm, const double *et, const double *etm, const double *dx,
                       const double *dxm, int ix, const double *dy, const double *dym,
                       int jx, const double *dz, const double *dzm, int kx) {
  mlw_m_3d_core(ro, pr, vx, vy, vz, bx, by, bz, dt, qav, gm, NULL, et, etm, dx, dxm, ix, dy,
                dym, jx, dz, dzm, kx);
}

/* cans3d/common/cfl_m_e.f: the wave limit of cfl_m (single-precision pi)
 * and the diffusion limit safety*0.5*dmesh**2/max(et,1.d-10) */
void oracle_cfl_m_e_3d(double *dt, double safety, double dtmin, int *merr, double gm,
                       const double *ro, const double *pr, const double *vx,
                       const double *vy, const double *vz, const double *bx,
                       const double *by, const double *bz, const double *et,
                       const double *dx, int ix, const double *dy, int jx,
                       const double *dz, int kx) {
  const double pai = (double)acosf(-1.0f);
  const double onep4 = 0.25 / pai;
  double dmin = R4_1E20;
#ifdef _OPENMP
#pragma omp parallel for reduction(min : dmin) schedule(static)
#endif
  for (int k = 1; k <= kx; k++)
    for (int j = 1; j <= jx; j++)
      for (int i = 1; i <= ix; i++) {
        size_t c = I3(i, j, k);
        double dmesh = fmin2(fmin2(dx[I1(i)], dy[I1(j)]), dz[I1(k)]);
        double b2 = bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c];
        double ca2 = b2 * onep4 / ro[c];
        double cs2 = gm * pr[c] / ro[c];
        double v2 = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
        double dtcfl = dmesh / sqrt(v2 + cs2 + ca2);
        double dtwav = safety * dtcfl;
        double dtdif = safety * 0.5 * (dmesh * dmesh) / fmax2(et[c], 1.e-10);
        double dtq = fmin2(dtwav, dtdif);
        if (dtq < dmin) dmin = dtq;
      }
  *dt = dmin;
  *merr = 0;
  if (*dt < dtmin) *merr = 9001;
}

/* cans3d/common/cfl_m.f:39-85; pai = acos(-1.0) is evaluated in single
 * precision and then widened, as in the reference. */
void oracle_cfl_m_3d(double *dt, double safety, double dtmin, int *merr,
                     double gm, const double *ro, const double *pr,
                     const double *vx, const double *vy, const double *vz,
                     const double *bx, const double *by, const double *bz,
                     const double *dx, int ix, const double *dy, int jx,
                     const double *dz, int kx) {
  const double pai = (double)acosf(-1.0f);
  const double onep4 = 0.25 / pai;
  double dmin = R4_1E20;
#ifdef _OPENMP
#pragma omp parallel for reduction(min : dmin) schedule(static)
#endif
  for (int k = 1; k <= kx; k++)
    for (int j = 1; j <= jx; j++)
      for (int i = 1; i <= ix; i++) {
        size_t c = I3(i, j, k);
        double b2 = bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c];
        double ca2 = b2 * onep4 / ro[c];
        double cs2 = gm * pr[c] / ro[c];
        double v2 = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
        double dtcfl =
            fmin2(fmin2(dx[I1(i)], dy[I1(j)]), dz[I1(k)]) / sqrt(v2 + cs2 + ca2);
        double dtq = safety * dtcfl;
        if (dtq < dmin) dmin = dtq;
      }
  *dt = dmin;
  *merr = 0;
  if (*dt < dtmin) *merr = 9001;
}
