/*
 * 2-D Roe-MUSCL step: line-faithful C restatement of the CANS Fortran
 * (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 *   roe_m3      cans2d/hdroe/roe_m3.f:1-204     two-stage driver
 *   roeflux_m3  cans2d/hdroe/roeflux_m3.f        Roe flux of one face
 *                (oracle_roe_face with fix = 0)
 *   tvdminmod   cans2d/hdroe/tvdminmod.f:1-37    minmod MUSCL reconstruction
 *
 * The y faces swap x and y (roe_m3.f:106-107, 167-168): normal y, first
 * tangential x, second z.  As in the 3-D restatement, the half-step
 * primitives the reference leaves unset on the outer cell layer
 * (roe_m3.f:123-132 fills 2..n-1) hold the input primitives of the cell,
 * and the corrector evaluates the faces tvdminmod reconstructs (2..n-2 in
 * both indices), which contain every face the updates of roe_m3.f:145-182
 * read.
 */
#include "oracle.h"
#include "oracle_common.h"

static oracle_arena arena_roe2;

enum { V_RO, V_PR, V_VX, V_VY, V_VZ, V_BX, V_BY, V_BZ };
enum { F_RO, F_EE, F_RX, F_RY, F_RZ, F_BX, F_BY, F_BZ };

/* components (normal, tangential 1, tangential 2) of the x and y faces */
static const int rot2[2][3] = {{0, 1, 2}, {1, 0, 2}};

/* Fortran sign(a, b) for a >= 0 */
static inline double fsign2(double a, double b) { return copysign(fabs(a), b); }

/* cans2d/hdroe/tvdminmod.f:8 */
static inline double flmt2(double a, double b) {
  const double s = fsign2(1.0, a);
  return fmax2(0.0, fmin2(b * s, fabs(a))) * s;
}

/* fluxes of the faces (c, c + e_axis), i in ilo..ihi, j in jlo..jhi */
static void flux_axis(double *const *fl, double gm, const double *const *wl,
                      const double *const *wr, int axis, int ilo, int ihi,
                      int jlo, int jhi, int ix) {
  const int *r = rot2[axis];
  OMP_FOR
  for (int j = jlo; j <= jhi; j++)
    for (int i = ilo; i <= ihi; i++) {
      const size_t c = I2(i, j);
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
      oracle_roe_face(gm, L, R, f, 0);
      fl[F_RO][c] = f[0];
      fl[F_EE][c] = f[1];
      for (int m = 0; m < 3; m++) fl[F_RX + r[m]][c] = f[2 + m];
      fl[F_BX + r[1]][c] = f[5];
      fl[F_BX + r[2]][c] = f[6];
    }
}

/* cans2d/hdroe/tvdminmod.f:14-33 on one variable */
static void tvdminmod2(int mdir, const double *da, double *dl, double *dr, int ix,
                       int jx) {
  const size_t st = mdir == 1 ? 1 : (size_t)ix;
  OMP_FOR
  for (int j = 2; j <= jx - 2; j++)
    for (int i = 2; i <= ix - 2; i++) {
      const size_t c = I2(i, j);
      const double dm = da[c - st], d0 = da[c], d1 = da[c + st], d2 = da[c + 2 * st];
      dl[c] = d0 + 0.5 * flmt2(d1 - d0, d0 - dm);
      dr[c] = d1 - 0.5 * flmt2(d1 - d0, d2 - d1);
    }
}

/* cans2d/hdroe/roe_m3.f:1-204 */
void oracle_roe_m3_2d(double *ro, double *pr, double *vx, double *vy, double *vz,
                      double *bx, double *by, double *bz, double *az, double dt,
                      double gm, const double *dx, int ix, const double *dy, int jx) {
  const size_t n = (size_t)ix * jx;
  /* arena: ee rx ry rz | 8 conserved half | 8 primitive half | 8 fluxes |
   * 8 left + 8 right face states */
  double *w = arena_get(&arena_roe2, n * 44);
  double *ee = w, *rx = w + n, *ry = w + 2 * n, *rz = w + 3 * n;
  double *Hc[8], *Hp[8], *Fl[8], *Wl[8], *Wr[8];
  for (int v = 0; v < 8; v++) {
    Hc[v] = w + (4 + v) * n;
    Hp[v] = w + (12 + v) * n;
    Fl[v] = w + (20 + v) * n;
    Wl[v] = w + (28 + v) * n;
    Wr[v] = w + (36 + v) * n;
  }
  double *P[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  const double pi = 4.0 * atan(1.0);
  const double pi4 = 4.0 * pi;
  const double pi4i = 1.0 / pi4;
  const double pi8i = 5.0e-1 * pi4i;

  /* :24-45 conserved variables and the half-step copies */
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

  /* predictor (:48-120): first-order states, fluxes, dt/2 updates; the y
   * fluxes are taken from the same input state as the x fluxes */
  for (int a = 0; a < 2; a++) {
    const size_t st = a == 0 ? 1 : (size_t)ix;
    const size_t nf = n - st;
    for (int v = 0; v < 8; v++) {
      OMP_FOR
      for (size_t c = 0; c < nf; c++) {
        Wl[v][c] = P[v][c];
        Wr[v][c] = P[v][c + st];
      }
    }
    if (a == 0) flux_axis(Fl, gm, (const double *const *)Wl, (const double *const *)Wr,
                          0, 1, ix - 1, 1, jx - 1, ix);
    else flux_axis(Fl, gm, (const double *const *)Wl, (const double *const *)Wr, 1, 1,
                   ix - 1, 1, jx - 1, ix);
    OMP_FOR
    for (int j = 2; j <= jx - 1; j++)
      for (int i = 2; i <= ix - 1; i++) {
        const size_t c = I2(i, j);
        const double h = a == 0 ? dx[I1(i)] : dy[I1(j)];
        for (int v = 0; v < 8; v++) {
          if (v == F_BX + a) continue;
          Hc[v][c] = Hc[v][c] + 0.5 * dt * ((Fl[v][c - st] - Fl[v][c]) / h);
        }
      }
  }

  /* :123-132 half-step primitives; the outer layer keeps the input ones */
  OMP_FOR
  for (int j = 1; j <= jx; j++)
    for (int i = 1; i <= ix; i++) {
      const size_t c = I2(i, j);
      Hp[V_RO][c] = Hc[F_RO][c];
      Hp[V_BX][c] = Hc[F_BX][c];
      Hp[V_BY][c] = Hc[F_BY][c];
      Hp[V_BZ][c] = Hc[F_BZ][c];
      if (i == 1 || i == ix || j == 1 || j == jx) {
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

  /* corrector (:133-182): x, then y */
  double *U[8] = {ro, ee, rx, ry, rz, bx, by, bz};
  for (int a = 0; a < 2; a++) {
    const size_t st = a == 0 ? 1 : (size_t)ix;
    for (int v = 0; v < 8; v++) tvdminmod2(a + 1, Hp[v], Wl[v], Wr[v], ix, jx);
    flux_axis(Fl, gm, (const double *const *)Wl, (const double *const *)Wr, a, 2,
              ix - 2, 2, jx - 2, ix);
    OMP_FOR
    for (int j = 3; j <= jx - 2; j++)
      for (int i = 3; i <= ix - 2; i++) {
        const size_t c = I2(i, j);
        const double h = a == 0 ? dx[I1(i)] : dy[I1(j)];
        for (int v = 0; v < 8; v++) {
          if (v == F_BX + a) continue;
          U[v][c] = U[v][c] + dt * ((Fl[v][c - st] - Fl[v][c]) / h);
        }
      }
  }

  /* :185-191 az with the half-step E_z */
  OMP_FOR
  for (int j = 3; j <= jx - 2; j++)
    for (int i = 3; i <= ix - 2; i++) {
      const size_t c = I2(i, j);
      double ez = -Hp[V_VX][c] * Hp[V_BY][c] + Hp[V_VY][c] * Hp[V_BX][c];
      double saz = -ez;
      az[c] = az[c] + dt * saz;
    }

  /* :193-202 primitives */
  OMP_FOR
  for (int j = 3; j <= jx - 2; j++)
    for (int i = 3; i <= ix - 2; i++) {
      const size_t c = I2(i, j);
      vx[c] = rx[c] / ro[c];
      vy[c] = ry[c] / ro[c];
      vz[c] = rz[c] / ro[c];
      double v2 = vx[c] * vx[c] + vy[c] * vy[c] + vz[c] * vz[c];
      double b2 = bx[c] * bx[c] + by[c] * by[c] + bz[c] * bz[c];
      pr[c] = (gm - 1.0) * (ee[c] - 0.5 * ro[c] * v2 - pi8i * b2);
    }
}
