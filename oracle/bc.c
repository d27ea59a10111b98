/*
 * Ghost-cell fill (bd* family) and grid metrics: C restatement of the CANS
 * Fortran (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 * Every bd* routine applies the same one-dimensional rule to each grid line
 * that runs along its axis, so one line kernel serves 1-D, 2-D and 3-D:
 *   periodic    cans2d/bc/bdperx.f:33-46   (also bdpery, cans3d/bc/bdperz.f)
 *   spp         cans2d/bc/bdsppx.f:31-47   ghost = +q(bnd-1+i)
 *   spn         cans2d/bc/bdspnx.f         ghost = -q(bnd-1+i)
 *   smp         cans2d/bc/bdsmpx.f         ghost = +q(bnd+i)
 *   smn         cans2d/bc/bdsmnx.f:31-55   ghost = -q(bnd+i), q(bnd) = 0
 *   fre         cans2d/bc/bdfrex.f         ghost = q(bnd)
 *   cns         cans2d/bc/bdcnsx.f         ghost = q0
 *   frd         cans2d/bc/bdfrdx.f         constant-gradient extrapolation
 * The reference loops ghost layer outermost and line innermost; lines never
 * read one another, so the per-line order used here gives the same values.
 *   grdrdy      cans1d/common/grdrdy.f (identical in cans2d/cans3d)
 */
#include "oracle.h"
#include "oracle_common.h"

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int oracle_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* q(l) for 1-based l along the line */
#define QL(l) q[(size_t)((l)-1) * stride]

static void bd_line(int kind, int mbnd, int m, double *q, size_t n,
                    size_t stride, double q0, const double *dxm) {
  const int nn = (int)n;
  if (kind == BD_PER) {
    const int b0 = 1 + m, b1 = nn - m;
    if (mbnd == 0)
      for (int i = 1; i <= m; i++) QL(b0 - i) = QL(b1 + 1 - i);
    else
      for (int i = 1; i <= m; i++) QL(b1 + i) = QL(b0 - 1 + i);
    return;
  }
  if (mbnd == 0) {
    const int b = 1 + m;
    switch (kind) {
    case BD_SPP: for (int i = 1; i <= m; i++) QL(b - i) = QL(b - 1 + i); break;
    case BD_SPN: for (int i = 1; i <= m; i++) QL(b - i) = -QL(b - 1 + i); break;
    case BD_SMP: for (int i = 1; i <= m; i++) QL(b - i) = QL(b + i); break;
    case BD_SMN:
      for (int i = 1; i <= m; i++) QL(b - i) = -QL(b + i);
      QL(b) = 0.;
      break;
    case BD_FRE: for (int i = 1; i <= m; i++) QL(b - i) = QL(b); break;
    case BD_CNS: for (int i = 1; i <= m; i++) QL(b - i) = q0; break;
    case BD_FRD:
      for (int i = 1; i <= m; i++) {
        double dqq = (QL(b + 1) - QL(b)) / dxm[I1(b)];
        QL(b - i) = QL(b - i + 1) - dqq * dxm[I1(b - i)];
      }
      break;
    default: break;
    }
  } else {
    const int b = nn - m;
    switch (kind) {
    case BD_SPP: for (int i = 1; i <= m; i++) QL(b + i) = QL(b + 1 - i); break;
    case BD_SPN: for (int i = 1; i <= m; i++) QL(b + i) = -QL(b + 1 - i); break;
    case BD_SMP: for (int i = 1; i <= m; i++) QL(b + i) = QL(b - i); break;
    case BD_SMN:
      for (int i = 1; i <= m; i++) QL(b + i) = -QL(b - i);
      QL(b) = 0.;
      break;
    case BD_FRE: for (int i = 1; i <= m; i++) QL(b + i) = QL(b); break;
    case BD_CNS: for (int i = 1; i <= m; i++) QL(b + i) = q0; break;
    case BD_FRD:
      for (int i = 1; i <= m; i++) {
        double dqq = (QL(b) - QL(b - 1)) / dxm[I1(b - 1)];
        QL(b + i) = QL(b + i - 1) + dqq * dxm[I1(b + i - 1)];
      }
      break;
    default: break;
    }
  }
}

/* Apply the rule along `axis` of an array with extents (n0, n1, n2). */
static void bd_nd(int kind, int axis, int mbnd, int m, double *qq, double q0,
                  const double *dxm, size_t n0, size_t n1, size_t n2) {
  size_t ext[3] = {n0, n1, n2};
  size_t stride = 1;
  for (int a = 0; a < axis; a++) stride *= ext[a];
  size_t n = ext[axis];
  size_t pre = stride;       /* lines below the axis */
  size_t post = 1;           /* lines above the axis */
  for (int a = axis + 1; a < 3; a++) post *= ext[a];
  for (size_t hi = 0; hi < post; hi++)
    for (size_t lo = 0; lo < pre; lo++)
      bd_line(kind, mbnd, m, qq + lo + hi * pre * n, n, stride, q0, dxm);
}

void oracle_bd_1d(int kind, int mbnd, int margin, double *qq, double q0,
                  const double *dxm, int ix) {
  bd_nd(kind, 0, mbnd, margin, qq, q0, dxm, (size_t)ix, 1, 1);
}

void oracle_bd_2d(int kind, int axis, int mbnd, int margin, double *qq,
                  double q0, const double *dxm, int ix, int jx) {
  bd_nd(kind, axis, mbnd, margin, qq, q0, dxm, (size_t)ix, (size_t)jx, 1);
}

void oracle_bd_3d(int kind, int axis, int mbnd, int margin, double *qq,
                  double q0, const double *dxm, int ix, int jx, int kx) {
  bd_nd(kind, axis, mbnd, margin, qq, q0, dxm, (size_t)ix, (size_t)jx,
        (size_t)kx);
}

/* cans1d/common/grdrdy.f */
void oracle_grdrdy(double *dx, double *xm, double *dxm, const double *x,
                   int ix) {
  for (int i = 1; i <= ix - 1; i++) dxm[I1(i)] = x[I1(i + 1)] - x[I1(i)];
  dxm[I1(ix)] = dxm[I1(ix - 1)];
  for (int i = 2; i <= ix - 1; i++)
    dx[I1(i)] = 0.5 * (dxm[I1(i - 1)] + dxm[I1(i)]);
  dx[I1(1)] = dx[I1(2)];
  dx[I1(ix)] = dx[I1(ix - 1)];
  for (int i = 1; i <= ix - 1; i++) xm[I1(i)] = 0.5 * (x[I1(i)] + x[I1(i + 1)]);
  xm[I1(ix)] = xm[I1(ix - 1)] + dx[I1(ix - 1)];
}
