/*
 * Shared helpers of the CPU oracle (TEST INFRASTRUCTURE ONLY; see oracle.h).
 */
#ifndef CANS_ORACLE_COMMON_H
#define CANS_ORACLE_COMMON_H

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

/* Fortran real*4 literals that are not exact in binary. */
#define R4_1EM4 ((double)1.0e-4f) /* 1.0e-4 in the artificial viscosity */
#define R4_1E20 ((double)1.e20f)  /* dt=1.e20 initial CFL minimum     */

/* 1-based, column-major index helpers. */
#define I1(i) ((size_t)((i)-1))
#define I2(i, j) ((size_t)((i)-1) + (size_t)((j)-1) * (size_t)ix)
#define I3(i, j, k)                                                            \
  ((size_t)((i)-1) +                                                           \
   (size_t)ix * ((size_t)((j)-1) + (size_t)jx * (size_t)((k)-1)))

/* Fortran max/min/abs on finite doubles. */
static inline double fmax2(double a, double b) { return a > b ? a : b; }
static inline double fmin2(double a, double b) { return a < b ? a : b; }

/* Cached arena standing in for the Fortran automatic arrays: ntmp arrays of n
 * doubles each, zero-initialised on first allocation and reused afterwards.
 * One arena per dimension family keeps the sizes stable between calls. */
typedef struct {
  double *buf;
  size_t cap;
} oracle_arena;

static inline double *arena_get(oracle_arena *a, size_t total) {
  if (a->cap < total) {
    free(a->buf);
    a->buf = (double *)calloc(total, sizeof(double));
    a->cap = a->buf ? total : 0;
  }
  return a->buf;
}

/* Roe flux of one face (roe3d.c), shared by the 3-D and 2-D steps. */
void oracle_roe_face(double gm, const double *L, const double *R, double *f, int fix);

#endif
