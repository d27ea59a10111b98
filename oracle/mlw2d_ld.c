/*
 * The 2-D mLW step of mlw2d.c evaluated in long double -- TEST
 * INFRASTRUCTURE ONLY, for the finite-difference check of the adjoint.
 *
 * A central difference of the final magnetic energy over a 2000-step
 * shear-layer run is limited by the rounding noise of the run itself: in
 * double the perturbed and unperturbed runs round differently by about 1e-14
 * of J, a few 1e-6 of the directional derivative at h = 1e-6.  The same
 * restatement in long double (the 64-bit significand of x87 extended
 * precision on x86-64) lowers that noise by more than three orders, so the
 * difference measures the derivative itself.  The file is mlw2d.c compiled
 * with every double widened; its exported symbols carry an oracle_ld_
 * prefix, and the real*4 literals keep their single-precision values.
 */
#define oracle_set_av_branch oracle_ld_set_av_branch
#define oracle_mlw_m3_2d oracle_ld_mlw_m3_2d
#define oracle_mlw_m3_g_2d oracle_ld_mlw_m3_g_2d
#define oracle_mlw_m_2d oracle_ld_mlw_m_2d
#define oracle_mlw_m_g_2d oracle_ld_mlw_m_g_2d
#define oracle_mlw_m3_ge_2d oracle_ld_mlw_m3_ge_2d
#define oracle_mlw_m_ge_2d oracle_ld_mlw_m_ge_2d
#define oracle_cfl_m3_e_2d oracle_ld_cfl_m3_e_2d
#define oracle_cfl_m3_2d oracle_ld_cfl_m3_2d
#define oracle_cfl_m_2d oracle_ld_cfl_m_2d
#define oracle_bbtoaa_2d oracle_ld_bbtoaa_2d
#define oracle_roe_face oracle_ld_roe_face_unused
/* the C library's math headers are included before double is widened */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <tgmath.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#define double long double
#include "mlw2d.c"
