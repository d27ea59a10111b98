/*
 * CPU oracle for the CANS modified Lax-Wendroff (mLW) MHD step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a line-faithful C restatement of the
 * reference Fortran-77 routines (CANS, cans{1,2,3}d/hdmlw, common, bc).  It is
 * used by the test-suite as the checker, by __graft_entry__.smoke() and by the
 * CPU-baseline leg of bench.py.  No product code path links or calls it.
 *
 * Parity status.  The 1-D spicule loop (mlw_m_bg, chkdav, the torque, the
 * boundary program) is pinned against the output the reference ships for its
 * spicule run (tests/golden/spicule_reference.npz): the set-up to the last
 * bits of an 80-bit evaluation, the 100000-step run to 2.6e-8 in time and
 * 2e-4 in the density and pressure profiles.  The mLW step in 1-D, 2-D and
 * 3-D, the Roe-MUSCL step in 1-D, 2-D and 3-D and the HLLD engine, each with
 * its CFL loop, are pinned against the reference's own known answer for its
 * shock-tube model, the exact solution of cans1d/md_shktb/hdmlw/
 * shktb_analytic.pro (shktb_analytic.py; tests/test_sod.py): they converge
 * to it under refinement.  No output of the Fortran itself exists for these
 * (no Fortran compiler in the build or GPU environment, no golden vectors in
 * the reference), so beyond that they are pinned by hand-checkable
 * invariants (uniform-state invariance, mirror symmetry, exact periodic
 * conservation, axis rotation) and by the committed fixtures in
 * tests/golden/ that freeze their outputs.
 *
 * Fidelity rules followed throughout:
 *   - same loop bounds and the same left-to-right operation order as the
 *     Fortran source (C and Fortran share associativity for + - * /);
 *   - x**2 is x*x, as gfortran expands it;
 *   - real*4 literals are kept in single precision where the value is not
 *     exactly representable (1.0e-4 in the artificial viscosity, 1.e20 as the
 *     initial CFL minimum, acos(-1.0) in the 3-D CFL);
 *   - build with -O2 -ffp-contract=off -fno-fast-math (no FMA contraction);
 *   - the Fortran automatic arrays become one cached, zero-initialised heap
 *     arena, reused between calls of the same size.
 *
 * Arrays are column-major with 1-based Fortran indices mapped by the I1/I2/I3
 * macros below; ghost cells are included exactly as in the reference.
 */
#ifndef CANS_ORACLE_H
#define CANS_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- threading (OpenMP when compiled with -fopenmp) ---------------------- */
void oracle_set_threads(int n);
int oracle_get_threads(void);

/* ---- 1-D  (cans1d) ------------------------------------------------------- */
void oracle_grdrdy(double *dx, double *xm, double *dxm, const double *x, int ix);
void oracle_mlw_m_1d(double *ro, double *pr, double *vx, double *vy, double *by,
                     const double *bx, const double *bxm, double dt, double qav,
                     double gm, const double *dx, const double *dxm, int ix);
void oracle_cfl_m_1d(double *dt, double safety, double dtmin, int *merr,
                     double gm, const double *bx, const double *ro,
                     const double *pr, const double *vx, const double *vy,
                     const double *by, const double *dx, int ix);
void oracle_bd_1d(int kind, int mbnd, int margin, double *qq, double q0,
                  const double *dxm, int ix);
/* mlw_m_bg (cans1d/hdmlw/mlw_m_bg.f:2): gravity, flux-tube cross section and
 * rotation; chkdav (cans1d/common/chkdav.f:2) returns the event count;
 * trqalfven (cans1d/md_spicule/hdmlw/trqalfven.f:2) with a counter-based
 * random stream in place of random_number (see mlw1d_bg.c). */
void oracle_mlw_m_bg_1d(double *ro, double *pr, double *vx, double *vy, double *by,
                        const double *bx, const double *bxm, double dt, double qav,
                        double gm, const double *gx, const double *gxm,
                        const double *sc, const double *dsc, const double *scm,
                        const double *dscm, const double *rr, const double *rrm,
                        const double *drr, const double *drrm, const double *dx,
                        const double *dxm, int ix);
int oracle_chkdav(double *da, double *vx, double floor_, int ix);
double oracle_torque_uniform(unsigned long long seed, long long ns, int g, int ix);
void oracle_trqalfven(double *vy, double dt, const double *trq, const double *rr,
                      double trq0, unsigned long long seed, long long ns, int ix);
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
                       double *t_out, long long *ns_out, long long *nev_out);

/* ---- 2-D  (cans2d) ------------------------------------------------------- */
void oracle_mlw_m3_2d(double *ro, double *pr, double *vx, double *vy,
                      double *vz, double *bx, double *by, double *bz,
                      double *az, double dt, double qav, double gm,
                      const double *dx, const double *dxm, int ix,
                      const double *dy, const double *dym, int jx);
void oracle_mlw_m_2d(double *ro, double *pr, double *vx, double *vy,
                     double *bx, double *by, double *az, double dt, double qav,
                     double gm, const double *dx, const double *dxm, int ix,
                     const double *dy, const double *dym, int jx);
/* mlw_m3_g (cans2d/hdmlw/mlw_m3_g.f:1) and mlw_m_g (cans2d/hdmlw/mlw_m_g.f:1):
 * the steps with gravity; gx, gy at cells and gxm, gym at cell corners, all
 * ix*jx. */
void oracle_mlw_m3_g_2d(double *ro, double *pr, double *vx, double *vy,
                        double *vz, double *bx, double *by, double *bz,
                        double *az, double dt, double qav, double gm,
                        const double *gx, const double *gxm, const double *gy,
                        const double *gym, const double *dx, const double *dxm,
                        int ix, const double *dy, const double *dym, int jx);
void oracle_mlw_m_g_2d(double *ro, double *pr, double *vx, double *vy,
                       double *bx, double *by, double *az, double dt, double qav,
                       double gm, const double *gx, const double *gxm,
                       const double *gy, const double *gym, const double *dx,
                       const double *dxm, int ix, const double *dy,
                       const double *dym, int jx);
/* mlw_m3_e / mlw_m3_ge and mlw_m_e / mlw_m_ge (cans2d/hdmlw/mlw_m3_e.f:2,
 * mlw_m3_ge.f:2, mlw_m_e.f:2, mlw_m_ge.f:2): resistivity et at the cells and
 * etm at the corners (ix*jx each); gx..gym NULL for the steps without
 * gravity. */
void oracle_mlw_m3_ge_2d(double *ro, double *pr, double *vx, double *vy,
                         double *vz, double *bx, double *by, double *bz,
                         double *az, double dt, double qav, double gm,
                         const double *gx, const double *gxm, const double *gy,
                         const double *gym, const double *et, const double *etm,
                         const double *dx, const double *dxm, int ix,
                         const double *dy, const double *dym, int jx);
void oracle_mlw_m_ge_2d(double *ro, double *pr, double *vx, double *vy,
                        double *bx, double *by, double *az, double dt, double qav,
                        double gm, const double *gx, const double *gxm,
                        const double *gy, const double *gym, const double *et,
                        const double *etm, const double *dx, const double *dxm,
                        int ix, const double *dy, const double *dym, int jx);
/* cfl_m3_e / cfl_m_e (cans2d/common/cfl_m3_e.f:2, cfl_m_e.f:2); vz, bz NULL
 * for cfl_m_e */
void oracle_cfl_m3_e_2d(double *dt, double safety, double dtmin, int *merr,
                        double gm, const double *ro, const double *pr,
                        const double *vx, const double *vy, const double *vz,
                        const double *bx, const double *by, const double *bz,
                        const double *et, const double *dx, int ix,
                        const double *dy, int jx);
void oracle_cfl_m3_2d(double *dt, double safety, double dtmin, int *merr,
                      double gm, const double *ro, const double *pr,
                      const double *vx, const double *vy, const double *vz,
                      const double *bx, const double *by, const double *bz,
                      const double *dx, int ix, const double *dy, int jx);
void oracle_cfl_m_2d(double *dt, double safety, double dtmin, int *merr,
                     double gm, const double *ro, const double *pr,
                     const double *vx, const double *vy, const double *bx,
                     const double *by, const double *dx, int ix,
                     const double *dy, int jx);
void oracle_bbtoaa_2d(double *az, const double *bx, const double *by,
                      const double *dxm, const double *dym, int margin, int ix,
                      int jx);
/* kind: see BD_* below; axis 0 = x, 1 = y; mbnd 0 = lower, 1 = upper face.
 * q0 is the constant for BD_CNS; dxm the spacing for BD_FRD. */
void oracle_bd_2d(int kind, int axis, int mbnd, int margin, double *qq,
                  double q0, const double *dxm, int ix, int jx);

/* ---- 3-D  (cans3d) ------------------------------------------------------- */
void oracle_mlw_m_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                     double *bx, double *by, double *bz, double dt, double qav,
                     double gm, const double *dx, const double *dxm, int ix,
                     const double *dy, const double *dym, int jx,
                     const double *dz, const double *dzm, int kx);
/* mlw_m_g (cans3d/hdmlw/mlw_m_g.f:2-4): the 3-D step with gravity; gx, gy,
 * gz at the cells, gxm, gym, gzm at the cell corners, ix*jx*kx each */
void oracle_mlw_m_g_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                       double *bx, double *by, double *bz, double dt, double qav,
                       double gm, const double *gx, const double *gxm,
                       const double *gy, const double *gym, const double *gz,
                       const double *gzm, const double *dx, const double *dxm,
                       int ix, const double *dy, const double *dym, int jx,
                       const double *dz, const double *dzm, int kx);
/* mlw_m_e (cans3d/hdmlw/mlw_m_e.f:2-3): the 3-D step with resistivity et
 * (cells) and etm (corners); cfl_m_e (cans3d/common/cfl_m_e.f) */
void oracle_mlw_m_e_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                       double *bx, double *by, double *bz, double dt, double qav,
                       double gm, const double *et, const double *etm, const double *dx,
                       const double *dxm, int ix, const double *dy, const double *dym,
                       int jx, const double *dz, const double *dzm, int kx);
void oracle_cfl_m_e_3d(double *dt, double safety, double dtmin, int *merr, double gm,
                       const double *ro, const double *pr, const double *vx,
                       const double *vy, const double *vz, const double *bx,
                       const double *by, const double *bz, const double *et,
                       const double *dx, int ix, const double *dy, int jx,
                       const double *dz, int kx);
void oracle_cfl_m_3d(double *dt, double safety, double dtmin, int *merr,
                     double gm, const double *ro, const double *pr,
                     const double *vx, const double *vy, const double *vz,
                     const double *bx, const double *by, const double *bz,
                     const double *dx, int ix, const double *dy, int jx,
                     const double *dz, int kx);
void oracle_bd_3d(int kind, int axis, int mbnd, int margin, double *qq,
                  double q0, const double *dxm, int ix, int jx, int kx);
/* Roe-MUSCL step (cans3d/hdroe/roe_m.f:2); see roe3d.c for the one
 * deviation (a definite value where the reference reads unset memory). */
void oracle_roe_m_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                     double *bx, double *by, double *bz, double dt, double gm,
                     const double *dx, int ix, const double *dy, int jx,
                     const double *dz, int kx);

/* 1-D Roe-MUSCL step roe_m (cans1d/hdroe/roe_m.f:2), two-component. */
void oracle_roe_m_1d(double *ro, double *pr, double *vx, double *vy, double *by,
                     const double *bx, const double *bxm, double dt, double gm,
                     const double *dx, int ix);

/* 2-D Roe-MUSCL step roe_m3 (cans2d/hdroe/roe_m3.f:1) on ix*jx arrays. */
void oracle_roe_m3_2d(double *ro, double *pr, double *vx, double *vy, double *vz,
                      double *bx, double *by, double *bz, double *az, double dt,
                      double gm, const double *dx, int ix, const double *dy, int jx);

/* HLLD step of the cansxx engine (cansxx-nosupport/md_mhdshktb/hdhlld-x/
 * engine.f:2), Heaviside units with permeability mu; mfdim[3] marks the
 * active axes (1) as in the reference.  See hlld.c for the two places where
 * the reference reads memory it never wrote. */
void oracle_hlld_engine_3d(double *ro, double *pr, double *vx, double *vy,
                           double *vz, double *bx, double *by, double *bz,
                           double gm, double mu, double dt, const double *dx,
                           int ix, const double *dy, int jx, const double *dz,
                           int kx, const int *mfdim);

/* Boundary kinds (reference routine family in parentheses). */
enum {
  BD_PER = 0, /* periodic            (bdperx/bdpery/bdperz)          */
  BD_SPP = 1, /* symmetric, even     (bdsppx/...) ghost(i)=q(bnd-1+i) */
  BD_SPN = 2, /* symmetric, odd      (bdspnx/...) ghost=-q(bnd-1+i)   */
  BD_SMP = 3, /* symmetric about cell, even (bdsmpx/...)              */
  BD_SMN = 4, /* symmetric about cell, odd, boundary cell zeroed (bdsmnx) */
  BD_FRE = 5, /* free, zero gradient (bdfrex/...)                     */
  BD_CNS = 6, /* constant value      (bdcnsx/...)                     */
  BD_FRD = 7  /* free, constant gradient (bdfrdx/...)                 */
};

#ifdef __cplusplus
}
#endif
#endif
