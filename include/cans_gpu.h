/*
 * cans_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the CANS
 * ideal-MHD modified Lax-Wendroff step.
 *
 * Three layers, all plain C (pointers and sizes only):
 *
 *  1. Drop-in entry points with the argument lists of the reference Fortran
 *     routines.  Every argument is passed by reference, as a Fortran-77 caller
 *     passes it, so a bind(C) interface maps each call one to one.  The same
 *     routine name exists in the reference's 1-D, 2-D and 3-D libraries with
 *     different arguments (libcans1d.a / libcans2d.a / libcans3d.a), so each C
 *     symbol carries a _1d/_2d/_3d suffix.  Arrays are column-major with their
 *     ghost cells, exactly as the caller holds them.
 *       - If the arrays were registered with cans_gpu_register(), the call
 *         works on their device-resident mirrors and moves no field data
 *         (cfl_m returns only dt and merr to the host).
 *       - Otherwise the call copies its arrays to the device, runs there and
 *         copies the results back before returning.
 *     There is no CPU fallback: without a usable GPU every call returns
 *     CANS_ERR_CUDA.
 *
 *  2. Residency registry (cans_gpu_register / pull / push / release), the
 *     only calls a reference driver adds: register the state after the model
 *     set-up and pull it before each output write.
 *
 *  3. A device-resident run handle (cans_run_*) that keeps the whole
 *     reference time loop -- cfl, step, boundary fill, t += dt, the
 *     tend/nstop/dtmin tests -- on the GPU, replayed as a CUDA graph.
 *
 * Status codes: every entry point returns 0 on success or one of CANS_ERR_*.
 * Where the reference sets merr, the entry point sets it too.
 */
#ifndef CANS_GPU_H
#define CANS_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define CANS_OK 0
#define CANS_ERR_DTMIN 9001    /* dt < dtmin, as the reference merr=9001 */
#define CANS_ERR_NONFINITE 9100 /* a loop with stop_on_bad met a bad cell */
#define CANS_ERR_CUDA 9200     /* CUDA failure; see cans_last_error()     */
#define CANS_ERR_TIMEOUT 9300  /* a bounded device wait gave up           */
#define CANS_ERR_ARG 9400      /* invalid argument                        */

/* ------------------------------------------------------------------------ */
/* Library settings                                                          */
/* ------------------------------------------------------------------------ */
/* Arithmetic policy of the drop-in entry points: 0 = fast (FMA contraction,
 * one reciprocal per cell), 1 = exact (reference operation order, no
 * contraction; bit-identical to the reference arithmetic).  The initial value
 * comes from the environment variable CANS_GPU_EXACT (default 0). */
int cans_set_exact(int exact);
int cans_get_exact(void);
/* CUDA stream (cudaStream_t) used by the drop-in entry points; NULL selects
 * the library's own stream. */
int cans_set_stream(void *stream);
/* Text of the last CUDA error seen by the library (thread-compatible). */
const char *cans_last_error(void);
/* Number of kernel launches issued by this library so far (graph replays
 * count every kernel node). */
unsigned long long cans_launch_count(void);
/* 1 if a CUDA device of compute capability 10.3 is usable, else 0. */
int cans_device_ok(void);

/* ------------------------------------------------------------------------ */
/* 1. Drop-in entry points: 2-D                                              */
/* ------------------------------------------------------------------------ */
/* replaces subroutine mlw_m3  (cans2d/hdmlw/mlw_m3.f:2-3) */
int cans_mlw_m3_2d(double *ro, double *pr, double *vx, double *vy, double *vz,
                   double *bx, double *by, double *bz, double *az,
                   const double *dt, const double *qav, const double *gm,
                   const double *dx, const double *dxm, const int *ix,
                   const double *dy, const double *dym, const int *jx);
/* replaces subroutine mlw_m3_g (cans2d/hdmlw/mlw_m3_g.f:1) and mlw_m_g
 * (cans2d/hdmlw/mlw_m_g.f:1): the steps with gravity; gx, gy at the cells,
 * gxm, gym at the cell corners, ix*jx each */
int cans_mlw_m3_g_2d(double *ro, double *pr, double *vx, double *vy, double *vz,
                     double *bx, double *by, double *bz, double *az,
                     const double *dt, const double *qav, const double *gm,
                     const double *gx, const double *gxm, const double *gy,
                     const double *gym, const double *dx, const double *dxm,
                     const int *ix, const double *dy, const double *dym,
                     const int *jx);
int cans_mlw_m_g_2d(double *ro, double *pr, double *vx, double *vy, double *bx,
                    double *by, double *az, const double *dt, const double *qav,
                    const double *gm, const double *gx, const double *gxm,
                    const double *gy, const double *gym, const double *dx,
                    const double *dxm, const int *ix, const double *dy,
                    const double *dym, const int *jx);
/* replaces subroutine mlw_m3_e (cans2d/hdmlw/mlw_m3_e.f:2-3) and mlw_m_e
 * (cans2d/hdmlw/mlw_m_e.f:2-3): the resistive steps; et at the cells, etm at
 * the cell corners, ix*jx each.  The reference leaves the current density
 * on the outer ring of cells, and the half-step field at corner ix / row jx,
 * undefined; both are taken as zero. */
int cans_mlw_m3_e_2d(double *ro, double *pr, double *vx, double *vy, double *vz,
                     double *bx, double *by, double *bz, double *az,
                     const double *dt, const double *qav, const double *gm,
                     const double *et, const double *etm, const double *dx,
                     const double *dxm, const int *ix, const double *dy,
                     const double *dym, const int *jx);
int cans_mlw_m_e_2d(double *ro, double *pr, double *vx, double *vy, double *bx,
                    double *by, double *az, const double *dt, const double *qav,
                    const double *gm, const double *et, const double *etm,
                    const double *dx, const double *dxm, const int *ix,
                    const double *dy, const double *dym, const int *jx);
/* replaces subroutine mlw_m3_ge (cans2d/hdmlw/mlw_m3_ge.f:2-3) and mlw_m_ge
 * (cans2d/hdmlw/mlw_m_ge.f:2-3): gravity and resistivity together */
int cans_mlw_m3_ge_2d(double *ro, double *pr, double *vx, double *vy, double *vz,
                      double *bx, double *by, double *bz, double *az,
                      const double *dt, const double *qav, const double *gm,
                      const double *gx, const double *gxm, const double *gy,
                      const double *gym, const double *et, const double *etm,
                      const double *dx, const double *dxm, const int *ix,
                      const double *dy, const double *dym, const int *jx);
int cans_mlw_m_ge_2d(double *ro, double *pr, double *vx, double *vy, double *bx,
                     double *by, double *az, const double *dt, const double *qav,
                     const double *gm, const double *gx, const double *gxm,
                     const double *gy, const double *gym, const double *et,
                     const double *etm, const double *dx, const double *dxm,
                     const int *ix, const double *dy, const double *dym,
                     const int *jx);
/* replaces subroutine cfl_m3_e (cans2d/common/cfl_m3_e.f:2-3) and cfl_m_e
 * (cans2d/common/cfl_m_e.f:2-3): the wave limit and the resistive diffusion
 * limit safety*0.5*min(dx,dy)**2/max(et,1.e-5) */
int cans_cfl_m3_e_2d(double *dt, const double *safety, const double *dtmin,
                     int *merr, const double *gm, const double *ro,
                     const double *pr, const double *vx, const double *vy,
                     const double *vz, const double *bx, const double *by,
                     const double *bz, const double *et, const double *dx,
                     const int *ix, const double *dy, const int *jx);
int cans_cfl_m_e_2d(double *dt, const double *safety, const double *dtmin,
                    int *merr, const double *gm, const double *ro,
                    const double *pr, const double *vx, const double *vy,
                    const double *bx, const double *by, const double *et,
                    const double *dx, const int *ix, const double *dy,
                    const int *jx);
/* replaces subroutine mlw_m   (cans2d/hdmlw/mlw_m.f:2-3) */
int cans_mlw_m_2d(double *ro, double *pr, double *vx, double *vy, double *bx,
                  double *by, double *az, const double *dt, const double *qav,
                  const double *gm, const double *dx, const double *dxm,
                  const int *ix, const double *dy, const double *dym,
                  const int *jx);
/* replaces subroutine cfl_m3  (cans2d/common/cfl_m3.f:2-3) */
int cans_cfl_m3_2d(double *dt, const double *safety, const double *dtmin,
                   int *merr, const double *gm, const double *ro,
                   const double *pr, const double *vx, const double *vy,
                   const double *vz, const double *bx, const double *by,
                   const double *bz, const double *dx, const int *ix,
                   const double *dy, const int *jx);
/* replaces subroutine cfl_m   (cans2d/common/cfl_m.f:2-3) */
int cans_cfl_m_2d(double *dt, const double *safety, const double *dtmin,
                  int *merr, const double *gm, const double *ro,
                  const double *pr, const double *vx, const double *vy,
                  const double *bx, const double *by, const double *dx,
                  const int *ix, const double *dy, const int *jx);

/* No counterpart in the reference.  cfl_m3 for callers that cannot allocate
 * device memory (a host code whose pool owns all device memory, a run under a
 * memory budget fixed at start-up, a caller that may not allocate while it
 * times its steps).  Same arguments and result as cans_cfl_m3_2d, but ro..bz,
 * dx and dy are DEVICE pointers the caller already holds; dt and merr are
 * written on the host.  The library allocates nothing for it: its scratch is
 * a fixed 32 KiB array in device memory, held by every GPU that loads the
 * library until the process exits, which limits the grid to
 * ix*jx <= 1,048,576 cells (larger grids return CANS_ERR_ARG).  The first
 * call on a device looks up that array's device address; make the first call
 * before any stream capture.  All calls share the array, so calls that
 * overlap on the GPU race; runs on the stream set by cans_set_stream (else
 * the default stream) and waits for it. */
int cans_cfl_m3_2d_noalloc(double *dt, const double *safety,
                           const double *dtmin, int *merr, const double *gm,
                           const double *ro, const double *pr,
                           const double *vx, const double *vy,
                           const double *vz, const double *bx,
                           const double *by, const double *bz,
                           const double *dx, const int *ix, const double *dy,
                           const int *jx);

/* Ghost-cell fill, 2-D (cans2d/bc/bd*.f:2).  bdper* take (margin0, margin1);
 * the others take (mbnd, margin) with mbnd 0 = lower face, 1 = upper face. */
int cans_bdperx_2d(const int *margin0, const int *margin1, double *qq, const int *ix, const int *jx); /* bdperx.f:2 */
int cans_bdpery_2d(const int *margin0, const int *margin1, double *qq, const int *ix, const int *jx); /* bdpery.f:2 */
int cans_bdsppx_2d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx);    /* bdsppx.f:2 */
int cans_bdsppy_2d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx);    /* bdsppy.f:2 */
int cans_bdspnx_2d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx);    /* bdspnx.f:2 */
int cans_bdspny_2d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx);    /* bdspny.f:2 */
int cans_bdsmpx_2d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx);    /* bdsmpx.f:2 */
int cans_bdsmpy_2d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx);    /* bdsmpy.f:2 */
int cans_bdsmnx_2d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx);    /* bdsmnx.f:2 */
int cans_bdsmny_2d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx);    /* bdsmny.f:2 */
int cans_bdfrex_2d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx);    /* bdfrex.f:2 */
int cans_bdfrey_2d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx);    /* bdfrey.f:2 */
int cans_bdcnsx_2d(const int *mbnd, const int *margin, double *qq, const double *q0, const int *ix, const int *jx); /* bdcnsx.f:2 */
int cans_bdcnsy_2d(const int *mbnd, const int *margin, double *qq, const double *q0, const int *ix, const int *jx); /* bdcnsy.f:2 */
int cans_bdfrdx_2d(const int *mbnd, const int *margin, double *qq, const double *dxm, const int *ix, const int *jx); /* bdfrdx.f:2 */
int cans_bdfrdy_2d(const int *mbnd, const int *margin, double *qq, const double *dym, const int *ix, const int *jx); /* bdfrdy.f:2 */

/* ------------------------------------------------------------------------ */
/* 1. Drop-in entry points: 1-D                                              */
/* ------------------------------------------------------------------------ */
/* replaces subroutine mlw_m   (cans1d/hdmlw/mlw_m.f:2) */
int cans_mlw_m_1d(double *ro, double *pr, double *vx, double *vy, double *by,
                  const double *bx, const double *bxm, const double *dt,
                  const double *qav, const double *gm, const double *dx,
                  const double *dxm, const int *ix);
/* replaces subroutine cfl_m   (cans1d/common/cfl_m.f:2) */
int cans_cfl_m_1d(double *dt, const double *safety, const double *dtmin,
                  int *merr, const double *gm, const double *bx,
                  const double *ro, const double *pr, const double *vx,
                  const double *vy, const double *by, const double *dx,
                  const int *ix);
/* replaces subroutine mlw_m_bg (cans1d/hdmlw/mlw_m_bg.f:2-3): mLW step
 * with gravity gx/gxm, flux-tube cross section sc/scm (gradients dsc/dscm)
 * and distance from the rotation axis rr/rrm (gradients drr/drrm) */
int cans_mlw_m_bg(double *ro, double *pr, double *vx, double *vy, double *by,
                  const double *bx, const double *bxm, const double *dt,
                  const double *qav, const double *gm, const double *gx,
                  const double *gxm, const double *sc, const double *dsc,
                  const double *scm, const double *dscm, const double *rr,
                  const double *rrm, const double *drr, const double *drrm,
                  const double *dx, const double *dxm, const int *ix);
/* replaces subroutine roe_m   (cans1d/hdroe/roe_m.f:2): one 1-D Roe-MUSCL
 * step with the two-component roeflux_m.f; bx, bxm fixed; cells 3..ix-2
 * are updated (margin 3 as md_mhdshktb/hdroe/main.f:5); ix >= 5 */
int cans_roe_m_1d(double *ro, double *pr, double *vx, double *vy, double *by,
                  const double *bx, const double *bxm, const double *dt,
                  const double *gm, const double *dx, const int *ix);
/* replaces subroutine chkdav  (cans1d/common/chkdav.f:2): da below floor is
 * raised to it and vx set to zero there; n_events receives the count */
int cans_chkdav(int *n_events, double *da, double *vx, const double *floor,
                const int *ix);
/* replaces subroutine chkdav (cans2d/common/chkdav.f:2 and
 * cans3d/common/chkdav.f:2): da below floor is raised to it and the velocity
 * components set to zero there; n_events receives the count */
int cans_chkdav_2d(int *n_events, double *da, double *vx, double *vy,
                   const double *floor, const int *ix, const int *jx);
int cans_chkdav_3d(int *n_events, double *da, double *vx, double *vy, double *vz,
                   const double *floor, const int *ix, const int *jx, const int *kx);
/* Ghost-cell fill, 1-D (cans1d/bc/bd*.f:2). */
int cans_bdperx_1d(const int *margin0, const int *margin1, double *qq, const int *ix); /* bdperx.f:2 */
int cans_bdsppx_1d(const int *mbnd, const int *margin, double *qq, const int *ix);    /* bdsppx.f:2 */
int cans_bdspnx_1d(const int *mbnd, const int *margin, double *qq, const int *ix);    /* bdspnx.f:2 */
int cans_bdsmpx_1d(const int *mbnd, const int *margin, double *qq, const int *ix);    /* bdsmpx.f:2 */
int cans_bdsmnx_1d(const int *mbnd, const int *margin, double *qq, const int *ix);    /* bdsmnx.f:2 */
int cans_bdfrex_1d(const int *mbnd, const int *margin, double *qq, const int *ix);    /* bdfrex.f:2 */
int cans_bdcnsx_1d(const int *mbnd, const int *margin, double *qq, const double *q0, const int *ix); /* bdcnsx.f:2 */
int cans_bdfrdx_1d(const int *mbnd, const int *margin, double *qq, const double *dxm, const int *ix); /* bdfrdx.f:2 */

/* ------------------------------------------------------------------------ */
/* 1. Drop-in entry points: 3-D                                              */
/* ------------------------------------------------------------------------ */
/* replaces subroutine mlw_m   (cans3d/hdmlw/mlw_m.f:2-3) */
int cans_mlw_m_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                  double *bx, double *by, double *bz, const double *dt,
                  const double *qav, const double *gm, const double *dx,
                  const double *dxm, const int *ix, const double *dy,
                  const double *dym, const int *jx, const double *dz,
                  const double *dzm, const int *kx);
/* replaces subroutine mlw_m_g (cans3d/hdmlw/mlw_m_g.f:2-4): the 3-D step with
 * gravity; gx, gy, gz at the cells, gxm, gym, gzm at the cell corners,
 * ix*jx*kx each */
int cans_mlw_m_g_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                    double *bx, double *by, double *bz, const double *dt,
                    const double *qav, const double *gm, const double *gx,
                    const double *gxm, const double *gy, const double *gym,
                    const double *gz, const double *gzm, const double *dx,
                    const double *dxm, const int *ix, const double *dy,
                    const double *dym, const int *jx, const double *dz,
                    const double *dzm, const int *kx);
/* replaces subroutine mlw_m_e (cans3d/hdmlw/mlw_m_e.f:2-3): the 3-D
 * resistive step; et at the cells, etm at the cell corners, ix*jx*kx each.
 * J on the outer layer of cells and of corners is taken as zero (the
 * reference leaves it undefined there). */
int cans_mlw_m_e_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                    double *bx, double *by, double *bz, const double *dt,
                    const double *qav, const double *gm, const double *et,
                    const double *etm, const double *dx, const double *dxm,
                    const int *ix, const double *dy, const double *dym,
                    const int *jx, const double *dz, const double *dzm,
                    const int *kx);
/* replaces subroutine cfl_m   (cans3d/common/cfl_m.f:2-3) */
int cans_cfl_m_3d(double *dt, const double *safety, const double *dtmin,
                  int *merr, const double *gm, const double *ro,
                  const double *pr, const double *vx, const double *vy,
                  const double *vz, const double *bx, const double *by,
                  const double *bz, const double *dx, const int *ix,
                  const double *dy, const int *jx, const double *dz,
                  const int *kx);
/* replaces subroutine cfl_m_e (cans3d/common/cfl_m_e.f:2-4): cfl_m with the
 * diffusion limit safety*0.5*min(dx,dy,dz)**2/max(et,1.d-10) */
int cans_cfl_m_e_3d(double *dt, const double *safety, const double *dtmin,
                    int *merr, const double *gm, const double *ro,
                    const double *pr, const double *vx, const double *vy,
                    const double *vz, const double *bx, const double *by,
                    const double *bz, const double *et, const double *dx,
                    const int *ix, const double *dy, const int *jx,
                    const double *dz, const int *kx);
/* replaces subroutine engine  (cansxx-nosupport/md_mhdshktb/hdhlld-x/
 * engine.f:2): one two-stage HLLD step (hlld_mh.f, hlld_flux.f90,
 * inp_const.f, inp_tvdminmod.f, adddfdx.f) on 8 arrays in Heaviside units
 * with permeability mu.  mfdim[3]: 1 = active axis.  dxm, dym, dzm are
 * accepted for the reference signature and not read.  An active axis needs
 * an extent >= 4. */
int cans_hlld_engine_3d(double *ro, double *pr, double *vx, double *vy,
                        double *vz, double *bx, double *by, double *bz,
                        const double *gm, const double *mu, const double *dt,
                        const double *dx, const double *dxm, const double *dy,
                        const double *dym, const double *dz, const double *dzm,
                        const int *ix, const int *jx, const int *kx,
                        const int *mfdim);
/* Ghost-cell fill, 3-D (cans3d/bc/bd*.f:2), same conventions as 2-D. */
int cans_bdperx_3d(const int *margin0, const int *margin1, double *qq, const int *ix, const int *jx, const int *kx); /* bdperx.f:2 */
int cans_bdpery_3d(const int *margin0, const int *margin1, double *qq, const int *ix, const int *jx, const int *kx); /* bdpery.f:2 */
int cans_bdperz_3d(const int *margin0, const int *margin1, double *qq, const int *ix, const int *jx, const int *kx); /* bdperz.f:2 */
int cans_bdsppx_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdsppx.f:2 */
int cans_bdsppy_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdsppy.f:2 */
int cans_bdsppz_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdsppz.f:2 */
int cans_bdspnx_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdspnx.f:2 */
int cans_bdspny_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdspny.f:2 */
int cans_bdspnz_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdspnz.f:2 */
int cans_bdsmpx_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdsmpx.f:2 */
int cans_bdsmpy_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdsmpy.f:2 */
int cans_bdsmpz_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdsmpz.f:2 */
int cans_bdsmnx_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdsmnx.f:2 */
int cans_bdsmny_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdsmny.f:2 */
int cans_bdsmnz_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdsmnz.f:2 */
int cans_bdfrex_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdfrex.f:2 */
int cans_bdfrey_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdfrey.f:2 */
int cans_bdfrez_3d(const int *mbnd, const int *margin, double *qq, const int *ix, const int *jx, const int *kx);    /* bdfrez.f:2 */
int cans_bdcnsx_3d(const int *mbnd, const int *margin, double *qq, const double *q0, const int *ix, const int *jx, const int *kx); /* bdcnsx.f:2 */
int cans_bdcnsy_3d(const int *mbnd, const int *margin, double *qq, const double *q0, const int *ix, const int *jx, const int *kx); /* bdcnsy.f:2 */
int cans_bdcnsz_3d(const int *mbnd, const int *margin, double *qq, const double *q0, const int *ix, const int *jx, const int *kx); /* bdcnsz.f:2 */
int cans_bdfrdx_3d(const int *mbnd, const int *margin, double *qq, const double *dxm, const int *ix, const int *jx, const int *kx); /* bdfrdx.f:2 */
int cans_bdfrdy_3d(const int *mbnd, const int *margin, double *qq, const double *dym, const int *ix, const int *jx, const int *kx); /* bdfrdy.f:2 */
int cans_bdfrdz_3d(const int *mbnd, const int *margin, double *qq, const double *dzm, const int *ix, const int *jx, const int *kx); /* bdfrdz.f:2 */
/* replaces subroutine roe_m   (cans3d/hdroe/roe_m.f:2): one Roe-MUSCL step
 * (roeflux_m.f, tvdminmod.f) on 8 arrays; cells 3..n-2 are updated, margin 3
 * as hdroe/main.f:5.  Extents must be >= 5. */
int cans_roe_m_3d(double *ro, double *pr, double *vx, double *vy, double *vz,
                  double *bx, double *by, double *bz, const double *dt,
                  const double *gm, const double *dx, const int *ix,
                  const double *dy, const int *jx, const double *dz,
                  const int *kx);
/* replaces subroutine roe_m3  (cans2d/hdroe/roe_m3.f:1): one 2-D Roe-MUSCL
 * step (roeflux_m3.f, tvdminmod.f of cans2d/hdroe) on the 9 arrays,
 * az advanced by the half-step E_z; cells 3..n-2 are updated (margin 2 or 3
 * as the md_mhdkh / md_mhd3shktb Roe packages).  Extents must be >= 5. */
int cans_roe_m3_2d(double *ro, double *pr, double *vx, double *vy, double *vz,
                   double *bx, double *by, double *bz, double *az,
                   const double *dt, const double *gm, const double *dx,
                   const int *ix, const double *dy, const int *jx);

/* ------------------------------------------------------------------------ */
/* 2. Residency registry                                                     */
/* ------------------------------------------------------------------------ */
/* Register `narr` host arrays of ix*jx*kx doubles each (jx = kx = 1 for
 * fewer dimensions) as one device-resident set and copy them to the device.
 * Later drop-in calls that pass these host pointers run on the mirrors.  A
 * step call must pass the arrays of one set in the set's order, which must
 * be the step's argument order (e.g. ro,pr,vx,vy,vz,bx,by,bz,az for mlw_m3). */
int cans_gpu_register(double *const *arrays, const int *narr, const int *ix,
                      const int *jx, const int *kx);
/* Copy the whole set containing `any` between device and host. */
int cans_gpu_pull(const double *any);
int cans_gpu_push(const double *any);
/* Forget the set containing `any` and free its device memory. */
int cans_gpu_release(const double *any);

/* ------------------------------------------------------------------------ */
/* 3. Device-resident run handle                                             */
/* ------------------------------------------------------------------------ */
#define CANS_SOLVER_MLW_M_2D 0   /* mlw_m  2-D: ro,pr,vx,vy,bx,by,az         */
#define CANS_SOLVER_MLW_M3_2D 1  /* mlw_m3 2-D: ro,pr,vx,vy,vz,bx,by,bz,az   */
#define CANS_SOLVER_MLW_M_3D 2   /* mlw_m  3-D: ro,pr,vx,vy,vz,bx,by,bz      */
#define CANS_SOLVER_MLW_M_1D 3   /* mlw_m  1-D: ro,pr,vx,vy,by (+ bx, bxm)   */
#define CANS_SOLVER_ROE_M_3D 4   /* roe_m  3-D: ro,pr,vx,vy,vz,bx,by,bz      */
#define CANS_SOLVER_HLLD_3D 5    /* HLLD engine: ro,pr,vx,vy,vz,bx,by,bz     */
#define CANS_SOLVER_MLW_M_BG_1D 6 /* mlw_m_bg 1-D: ro,pr,vx,vy,by (+ bx, bxm
                                    and the ten gravity / flux-tube profiles) */
#define CANS_SOLVER_ROE_M3_2D 7  /* roe_m3 2-D: ro,pr,vx,vy,vz,bx,by,bz,az    */

/* Boundary kinds, one per reference bd* family. */
#define CANS_BD_NONE (-1)
#define CANS_BD_PER 0  /* bdper*  periodic                               */
#define CANS_BD_SPP 1  /* bdspp*  symmetric about the face, even         */
#define CANS_BD_SPN 2  /* bdspn*  symmetric about the face, odd          */
#define CANS_BD_SMP 3  /* bdsmp*  symmetric about the boundary cell, even */
#define CANS_BD_SMN 4  /* bdsmn*  ... odd, boundary cell set to zero      */
#define CANS_BD_FRE 5  /* bdfre*  zero gradient                          */
#define CANS_BD_CNS 6  /* bdcns*  constant value q0                      */
#define CANS_BD_FRD 7  /* bdfrd*  constant gradient                      */

typedef struct cans_run cans_run;

typedef struct {
  int solver;                 /* CANS_SOLVER_*                              */
  int ix, jx, kx;             /* extents including ghost cells (kx=1 in 2-D) */
  int margin;                 /* ghost layers filled by the boundary program */
  double gm, qav;             /* gamma and the artificial-viscosity factor  */
  const double *dx, *dxm;     /* host metric arrays (grdrdy output)         */
  const double *dy, *dym;
  const double *dz, *dzm;
  int exact;                  /* 1 = exact arithmetic policy                */
  int tile;                   /* tile configuration, -1 = library default   */
  void *stream;               /* cudaStream_t or NULL (library stream)      */
  const double *bx, *bxm;     /* 1-D only: the constant bx(ix), bxm(ix)     */
  double mu;                  /* HLLD: permeability (0 = 1)                 */
  int mfdim[3];               /* HLLD: active axes; all 0 = every axis with
                                 an extent > 1                              */
  /* mlw_m_bg (CANS_SOLVER_MLW_M_BG_1D): the static profiles of
   * cans1d/hdmlw/mlw_m_bg.f:2-3, ix doubles each (gravity, cross section,
   * distance from the rotation axis and their gradients).  For the 2-D mLW
   * solvers gx and gxm, with gy and gym below, are the gravity fields of
   * mlw_m_g / mlw_m3_g (ix*jx doubles each; gxm, gym at the cell corners):
   * when gx is set the run takes the step with gravity. */
  const double *gx, *gxm, *sc, *scm, *dsc, *dscm, *rr, *rrm, *drr, *drrm;
  /* chkdav (cans1d/common/chkdav.f:2 and its 2-D / 3-D twins) of ro, then
   * pr, with `floor` after every boundary fill when chkdav = 1; the events
   * are counted in cans_run_state.n_floor */
  int chkdav;
  double floor;
  /* mlw_m_bg loops: the random torque source of the spicule model
   * (cans1d/md_spicule/hdmlw/trqalfven.f:2) after every step when trq (the
   * profile tanh((x-0.75)/0.075)-1, ix doubles) is not NULL; amplitude trq0,
   * random stream keyed by seed */
  const double *trq;
  double trq0;
  unsigned long long seed;
  /* 2-D mLW with gravity: gy(ix,jx) at the cells, gym(ix,jx) at the corners */
  const double *gy, *gym;
  /* mLW with resistivity (2-D mlw_m_e / mlw_m3_e, with gx also mlw_m_ge /
   * mlw_m3_ge; 3-D mlw_m_e, without gravity): et at the cells, etm at the
   * corners, ix*jx(*kx) each; the time step then includes the diffusion
   * limit of cfl_m_e / cfl_m3_e */
  const double *et, *etm;
  /* 3-D mLW with gravity (mlw_m_g, cans3d/hdmlw/mlw_m_g.f): gx, gxm, gy, gym
   * above and gz, gzm here, ix*jx*kx each (the *m fields at the corners) */
  const double *gz, *gzm;
  /* Loop-state check: the CFL of every step counts the warps that
   * met a cell with a non-positive density or pressure, or a non-finite value
   * (cans_run_state.n_bad); the reference's scan just skips such a cell.
   * stop_on_bad = 1 ends the loop at the start of the next iteration with
   * merr = CANS_ERR_NONFINITE. */
  int stop_on_bad;
} cans_run_desc;

typedef struct {
  double t, dt;               /* time after the last step; its dt           */
  long long ns;               /* loop counter of the reference driver       */
  long long nexec;            /* steps executed since cans_run_start        */
  int merr;                   /* 0 or 9001                                  */
  int done;                   /* 1 when tend/nstop/merr ended the loop      */
  int pause;                  /* 1 when an output time was crossed          */
  long long n_floor;          /* chkdav events since cans_run_start         */
  long long n_bad;            /* warps whose CFL met a bad cell (see
                                 cans_run_desc.stop_on_bad) since the start */
} cans_run_state;

int cans_run_create(cans_run **h, const cans_run_desc *d);
int cans_run_destroy(cans_run *h);
/* Boundary program entry: variable index in solver order, face 0..5
 * (x-lo, x-hi, y-lo, y-hi, z-lo, z-hi), CANS_BD_* kind and constant q0. */
int cans_run_set_bc(cans_run *h, int var, int face, int kind, double q0);
/* Copy the state between host arrays (solver order) and the device. */
int cans_run_push(cans_run *h, double *const *host);
int cans_run_pull(cans_run *h, double *const *host);
/* Start the reference loop: t=t0, ns=0, first CFL and t+=dt on the device.
 * pause_on_output=1 stops the loop whenever int(tp/dtout) < int(t/dtout). */
int cans_run_start(cans_run *h, double t0, double tend, long long nstop,
                   double safety, double dtmin, double dtout,
                   int pause_on_output);
/* Enqueue up to `iters` further loop iterations (asynchronous). */
int cans_run_advance(cans_run *h, int iters);
/* No counterpart in the reference: its parameter studies (cans_beta_one,
 * cans_beta_vary: cans1d/md_spicule/hdmlw at several plasma betas, the
 * onebeta of model.f) run every 1-D model as its own process.  This advances
 * `nruns` started 1-D runs (MLW_M_1D or MLW_M_BG_1D, all of one solver
 * family and one arithmetic policy, each run once) by up to `iters` loop
 * iterations each, in one kernel launch: one cluster per run, so runs too
 * small to use the GPU alone share it (a run of up to about 7800 cells, 6000
 * with mlw_m_bg; a larger one is refused with CANS_ERR_ARG).  Each run ends where its own
 * loop would (tend, nstop, dtmin, output pause).  In the exact policy its state
 * and loop state are those cans_run_advance gives, bit for bit; in the fast
 * policy the group kernel may fuse multiply-adds differently, within that
 * policy's tolerance.  Asynchronous, on the first run's stream; the other
 * runs' streams are ordered before and after it. */
int cans_run_advance_group(cans_run *const *runs, int nruns, int iters);
/* Wait for the stream and read the loop state. */
int cans_run_query(cans_run *h, cans_run_state *st);
/* Clear a pause after the host has read the output state. */
int cans_run_resume(cans_run *h);
/* One step with a given dt, optionally followed by the boundary program
 * (no CFL, no loop bookkeeping); asynchronous. */
int cans_run_step(cans_run *h, const double *dt, int apply_bc);
/* Full-grid CFL of the current state (cfl_m3 / cfl_m); synchronous. */
int cans_run_cfl(cans_run *h, double safety, double *dt);
/* Time each tile configuration on `trial_steps` steps of the current state
 * and keep the fastest; returns its index in *tile. */
int cans_run_autotune(cans_run *h, int trial_steps, int *tile);
/* Device pointers of the current state arrays (solver order). */
int cans_run_device_state(cans_run *h, double **dev);
/* Run `iters` loop iterations without a graph, timing each with CUDA events
 * on the run's stream: *step_ms = summed duration of the step kernels,
 * *iter_ms = summed duration of whole iterations.  Synchronous. */
int cans_run_profile(cans_run *h, int iters, double *step_ms, double *iter_ms);

/* Advance with one kernel launch per stage instead of graph replays
 * (use_graph = 0); the default is 1. */
int cans_run_set_graph(cans_run *h, int use_graph);

/* Select the step's tile configuration (0 .. count-1 of the run's step
 * kernel; cans_run_autotune picks one by timing them all). */
int cans_run_set_tile(cans_run *h, int tile);

/* The double-float policy of the 2-D mlw_m3 and the 3-D mlw_m step, of the
 * face flux of the Roe-MUSCL and HLLD steps, and of the 1-D mlw_m and
 * mlw_m_bg loops (no counterpart in the reference: an arithmetic policy
 * beside exact and fast).
 * With on = 1 the step's arithmetic runs as pairs of floats on the FP32
 * pipes (48-bit significands; the exponent range of float, about
 * 1e-38..1e38, bounds the values it holds) and the conserved density and
 * field are accumulated in FP64; the CFL, boundary fill and loop
 * bookkeeping are unchanged.  Held to a relative 1e-10 per variable against
 * the reference arithmetic after 100 steps (mlw_m_bg: the fast policy's
 * bounds, 1e-10 and vx 1e-4, whose static B_x terms stay in FP64).  Only
 * fast-policy CANS_SOLVER_MLW_M3_2D, CANS_SOLVER_MLW_M_3D,
 * CANS_SOLVER_MLW_M_1D, CANS_SOLVER_MLW_M_BG_1D, CANS_SOLVER_ROE_M3_2D,
 * CANS_SOLVER_ROE_M_3D and CANS_SOLVER_HLLD_3D runs without gravity or
 * resistivity take it (else CANS_ERR_ARG); the 2-D and 3-D mLW steps
 * select among their own tile shapes (cans_run_autotune).  A group of 1-D
 * runs (cans_run_advance_group) must share the policy. */
int cans_run_set_df64(cans_run *h, int on);

/* ------------------------------------------------------------------------ */
/* 4. Batches of independent 2-D runs                                        */
/* ------------------------------------------------------------------------ */
/* Many 2-D runs of the same solver (sizes, gamma, metrics and boundary
 * programs may differ) advanced together: each loop iteration of every run
 * is one persistent step launch fed by a device work queue of (run, tile)
 * items, two boundary-fill launches and one bookkeeping launch, replayed as
 * a CUDA graph.  Each run keeps its own dt, t, ns and stop tests, and its
 * results equal those of the same run done alone. */
typedef struct cans_batch cans_batch;
int cans_batch_create(cans_batch **b, int ngrids, const cans_run_desc *descs);
int cans_batch_destroy(cans_batch *b);
int cans_batch_set_bc(cans_batch *b, int grid, int var, int face, int kind,
                      double q0);
int cans_batch_push(cans_batch *b, int grid, double *const *host);
int cans_batch_pull(cans_batch *b, int grid, double *const *host);
/* Every run starts its loop: first CFL, ns=1, t=t0+dt. */
int cans_batch_start(cans_batch *b, double t0, double tend, long long nstop,
                     double safety, double dtmin);
/* Enqueue `iters` iterations of every run (asynchronous); use_graph = 0
 * launches the kernels one by one. */
int cans_batch_advance(cans_batch *b, int iters, int use_graph);
int cans_batch_query(cans_batch *b, int grid, cans_run_state *st);
/* Tile shape / cells-per-thread configurations, and the choice among them. */
int cans_batch_configs(void);
int cans_batch_set_config(cans_batch *b, int config);
/* Time every configuration on `trial_steps` steps and keep the fastest;
 * call after cans_batch_start (the current states are left unchanged). */
int cans_batch_autotune(cans_batch *b, int trial_steps, int *config);

/* ------------------------------------------------------------------------ */
/* Discrete adjoint of the 2-D mlw_m3 run (no counterpart in the reference:  */
/* the reverse sweep the differentiation pattern adds beside the step)       */
/* ------------------------------------------------------------------------ */
/* The run's current state is P_0; every call leaves it unchanged.  The step
 * k+1 state is bnd(mlw_m3(P_k, dts[k])) with the run's boundary program.
 * The objective is J = sum over the interior cells of (bx^2+by^2+bz^2)/(8 pi)
 * dx(i) dy(j) of the final state.  Only CANS_SOLVER_MLW_M3_2D runs. */
/* Forward run with the CFL step of cfl_m3 (safety as given): the dt of every
 * step into dts[nsteps] and, if J is not NULL, the objective. */
int cans_run_record_dts(cans_run *h, long long nsteps, double safety,
                        double *dts, double *J);
/* Forward run with the frozen dts: the objective only. */
int cans_run_objective(cans_run *h, long long nsteps, const double *dts,
                       double *J);
/* Forward run and reverse sweep with binomial checkpointing in at most nsnap
 * stored states (nsnap >= 2; the schedule minimises the recomputed steps):
 * J, and dJ/dP_0 into grad[v] (host arrays of ix*jx doubles, one per state
 * variable, NULL entries skipped; ghost cells included).  *nfwd (if not
 * NULL) receives the number of forward steps executed. */
int cans_run_adjoint(cans_run *h, long long nsteps, const double *dts,
                     int nsnap, double *J, double *const *grad,
                     long long *nfwd);
/* The finite-difference check of the adjoint with the artificial viscosity's
 * branch held.  q = qav dxm max(0, |dv| - 1e-4) (cans2d/hdmlw/mlw_m3.f:
 * 325-334) is piecewise affine in dv; the reverse sweep differentiates the
 * branch each face took in the recorded run.  cans_run_av_record runs the
 * nsteps steps of dts from P_0 and keeps, for every step and face, whether
 * the face was active (|dv| > 1e-4) and the sign of dv (2*ix*jx bytes per
 * step on the device, held until the next record or cans_run_destroy; at
 * most 64 GiB).  cans_run_objective_frozen_av is cans_run_objective with
 * every face held at its recorded branch: q = qav dxm (s dv - 1e-4) on the
 * faces recorded active, s the recorded sign, 0 on the others.  *nflip (if
 * not NULL) receives the number of face-steps whose own branch differs from
 * the recorded one: the switches a perturbed run crosses. */
int cans_run_av_record(cans_run *h, long long nsteps, const double *dts);
/* Copy the branches cans_run_av_record kept for step `step` (2*ix*jx bytes:
 * x faces at i + j*ix, then y faces; bit 0 active, bit 1 dv < 0) to host
 * memory, so that a check run elsewhere can hold the same branches.
 * Synchronous. */
int cans_run_av_branches(cans_run *h, long long step, unsigned char *out);
int cans_run_objective_frozen_av(cans_run *h, long long nsteps, const double *dts,
                                 double *J, long long *nflip);
/* The arithmetic of the reverse sweep: double-float on the FP32 pipes (on =
 * 1, the default; about 2^-46 per operation, far below the gradient's use)
 * or FP64 (on = 0).  The forward steps the sweep recomputes and linearises
 * about are the run's own FP64 steps either way. */
int cans_run_set_adjoint_df64(cans_run *h, int on);
/* Transpose of the run's boundary program applied in place to host arrays
 * (one per state variable): folds ghost-cell sensitivities into the cells
 * they are copied from. */
int cans_run_bc_transpose(cans_run *h, double *const *arrays);

#ifdef __cplusplus
}
#endif
#endif /* CANS_GPU_H */
