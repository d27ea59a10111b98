// Internal host-side declarations shared by the kernel translation units and
// the C-ABI layer.  Not part of the public interface (include/cans_gpu.h).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "cans_common.cuh"
#include <nvtx3/nvToolsExt.h>

namespace cans {

// NVTX range over one host API call (a no-op unless a profiler such as nsys
// or ncu --nvtx is attached); the names are the C-ABI entry points.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// Device copies of the per-axis metric arrays of the reference step
// (cans2d/hdmlw/mlw_m3.f:70-86): spacing d/dm, their inverses di/dim and
// the corner weights u0/u1, plus the host copies they were computed from.
struct Axis {
  int n = 0;
  double *d = nullptr, *dm = nullptr, *di = nullptr, *dim = nullptr,
         *u0 = nullptr, *u1 = nullptr;
};

// Physical constants of one run, computed on the host exactly as the
// reference computes them.
struct Phys {
  double gm, gm1, gm1i, ggm1, pi8i, pi4i, qav;
  double pi4i_cfl;  // 3-D cfl_m uses a single-precision pi
};

// Boundary program: per variable and face (x-lo, x-hi, y-lo, y-hi, z-lo,
// z-hi) a bd* kind and its constant; applied axis by axis (x, then y, then z)
// after each step, as the reference model packages do.
constexpr int kMaxVar = 9;
struct BcTable {
  int margin;
  int kind[kMaxVar][6];
  double q0[kMaxVar][6];
};

enum BdKind { BD_NONE = -1, BD_PER = 0, BD_SPP = 1, BD_SPN = 2, BD_SMP = 3,
              BD_SMN = 4, BD_FRE = 5, BD_CNS = 6, BD_FRD = 7 };

// Region whose CFL the step kernel reduces (0-based inclusive box).  Cells
// outside it are reduced after the boundary fill by the frame kernel.
struct Box3 { int lo[3], hi[3]; };

// ---- 2-D ------------------------------------------------------------------
// solver: 0 = mlw_m (7 arrays), 1 = mlw_m3 (9 arrays).  A and B hold nvar
// contiguous arrays of ix*jx doubles.  If ctl is non-null the kernel takes dt
// from it, skips when the run is done or paused, and reduces the CFL of the
// cells inside `box` into ctl->cfl_bits.
cudaError_t launch_mlw2d(int solver, bool exact, int tile, const double *A,
                         double *B, int ix, int jx, const Axis &ax,
                         const Axis &ay, const Phys &ph, double dt, Ctl *ctl,
                         Box3 box, cudaStream_t s);
int mlw2d_tile_count();
// The mlw_m3 step in the double-float policy (mlw2d_df.cu); tile selects
// one of mlw2d_df_tile_count() shapes.
cudaError_t launch_mlw2d_df(int tile, const double *A, double *B, int ix, int jx,
                            const Axis &ax, const Axis &ay, const Phys &ph, double dt,
                            Ctl *ctl, Box3 box, cudaStream_t s);
int mlw2d_df_tile_count();
// The fast policy's mlw_m3 step with the y-marching tile (the FP64 instance
// of the marching kernel of mlw2d_df.cu); waves selects the segment balance
// by waves of resident blocks instead of by blocks per SM.
cudaError_t launch_mlw2d_march_fast(const double *A, double *B, int ix, int jx,
                                    const Axis &ax, const Axis &ay, const Phys &ph, double dt,
                                    Ctl *ctl, Box3 box, cudaStream_t s, bool waves = false);
// The 3-D mlw_m step in the double-float policy (mlw3d_df.cu).
cudaError_t launch_mlw3d_df(int tile, const double *A, double *B, int ix, int jx, int kx,
                            const Axis &ax, const Axis &ay, const Axis &az, const Phys &ph,
                            double dt, Ctl *ctl, Box3 box, cudaStream_t s);
int mlw3d_df_tile_count();
// The mlw_m3 step (no control block) with the artificial viscosity's branch
// recorded (mode 1) into, or held at (mode 2) the bytes of, avb: 2*ix*jx
// bytes, x faces then y faces.  Mode 2 adds to *nflip the faces whose own
// branch differs from the recorded one.
cudaError_t launch_mlw2d_av(bool exact, int mode, const double *A, double *B, int ix, int jx,
                            const Axis &ax, const Axis &ay, const Phys &ph, double dt,
                            unsigned char *avb, unsigned long long *nflip, cudaStream_t s);
// The same steps with gravity (mlw_m_g / mlw_m3_g): grav holds gx, gxm, gy,
// gym, ix*jx doubles each, on the device.
cudaError_t launch_mlw2d_g(int solver, bool exact, int tile, const double *A,
                           double *B, int ix, int jx, const Axis &ax,
                           const Axis &ay, const Phys &ph, const double *grav,
                           double dt, Ctl *ctl, Box3 box, cudaStream_t s);
int mlw2d_g_tile_count();
// Resistive 2-D mLW steps (mlw2d_e.cu): eta = et, etm (ix*jx each), res the
// eta*J scratch of mlw2d_e_scratch_doubles doubles, grav optional.
size_t mlw2d_e_scratch_doubles(int solver, int ix, int jx);
cudaError_t launch_mlw2d_e(int solver, bool exact, const double *A, double *B, int ix,
                           int jx, const Axis &ax, const Axis &ay, const Phys &ph,
                           const double *grav, const double *eta, double *res,
                           double dt, Ctl *ctl, Box3 box, cudaStream_t s);
// cfl_m_e / cfl_m3_e over all cells into out_bits; wave = 0 reduces the
// diffusion limit alone.
cudaError_t launch_cfl2d_e(int solver, bool exact, const double *S, int ix, int jx,
                           const Axis &ax, const Axis &ay, const Phys &ph,
                           const double *et, double safety, int wave,
                           unsigned long long *out_bits, cudaStream_t s);
cudaError_t launch_cfl2d_full(int solver, bool exact, const double *S, int ix,
                              int jx, const Axis &ax, const Axis &ay,
                              const Phys &ph, double safety,
                              unsigned long long *out_bits, cudaStream_t s);
cudaError_t launch_bc2d(int nvar, double *S, int ix, int jx, const Axis &ax,
                        const Axis &ay, const BcTable &bc, const Ctl *ctl,
                        cudaStream_t s);
cudaError_t launch_frame2d(int solver, bool exact, const double *S, int ix,
                           int jx, const Axis &ax, const Axis &ay,
                           const Phys &ph, int margin, Ctl *ctl,
                           cudaStream_t s, int all = 0);
// launch_bc2d (with ctl) followed by launch_frame2d (all = 0) as one launch:
// the boundary program of the state the step just wrote, the frame CFL and
// the end of the loop iteration.  nvar must be that of the solver's layout
// (9 or 7) and each extent at least 2 margin + 3.
cudaError_t launch_bcframe2d(int solver, bool exact, int nvar, int ix, int jx, const Axis &ax,
                             const Axis &ay, const Phys &ph, const BcTable &bc, Ctl *ctl,
                             cudaStream_t s);

// ---- 3-D ------------------------------------------------------------------
// mlw_m 3-D on 8 arrays (ro,pr,vx,vy,vz,bx,by,bz) of ix*jx*kx doubles.
cudaError_t launch_mlw3d(bool exact, int tile, const double *A, double *B,
                         int ix, int jx, int kx, const Axis &ax,
                         const Axis &ay, const Axis &az, const Phys &ph,
                         double dt, Ctl *ctl, Box3 box, cudaStream_t s);
// 3-D mlw_m_g (mlw3d.cu): grav = gx, gxm, gy, gym, gz, gzm (n each)
int mlw3d_g_tile_count();
cudaError_t launch_mlw3d_g(bool exact, int tile, const double *A, double *B, int ix,
                           int jx, int kx, const Axis &ax, const Axis &ay, const Axis &az,
                           const Phys &ph, const double *grav, double dt, Ctl *ctl,
                           Box3 box, cudaStream_t s);
int mlw3d_tile_count();
// 3-D mlw_m_e, the step kernel part (mlw3d.cu): res = et*J at the cells and
// etm*Jh at the corners (x, y, z each, n doubles per component)
cudaError_t launch_mlw3d_res(bool exact, int tile, const double *A, double *B, int ix,
                             int jx, int kx, const Axis &ax, const Axis &ay, const Axis &az,
                             const Phys &ph, const double *res, double dt, Ctl *ctl,
                             Box3 box, cudaStream_t s);
// 3-D mlw_m_e (mlw3d_e.cu): eta = et, etm (n each); res scratch of
// mlw3d_e_scratch_doubles doubles; the tile as launch_mlw3d_res
size_t mlw3d_e_scratch_doubles(int ix, int jx, int kx);
cudaError_t launch_mlw3d_e(bool exact, int tile, const double *A, double *B, int ix, int jx,
                           int kx, const Axis &ax, const Axis &ay, const Axis &az,
                           const Phys &ph, const double *eta, double *res, double dt,
                           Ctl *ctl, Box3 box, cudaStream_t s);
// cfl_m_e 3-D: min over the cells of the wave (wave = 1) and diffusion limits
cudaError_t launch_cfl3d_e(bool exact, const double *S, int ix, int jx, int kx,
                           const Axis &ax, const Axis &ay, const Axis &az, const Phys &ph,
                           const double *et, double safety, int wave,
                           unsigned long long *out_bits, cudaStream_t s);
cudaError_t launch_cfl3d_full(bool exact, const double *S, int ix, int jx,
                              int kx, const Axis &ax, const Axis &ay,
                              const Axis &az, const Phys &ph, double safety,
                              unsigned long long *out_bits, cudaStream_t s);
cudaError_t launch_bc3d(int nvar, double *S, int ix, int jx, int kx,
                        const Axis &ax, const Axis &ay, const Axis &az,
                        const BcTable &bc, const Ctl *ctl, cudaStream_t s);
cudaError_t launch_frame3d(bool exact, int ix, int jx, int kx, const Axis &ax,
                           const Axis &ay, const Axis &az, const Phys &ph,
                           int margin, Ctl *ctl, cudaStream_t s, int all = 0);

// ---- 3-D Roe-MUSCL (roe_m) -------------------------------------------------
// One two-stage step on 8 arrays (ro,pr,vx,vy,vz,bx,by,bz); A -> B, cells
// outside 3..n-2 copied.  scratch holds roe3d_scratch_doubles(ix*jx*kx)
// doubles (half-step primitives and the face fluxes of one stage).  With ctl
// the kernels take dt and the buffers from it and reduce the CFL of `box`.
size_t roe3d_scratch_doubles(size_t ncells);
cudaError_t launch_roe3d(bool exact, const double *A, double *B,
                         double *scratch, int ix, int jx, int kx,
                         const Axis &ax, const Axis &ay, const Axis &az,
                         const Phys &ph, double dt, Ctl *ctl, Box3 box,
                         cudaStream_t s, bool df = false);

// 2-D roe_m3 (9 arrays ro,pr,vx,vy,vz,bx,by,bz,az of ix*jx); A -> B, cells
// outside 3..n-2 copied; scratch of roe3d_scratch_doubles(ix*jx).
cudaError_t launch_roe2d(bool exact, const double *A, double *B,
                         double *scratch, int ix, int jx, const Axis &ax,
                         const Axis &ay, const Phys &ph, double dt, Ctl *ctl,
                         Box3 box, cudaStream_t s, bool df = false);

// 1-D roe_m (5 arrays ro,pr,vx,vy,by of ix; bx, bxm, dx device arrays);
// A -> B, cells outside 3..ix-2 copied; scratch of roe1d_scratch_doubles(ix).
size_t roe1d_scratch_doubles(size_t ncells);
cudaError_t launch_roe1d(bool exact, const double *A, double *B, double *scratch,
                         const double *bx, const double *bxm, const double *dx,
                         int ix, double gm, double dt, cudaStream_t s);

// ---- 3-D HLLD (cansxx engine) ----------------------------------------------
// One two-stage HLLD step on 8 arrays (Heaviside units, permeability mu);
// A -> B for every cell.  mfdim[a] = 1 marks an active axis.  scratch holds
// hlld3d_scratch_doubles(ix*jx*kx) doubles.  With ctl the kernels take dt and
// the buffers from it; launch_hlld3d_finish then reduces the CFL of every
// cell of the new state and ends the loop iteration.  df (with exact false)
// evaluates the face flux in double-float arithmetic.
size_t hlld3d_scratch_doubles(size_t ncells);
cudaError_t launch_hlld3d(bool exact, const double *A, double *B,
                          double *scratch, int ix, int jx, int kx,
                          const int *mfdim, const Axis &ax, const Axis &ay,
                          const Axis &az, double gm, double mu, double dt,
                          const Ctl *ctl, cudaStream_t s, bool df = false);
cudaError_t launch_hlld3d_finish(bool exact, int ix, int jx, int kx,
                                 const Axis &ax, const Axis &ay,
                                 const Axis &az, const Phys &ph, Ctl *ctl,
                                 cudaStream_t s);

// ---- discrete adjoint of the 2-D mlw_m3 step ---------------------------------
// P: input state (9 arrays), R: the step's raw output, lam_in: adjoint of R
// (after the transposed boundary fill), lam_out: adjoint of P.  scratch holds
// adj2d_scratch_doubles(ix*jx) doubles.  df: the reverse arithmetic in
// double-float on the FP32 pipes (else FP64).
size_t adj2d_scratch_doubles(size_t ncells);
cudaError_t launch_adj2d_step(const double *P, const double *R,
                              const double *lam_in, double *lam_out,
                              double *scratch, int ix, int jx, const Axis &ax,
                              const Axis &ay, const Phys &ph, double dt, bool df,
                              cudaStream_t s);
// raw output of a step (margin 1, no bdsmn* rule) from the filled states
// before (P_cur: outer layer) and after it (P_next: every other cell)
cudaError_t launch_adj2d_merge(const double *P_next, const double *P_cur, double *R,
                               int nvar, int ix, int jx, cudaStream_t s);
// transpose of the 2-D boundary program, in place on nvar adjoint arrays
cudaError_t launch_bc2d_transpose(int nvar, double *lam, int ix, int jx,
                                  const Axis &ax, const Axis &ay,
                                  const BcTable &bc, cudaStream_t s);
// J = sum over the interior of |B|^2/(8 pi) dx dy into *J (device), and, if
// lam is not null, dJ/dP into lam (9 arrays); scratch >= 256 doubles
cudaError_t launch_adj2d_objective(const double *P, double *lam, double *J,
                                   double *scratch, int ix, int jx,
                                   const Axis &ax, const Axis &ay,
                                   const Phys &ph, cudaStream_t s);

// ---- 1-D ------------------------------------------------------------------
// The whole 1-D loop (or one fixed-dt step) as one cluster launch, in place
// on 5 arrays (ro,pr,vx,vy,by) of ix doubles.
int mlw1d_min_cells();
// Options of the 1-D loop: bg (10 arrays of ix: gx gxm sc scm dsc dscm rr
// rrm drr drrm) selects the mlw_m_bg step; trq (ix, needs bg) adds the
// torque source of the spicule model with amplitude trq0 and random-stream
// key seed; chk applies chkdav of ro and pr with `floor` after each boundary
// fill, counting the events into ctl->nfloor.  A fixed step uses bg only.
struct Loop1D {
  const double *bg = nullptr;
  const double *trq = nullptr;
  double trq0 = 0.0;
  unsigned long long seed = 0;
  double floor = 0.0;
  int chk = 0;
};
// The 1-D loop (or one fixed step) on one cluster; dfp: the double-float
// policy (exact false).
cudaError_t launch_mlw1d(bool exact, double *S, const double *bx,
                         const double *bxm, const Loop1D &opt, int ix,
                         const Axis &ax, const Phys &ph, const BcTable &bc,
                         Ctl *ctl, int max_steps, int fixed, double dt_fixed,
                         int start, cudaStream_t s, bool dfp = false);
// One run of a group advanced by launch_mlw1d_group (a started resident
// loop: ctl is its control block).
struct Run1DArgs {
  double *S;
  const double *bx, *bxm;
  Loop1D opt;
  int ix;
  Axis ax;
  Phys ph;
  BcTable bc;
  Ctl *ctl;
};
// Up to max_steps iterations of each run's loop, all runs in one launch (one
// cluster per run); every run has the BG variant or none has.
// dfp: the double-float policy (exact false).
cudaError_t launch_mlw1d_group(bool exact, bool bgv, const Run1DArgs *runs, int nruns,
                               int max_steps, cudaStream_t s, bool dfp = false);
// chkdav (cans1d/common/chkdav.f:68-76) on device arrays: da below floor is
// raised to it and vx zeroed there; the count is added to *count (device).
// chkdav of 2-D / 3-D states (mlw1d.cu): na density-like slots a0, a1 of S
// (n doubles each) floored in turn, each event zeroing nv velocity slots from
// v0; with ctl S is the state the loop's step just wrote.
cudaError_t launch_chkdav_nd(double *S, size_t n, int na, int a0, int a1, int nv, int v0,
                             double floor, const Ctl *ctl, unsigned long long *count,
                             cudaStream_t s);
cudaError_t launch_chkdav(double *da, double *vx, double floor, size_t n,
                          unsigned long long *count, cudaStream_t s);
cudaError_t launch_cfl1d(bool exact, const double *S, const double *bx, int ix,
                         const Axis &ax, const Phys &ph, double safety,
                         unsigned long long *out, cudaStream_t s);

// ---- single bd* operation on one array (literal entry points) -------------
// kind/axis/mbnd follow the reference routine; dims = (n0, n1, n2).
cudaError_t launch_bd_one(int kind, int axis, int mbnd, int margin0,
                          int margin1, double *q, double q0, const double *dxm,
                          int n0, int n1, int n2, cudaStream_t s);

// ---- control block helpers --------------------------------------------------
// Start of the reference loop body: ns+=1, dt from the CFL minimum, the dtmin
// test, tp=t, t+=dt.  Runs on one thread.
cudaError_t launch_prepare(Ctl *ctl, cudaStream_t s);

// Host-side metric construction with the reference expressions.
void build_axis_host(int n, const double *d, const double *dm, double *di,
                     double *dim, double *u0, double *u1);
Phys make_phys(double gm, double qav);

// The stream the drop-in entry points use if one exists already (set by
// cans_set_stream or created by an earlier call), else the default stream;
// never creates a stream.
cudaStream_t configured_stream();

// Kernel-launch counter (all launches issued by this library).
void count_launch(int n = 1);
unsigned long long launch_count();

}  // namespace cans
