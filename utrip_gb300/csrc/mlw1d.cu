// 1-D modified Lax-Wendroff time loop as one thread-block-cluster kernel
// (sm_103a, FP64).
//
// Replaces the 1-D reference loop of cans1d/md_mhdshktb/hdmlw/main.f:139-152:
// cfl_m (cans1d/common/cfl_m.f:42-71) -> t += dt -> mlw_m
// (cans1d/hdmlw/mlw_m.f:2-215 with mlwhalf.f:33-46, mlwfull.f:30-33,
// mlwartv.f:31-34) -> bnd (bdsppx / bdsmnx ...) -> output and loop tests.
//
// A 1-D grid of ~10^3 cells is far too small to fill the GPU and a kernel
// per stage would be launch-bound, so the whole loop runs inside one launch of
// a cluster of CS blocks.  Each block keeps its segment of the grid (plus one
// halo cell per side) in shared memory for the whole run; after each step
// neighbours exchange halo cells through distributed shared memory and the
// CFL minimum is reduced across the cluster, so no host round trip happens
// per step.  One cluster barrier per step (the CFL reduction, which also
// publishes the new cells for the halo exchange) when the boundary program
// reads only the cells of the blocks that run it; a second one before the
// boundary fill when a rule is periodic.
//
// The BG variant is mlw_m_bg (cans1d/hdmlw/mlw_m_bg.f:2-271): the same
// two-stage step on the cross-section-weighted variables (ro, e, rx, ry r,
// by/r) x sc with gravity, cross-section and rotation sources added by
// mlwsrch.f / mlwsrcf.f, and bx included in the energy.  The spicule loop
// (cans1d/md_spicule/hdmlw/main.f:160-219) adds two options that any 1-D
// loop may use: the torque source of trqalfven.f after the step, and the
// chkdav floor of ro and pr after the boundary fill (one extra cluster
// barrier), with the events counted in the control block.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "df64.cuh"

namespace cg = cooperative_groups;

namespace cans {

namespace {
// primitive order: ro pr vx vy by ; conserved order: ro ee rx ry by
constexpr int NV1 = 5;
}  // namespace

struct Run1D {
  double *S;             // global state, 5 arrays of ix (read at start, written at end)
  const double *bx, *bxm;
  const double *bg;      // BG: gx gxm sc scm dsc dscm rr rrm drr drrm (10 x ix)
  const double *trq;     // torque profile trq(ix), or nullptr
  double trq0;           // torque amplitude
  unsigned long long seed;  // key of the torque's random stream
  double floor;          // chkdav floor of ro and pr (used when chk)
  int chk;
  int bnd_local;         // 1: no boundary rule reads another block's cells
  Axis ax;
  Phys ph;
  BcTable bc;
  Ctl *ctl;              // loop control (resident run) or nullptr
  int ix;
  int q, rem;            // blocks r < rem own q+1 interior cells, the rest q
  int lmax;              // q + 3: largest own count plus two halo cells
  int max_steps;         // steps this launch may take
  int fixed;             // 1: one step with dt_fixed, no CFL / boundary fill
  double dt_fixed;
  int start;             // 1: compute the first CFL and start the loop
};

// one reference bd* rule on the global line, through an accessor
template <class Get, class Put>
__device__ void bd1_face(int kind, int mbnd, int m, int n, double q0,
                         const double *dxm, Get get, Put put) {
  if (kind < 0) return;
  if (kind == BD_PER) {
    const int b0 = 1 + m, b1 = n - m;
    if (mbnd == 0)
      for (int i = 1; i <= m; i++) put(b0 - i, get(b1 + 1 - i));
    else
      for (int i = 1; i <= m; i++) put(b1 + i, get(b0 - 1 + i));
    return;
  }
  if (mbnd == 0) {
    const int b = 1 + m;
    switch (kind) {
      case BD_SPP: for (int i = 1; i <= m; i++) put(b - i, get(b - 1 + i)); break;
      case BD_SPN: for (int i = 1; i <= m; i++) put(b - i, -get(b - 1 + i)); break;
      case BD_SMP: for (int i = 1; i <= m; i++) put(b - i, get(b + i)); break;
      case BD_SMN:
        for (int i = 1; i <= m; i++) put(b - i, -get(b + i));
        put(b, 0.0);
        break;
      case BD_FRE: for (int i = 1; i <= m; i++) put(b - i, get(b)); break;
      case BD_CNS: for (int i = 1; i <= m; i++) put(b - i, q0); break;
      case BD_FRD:
        for (int i = 1; i <= m; i++) {
          const double dqq = __ddiv_rn(__dsub_rn(get(b + 1), get(b)), dxm[b - 1]);
          put(b - i, __dsub_rn(get(b - i + 1), __dmul_rn(dqq, dxm[b - i - 1])));
        }
        break;
      default: break;
    }
  } else {
    const int b = n - m;
    switch (kind) {
      case BD_SPP: for (int i = 1; i <= m; i++) put(b + i, get(b + 1 - i)); break;
      case BD_SPN: for (int i = 1; i <= m; i++) put(b + i, -get(b + 1 - i)); break;
      case BD_SMP: for (int i = 1; i <= m; i++) put(b + i, get(b - i)); break;
      case BD_SMN:
        for (int i = 1; i <= m; i++) put(b + i, -get(b - i));
        put(b, 0.0);
        break;
      case BD_FRE: for (int i = 1; i <= m; i++) put(b + i, get(b)); break;
      case BD_CNS: for (int i = 1; i <= m; i++) put(b + i, q0); break;
      case BD_FRD:
        for (int i = 1; i <= m; i++) {
          const double dqq = __ddiv_rn(__dsub_rn(get(b), get(b - 1)), dxm[b - 2]);
          put(b + i, __dadd_rn(get(b + i - 1), __dmul_rn(dqq, dxm[b + i - 2])));
        }
        break;
      default: break;
    }
  }
}

// Uniform deviate in [0, 1) for cell g of loop step ns: SplitMix64 (Steele,
// Lea and Flood, "Fast splittable pseudorandom number generators", OOPSLA
// 2014) of the counter ns*ix + g offset by the seed, top 53 bits.  Integer
// arithmetic only, so every device and the host give the same stream.  It
// stands in for the Fortran random_number of trqalfven.f:23, whose stream
// belongs to the compiler's runtime library.
__device__ __forceinline__ double torque_uniform(unsigned long long seed, long long ns,
                                                 int g, int ix) {
  unsigned long long z =
      seed + ((unsigned long long)ns * (unsigned long long)ix + (unsigned long long)g + 1ull) *
                 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * 0x1.0p-53;
}

// trqalfven.f:25-36 for global cell g: vy + dt*trq0*q*trq with
// q = 2 rr (anum - 0.5); cell ix takes q of cell ix-2 (trqalfven.f:30)
template <bool E>
__device__ __forceinline__ F<E> torque_add(const Run1D &p, F<E> vy, F<E> dt, long long ns,
                                           int g) {
  using FT = F<E>;
  const int gq = (g == p.ix - 1) ? p.ix - 3 : g;
  const FT anum(torque_uniform(p.seed, ns, gq, p.ix));
  const FT q = 2.0 * FT(p.bg[6 * (size_t)p.ix + gq]) * (anum - 0.5);
  return vy + dt * FT(p.trq0) * q * FT(p.trq[g]);
}

// ---- the double-float policy of the 1-D step -------------------------------
// The stages below are the fast policy's algebra evaluated in double-float
// (df64.cuh) on the FP32 pipes: the state stays in FP64 (converted on load
// and store), the scratch arrays hold double-float values in their 8-byte
// slots, and the torque, boundary program, chkdav and the cluster's CFL
// minimum stay in FP64.
//
// mlw_m_bg carries bx^2/8pi in the energy, and -bx^2/8pi sc and bx^2/8pi dsc
// in the x-momentum flux and source.  In a low-beta corona those static terms
// are many orders above the gas pressure, and p = (gm-1)(e - ek - b^2/8pi)
// and the force balance of the tube would lose their digits to the 48-bit
// significand.  So the double-float values leave them out (they are constant
// in time), and the scheme gets them back through static arrays formed once
// in FP64, where it sees them:
//   XS[0][l] = es(l+1) - es(l), es = pi8i bx^2 sc: the viscosity term of the
//            energy update;
//   XS[1][l] = the corner average of es over scm, minus pi8i bxm^2: the
//            corner pressure;
//   XS[2][l] = the static x-momentum flux difference and source of the
//            corner predictor (times dt);
//   XS[3][l] = those of the cell update, cell and corner terms (times dt/2).
namespace d1 {
using R = df::DF;
__device__ __forceinline__ R in(double x) { return num_in<R>(x); }
__device__ __forceinline__ R ld(const double *p) { return num_ld<R>(p); }
__device__ __forceinline__ void st(double *p, R v) { num_st(p, v); }
__device__ __forceinline__ R half(R x) { return R(df::scale(x.d, 0.5f)); }
__device__ __forceinline__ R sq(R x) { return R(df::sqr(x.d)); }
__device__ __forceinline__ R rcp(R x) { return R(df::rcp(x.d)); }
// square root: the correctly rounded float root s, then one Newton step
// s + (x - s^2) / (2 s), with s^2 exact as a float pair and x - s^2 formed
// to float precision (the head difference is exact: s^2 and x.h are within
// an ulp of each other)
__device__ __forceinline__ R sqrt_(R x) {
  const float s = __fsqrt_rn(x.d.h);
  if (!(s > 0.0f) || s == __int_as_float(0x7f800000)) return R(s);  // 0, NaN, inf
  const float ph = __fmul_rn(s, s), pl = __fmaf_rn(s, s, -ph);
  const float e = __fadd_rn(__fsub_rn(__fsub_rn(x.d.h, ph), pl), x.d.l);
  return R(df::fast_two_sum(s, __fmul_rn(e, __fmul_rn(0.5f, __frcp_rn(s)))));
}
struct Phys1 {
  R gm, gm1, gm1i, ggm1, pi4i, pi8i, qav;
};
__device__ __forceinline__ Phys1 phys1(const Phys &ph) {
  return {in(ph.gm), in(ph.gm1), in(ph.gm1i), in(ph.ggm1), in(ph.pi4i), in(ph.pi8i),
          in(ph.qav)};
}

// cell stage of local cell l (global g): conserved values U, fluxes FX and
// (BG) cell sources SS from the primitives pc (5 arrays of stride L)
template <bool BG>
__device__ __forceinline__ void cell(const Run1D &p, const double *pc, int L, int l, int g,
                                     const double *RI, double *U, double *FX, double *SS,
                                     const Phys1 &c) {
  const size_t nx = (size_t)p.ix;
  const R ro = in(pc[l]), pr = in(pc[L + l]), vx = in(pc[2 * L + l]), vy = in(pc[3 * L + l]),
          by = in(pc[4 * L + l]);
  const R bx = in(p.bx[g]);
  const R ek = half(ro) * fma(vy, vy, sq(vx));
  const R rx = ro * vx;
  const R ez = fma(vy, bx, -(vx * by));
  if constexpr (BG) {
    const double *bg = p.bg;
    const R sc = in(bg[2 * nx + g]), rr = in(bg[6 * nx + g]), gx = in(bg[g]),
            dsc = in(bg[4 * nx + g]), drr = in(bg[8 * nx + g]), rri = in(RI[2 * L + l]);
    const R pty = fma(sq(by), c.pi8i, pr);  // pressure without pi8i bx^2
    const R eey = fma(pr, c.gm1i, fma(c.pi8i, sq(by), ek));
    const R ep = fma(pr, c.ggm1, ek);
    const R rxs = rx * sc, scri = sc * rri;
    st(&U[l], ro * sc);
    st(&U[L + l], eey * sc);
    st(&U[2 * L + l], rxs);
    st(&U[3 * L + l], (ro * vy) * (sc * rr));
    st(&U[4 * L + l], by * scri);
    st(&FX[l], rxs);
    st(&FX[L + l], fma(-(by * ez), c.pi4i, ep * vx) * sc);
    st(&FX[2 * L + l], fma(rx, vx, pty) * sc);
    st(&FX[3 * L + l], fma(rx, vy, -(bx * by * c.pi4i)) * (sc * rr));
    st(&FX[4 * L + l], -(ez * scri));
    st(&SS[l], rxs * gx);
    st(&SS[L + l], fma(fma(fma(ro * vy, vy, -(sq(by) * c.pi4i)), rri * drr, ro * gx), sc,
                       pty * dsc));
  } else {
    const R bb = sq(by);
    const R ee = fma(pr, c.gm1i, fma(c.pi8i, bb, ek));
    const R ep = fma(pr, c.ggm1, ek);
    st(&U[l], ro);
    st(&U[L + l], ee);
    st(&U[2 * L + l], rx);
    st(&U[3 * L + l], ro * vy);
    st(&U[4 * L + l], by);
    st(&FX[l], rx);
    st(&FX[L + l], fma(-(by * ez), c.pi4i, ep * vx));
    st(&FX[2 * L + l], fma(rx, vx, fma(bb, c.pi8i, pr)));
    st(&FX[3 * L + l], fma(rx, vy, -(bx * by * c.pi4i)));
    st(&FX[4 * L + l], -ez);
  }
}

// corner between local cells l and l+1 (global g, g+1): half-step fluxes K,
// (BG) corner sources SH and the viscosity coefficient Q
template <bool BG>
__device__ __forceinline__ void corner(const Run1D &p, const double *pc, int L, int l, int g,
                                       const double *RI, const double *XS, const double *U,
                                       const double *FX,
                                       const double *SS, double *K, double *SH, double *Q,
                                       R dt, const Phys1 &c) {
  const size_t nx = (size_t)p.ix;
  const R dxim = in(p.ax.dim[g]);
  R un[NV1];
#pragma unroll
  for (int v = 0; v < NV1; v++) {
    const R uh = half(ld(&U[v * L + l + 1]) + ld(&U[v * L + l]));
    un[v] = fma(-dt, dxim * (ld(&FX[v * L + l + 1]) - ld(&FX[v * L + l])), uh);
  }
  const R bxm = in(p.bxm[g]);
  if constexpr (BG) {
    const double *bg = p.bg;
    un[1] = fma(dt, half(ld(&SS[l + 1]) + ld(&SS[l])), un[1]);
    un[2] = fma(dt, half(ld(&SS[L + l + 1]) + ld(&SS[L + l])) + ld(&XS[2 * L + l]), un[2]);
    const R scm = in(bg[3 * nx + g]), rrm = in(bg[7 * nx + g]), gxm = in(bg[nx + g]),
            dscm = in(bg[5 * nx + g]), drrm = in(bg[9 * nx + g]);
    const R si = in(RI[L + l]), rrmi = in(RI[3 * L + l]), ri = rcp(un[0]);
    const R roh = un[0] * si, eeh = un[1] * si, vxh = un[2] * ri, vyh = un[3] * ri * rrmi,
            byh = un[4] * si * rrm;
    const R ek = half(roh) * fma(vyh, vyh, sq(vxh));
    const R prh = c.gm1 * (eeh - ek - c.pi8i * sq(byh) + ld(&XS[L + l]));
    const R pty = fma(sq(byh), c.pi8i, prh);  // without pi8i bxm^2
    const R ezh = fma(vyh, bxm, -(vxh * byh));
    const R eph = fma(prh, c.ggm1, ek);
    const R rvx = roh * vxh;
    st(&K[l], rvx * scm);
    st(&K[L + l], fma(-(byh * ezh), c.pi4i, eph * vxh) * scm);
    st(&K[2 * L + l], fma(rvx, vxh, pty) * scm);
    st(&K[3 * L + l], fma(rvx, vyh, -(bxm * byh * c.pi4i)) * (scm * rrm));
    st(&K[4 * L + l], -(ezh * (scm * rrmi)));
    st(&SH[l], rvx * gxm * scm);
    st(&SH[L + l], fma(fma(fma(roh * vyh, vyh, -(sq(byh) * c.pi4i)), rrmi * drrm, roh * gxm),
                       scm, pty * dscm));
  } else {
    const R roh = un[0], ri = rcp(roh);
    const R vxh = un[2] * ri, vyh = un[3] * ri, byh = un[4];
    const R bb = sq(byh);
    const R ek = half(roh) * fma(vyh, vyh, sq(vxh));
    const R prh = c.gm1 * (un[1] - ek - c.pi8i * bb);
    const R ezh = fma(vyh, bxm, -(vxh * byh));
    const R eph = fma(prh, c.ggm1, ek);
    const R rvx = roh * vxh;
    st(&K[l], rvx);
    st(&K[L + l], fma(-(byh * ezh), c.pi4i, eph * vxh));
    st(&K[2 * L + l], fma(rvx, vxh, fma(bb, c.pi8i, prh)));
    st(&K[3 * L + l], fma(rvx, vyh, -(bxm * byh * c.pi4i)));
    st(&K[4 * L + l], -ezh);
  }
  // q = qav dxm max(0, |vx(i+1) - vx(i)| - 1.0e-4), the threshold a
  // single-precision literal in the reference, so exactly the float 1.0e-4f
  const R a = fabs(in(pc[2 * L + l + 1]) - in(pc[2 * L + l])) - 1.0e-4f;
  const R q = a > 0.0f ? c.qav * in(p.ax.dm[g]) * a : R(0.0f);
  st(&Q[l], q * dxim);
}

// full step of own local cell l (global g): the new primitives into pn
template <bool BG>
__device__ __forceinline__ void update(const Run1D &p, double *pn, int L, int l, int g,
                                       const double *RI, const double *XS, const double *U,
                                       const double *FX,
                                       const double *SS, const double *K, const double *SH,
                                       const double *Q, R dt, const Phys1 &c) {
  const R hdt = half(dt), dxi = in(p.ax.di[g]), hdx = half(dxi);
  const R ql = ld(&Q[l]), qm = ld(&Q[l - 1]);
  R u[NV1];
#pragma unroll
  for (int v = 0; v < NV1; v++) {
    R du = -(hdt * (hdx * (ld(&FX[v * L + l + 1]) - ld(&FX[v * L + l - 1]))));
    if (BG && (v == 1 || v == 2)) du = fma(hdt, ld(&SS[(v - 1) * L + l]), du);
    du = fma(-hdt, dxi * (ld(&K[v * L + l]) - ld(&K[v * L + l - 1])), du);
    if (BG && (v == 1 || v == 2))
      du = fma(hdt,
               fma(in(p.ax.u0[g]), ld(&SH[(v - 1) * L + l - 1]),
                   in(p.ax.u1[g]) * ld(&SH[(v - 1) * L + l])),
               du);
    const R uc = ld(&U[v * L + l]);
    du = fma(dt, dxi * (ql * (ld(&U[v * L + l + 1]) - uc) - qm * (uc - ld(&U[v * L + l - 1]))),
             du);
    if (BG && v == 1) du = fma(dt, dxi * (ql * ld(&XS[l]) - qm * ld(&XS[l - 1])), du);
    if (BG && v == 2) du = fma(hdt, ld(&XS[3 * L + l]), du);
    u[v] = uc + du;
  }
  const R rinv = rcp(u[0]);
  R ro, ee, vx, vy, by;
  if constexpr (BG) {
    const R si = in(RI[l]);
    ro = u[0] * si;
    ee = u[1] * si;
    vx = u[2] * rinv;
    vy = u[3] * rinv * in(RI[2 * L + l]);
    by = u[4] * si * in(p.bg[6 * (size_t)p.ix + g]);
  } else {
    ro = u[0];
    ee = u[1];
    vx = u[2] * rinv;
    vy = u[3] * rinv;
    by = u[4];
  }
  // (BG: ee without pi8i bx^2, as the cell stage stores it)
  const R pr = c.gm1 * (ee - half(ro) * fma(vy, vy, sq(vx)) - c.pi8i * sq(by));
  pn[l] = num_out(ro);
  pn[L + l] = num_out(pr);
  pn[2 * L + l] = num_out(vx);
  pn[3 * L + l] = num_out(vy);
  pn[4 * L + l] = num_out(by);
}

// safety * dx / (|vx| + c_f) of one cell (cfl_m.f:53-60), c_f from the
// fast magnetosonic speed squared (b^2 pi4i + gm pr) / ro
__device__ __forceinline__ double cfl(const Run1D &p, const double *pc, int L, int l, int g,
                                      double safety, const Phys1 &c) {
  const R ro = in(pc[l]), pr = in(pc[L + l]), vx = in(pc[2 * L + l]), by = in(pc[4 * L + l]);
  const R bx = in(p.bx[g]);
  const R s = fma(c.gm, pr, fma(bx, bx, sq(by)) * c.pi4i) * rcp(ro);
  const R den = fabs(vx) + sqrt_(s);
  return num_out(in(safety) * in(p.ax.d[g]) * rcp(den));
}
}  // namespace d1

// The loop of one run on one cluster (the kernels below): p lives in the
// kernel parameters (one run) or in shared memory (a group of runs).  DFP:
// the double-float policy (E false).
template <bool E, bool BG, bool DFP = false>
__device__ __forceinline__ void mlw1d_body(const Run1D &p) {
  static_assert(!(E && DFP), "the double-float policy is a fast policy");
  using FT = F<E>;
  cg::cluster_group cluster = cg::this_cluster();
  const int CS = (int)cluster.num_blocks();
  const int r = (int)cluster.block_rank();
  const int tid = threadIdx.x, NT = blockDim.x;
  const int ix = p.ix, L = p.lmax;
  extern __shared__ double sm[];
  // layout: prim[2][5][L], U[5][L], FX[5][L], K[5][L], Q[L],
  // (BG: SS[2][L] cell sources, SH[2][L] corner sources, RI[4][L] the
  // reciprocals 1/sc, 1/scm, 1/rr, 1/rrm of the own cells; BG and DFP: XS[4][L]
  // the static-field terms of the double-float stages), slots[2][CS],
  // bad[2][CS], red[32]
  double *prim = sm;
  double *U = prim + 2 * NV1 * L;
  double *FX = U + NV1 * L;
  double *K = FX + NV1 * L;
  double *Q = K + NV1 * L;
  double *SS = Q + L;
  double *SH = SS + (BG ? 2 * L : 0);
  double *RI = SH + (BG ? 2 * L : 0);
  double *XS = RI + (BG ? 4 * L : 0);
  double *slots = XS + ((BG && DFP) ? 4 * L : 0);
  double *bslots = slots + 2 * CS;  // per block: 1 if its CFL saw a bad cell
  double *red = bslots + 2 * CS;
  const double *bg = p.bg;
  const size_t nx = (size_t)ix;
  __shared__ double s_dt, s_t, s_tp, s_pending;
  __shared__ long long s_ns, s_nexec;
  __shared__ int s_done, s_merr, s_pause;

  // interior cells (0-based 1..ix-2) split evenly; local l <-> global lo-1+l
  // balanced split of the ix-2 interior cells over the cluster
  auto first_cell = [&](int rr) { return 1 + rr * p.q + min(rr, p.rem); };
  auto own_count = [&](int rr) { return p.q + (rr < p.rem ? 1 : 0); };
  const int lo = first_cell(r);
  const int hi = lo + own_count(r) - 1;
  const int nl = hi - lo + 3;  // local cells incl. one halo each side
  d1::Phys1 cdf;  // the double-float policy's constants
  if constexpr (DFP) cdf = d1::phys1(p.ph);
  const FT gm(p.ph.gm), gm1(p.ph.gm1), pi8i(p.ph.pi8i), pi4i(p.ph.pi4i),
      qav(p.ph.qav);
  const Axis &ax = p.ax;
  const int NVS = NV1 * L;  // stride of one prim buffer

  auto P = [&](int buf, int v, int l) -> double & {
    return prim[(size_t)buf * NVS + (size_t)v * L + l];
  };
  // load own segment, halos and ghosts from global memory
  for (int l = tid; l < nl; l += NT) {
    const int g = lo - 1 + l;
#pragma unroll
    for (int v = 0; v < NV1; v++) P(0, v, l) = p.S[(size_t)v * ix + g];
    if constexpr (BG) {
      // the cross-section and radius profiles are constant through the run:
      // the fast policy multiplies by their reciprocals instead of dividing
      // by them every step (1.0 / x, the value the step's own 1.0 / sc gave)
      RI[0 * L + l] = 1.0 / bg[2 * nx + g];
      RI[1 * L + l] = 1.0 / bg[3 * nx + g];
      RI[2 * L + l] = 1.0 / bg[6 * nx + g];
      RI[3 * L + l] = 1.0 / bg[7 * nx + g];
    }
    if constexpr (BG && DFP) {
      // formed in FP64: differences of nearly equal terms
      const double c8 = p.ph.pi8i;
      auto b2 = [&](int gg) { return p.bx[gg] * p.bx[gg]; };
      auto bm2 = [&](int gg) { return p.bxm[gg] * p.bxm[gg]; };
      auto es = [&](int gg) { return c8 * b2(gg) * bg[2 * nx + gg]; };       // energy
      auto fxs = [&](int gg) { return -(c8 * b2(gg)) * bg[2 * nx + gg]; };   // x-momentum flux
      auto sss = [&](int gg) { return c8 * b2(gg) * bg[4 * nx + gg]; };      // and source
      auto kxs = [&](int gg) { return -(c8 * bm2(gg)) * bg[3 * nx + gg]; };  // at corners
      auto shs = [&](int gg) { return c8 * bm2(gg) * bg[5 * nx + gg]; };
      if (l <= nl - 2) {
        num_st(&XS[l], d1::in(es(g + 1) - es(g)));
        num_st(&XS[L + l], d1::in(0.5 * (es(g + 1) + es(g)) / bg[3 * nx + g] - c8 * bm2(g)));
        num_st(&XS[2 * L + l], d1::in(-ax.dim[g] * (fxs(g + 1) - fxs(g)) +
                                      0.5 * (sss(g + 1) + sss(g))));
      }
      if (l >= 1 && l <= nl - 2)
        num_st(&XS[3 * L + l],
               d1::in(-(0.5 * ax.di[g]) * (fxs(g + 1) - fxs(g - 1)) + sss(g) -
                      ax.di[g] * (kxs(g) - kxs(g - 1)) + ax.u0[g] * shs(g - 1) +
                      ax.u1[g] * shs(g)));
    }
  }
  if (tid == 0) {
    if (p.ctl) {
      s_dt = p.ctl->dt; s_t = p.ctl->t; s_tp = p.ctl->tp; s_ns = p.ctl->ns;
      s_nexec = p.ctl->nexec; s_done = p.ctl->done; s_merr = p.ctl->merr;
      s_pause = p.ctl->pause;
    } else {
      s_dt = p.dt_fixed; s_t = 0.0; s_tp = 0.0; s_ns = 0; s_nexec = 0;
      s_done = 0; s_merr = 0; s_pause = 0;
    }
  }
  int cur = 0;
  __syncthreads();

  // CFL of the own cells (cfl_m.f:53-60) reduced over the cluster into
  // slots[par] of block 0; returns the minimum after a cluster barrier, and
  // in any_bad whether a cell of any block had a non-positive density or
  // pressure or a time step that is not a number (counted in ctl->nonfinite).
  auto cluster_cfl = [&](int buf, int par, bool &any_bad) -> double {
    double dmin = __longlong_as_double(0x7ff0000000000000LL);
    bool bad = false;
    const FT safety(p.ctl ? p.ctl->safety : 1.0), pi4c(p.ph.pi4i);
    for (int l = 1 + tid; l <= nl - 2; l += NT) {
      const int g = lo - 1 + l;
      if constexpr (DFP) {
        const double dtq = d1::cfl(p, &P(buf, 0, 0), L, l, g, safety.v, cdf);
        if (dtq < dmin || dmin != dmin) dmin = dtq;
        bad |= bad_cell(P(buf, 0, l), P(buf, 1, l), dtq);
        continue;
      }
      const FT ro(P(buf, 0, l)), pr(P(buf, 1, l)), vx(P(buf, 2, l)), by(P(buf, 4, l));
      const FT bx(p.bx[g]);
      const FT onero = 1.0 / ro;
      const FT ca2 = (bx * bx + by * by) * pi4c * onero;
      const FT cs2 = gm * pr * onero;
      const FT dtcfl = FT(ax.d[g]) / (fabs_(vx) + fsqrt(cs2 + ca2));
      const double dtq = (safety * dtcfl).v;
      if (dtq < dmin || dmin != dmin) dmin = dtq;
      bad |= bad_cell(ro.v, pr.v, dtq);
    }
    dmin = warp_min(dmin);
    if ((tid & 31) == 0) red[tid >> 5] = dmin;
    const int blk_bad = __syncthreads_or(bad);
    if (tid == 0) {
      double x = red[0];
      for (int w = 1; w < (NT + 31) / 32; w++) x = (red[w] < x || x != x) ? red[w] : x;
      double *dst = cluster.map_shared_rank(slots, 0);
      dst[par * CS + r] = x;
      double *dstb = cluster.map_shared_rank(bslots, 0);
      dstb[par * CS + r] = blk_bad ? 1.0 : 0.0;
      if (blk_bad && p.ctl) atomicAdd(&p.ctl->nonfinite, 1);
    }
    cluster.sync();
    double *src = cluster.map_shared_rank(slots, 0);
    double *srcb = cluster.map_shared_rank(bslots, 0);
    double m = (double)1.e20f;  // the reference's starting minimum
    any_bad = false;
    for (int k = 0; k < CS; k++) {
      const double x = src[par * CS + k];
      if (x < m) m = x;
      any_bad |= srcb[par * CS + k] != 0.0;
    }
    return m;
  };

  int par = 0;
  if (!p.fixed && p.start) {
    bool bad0;
    const double dt0 = cluster_cfl(cur, par, bad0);
    par ^= 1;
    if (tid == 0) {  // first iteration always starts (do-while loop)
      s_ns += 1;
      s_dt = dt0;
      if (dt0 < p.ctl->dtmin) {
        s_merr = 9001;
        s_done = 1;
      } else {
        s_tp = s_t;
        s_t = s_t + dt0;
      }
    }
    __syncthreads();
  }

  for (int step = 0; step < p.max_steps; step++) {
    if (s_done || s_pause) break;
    const FT dt(s_dt);
    const long long ns_now = s_ns;
    const int nb = cur ^ 1;
    // ---- cell stage (mlw_m.f:37-73; mlw_m_bg.f:97-166) ---------------------
    if constexpr (DFP) {
      for (int l = tid; l < nl; l += NT)
        d1::cell<BG>(p, &P(cur, 0, 0), L, l, lo - 1 + l, RI, U, FX, SS, cdf);
    } else if constexpr (BG) {
      for (int l = tid; l < nl; l += NT) {
        const int g = lo - 1 + l;
        const FT ro(P(cur, 0, l)), pr(P(cur, 1, l)), vx(P(cur, 2, l)), vy(P(cur, 3, l)),
            by(P(cur, 4, l));
        const FT bx(p.bx[g]), gx(bg[g]), sc(bg[2 * nx + g]), dsc(bg[4 * nx + g]),
            rr(bg[6 * nx + g]), drr(bg[8 * nx + g]);
        const FT vv = vx * vx + vy * vy;
        const FT bb = by * by + bx * bx;
        FT ee, ep;
        if constexpr (E) {
          ee = pr / gm1 + 0.5 * ro * vv + pi8i * bb;
          ep = pr * gm / gm1 + 0.5 * ro * vv;
        } else {
          ee = pr * p.ph.gm1i + 0.5 * ro * vv + pi8i * bb;
          ep = pr * p.ph.ggm1 + 0.5 * ro * vv;
        }
        const FT rx = ro * vx;
        const FT ez = -vx * by + vy * bx;
        const FT bbm = by * by - bx * bx;
        U[0 * L + l] = (ro * sc).v; U[1 * L + l] = (ee * sc).v; U[2 * L + l] = (rx * sc).v;
        U[3 * L + l] = (ro * vy * sc * rr).v;
        FX[0 * L + l] = (rx * sc).v;                                          // :121-122
        FX[1 * L + l] = ((ep * vx - by * ez * pi4i) * sc).v;                  // :130-131
        SS[0 * L + l] = (rx * gx * sc).v;                                     // :132-133
        FX[2 * L + l] = ((ro * (vx * vx) + pr + bbm * pi8i) * sc).v;          // :144,147
        FX[3 * L + l] = ((ro * vx * vy - bx * by * pi4i) * sc * rr).v;        // :155-156
        if constexpr (E) {
          U[4 * L + l] = (by * sc / rr).v;
          SS[1 * L + l] = ((ro * gx + (ro * (vy * vy) - (by * by) * pi4i) / rr * drr) * sc +
                           (pr + bb * pi8i) * dsc).v;                         // :145-148
          FX[4 * L + l] = ((-ez) * sc / rr).v;                                // :162-164
        } else {
          const FT rri(RI[2 * L + l]);
          U[4 * L + l] = (by * sc * rri).v;
          SS[1 * L + l] = ((ro * gx + (ro * (vy * vy) - (by * by) * pi4i) * rri * drr) * sc +
                           (pr + bb * pi8i) * dsc).v;
          FX[4 * L + l] = ((-ez) * sc * rri).v;
        }
      }
    } else
    for (int l = tid; l < nl; l += NT) {
      const int g = lo - 1 + l;
      const FT ro(P(cur, 0, l)), pr(P(cur, 1, l)), vx(P(cur, 2, l)), vy(P(cur, 3, l)),
          by(P(cur, 4, l));
      const FT bx(p.bx[g]);
      const FT vv = vx * vx + vy * vy;
      const FT bb = by * by;
      FT ee, ep;
      if constexpr (E) {
        ee = pr / gm1 + 0.5 * ro * vv + pi8i * bb;
        ep = pr * gm / gm1 + 0.5 * ro * vv;
      } else {
        ee = pr * p.ph.gm1i + 0.5 * ro * vv + pi8i * bb;
        ep = pr * p.ph.ggm1 + 0.5 * ro * vv;
      }
      const FT rx = ro * vx;
      const FT ez = -vx * by + vy * bx;
      U[0 * L + l] = ro.v; U[1 * L + l] = ee.v; U[2 * L + l] = rx.v;
      U[3 * L + l] = (ro * vy).v; U[4 * L + l] = by.v;
      FX[0 * L + l] = rx.v;                                        // ro*vx
      FX[1 * L + l] = (ep * vx - by * ez * pi4i).v;                 // :55
      FX[2 * L + l] = (ro * (vx * vx) + pr + by * by * pi8i).v;     // :60-61
      FX[3 * L + l] = (ro * vx * vy - bx * by * pi4i).v;            // :66
      FX[4 * L + l] = (-ez).v;                                      // :71
    }
    __syncthreads();
    // ---- corners (mlwhalf.f:42-46, mlw_m.f:74-110) and AV faces -----------
    if constexpr (DFP) {
      const d1::R dtr = d1::in(s_dt);
      for (int l = tid; l < nl - 1; l += NT)
        d1::corner<BG>(p, &P(cur, 0, 0), L, l, lo - 1 + l, RI, XS, U, FX, SS, K, SH, Q, dtr,
                       cdf);
    } else if constexpr (BG) {
      // mlwhalf + mlwsrch, conversion (mlw_m_bg.f:170-183), corner fluxes
      // and sources (:188-234)
      for (int l = tid; l < nl - 1; l += NT) {
        const int g = lo - 1 + l;
        const FT dxim(ax.dim[g]);
        FT un[NV1];
#pragma unroll
        for (int v = 0; v < NV1; v++) {
          const FT uh = 0.5 * (FT(U[v * L + l + 1]) + FT(U[v * L + l]));
          const FT dfdx = dxim * (FT(FX[v * L + l + 1]) - FT(FX[v * L + l]));
          un[v] = uh - dt * dfdx;
        }
        un[1] = un[1] + dt * (0.5 * (FT(SS[0 * L + l + 1]) + FT(SS[0 * L + l])));
        un[2] = un[2] + dt * (0.5 * (FT(SS[1 * L + l + 1]) + FT(SS[1 * L + l])));
        const FT scm(bg[3 * nx + g]), rrm(bg[7 * nx + g]), gxm(bg[nx + g]),
            dscm(bg[5 * nx + g]), drrm(bg[9 * nx + g]), bxm(p.bxm[g]);
        FT roh, eeh, vxh, vyh, byh;
        if constexpr (E) {
          roh = un[0] / scm;
          eeh = un[1] / scm;
          vxh = un[2] / un[0];
          vyh = un[3] / un[0] / rrm;
          byh = un[4] / scm * rrm;
        } else {
          const FT si(RI[1 * L + l]), ri(1.0 / un[0].v);
          roh = un[0] * si;
          eeh = un[1] * si;
          vxh = un[2] * ri;
          vyh = un[3] * ri * FT(RI[3 * L + l]);
          byh = un[4] * si * rrm;
        }
        const FT vv = vxh * vxh + vyh * vyh;
        const FT bb = bxm * bxm + byh * byh;
        const FT prh = gm1 * (eeh - 0.5 * roh * vv - pi8i * bb);
        const FT ezh = -vxh * byh + vyh * bxm;
        FT eph;
        if constexpr (E) eph = prh * gm / gm1 + 0.5 * roh * vv;
        else eph = prh * p.ph.ggm1 + 0.5 * roh * vv;
        const FT bbm = byh * byh - bxm * bxm;
        K[0 * L + l] = (roh * vxh * scm).v;
        K[1 * L + l] = ((eph * vxh - byh * ezh * pi4i) * scm).v;
        SH[0 * L + l] = (roh * vxh * gxm * scm).v;
        K[2 * L + l] = ((roh * (vxh * vxh) + prh + bbm * pi8i) * scm).v;
        K[3 * L + l] = ((roh * vxh * vyh - bxm * byh * pi4i) * scm * rrm).v;
        if constexpr (E) {
          SH[1 * L + l] = ((roh * gxm + (roh * (vyh * vyh) - (byh * byh) * pi4i) / rrm * drrm) *
                               scm +
                           (prh + bb * pi8i) * dscm).v;
          K[4 * L + l] = ((-ezh) * scm / rrm).v;
        } else {
          const FT rrmi(RI[3 * L + l]);
          SH[1 * L + l] = ((roh * gxm + (roh * (vyh * vyh) - (byh * byh) * pi4i) * rrmi * drrm) *
                               scm +
                           (prh + bb * pi8i) * dscm).v;
          K[4 * L + l] = ((-ezh) * scm * rrmi).v;
        }
        const FT q = qav * FT(ax.dm[g]) *
                     max0(fabs_(FT(P(cur, 2, l + 1)) - FT(P(cur, 2, l))) - CANS_AV_EPS);
        Q[l] = (q * dxim).v;
      }
    } else
    for (int l = tid; l < nl - 1; l += NT) {
      const int g = lo - 1 + l;  // corner between g and g+1
      const FT dxim(ax.dim[g]);
      FT un[NV1];
#pragma unroll
      for (int v = 0; v < NV1; v++) {
        const FT uh = 0.5 * (FT(U[v * L + l + 1]) + FT(U[v * L + l]));
        const FT dfdx = dxim * (FT(FX[v * L + l + 1]) - FT(FX[v * L + l]));
        un[v] = uh - dt * dfdx;
      }
      const FT roh = un[0], eeh = un[1], rxh = un[2], ryh = un[3], byh = un[4];
      FT vxh, vyh;
      if constexpr (E) {
        vxh = rxh / roh;
        vyh = ryh / roh;
      } else {
        const FT rinv(1.0 / roh.v);
        vxh = rxh * rinv;
        vyh = ryh * rinv;
      }
      const FT vv = vxh * vxh + vyh * vyh;
      const FT bb = byh * byh;
      const FT prh = gm1 * (eeh - 0.5 * roh * vv - pi8i * bb);
      const FT bxm(p.bxm[g]);
      const FT ezh = -vxh * byh + vyh * bxm;
      FT eph;
      if constexpr (E) eph = prh * gm / gm1 + 0.5 * roh * vv;
      else eph = prh * p.ph.ggm1 + 0.5 * roh * vv;
      K[0 * L + l] = (roh * vxh).v;
      K[1 * L + l] = (eph * vxh - byh * ezh * pi4i).v;
      K[2 * L + l] = (roh * (vxh * vxh) + prh + byh * byh * pi8i).v;
      K[3 * L + l] = (roh * vxh * vyh - bxm * byh * pi4i).v;
      K[4 * L + l] = (-ezh).v;
      const FT q = qav * FT(ax.dm[g]) *
                   max0(fabs_(FT(P(cur, 2, l + 1)) - FT(P(cur, 2, l))) - CANS_AV_EPS);
      Q[l] = (q * dxim).v;
    }
    __syncthreads();
    // ---- full step of the own cells ---------------------------------------
    if constexpr (DFP) {
      const d1::R dtr = d1::in(s_dt);
      for (int l = 1 + tid; l <= nl - 2; l += NT) {
        const int g = lo - 1 + l;
        d1::update<BG>(p, &P(nb, 0, 0), L, l, g, RI, XS, U, FX, SS, K, SH, Q, dtr, cdf);
        if (BG && p.trq) P(nb, 3, l) = torque_add<false>(p, FT(P(nb, 3, l)), dt, ns_now, g).v;
      }
    } else if constexpr (BG) {
      // mlwhalf/mlwsrch increments, mlwfull + mlwsrcf, mlwartv, then the
      // update and conversion (mlw_m_bg.f:251-268) and the torque
      for (int l = 1 + tid; l <= nl - 2; l += NT) {
        const int g = lo - 1 + l;
        const FT hdt = 0.5 * dt, dxi(ax.di[g]);
        const FT hdx = 0.5 * dxi;
        FT u[NV1];
#pragma unroll
        for (int v = 0; v < NV1; v++) {
          FT du(0.0);
          du = du - hdt * (hdx * (FT(FX[v * L + l + 1]) - FT(FX[v * L + l - 1])));
          if (v == 1 || v == 2) du = du + hdt * FT(SS[(v - 1) * L + l]);
          du = du - hdt * (dxi * (FT(K[v * L + l]) - FT(K[v * L + l - 1])));
          if (v == 1 || v == 2)
            du = du + hdt * (FT(ax.u0[g]) * FT(SH[(v - 1) * L + l - 1]) +
                             FT(ax.u1[g]) * FT(SH[(v - 1) * L + l]));
          const FT uc(U[v * L + l]);
          du = du + dt * (dxi * (FT(Q[l]) * (FT(U[v * L + l + 1]) - uc) -
                                 FT(Q[l - 1]) * (uc - FT(U[v * L + l - 1]))));
          u[v] = uc + du;
        }
        const FT sc(bg[2 * nx + g]), rr(bg[6 * nx + g]), bx(p.bx[g]);
        FT ro, ee, rx, ry, by, vx, vy;
        if constexpr (E) {
          ro = u[0] / sc;
          ee = u[1] / sc;
          rx = u[2] / sc;
          ry = u[3] / sc / rr;
          by = u[4] / sc * rr;
          vx = rx / ro;
          vy = ry / ro;
        } else {
          const FT si(RI[0 * L + l]);
          ro = u[0] * si;
          ee = u[1] * si;
          const FT rinv(1.0 / u[0].v);  // 1/(ro sc)
          vx = u[2] * rinv;
          vy = u[3] * rinv * FT(RI[2 * L + l]);
          by = u[4] * si * rr;
        }
        const FT pr = gm1 * (ee - 0.5 * ro * (vx * vx + vy * vy) - pi8i * (bx * bx + by * by));
        if (p.trq) vy = torque_add<E>(p, vy, dt, ns_now, g);
        P(nb, 0, l) = ro.v; P(nb, 1, l) = pr.v; P(nb, 2, l) = vx.v;
        P(nb, 3, l) = vy.v; P(nb, 4, l) = by.v;
      }
    } else
    for (int l = 1 + tid; l <= nl - 2; l += NT) {
      const int g = lo - 1 + l;
      const FT hdt = 0.5 * dt, dxi(ax.di[g]);
      const FT hdx = 0.5 * dxi;
      FT u[NV1];
#pragma unroll
      for (int v = 0; v < NV1; v++) {
        FT du(0.0);
        du = du - hdt * (hdx * (FT(FX[v * L + l + 1]) - FT(FX[v * L + l - 1])));
        du = du - hdt * (dxi * (FT(K[v * L + l]) - FT(K[v * L + l - 1])));
        const FT uc(U[v * L + l]);
        du = du + dt * (dxi * (FT(Q[l]) * (FT(U[v * L + l + 1]) - uc) -
                               FT(Q[l - 1]) * (uc - FT(U[v * L + l - 1]))));
        u[v] = uc + du;
      }
      const FT ro = u[0], ee = u[1], rx = u[2], ry = u[3], by = u[4];
      FT vx, vy;
      if constexpr (E) {
        vx = rx / ro;
        vy = ry / ro;
      } else {
        const FT rinv(1.0 / ro.v);
        vx = rx * rinv;
        vy = ry * rinv;
      }
      const FT pr = gm1 * (ee - 0.5 * ro * (vx * vx + vy * vy) - pi8i * (by * by));
      P(nb, 0, l) = ro.v; P(nb, 1, l) = pr.v; P(nb, 2, l) = vx.v;
      P(nb, 3, l) = vy.v; P(nb, 4, l) = by.v;
    }
    // ghost cells keep their values through the step; the torque source
    // runs over every cell (trqalfven.f:35-37), ghosts included
    if (tid == 0) {
      if (lo == 1) {
        for (int v = 0; v < NV1; v++) P(nb, v, 0) = P(cur, v, 0);
        if (BG && p.trq) P(nb, 3, 0) = torque_add<E>(p, FT(P(nb, 3, 0)), dt, ns_now, 0).v;
      }
      if (hi == ix - 2) {
        for (int v = 0; v < NV1; v++) P(nb, v, nl - 1) = P(cur, v, nl - 1);
        if (BG && p.trq)
          P(nb, 3, nl - 1) = torque_add<E>(p, FT(P(nb, 3, nl - 1)), dt, ns_now, ix - 1).v;
      }
    }
    if (p.fixed) {
      cluster.sync();
      cur = nb;
      break;
    }
    // The boundary program reads only cells of the block that runs it unless
    // a rule is periodic or reaches past that block's cells (bnd_local = 0);
    // then it must wait for the whole cluster.
    if (p.bnd_local) __syncthreads();
    else cluster.sync();
    // ---- boundary program (bnd.f:9-19): lower face by block 0, upper face
    // by the last block; cells of other blocks are read through DSMEM -------
    if (tid < NV1 && (r == 0 || r == CS - 1)) {
      const int v = tid;
      auto owner = [&](int g1) {  // 1-based global cell -> (rank, local)
        const int g = g1 - 1;
        int rr;
        if (g <= 0) rr = 0;
        else if (g >= ix - 1) rr = CS - 1;
        else if (g - 1 < p.rem * (p.q + 1)) rr = (g - 1) / (p.q + 1);
        else rr = p.rem + (g - 1 - p.rem * (p.q + 1)) / p.q;
        const int l = g - first_cell(rr) + 1;
        return make_int2(rr, l);
      };
      auto get = [&](int g1) -> double {
        const int2 o = owner(g1);
        double *base = cluster.map_shared_rank(prim, o.x);
        return base[(size_t)nb * NVS + (size_t)v * L + o.y];
      };
      auto put = [&](int g1, double x) {
        const int2 o = owner(g1);
        P(nb, v, o.y) = x;  // faces only write cells of this block
      };
      if (r == 0)
        bd1_face(p.bc.kind[v][0], 0, p.bc.margin, ix, p.bc.q0[v][0], ax.dm, get, put);
      if (r == CS - 1)
        bd1_face(p.bc.kind[v][1], 1, p.bc.margin, ix, p.bc.q0[v][1], ax.dm, get, put);
    }
    __syncthreads();
    // ---- chkdav of ro, then pr (chkdav.f:68-76), every cell incl. ghosts ----
    if (p.chk) {
      unsigned int nev = 0;
      const int l0 = (lo == 1) ? 0 : 1, l1 = (hi == ix - 2) ? nl - 1 : nl - 2;
      for (int l = l0 + tid; l <= l1; l += NT) {
        if (P(nb, 0, l) < p.floor) {
          P(nb, 0, l) = p.floor;
          P(nb, 2, l) = 0.0;
          nev++;
        }
        if (P(nb, 1, l) < p.floor) {
          P(nb, 1, l) = p.floor;
          P(nb, 2, l) = 0.0;
          nev++;
        }
      }
      if (nev) atomicAdd(&p.ctl->nfloor, (unsigned long long)nev);
      __syncthreads();
    }
    // ---- CFL of the own cells, reduced over the cluster; its cluster barrier
    // also publishes every block's final cells for the halo exchange ---------
    bool badn;
    const double dtn = cluster_cfl(nb, par, badn);
    par ^= 1;
    if (tid < NV1) {
      if (r > 0) {
        const double *nbp = cluster.map_shared_rank(prim, r - 1);
        const int ln = own_count(r - 1);  // neighbour's last own cell
        P(nb, tid, 0) = nbp[(size_t)nb * NVS + (size_t)tid * L + ln];
      }
      if (r < CS - 1) {
        const double *nbp = cluster.map_shared_rank(prim, r + 1);
        P(nb, tid, nl - 1) = nbp[(size_t)nb * NVS + (size_t)tid * L + 1];
      }
    }
    cur = nb;
    if (tid == 0) {
      // end of the loop body (main.f:155-199) and start of the next
      s_nexec += 1;
      if (p.ctl->pause_on_output && p.ctl->dtout > 0.0) {
        const long long nt1 = (long long)(s_tp / p.ctl->dtout);
        const long long nt2 = (long long)(s_t / p.ctl->dtout);
        if (nt1 < nt2) s_pause = 1;
      }
      s_pending = dtn;  // CFL of the state just written, for a later resume
      if (!(s_ns < p.ctl->nstop && s_t < p.ctl->tend)) {
        s_done = 1;
      } else if (!s_pause && p.ctl->stop_on_bad && badn) {
        s_merr = 9100;  // CANS_ERR_NONFINITE: the state just written has a bad cell
        s_done = 1;
      } else if (!s_pause) {
        s_ns += 1;
        s_dt = dtn;
        if (dtn < p.ctl->dtmin) {
          s_merr = 9001;
          s_done = 1;
        } else {
          s_tp = s_t;
          s_t = s_t + dtn;
        }
      }
    }
    __syncthreads();
  }
  // keep remote reads of this block's shared memory valid until all are done
  cluster.sync();
  // write the own segment (and ghosts) back
  for (int l = tid; l < nl; l += NT) {
    const int g = lo - 1 + l;
    const bool own = (l >= 1 && l <= nl - 2) || (g == 0) || (g == ix - 1);
    if (!own) continue;
#pragma unroll
    for (int v = 0; v < NV1; v++) p.S[(size_t)v * ix + g] = P(cur, v, l);
  }
  if (r == 0 && tid == 0 && p.ctl) {
    p.ctl->dt = s_dt; p.ctl->t = s_t; p.ctl->tp = s_tp; p.ctl->ns = s_ns;
    p.ctl->nexec = s_nexec; p.ctl->done = s_done; p.ctl->merr = s_merr;
    p.ctl->pause = s_pause;
    if (s_pause)  // resume starts the next iteration from this CFL minimum
      p.ctl->cfl_bits = (unsigned long long)__double_as_longlong(s_pending);
  }
}

template <bool E, bool BG, bool DFP>
__global__ void __launch_bounds__(256, 1) k_mlw1d(Run1D p) {
  mlw1d_body<E, BG, DFP>(p);
}

// A group of independent runs, one cluster each: cluster c runs runs[c].  The
// run's parameters are copied to shared memory once; the runs share nothing
// else, so a cluster that finishes early leaves its SMs to the next ones.
// Two blocks a SM; the double-float instance takes up to 288 threads (96
// registers), so that the two halo cells of a 256-cell block get a warp of
// their own instead of a second pass of warp 0 that the others wait for.
template <bool E, bool BG, bool DFP>
__global__ void __launch_bounds__(DFP ? 288 : 256, 2)
    k_mlw1d_group(const Run1D *__restrict__ runs) {
  __shared__ Run1D sp;
  const unsigned c = blockIdx.x / cg::this_cluster().num_blocks();
  if (threadIdx.x == 0) sp = runs[c];
  __syncthreads();
  mlw1d_body<E, BG, DFP>(sp);
}

// the kernel instance of a policy (exact, fast or double-float) and variant
template <class K>
K pick1d(bool exact, bool bgv, bool dfp, K ef, K eb, K ff, K fb, K df, K db) {
  if (dfp) return bgv ? db : df;
  if (exact) return bgv ? eb : ef;
  return bgv ? fb : ff;
}

// Smallest grid the 1-D loop kernel accepts (one block of 4 interior cells).
int mlw1d_min_cells() { return 6; }

// Cluster size for ix cells: up to `cmax` blocks, each owning at least 4
// interior cells so a face rule of margin <= 3 stays inside its block.  The
// step is FP64-bound even at 10^3 cells (2 FP64 lanes per SM), so more SMs
// per cluster shorten every step.
static int cluster_for(int ix, int cmax) {
  int cs = cmax;
  while (cs > 1 && (ix - 2) / cs < 4) cs >>= 1;
  return cs;
}

// Largest cluster the device co-schedules for this kernel: 16 blocks where
// non-portable cluster sizes are available, else the portable 8.  Asked once
// per device (the same answer for every instance of the kernel), under a lock:
// launches may come from several host threads and devices.
static int cluster_max(void (*kern)(Run1D), size_t smem) {
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static int cached_of[kMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return 8;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (cached_of[dev]) return cached_of[dev];
  int best = 8;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
      cudaSuccess) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(16, 1, 1);
    cfg.blockDim = dim3(256, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) == cudaSuccess && n > 0) best = 16;
  }
  cudaGetLastError();  // a refused query leaves no error behind
  cached_of[dev] = best;
  return best;
}

namespace {
constexpr size_t per_cell_doubles(bool bgv, bool dfp) {
  return (size_t)(2 * NV1 + 3 * NV1 + 1) + (bgv ? 8 : 0) + (bgv && dfp ? 4 : 0);
}

// The parameters of one run on a cluster of CS blocks; false when a block
// would own too few cells for the boundary rules.
bool fill_run1d(Run1D &p, double *S, const double *bx, const double *bxm, const Loop1D &opt,
                int ix, const Axis &ax, const Phys &ph, const BcTable &bc, Ctl *ctl,
                int max_steps, int fixed, double dt_fixed, int start, int CS) {
  p = Run1D{};
  p.S = S; p.bx = bx; p.bxm = bxm; p.ax = ax; p.ph = ph; p.bc = bc; p.ctl = ctl;
  p.bg = opt.bg;
  p.trq = fixed ? nullptr : opt.trq;
  p.trq0 = opt.trq0;
  p.seed = opt.seed;
  p.floor = opt.floor;
  p.chk = fixed ? 0 : opt.chk;
  p.ix = ix;
  p.q = (ix - 2) / CS;
  p.rem = (ix - 2) % CS;
  p.lmax = p.q + 3;
  p.max_steps = max_steps;
  p.fixed = fixed;
  p.dt_fixed = dt_fixed;
  p.start = start;
  // each block must own at least margin+1 cells for the boundary rules
  if (p.q < bc.margin + 1) return false;
  // a face rule reads at most 2*margin cells in from its end of the line
  // (bdsmp*: cell b+margin); block 0 and the last block own at least q cells
  p.bnd_local = 2 * bc.margin <= p.q ? 1 : 0;
  for (int v = 0; v < NV1; v++)
    for (int f = 0; f < 2; f++)
      if (bc.kind[v][f] == BD_PER) p.bnd_local = 0;
  return true;
}
}  // namespace

// Host launcher: the cluster kernel over a state of 5 arrays of ix doubles,
// updated in place.
cudaError_t launch_mlw1d(bool exact, double *S, const double *bx,
                         const double *bxm, const Loop1D &opt, int ix,
                         const Axis &ax, const Phys &ph, const BcTable &bc,
                         Ctl *ctl, int max_steps, int fixed, double dt_fixed,
                         int start, cudaStream_t s, bool dfp) {
  if (ix < mlw1d_min_cells() || (dfp && exact)) return cudaErrorInvalidValue;
  const bool bgv = opt.bg != nullptr;
  // the torque reads the rr profile; the floor counts into the control block
  if ((opt.trq && !bgv) || (opt.chk && !ctl && !fixed)) return cudaErrorInvalidValue;
  void (*kern)(Run1D) =
      pick1d(exact, bgv, dfp, k_mlw1d<true, false, false>, k_mlw1d<true, true, false>,
             k_mlw1d<false, false, false>, k_mlw1d<false, true, false>,
             k_mlw1d<false, false, true>, k_mlw1d<false, true, true>);
  const size_t per_cell = per_cell_doubles(bgv, dfp);
  // shared memory of the largest block the grid can have (16 blocks)
  const size_t smem_probe = sizeof(double) * (per_cell * ((ix - 2) / 16 + 4) + 64 + 32);
  const int CS = cluster_for(ix, cluster_max(kern, smem_probe));
  Run1D p;
  if (!fill_run1d(p, S, bx, bxm, opt, ix, ax, ph, bc, ctl, max_steps, fixed, dt_fixed, start,
                  CS))
    return cudaErrorInvalidValue;
  const size_t smem = sizeof(double) * (per_cell * p.lmax + 4 * CS + 32);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  if (CS > 8) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  // one thread per cell of the block's segment (whole warps, 256 at most):
  // threads without a cell would only wait at the barriers of every stage
  int nt = ((p.lmax + 31) / 32) * 32;
  nt = nt < 32 ? 32 : (nt > 256 ? 256 : nt);
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(CS, 1, 1);
  cfg.blockDim = dim3(nt, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, kern, p);
  count_launch();
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Host launcher of a group of runs (k_mlw1d_group): every run gets a cluster
// of the same size CS, at first the smallest power of two (at most 8) that
// leaves each block of every run at most 256 interior cells (a thread per
// cell, the two halo cells of a full block taken in a second pass), two
// blocks per SM.  A group too small to cover the SMs with one block each then
// takes larger clusters: 1024-cell runs step in 17 us on 8 SMs against 30 us
// on 4 (CS doubles while the grid stays within one block per SM and every
// block keeps 32 cells).  The runs' parameters go to the device in one
// stream-ordered allocation.  All runs share exact and the BG variant.
cudaError_t launch_mlw1d_group(bool exact, bool bgv, const Run1DArgs *runs, int nruns,
                               int max_steps, cudaStream_t s, bool dfp) {
  if (nruns < 1 || (dfp && exact)) return cudaErrorInvalidValue;
  int ixmax = 0, ixmin = 1 << 30;
  for (int k = 0; k < nruns; k++) {
    const Run1DArgs &a = runs[k];
    if (a.ix < mlw1d_min_cells() || !a.ctl) return cudaErrorInvalidValue;
    if ((a.opt.bg != nullptr) != bgv || (a.opt.trq && !bgv)) return cudaErrorInvalidValue;
    ixmax = a.ix > ixmax ? a.ix : ixmax;
    ixmin = a.ix < ixmin ? a.ix : ixmin;
  }
  int CS = 1;
  while (CS < 8 && (ixmax - 2 + CS - 1) / CS > 256) CS <<= 1;
  int devno = 0, nsm = 0;
  cudaError_t e = cudaGetDevice(&devno);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, devno);
  if (e != cudaSuccess) return e;
  while (CS < 8 && 2LL * CS * nruns <= nsm && (ixmin - 2) / (2 * CS) >= 32) CS <<= 1;
  std::vector<Run1D> host((size_t)nruns);
  int lmax = 0;
  for (int k = 0; k < nruns; k++) {
    const Run1DArgs &a = runs[k];
    if (!fill_run1d(host[k], a.S, a.bx, a.bxm, a.opt, a.ix, a.ax, a.ph, a.bc, a.ctl,
                    max_steps, 0, 0.0, 0, CS) ||
        host[k].q < 4)
      return cudaErrorInvalidValue;
    lmax = host[k].lmax > lmax ? host[k].lmax : lmax;
  }
  void (*kern)(const Run1D *) =
      pick1d(exact, bgv, dfp, k_mlw1d_group<true, false, false>,
             k_mlw1d_group<true, true, false>, k_mlw1d_group<false, false, false>,
             k_mlw1d_group<false, true, false>, k_mlw1d_group<false, false, true>,
             k_mlw1d_group<false, true, true>);
  const size_t smem = sizeof(double) * (per_cell_doubles(bgv, dfp) * lmax + 4 * CS + 32);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  Run1D *dev = nullptr;
  const size_t bytes = sizeof(Run1D) * (size_t)nruns;
  if ((e = cudaMallocAsync((void **)&dev, bytes, s)) != cudaSuccess) return e;
  // from pageable memory: the call returns once the bytes are staged, so the
  // host vector may go
  if ((e = cudaMemcpyAsync(dev, host.data(), bytes, cudaMemcpyHostToDevice, s)) !=
      cudaSuccess) {
    cudaFreeAsync(dev, s);
    return e;
  }
  const int ntmax = dfp ? 288 : 256;  // the kernel's launch bound
  int nt = ((lmax + 31) / 32) * 32;
  nt = nt < 32 ? 32 : (nt > ntmax ? ntmax : nt);
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)(CS * nruns), 1, 1);
  cfg.blockDim = dim3(nt, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, kern, (const Run1D *)dev);
  count_launch();
  const cudaError_t e2 = cudaFreeAsync(dev, s);
  if (e != cudaSuccess) return e;
  if (e2 != cudaSuccess) return e2;
  return cudaGetLastError();
}

// Standalone 1-D CFL (cfl_m.f:42-71) on interior cells, one block.
template <bool E>
__global__ void k_cfl1d(const double *S, const double *bx, int ix, Axis ax,
                        Phys ph, double safety, unsigned long long *out) {
  using FT = F<E>;
  __shared__ double red[32];
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  const FT gm(ph.gm), pi4i(ph.pi4i);
  for (int g = 1 + threadIdx.x; g <= ix - 2; g += blockDim.x) {
    const FT ro(S[g]), pr(S[(size_t)ix + g]), vx(S[2 * (size_t)ix + g]),
        by(S[4 * (size_t)ix + g]), b(bx[g]);
    const FT onero = 1.0 / ro;
    const FT ca2 = (b * b + by * by) * pi4i * onero;
    const FT cs2 = gm * pr * onero;
    const FT dtcfl = FT(ax.d[g]) / (fabs_(vx) + fsqrt(cs2 + ca2));
    const double dtq = (FT(safety) * dtcfl).v;
    if (dtq < dmin) dmin = dtq;
  }
  block_min_to(out, dmin, red, threadIdx.x, blockDim.x);
}

cudaError_t launch_cfl1d(bool exact, const double *S, const double *bx, int ix,
                         const Axis &ax, const Phys &ph, double safety,
                         unsigned long long *out, cudaStream_t s) {
  if (exact) k_cfl1d<true><<<1, 256, 0, s>>>(S, bx, ix, ax, ph, safety, out);
  else k_cfl1d<false><<<1, 256, 0, s>>>(S, bx, ix, ax, ph, safety, out);
  count_launch();
  return cudaGetLastError();
}

}  // namespace cans

namespace cans {

// chkdav on one array pair (the drop-in entry point); grid-stride loop,
// one atomic per block for the count.
__global__ void k_chkdav(double *da, double *vx, double floor, size_t n,
                         unsigned long long *count) {
  __shared__ unsigned int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  unsigned int mine = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    if (da[i] < floor) {
      da[i] = floor;
      vx[i] = 0.0;
      mine++;
    }
  }
  if (mine) atomicAdd(&cnt, mine);
  __syncthreads();
  if (threadIdx.x == 0 && cnt) atomicAdd(count, (unsigned long long)cnt);
}

// chkdav of the 2-D and 3-D model packages (cans2d/common/chkdav.f:33-44,
// cans3d/common/chkdav.f): where da < floor, da = floor and the velocity
// components vel[0..nv-1] are set to zero.  With ctl the arrays are slots of
// the state the step just wrote (da = slot a[0], then a[1]; velocities at
// slots v0..), and the kernel is a no-op once the loop is done or paused.
__global__ void k_chkdav_nd(double *S, size_t n, int na, int a0, int a1, int nv, int v0,
                            double floor, const Ctl *ctl, unsigned long long *count) {
  __shared__ unsigned int cnt;
  if (ctl != nullptr) {
    if (ctl->done | ctl->pause) return;
    S = ctl->buf[ctl->cur ^ 1];
  }
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  unsigned int mine = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
#pragma unroll 1
    for (int q = 0; q < na; q++) {  // chkdav of ro, then of pr
      double *da = S + (size_t)(q == 0 ? a0 : a1) * n;
      if (da[i] < floor) {
        da[i] = floor;
#pragma unroll 1
        for (int v = 0; v < nv; v++) S[(size_t)(v0 + v) * n + i] = 0.0;
        mine++;
      }
    }
  }
  if (mine) atomicAdd(&cnt, mine);
  __syncthreads();
  if (threadIdx.x == 0 && cnt) atomicAdd(count, (unsigned long long)cnt);
}

cudaError_t launch_chkdav_nd(double *S, size_t n, int na, int a0, int a1, int nv, int v0,
                             double floor, const Ctl *ctl, unsigned long long *count,
                             cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int threads = 256;
  const size_t want = (n + threads - 1) / threads;
  const int blocks = (int)(want < 1216 ? want : 1216);
  k_chkdav_nd<<<blocks, threads, 0, s>>>(S, n, na, a0, a1, nv, v0, floor, ctl, count);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_chkdav(double *da, double *vx, double floor, size_t n,
                          unsigned long long *count, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int threads = 256;
  const size_t want = (n + threads - 1) / threads;
  const int blocks = (int)(want < 1216 ? want : 1216);  // 8 blocks per SM at most
  k_chkdav<<<blocks, threads, 0, s>>>(da, vx, floor, n, count);
  count_launch();
  return cudaGetLastError();
}

}  // namespace cans
