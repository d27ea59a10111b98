// HLLD step of the cansxx engine (sm_103a, FP64): engine.f:2-73 with its two
// hlld_mh stages (hlld_mh.f:2-127) as four kernels over one thread per cell,
// in Heaviside units with permeability mu.
//
//   k_hlld_flux<1>    first-order face states (inp_const), bb = face average
//                     of the normal field, HLLD flux of the faces (c, c+e_a)
//                     of every active axis
//   k_hlld_update     U - dt/2 (F(c) - F(c-e_a))/d_a on 2..n-1 of each
//                     active axis (adddfdx.f:18-46), half-step primitives of
//                     every cell (rvtovv, ee2eh, eh2pr)
//   k_hlld_flux<2>    minmod face states of the half-step primitives
//                     (inp_tvdminmod.f, first order at both ends), HLLD flux
//   k_hlld_update     U - dt (...) from the conserved variables of the input
//                     state, primitives of the new state
//   k_hlld_finish     after the boundary fill: CFL of every cell and the end
//                     of the loop iteration (resident runs only)
//
// The normal-field flux of an axis is zero (hlld_mh.f:74,91,108), so that
// component is not updated in its own pass.
//
// The double-float policy (QF) evaluates the face flux in double-float
// arithmetic on the FP32 pipes, and a face whose star state is
// ill-conditioned for it (hlld_flux_t) in FP64; face states, updates and
// primitives stay FP64.
#include <cuda_runtime.h>

#include <cmath>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "cfl3.cuh"
#include "hlld_flux.cuh"

namespace cans {

namespace {

constexpr int kThreads = 128;
enum { U_RO = 0, U_EE = 1, U_RX = 2, U_BX = 5 };

struct Geo {
  int n3[3];
  size_t st[3];
  size_t n;
  int act[3];  // mfdim: 1 = active axis
};

__device__ __forceinline__ void cell_index(const Geo &g, size_t c, int &i,
                                           int &j, int &k) {
  const size_t plane = g.st[2];
  k = (int)(c / plane);
  const size_t r = c - (size_t)k * plane;
  j = (int)(r / (size_t)g.n3[0]);
  i = (int)(r - (size_t)j * g.n3[0]);
}
template <typename V>
__device__ __forceinline__ V pick3(int idx, V x, V y, V z) {
  return idx == 0 ? x : (idx == 1 ? y : z);
}
__device__ __forceinline__ int rot(int a, int m) {
  const int r = a + m;
  return r >= 3 ? r - 3 : r;
}

// Conserved variables of a primitive state: vvtorv, pr2eh, eh2ee.
template <bool E>
__device__ __forceinline__ void to_conserved(const double *p, double gm1,
                                             double gm1i, double mu2, F<E> *u) {
  using T = F<E>;
  const T ro(p[P3::RO]), pr(p[P3::PR]), vx(p[P3::VX]), vy(p[P3::VY]),
      vz(p[P3::VZ]), bx(p[P3::BX]), by(p[P3::BY]), bz(p[P3::BZ]);
  T eh;
  if constexpr (E) eh = pr / T(gm1);
  else eh = pr * T(gm1i);
  const T ek = (vx * vx + vy * vy + vz * vz) * ro / T(2.0);
  const T em = (bx * bx + by * by + bz * bz) / T(mu2);
  u[U_RO] = ro;
  u[U_EE] = eh + ek + em;
  u[U_RX] = vx * ro;
  u[U_RX + 1] = vy * ro;
  u[U_RX + 2] = vz * ro;
  u[U_BX] = bx;
  u[U_BX + 1] = by;
  u[U_BX + 2] = bz;
}

// Primitive variables of a conserved state: rvtovv, ee2eh, eh2pr.
template <bool E>
__device__ __forceinline__ void to_primitive(const F<E> *u, double gm1, double mu2,
                                             double *p) {
  using T = F<E>;
  const T ro = u[U_RO];
  T vx, vy, vz;
  if constexpr (E) {
    vx = u[U_RX] / ro;
    vy = u[U_RX + 1] / ro;
    vz = u[U_RX + 2] / ro;
  } else {
    const T roi = T(1.0) / ro;
    vx = u[U_RX] * roi;
    vy = u[U_RX + 1] * roi;
    vz = u[U_RX + 2] * roi;
  }
  const T ek = (vx * vx + vy * vy + vz * vz) * ro / T(2.0);
  const T em = (u[U_BX] * u[U_BX] + u[U_BX + 1] * u[U_BX + 1] + u[U_BX + 2] * u[U_BX + 2]) /
               T(mu2);
  const T eh = u[U_EE] - ek - em;
  p[P3::RO] = ro.v;
  p[P3::PR] = (T(gm1) * eh).v;
  p[P3::VX] = vx.v;
  p[P3::VY] = vy.v;
  p[P3::VZ] = vz.v;
  p[P3::BX] = u[U_BX].v;
  p[P3::BY] = u[U_BX + 1].v;
  p[P3::BZ] = u[U_BX + 2].v;
}

// The double-float policy's forecast of a face the double-float flux would
// hand to FP64 (hlld_flux_t's test of the star-state denominators): the
// field of both face states within about 1/32 of the face normal and the
// normal field's pressure above about a sixteenth of the gas pressure, the
// c_f = c_a degeneracy.  Judged on the exponent fields with integer
// operations.  When every active lane of a warp forecasts it, the warp takes
// the FP64 flux directly; a warp with any other face takes the double-float
// flux with its own test, so that no warp pays for both paths on a forecast
// alone.
__device__ __forceinline__ int exp_field(double x) {
  return (__double2hiint(x) >> 20) & 0x7ff;
}
__device__ __forceinline__ bool near_degenerate(const double *L, const double *R, double bn) {
  const int en = exp_field(bn);
  const int et = max(max(exp_field(L[6]), exp_field(L[7])), max(exp_field(R[6]), exp_field(R[7])));
  const int ep = max(exp_field(L[1]), exp_field(R[1]));
  return en > 0 && et + 6 <= en && 2 * en - 1019 >= ep;
}

// minmod of the fast policy (flmt of inp_tvdminmod.f:118 up to the sign of a
// zero result)
__device__ __forceinline__ double minmod(double a, double b) {
  const long long x = __double_as_longlong(a) ^ __double_as_longlong(b);
  return x >= 0 ? copysign(fmin(fabs(a), fabs(b)), a) : 0.0;
}

template <bool E, int STAGE, bool QF>
__global__ void __launch_bounds__(kThreads)
    k_hlld_flux(const double *__restrict__ P, double *__restrict__ Fl, Geo g,
                HlldK K, const Ctl *ctl) {
  if (ctl) {
    if (ctl->done | ctl->pause) return;
    if (STAGE == 1) P = ctl->buf[ctl->cur];
  }
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= g.n) return;
  int i, j, k;
  cell_index(g, c, i, j, k);
  using T = F<E>;
#pragma unroll 1
  for (int a = 0; a < 3; a++) {
    const int na = pick3(a, g.n3[0], g.n3[1], g.n3[2]);
    const int ca = pick3(a, i, j, k);
    if (!pick3(a, g.act[0], g.act[1], g.act[2]) || ca > na - 2) continue;
    const size_t s = pick3(a, g.st[0], g.st[1], g.st[2]);
    const bool first = STAGE == 1 || ca == 0 || ca == na - 2;
    double wl[8], wr[8];
#pragma unroll
    for (int v = 0; v < 8; v++) {
      const double *h = P + v * g.n + c;
      const double d0 = __ldg(h), d1 = __ldg(h + s);
      if (first) {
        wl[v] = d0;
        wr[v] = d1;
      } else {
        const double dm = __ldg(h - s), d2 = __ldg(h + 2 * s);
        if constexpr (E) {
          const T t0(d0), t1(d1);
          wl[v] = (t0 + T(0.5) * flmt(t0 - T(dm), t1 - t0)).v;
          wr[v] = (t1 - T(0.5) * flmt(T(d2) - t1, t1 - t0)).v;
        } else {
          const double gc = d1 - d0;
          wl[v] = fma(0.5, minmod(d0 - dm, gc), d0);
          wr[v] = fma(-0.5, minmod(d2 - d1, gc), d1);
        }
      }
    }
    double L[8], R[8], f[7];
    L[0] = wl[P3::RO];
    L[1] = wl[P3::PR];
    R[0] = wr[P3::RO];
    R[1] = wr[P3::PR];
#pragma unroll
    for (int m = 0; m < 3; m++) {
      const int r = rot(a, m);
      L[2 + m] = pick3(r, wl[P3::VX], wl[P3::VY], wl[P3::VZ]);
      L[5 + m] = pick3(r, wl[P3::BX], wl[P3::BY], wl[P3::BZ]);
      R[2 + m] = pick3(r, wr[P3::VX], wr[P3::VY], wr[P3::VZ]);
      R[5 + m] = pick3(r, wr[P3::BX], wr[P3::BY], wr[P3::BZ]);
    }
    // bb: the cell-centred normal field of the stage input averaged onto the face
    const double *bn = P + (P3::BX + a) * g.n + c;
    const double bb = ((T(__ldg(bn)) + T(__ldg(bn + s))) / T(2.0)).v;
    if constexpr (QF) {
      bool ill = __all_sync(__activemask(), near_degenerate(L, R, bb));
      if (!ill) hlld_flux_t<df::DF>(K, L, R, bb, f, &ill);
      if (ill) hlld_flux<false>(K, L, R, bb, f);  // ill-conditioned: FP64
    } else {
      hlld_flux<E>(K, L, R, bb, f);
    }
    double *Fa = Fl + (size_t)a * 8 * g.n;
    Fa[U_RO * g.n + c] = f[0];
    Fa[U_EE * g.n + c] = f[1];
#pragma unroll
    for (int m = 0; m < 3; m++) Fa[(U_RX + rot(a, m)) * g.n + c] = f[2 + m];
    Fa[(U_BX + rot(a, 1)) * g.n + c] = f[5];
    Fa[(U_BX + rot(a, 2)) * g.n + c] = f[6];
  }
}

// One stage update from the conserved variables of the primitive state A;
// writes the primitives of the result to B.  STAGE 1 uses dt/2.
template <bool E, int STAGE>
__global__ void __launch_bounds__(kThreads)
    k_hlld_update(const double *__restrict__ A, const double *__restrict__ Fl,
                  double *__restrict__ B, Geo g, Axis ax, Axis ay, Axis az,
                  HlldK K, double mu2, double dt, const Ctl *ctl) {
  if (ctl) {
    if (ctl->done | ctl->pause) return;
    A = ctl->buf[ctl->cur];
    if (STAGE == 2) B = ctl->buf[ctl->cur ^ 1];
    dt = ctl->dt;
  }
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= g.n) return;
  int i, j, k;
  cell_index(g, c, i, j, k);
  using T = F<E>;
  double p[8];
#pragma unroll
  for (int v = 0; v < 8; v++) p[v] = __ldg(A + v * g.n + c);
  T u[8];
  to_conserved<E>(p, K.gm1, K.gm1i, mu2, u);
  const T dts = STAGE == 1 ? T(0.5) * T(dt) : T(dt);
#pragma unroll 1
  for (int a = 0; a < 3; a++) {
    const int na = pick3(a, g.n3[0], g.n3[1], g.n3[2]);
    const int ca = pick3(a, i, j, k);
    if (!pick3(a, g.act[0], g.act[1], g.act[2]) || ca < 1 || ca > na - 2) continue;
    const size_t s = pick3(a, g.st[0], g.st[1], g.st[2]);
    const double *pd = pick3(a, ax.d, ay.d, az.d);
    const double *pdi = pick3(a, ax.di, ay.di, az.di);
    const double *Fa = Fl + (size_t)a * 8 * g.n;
#pragma unroll
    for (int v = 0; v < 8; v++) {
      if (v == U_BX + a) continue;
      const T f0(__ldg(Fa + v * g.n + c)), fm(__ldg(Fa + v * g.n + c - s));
      if constexpr (E) u[v] = u[v] - dts * ((f0 - fm) / T(pd[ca]));
      else u[v] = u[v] - dts * ((f0 - fm) * T(pdi[ca]));
    }
  }
  to_primitive<E>(u, K.gm1, mu2, p);
#pragma unroll
  for (int v = 0; v < 8; v++) B[v * g.n + c] = p[v];
}

// CFL (cans3d/common/cfl_m.f) of every cell of the new state after the
// boundary fill, then the end of the loop iteration by the last block.
template <bool E>
__global__ void k_hlld_finish(Geo g, Axis ax, Axis ay, Axis az, Phys ph, Ctl *ctl) {
  __shared__ double red[32];
  if (ctl->done | ctl->pause) return;
  const double *S = ctl->buf[ctl->cur ^ 1];
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  bool bad = false;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.n;
       c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_index(g, c, i, j, k);
    const double d = cfl3_cell<E>(S, g.n, c, i, j, k, ax, ay, az, ph, ctl->safety);
    if (d < dmin) dmin = d;
    bad |= bad_cell(S[P3::RO * g.n + c], S[P3::PR * g.n + c], d);
  }
  count_bad_block(bad, &ctl->nonfinite, threadIdx.x);
  block_min_to(&ctl->cfl_bits, dmin, red, threadIdx.x, blockDim.x);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(&ctl->frame_blocks_done, 1u);
    if (prev == gridDim.x - 1) {
      __threadfence();
      finish_iteration(ctl);
    }
  }
}

Geo make_geo(int ix, int jx, int kx, const int *mfdim) {
  Geo g{};
  g.n3[0] = ix;
  g.n3[1] = jx;
  g.n3[2] = kx;
  g.st[0] = 1;
  g.st[1] = (size_t)ix;
  g.st[2] = (size_t)ix * jx;
  g.n = g.st[2] * kx;
  for (int a = 0; a < 3; a++) g.act[a] = mfdim[a] == 1 ? 1 : 0;
  return g;
}

template <bool E, bool QF>
cudaError_t launch_all(const double *A, double *B, double *scratch, const Geo &g,
                       const Axis &ax, const Axis &ay, const Axis &az,
                       const HlldK &K, double mu2, double dt, const Ctl *ctl,
                       cudaStream_t s) {
  const unsigned blocks = (unsigned)((g.n + kThreads - 1) / kThreads);
  double *H = scratch, *Fl = scratch + 8 * g.n;
  k_hlld_flux<E, 1, QF><<<blocks, kThreads, 0, s>>>(A, Fl, g, K, ctl);
  k_hlld_update<E, 1><<<blocks, kThreads, 0, s>>>(A, Fl, H, g, ax, ay, az, K, mu2, dt, ctl);
  k_hlld_flux<E, 2, QF><<<blocks, kThreads, 0, s>>>(H, Fl, g, K, ctl);
  k_hlld_update<E, 2><<<blocks, kThreads, 0, s>>>(A, Fl, B, g, ax, ay, az, K, mu2, dt, ctl);
  count_launch(4);
  return cudaGetLastError();
}

}  // namespace

size_t hlld3d_scratch_doubles(size_t ncells) { return 32 * ncells; }

cudaError_t launch_hlld3d(bool exact, const double *A, double *B, double *scratch,
                          int ix, int jx, int kx, const int *mfdim, const Axis &ax,
                          const Axis &ay, const Axis &az, double gm, double mu,
                          double dt, const Ctl *ctl, cudaStream_t s, bool df) {
  const Geo g = make_geo(ix, jx, kx, mfdim);
  HlldK K{};
  K.gm = gm;
  K.gm1 = gm - 1.0;
  K.zfloor = 1.0e-10;
  K.gm1i = 1.0 / (gm - 1.0);
  const double mu2 = 2.0 * mu;
  if (exact) return launch_all<true, false>(A, B, scratch, g, ax, ay, az, K, mu2, dt, ctl, s);
  if (df) return launch_all<false, true>(A, B, scratch, g, ax, ay, az, K, mu2, dt, ctl, s);
  return launch_all<false, false>(A, B, scratch, g, ax, ay, az, K, mu2, dt, ctl, s);
}

cudaError_t launch_hlld3d_finish(bool exact, int ix, int jx, int kx,
                                 const Axis &ax, const Axis &ay, const Axis &az,
                                 const Phys &ph, Ctl *ctl, cudaStream_t s) {
  const int mf[3] = {1, 1, 1};
  const Geo g = make_geo(ix, jx, kx, mf);
  int blocks = (int)((g.n + 255) / 256);
  if (blocks < 1) blocks = 1;
  if (blocks > 152 * 4) blocks = 152 * 4;
  if (exact) k_hlld_finish<true><<<blocks, 256, 0, s>>>(g, ax, ay, az, ph, ctl);
  else k_hlld_finish<false><<<blocks, 256, 0, s>>>(g, ax, ay, az, ph, ctl);
  count_launch();
  return cudaGetLastError();
}

}  // namespace cans
