// 3-D Roe-MUSCL step (sm_103a, FP64): the two stages of
// cans3d/hdroe/roe_m.f:2-340 as four kernels over one thread per cell.
//
//   k_roe_flux1  first-order Roe fluxes of the faces (c, c+e_a), a = x,y,z
//                (roe_m.f:73-97, 123-147, 173-197)
//   k_roe_half   dt/2 update of the conserved variables on 2..n-1 and the
//                half-step primitives (roe_m.f:39-68, 99-118, 149-168,
//                199-233)
//   k_roe_flux2  minmod states of the half-step primitives and the Roe fluxes
//                of the faces the full update reads (roe_m.f:241-251,
//                269-279, 297-307; tvdminmod.f:18-55)
//   k_roe_full   dt update on 3..n-2, primitives, copy of the other cells,
//                CFL of the cells the boundary fill keeps (roe_m.f:253-336)
//
// Every face flux is evaluated once per stage (3 faces per cell) and kept in
// HBM between the flux and the update kernels; the step is bound by the FP64
// pipe, not by these 32 x 8 B per cell of scratch traffic.
//
// The same kernels with ND = 2 are the 2-D roe_m3 (cans2d/hdroe/roe_m3.f:
// 1-204), which differs from the 3-D step in four places: the y faces swap
// x and y (roe_m3.f:106-107) instead of rotating cyclically, the flux is
// roeflux_m3.f (alphs without the 3-D fix, roe_flux.cuh), the minmod
// arguments come in the order of cans2d/hdroe/tvdminmod.f:14-33, and the
// update also advances az with the half-step E_z (roe_m3.f:185-191).
//
// The reference leaves the half-step prh, vxh, vyh, vzh unset on the outer
// cell layer (index 1 or n) and the minmod states of the faces 2 and n-2
// read it; here that layer holds the input primitives of the cell.  Only
// cells with an index 3 or n-2 -- boundary cells at margin 3 -- depend on it.
// The 2-D md_mhdkh Roe package runs with margin 2 (cans2d/md_mhdkh/hdroe/
// main.f:5), where those are the first interior cells: the reference result
// there depends on stack contents, and here on the input primitives.
#include <cuda_runtime.h>

#include <cmath>

#include "cans_common.cuh"
#include "cans_internal.h"
#include "cfl3.cuh"
#include "roe_flux.cuh"

namespace cans {

namespace {

constexpr int kRoeThreads = 128;

// conserved-variable slots of the face-flux arrays (8 per axis; the slot of
// the normal field component of an axis is never written nor read)
enum { U_RO = 0, U_EE = 1, U_RX = 2, U_BX = 5 };

struct Geo {
  int n3[3];
  size_t st[3];
  size_t n;
};

__device__ __forceinline__ void cell_index(const Geo &g, size_t c, int &i,
                                           int &j, int &k) {
  const size_t plane = g.st[2];
  k = (int)(c / plane);
  const size_t r = c - (size_t)k * plane;
  j = (int)(r / (size_t)g.n3[0]);
  i = (int)(r - (size_t)j * g.n3[0]);
}

// Component `idx` of a triple, by selects (no local-memory indexing).
template <typename V>
__device__ __forceinline__ V pick3(int idx, V x, V y, V z) {
  return idx == 0 ? x : (idx == 1 ? y : z);
}

// Frame of axis a: component m (0 normal, 1, 2 tangential) is the
// Cartesian component rot(a, m).  3-D: (a+m) mod 3, the cyclic rotation of
// roe_m.f:96,146,196.  2-D: the y faces swap x and y and keep z
// (roe_m3.f:106-107).
template <int ND>
__device__ __forceinline__ int rot(int a, int m) {
  if constexpr (ND == 3) {
    const int r = a + m;
    return r >= 3 ? r - 3 : r;
  } else {
    return a == 0 ? m : (m == 0 ? 1 : (m == 1 ? 0 : 2));
  }
}

// face states (ro, pr, v[3], b[3]) in the frame of axis a
template <int ND>
__device__ __forceinline__ void to_frame(int a, const double *p, double *w) {
  w[0] = p[P3::RO];
  w[1] = p[P3::PR];
#pragma unroll
  for (int m = 0; m < 3; m++) {
    const int r = rot<ND>(a, m);
    w[2 + m] = pick3(r, p[P3::VX], p[P3::VY], p[P3::VZ]);
    w[5 + m] = pick3(r, p[P3::BX], p[P3::BY], p[P3::BZ]);
  }
}

// flux of the frame (ro, ee, rn, rt1, rt2, bt1, bt2) into the conserved slots
template <int ND>
__device__ __forceinline__ void store_flux(double *__restrict__ Fa, size_t n,
                                           size_t c, int a, const double *f) {
  Fa[U_RO * n + c] = f[0];
  Fa[U_EE * n + c] = f[1];
#pragma unroll
  for (int m = 0; m < 3; m++) Fa[(U_RX + rot<ND>(a, m)) * n + c] = f[2 + m];
  Fa[(U_BX + rot<ND>(a, 1)) * n + c] = f[5];
  Fa[(U_BX + rot<ND>(a, 2)) * n + c] = f[6];
}

// Is the face (c, c + e_a) in the box: index along a in [alo, n_a - ahi],
// indices across a in [tlo, n_t - thi] (0-based)?  A 2-D grid has no z.
template <int ND>
__device__ __forceinline__ bool face_in(int i, int j, int k, const Geo &g, int a,
                                        int alo, int ahi, int tlo, int thi) {
  const int ia = pick3(a, i, j, k), na = pick3(a, g.n3[0], g.n3[1], g.n3[2]);
  bool ok = ia >= alo && ia <= na - ahi;
  if (a != 0) ok = ok && i >= tlo && i <= g.n3[0] - thi;
  if (a != 1) ok = ok && j >= tlo && j <= g.n3[1] - thi;
  if (ND == 3 && a != 2) ok = ok && k >= tlo && k <= g.n3[2] - thi;
  return ok;
}

// cells 1..n-2 / 2..n-3 (0-based) of every axis the grid has
template <int ND>
__device__ __forceinline__ bool in_range(const Geo &g, int i, int j, int k, int w) {
  bool ok = i >= w && i <= g.n3[0] - 1 - w && j >= w && j <= g.n3[1] - 1 - w;
  if (ND == 3) ok = ok && k >= w && k <= g.n3[2] - 1 - w;
  return ok;
}

__device__ __forceinline__ size_t stride(const Geo &g, int a) {
  return pick3(a, g.st[0], g.st[1], g.st[2]);
}

// 3-D: roeflux_m.f; 2-D: roeflux_m3.f (alphs without the fix)
// QF: the fast flux in double-float (the double-float policy; the update
// kernels stay FP64)
template <bool E, int ND, bool QF = false>
__device__ __forceinline__ void roe_flux(const RoeK &K, const double *L,
                                         const double *R, double *f) {
  if constexpr (E) roe_flux_ref<true, ND == 3>(K, L, R, f);
  else if constexpr (QF) roe_flux_df<ND == 3>(K, L, R, f);
  else roe_flux_fast<ND == 3>(K, L, R, f);
}

// minmod(a, b) of the fast policy: equal to flmt(a, b) of tvdminmod.f:15 up
// to the sign of a zero result; the sign test runs on the integer pipe.
__device__ __forceinline__ double minmod(double a, double b) {
  const long long x = __double_as_longlong(a) ^ __double_as_longlong(b);
  return x >= 0 ? copysign(fmin(fabs(a), fabs(b)), a) : 0.0;
}

// Conserved variables of a primitive state (roe_m.f:42-47).
template <bool E>
__device__ __forceinline__ void to_conserved(const RoeK &K, const double *p,
                                             F<E> *u) {
  using T = F<E>;
  const T ro(p[P3::RO]), pr(p[P3::PR]), vx(p[P3::VX]), vy(p[P3::VY]),
      vz(p[P3::VZ]), bx(p[P3::BX]), by(p[P3::BY]), bz(p[P3::BZ]);
  const T v2 = vx * vx + vy * vy + vz * vz;
  const T b2 = bx * bx + by * by + bz * bz;
  u[U_RO] = ro;
  if constexpr (E) u[U_EE] = pr / T(K.gm1) + T(0.5) * ro * v2 + T(K.pi8i) * b2;
  else u[U_EE] = pr * T(K.gm1i) + T(0.5) * ro * v2 + T(K.pi8i) * b2;
  u[U_RX] = ro * vx;
  u[U_RX + 1] = ro * vy;
  u[U_RX + 2] = ro * vz;
  u[U_BX] = bx;
  u[U_BX + 1] = by;
  u[U_BX + 2] = bz;
}

// Primitive variables of a conserved state (roe_m.f:225-230, 328-333).
template <bool E>
__device__ __forceinline__ void to_primitive(const RoeK &K, const F<E> *u,
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
  const T v2 = vx * vx + vy * vy + vz * vz;
  const T b2 = u[U_BX] * u[U_BX] + u[U_BX + 1] * u[U_BX + 1] + u[U_BX + 2] * u[U_BX + 2];
  const T pr = T(K.gm1) * (u[U_EE] - T(0.5) * ro * v2 - T(K.pi8i) * b2);
  p[P3::RO] = ro.v;
  p[P3::PR] = pr.v;
  p[P3::VX] = vx.v;
  p[P3::VY] = vy.v;
  p[P3::VZ] = vz.v;
  p[P3::BX] = u[U_BX].v;
  p[P3::BY] = u[U_BX + 1].v;
  p[P3::BZ] = u[U_BX + 2].v;
}

// u += fac * (F(c - e_a) - F(c)) / d_a for every conserved variable but the
// normal field component of the axis (roe_m.f:102-115 and the like).
template <bool E>
__device__ __forceinline__ void add_divergence(F<E> *u, const double *__restrict__ Fl,
                                               const Geo &g, size_t c, int a,
                                               double fac, double d, double di) {
  using T = F<E>;
  const double *Fa = Fl + (size_t)a * 8 * g.n;
  const size_t st = stride(g, a);
#pragma unroll
  for (int v = 0; v < 8; v++) {
    if (v == U_BX + a) continue;
    const T fm(__ldg(Fa + v * g.n + c - st)), f0(__ldg(Fa + v * g.n + c));
    if constexpr (E) u[v] = u[v] + T(fac) * ((fm - f0) / T(d));
    else u[v] = u[v] + T(fac) * ((fm - f0) * T(di));
  }
}

// spacing d(i) of axis a and its inverse at the cell (i, j, k)
__device__ __forceinline__ void axis_h(const Axis &ax, const Axis &ay,
                                       const Axis &az, int a, int i, int j,
                                       int k, double &d, double &di) {
  const double *pd = pick3(a, ax.d, ay.d, az.d);
  const double *pi = pick3(a, ax.di, ay.di, az.di);
  const int ii = pick3(a, i, j, k);
  d = pd[ii];
  di = pi[ii];
}

// ---- predictor --------------------------------------------------------------

template <bool E, int ND, bool QF = false>
__global__ void __launch_bounds__(kRoeThreads)
    k_roe_flux1(const double *__restrict__ A, double *__restrict__ Fl, Geo g,
                RoeK K, const Ctl *ctl) {
  if (ctl) {
    if (ctl->done | ctl->pause) return;
    A = ctl->buf[ctl->cur];
  }
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= g.n) return;
  int i, j, k;
  cell_index(g, c, i, j, k);
  double p0[8];
#pragma unroll
  for (int v = 0; v < 8; v++) p0[v] = __ldg(A + v * g.n + c);
#pragma unroll 1
  for (int a = 0; a < ND; a++) {
    // faces 1..n-1 along a (1-based) of the cells 2..n-1 across it: every
    // face the dt/2 update reads
    if (!face_in<ND>(i, j, k, g, a, 0, 2, 1, 2)) continue;
    const size_t st = stride(g, a);
    double p1[8], L[8], R[8], f[7];
#pragma unroll
    for (int v = 0; v < 8; v++) p1[v] = __ldg(A + v * g.n + c + st);
    to_frame<ND>(a, p0, L);
    to_frame<ND>(a, p1, R);
    roe_flux<E, ND, QF>(K, L, R, f);
    store_flux<ND>(Fl + (size_t)a * 8 * g.n, g.n, c, a, f);
  }
}

template <bool E, int ND>
__global__ void __launch_bounds__(kRoeThreads)
    k_roe_half(const double *__restrict__ A, const double *__restrict__ Fl,
               double *__restrict__ H, Geo g, Axis ax, Axis ay, Axis az, RoeK K,
               double dt, const Ctl *ctl) {
  if (ctl) {
    if (ctl->done | ctl->pause) return;
    A = ctl->buf[ctl->cur];
    dt = ctl->dt;
  }
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= g.n) return;
  int i, j, k;
  cell_index(g, c, i, j, k);
  double p[8];
#pragma unroll
  for (int v = 0; v < 8; v++) p[v] = __ldg(A + v * g.n + c);
  if (in_range<ND>(g, i, j, k, 1)) {
    F<E> u[8];
    to_conserved<E>(K, p, u);
    const double hdt = (F<E>(0.5) * F<E>(dt)).v;
#pragma unroll 1
    for (int a = 0; a < ND; a++) {
      double d, di;
      axis_h(ax, ay, az, a, i, j, k, d, di);
      add_divergence<E>(u, Fl, g, c, a, hdt, d, di);
    }
    to_primitive<E>(K, u, p);
  }
#pragma unroll
  for (int v = 0; v < 8; v++) H[v * g.n + c] = p[v];
}

// ---- corrector --------------------------------------------------------------

template <bool E, int ND, bool QF = false>
__global__ void __launch_bounds__(kRoeThreads)
    k_roe_flux2(const double *__restrict__ H, double *__restrict__ Fl, Geo g,
                RoeK K, const Ctl *ctl) {
  if (ctl && (ctl->done | ctl->pause)) return;
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= g.n) return;
  int i, j, k;
  cell_index(g, c, i, j, k);
  using T = F<E>;
#pragma unroll 1
  for (int a = 0; a < ND; a++) {
    // faces 2..n-2 along a (1-based) of the cells 3..n-2 across it: every
    // face the dt update reads
    if (!face_in<ND>(i, j, k, g, a, 1, 3, 2, 3)) continue;
    const size_t s = stride(g, a);
    double wl[8], wr[8], L[8], R[8], f[7];
#pragma unroll
    for (int v = 0; v < 8; v++) {
      const double *h = H + v * g.n + c;
      const T dm(__ldg(h - s)), d0(__ldg(h)), d1(__ldg(h + s)), d2(__ldg(h + 2 * s));
      if constexpr (E && ND == 3) {  // cans3d/hdroe/tvdminmod.f:22-25
        wl[v] = (d0 + T(0.5) * flmt(d0 - dm, d1 - d0)).v;
        wr[v] = (d1 - T(0.5) * flmt(d2 - d1, d1 - d0)).v;
      } else if constexpr (E) {      // cans2d/hdroe/tvdminmod.f:16-19
        wl[v] = (d0 + T(0.5) * flmt(d1 - d0, d0 - dm)).v;
        wr[v] = (d1 - T(0.5) * flmt(d1 - d0, d2 - d1)).v;
      } else {
        const double gl = d0.v - dm.v, gc = d1.v - d0.v, gr = d2.v - d1.v;
        wl[v] = fma(0.5, minmod(gl, gc), d0.v);
        wr[v] = fma(-0.5, minmod(gr, gc), d1.v);
      }
    }
    to_frame<ND>(a, wl, L);
    to_frame<ND>(a, wr, R);
    roe_flux<E, ND, QF>(K, L, R, f);
    store_flux<ND>(Fl + (size_t)a * 8 * g.n, g.n, c, a, f);
  }
}

// Per-cell CFL time step of the 2-D step (cans2d/common/cfl_m3.f:46-55), the
// expression the 2-D mLW kernels and the frame kernel reduce.
template <bool E>
__device__ __forceinline__ double cfl2_cell(const double *__restrict__ S, size_t n,
                                            size_t g, int i, int j, const Axis &ax,
                                            const Axis &ay, const Phys &ph,
                                            double safety) {
  using FT = F<E>;
  const FT ro(S[P3::RO * n + g]), pr(S[P3::PR * n + g]);
  const FT vx(S[P3::VX * n + g]), vy(S[P3::VY * n + g]), vz(S[P3::VZ * n + g]);
  const FT bx(S[P3::BX * n + g]), by(S[P3::BY * n + g]), bz(S[P3::BZ * n + g]);
  const FT b2 = bx * bx + by * by + bz * bz;
  const FT v2 = vx * vx + vy * vy + vz * vz;
  const FT ca2 = b2 * FT(ph.pi4i) / ro;
  const FT cs2 = FT(ph.gm) * pr / ro;
  const FT dtcfl = fmin_(FT(ax.d[i]), FT(ay.d[j])) / fsqrt(v2 + cs2 + ca2);
  return (FT(safety) * dtcfl).v;
}

template <bool E, int ND>
__global__ void __launch_bounds__(kRoeThreads)
    k_roe_full(const double *__restrict__ A, const double *__restrict__ Fl,
               const double *__restrict__ H, double *__restrict__ B, Geo g,
               Axis ax, Axis ay, Axis az, RoeK K, Phys ph, double dt, Ctl *ctl,
               Box3 box) {
  __shared__ double red[kRoeThreads / 32];
  if (ctl) {
    if (ctl->done | ctl->pause) return;
    A = ctl->buf[ctl->cur];
    B = ctl->buf[ctl->cur ^ 1];
    dt = ctl->dt;
  }
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  bool bad = false;  // a cell of the new state the CFL cannot use
  if (c < g.n) {
    int i, j, k;
    cell_index(g, c, i, j, k);
    double p[8];
#pragma unroll
    for (int v = 0; v < 8; v++) p[v] = __ldg(A + v * g.n + c);
    const bool upd = in_range<ND>(g, i, j, k, 2);
    if (upd) {
      F<E> u[8];
      to_conserved<E>(K, p, u);
#pragma unroll 1
      for (int a = 0; a < ND; a++) {
        double d, di;
        axis_h(ax, ay, az, a, i, j, k, d, di);
        add_divergence<E>(u, Fl, g, c, a, dt, d, di);
      }
      to_primitive<E>(K, u, p);
    }
#pragma unroll
    for (int v = 0; v < 8; v++) B[v * g.n + c] = p[v];
    if constexpr (ND == 2) {
      // az += dt * (-E_z) of the half step (roe_m3.f:185-191)
      using T = F<E>;
      T az_(__ldg(A + 8 * g.n + c));
      if (upd) {
        const T vxh(__ldg(H + P3::VX * g.n + c)), vyh(__ldg(H + P3::VY * g.n + c));
        const T bxh(__ldg(H + P3::BX * g.n + c)), byh(__ldg(H + P3::BY * g.n + c));
        const T ez = -vxh * byh + vyh * bxh;
        const T saz = -ez;
        az_ = az_ + T(dt) * saz;
      }
      B[8 * g.n + c] = az_.v;
    }
    if (ctl && i >= box.lo[0] && i <= box.hi[0] && j >= box.lo[1] &&
        j <= box.hi[1] && k >= box.lo[2] && k <= box.hi[2]) {
      if constexpr (ND == 3)
        dmin = cfl3_cell<E>(B, g.n, c, i, j, k, ax, ay, az, ph, ctl->safety);
      else
        dmin = cfl2_cell<E>(B, g.n, c, i, j, ax, ay, ph, ctl->safety);
      bad = bad_cell(p[P3::RO], p[P3::PR], dmin);
    }
  }
  if (ctl) {
    count_bad_block(bad, &ctl->nonfinite, threadIdx.x);
    block_min_to(&ctl->cfl_bits, dmin, red, threadIdx.x, blockDim.x);
  }
}

template <bool E, int ND, bool QF = false>
cudaError_t launch_all(const double *A, double *B, double *scratch, const Geo &g,
                       const Axis &ax, const Axis &ay, const Axis &az,
                       const RoeK &K, const Phys &ph, double dt, Ctl *ctl,
                       Box3 box, cudaStream_t s) {
  const unsigned blocks = (unsigned)((g.n + kRoeThreads - 1) / kRoeThreads);
  double *H = scratch, *Fl = scratch + 8 * g.n;
  k_roe_flux1<E, ND, QF><<<blocks, kRoeThreads, 0, s>>>(A, Fl, g, K, ctl);
  k_roe_half<E, ND><<<blocks, kRoeThreads, 0, s>>>(A, Fl, H, g, ax, ay, az, K, dt, ctl);
  k_roe_flux2<E, ND, QF><<<blocks, kRoeThreads, 0, s>>>(H, Fl, g, K, ctl);
  k_roe_full<E, ND><<<blocks, kRoeThreads, 0, s>>>(A, Fl, H, B, g, ax, ay, az, K, ph,
                                                   dt, ctl, box);
  count_launch(4);
  return cudaGetLastError();
}

}  // namespace

static RoeK make_roek(double gm) {
  RoeK k{};
  const double pi = std::acos(-1.0);
  k.gm = gm;
  k.gm1 = gm - 1.0;
  k.gm2 = gm - 2.0;
  k.gm21 = (gm - 2.0) / (gm - 1.0);
  k.pi4 = 4.0 * pi;
  k.pi4i = 1.0 / k.pi4;
  k.pi8i = 5.0e-1 * k.pi4i;
  k.sqh = std::sqrt(0.5);
  k.gm1i = 1.0 / (gm - 1.0);
  k.ggm1 = gm / (gm - 1.0);
  k.sq4pi = std::sqrt(k.pi4);
  k.sq4pii = std::sqrt(k.pi4i);
  return k;
}

size_t roe3d_scratch_doubles(size_t ncells) { return 32 * ncells; }

cudaError_t launch_roe3d(bool exact, const double *A, double *B, double *scratch,
                         int ix, int jx, int kx, const Axis &ax, const Axis &ay,
                         const Axis &az, const Phys &ph, double dt, Ctl *ctl,
                         Box3 box, cudaStream_t s, bool df) {
  Geo g{};
  g.n3[0] = ix;
  g.n3[1] = jx;
  g.n3[2] = kx;
  g.st[0] = 1;
  g.st[1] = (size_t)ix;
  g.st[2] = (size_t)ix * jx;
  g.n = g.st[2] * kx;
  const RoeK K = make_roek(ph.gm);
  if (df && !exact)
    return launch_all<false, 3, true>(A, B, scratch, g, ax, ay, az, K, ph, dt, ctl, box, s);
  return exact ? launch_all<true, 3>(A, B, scratch, g, ax, ay, az, K, ph, dt, ctl, box, s)
               : launch_all<false, 3>(A, B, scratch, g, ax, ay, az, K, ph, dt, ctl, box, s);
}

cudaError_t launch_roe2d(bool exact, const double *A, double *B, double *scratch,
                         int ix, int jx, const Axis &ax, const Axis &ay,
                         const Phys &ph, double dt, Ctl *ctl, Box3 box,
                         cudaStream_t s, bool df) {
  Geo g{};
  g.n3[0] = ix;
  g.n3[1] = jx;
  g.n3[2] = 1;
  g.st[0] = 1;
  g.st[1] = (size_t)ix;
  g.st[2] = (size_t)ix * jx;
  g.n = g.st[2];
  const RoeK K = make_roek(ph.gm);
  const Axis none{};
  if (df && !exact)
    return launch_all<false, 2, true>(A, B, scratch, g, ax, ay, none, K, ph, dt, ctl, box, s);
  return exact ? launch_all<true, 2>(A, B, scratch, g, ax, ay, none, K, ph, dt, ctl, box, s)
               : launch_all<false, 2>(A, B, scratch, g, ax, ay, none, K, ph, dt, ctl, box, s);
}

}  // namespace cans
