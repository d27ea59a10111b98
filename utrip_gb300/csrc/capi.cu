// C-ABI layer: drop-in entry points with the reference argument lists, the
// residency registry, and the device-resident run handle.
//
// Host-side bookkeeping mirrors the reference drivers (for example
// cans2d/md_mhdkh/hdmlw/main.f:160-219): cfl -> t += dt -> step -> bnd ->
// output test -> loop test.  The run handle keeps that loop on the device
// and replays it as a CUDA graph; the drop-in entry points serve a Fortran
// driver that still calls cfl_m3 / mlw_m3 / bd* once per step.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <algorithm>
#include <vector>

#include "cans_gpu.h"
#include "cans_internal.h"

namespace cans {

static std::atomic<unsigned long long> g_launches{0};
void count_launch(int n) { g_launches += (unsigned long long)n; }
unsigned long long launch_count() { return g_launches.load(); }

// Reference metric set-up (cans2d/hdmlw/mlw_m3.f:70-86).  Index 0 and n-1 of
// u0/u1 are never read by the step.
void build_axis_host(int n, const double *d, const double *dm, double *di,
                     double *dim, double *u0, double *u1) {
  for (int i = 0; i < n; i++) {
    di[i] = 1.0 / d[i];
    dim[i] = 1.0 / dm[i];
    u0[i] = 0.0;
    u1[i] = 0.0;
  }
  for (int i = 1; i < n - 1; i++) {
    u1[i] = 0.5 * dm[i - 1] / d[i];
    u0[i] = 0.5 * dm[i] / d[i];
  }
}

Phys make_phys(double gm, double qav) {
  Phys p;
  const double pi = std::acos(-1.0);
  p.gm = gm;
  p.gm1 = gm - 1;
  p.gm1i = 1.0 / p.gm1;
  p.ggm1 = gm / p.gm1;
  p.pi8i = 1. / pi / 8.;
  p.pi4i = 1. / pi / 4.;
  p.qav = qav;
  p.pi4i_cfl = 0.25 / (double)std::acos(-1.0f);  // cans3d/common/cfl_m.f:39-40
  return p;
}

}  // namespace cans

using namespace cans;

// ---------------------------------------------------------------------------
// Library state
namespace {

thread_local std::string g_last_error;
std::mutex g_mu;
int g_exact = -1;            // -1: read CANS_GPU_EXACT on first use
cudaStream_t g_stream = nullptr;
bool g_stream_user = false;

int fail_cuda(cudaError_t e, const char *where) {
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return CANS_ERR_CUDA;
}
#define CK(call)                                             \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return fail_cuda(_e, #call);      \
  } while (0)

int exact_mode() {
  if (g_exact < 0) {
    const char *s = std::getenv("CANS_GPU_EXACT");
    g_exact = (s && s[0] == '1') ? 1 : 0;
  }
  return g_exact;
}

int lib_stream(cudaStream_t *s) {
  if (!g_stream && !g_stream_user) {
    CK(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking));
  }
  *s = g_stream;
  return CANS_OK;
}

// Device metric arrays of one axis (six arrays in one allocation).
struct DevAxis {
  Axis a;
  double *mem = nullptr;
  int cap = 0;
  std::vector<double> h;  // host staging: d, dm, di, dim, u0, u1
  int ensure(int n) {
    if (cap < n) {
      if (mem) cudaFree(mem);
      mem = nullptr;
      cap = 0;
      CK(cudaMalloc(&mem, sizeof(double) * 6 * (size_t)n));
      cap = n;
    }
    a.n = n;
    a.d = mem;
    a.dm = mem + n;
    a.di = mem + 2 * n;
    a.dim = mem + 3 * n;
    a.u0 = mem + 4 * n;
    a.u1 = mem + 5 * n;
    return CANS_OK;
  }
  // Upload d and dm, plus the derived arrays computed on the host with the
  // reference expressions.
  int upload(int n, const double *d, const double *dm, cudaStream_t s) {
    int rc = ensure(n);
    if (rc) return rc;
    h.assign(6 * (size_t)n, 0.0);
    std::memcpy(h.data(), d, sizeof(double) * n);
    std::memcpy(h.data() + n, dm, sizeof(double) * n);
    build_axis_host(n, d, dm, h.data() + 2 * n, h.data() + 3 * n,
                    h.data() + 4 * n, h.data() + 5 * n);
    CK(cudaMemcpyAsync(mem, h.data(), sizeof(double) * 6 * (size_t)n,
                       cudaMemcpyHostToDevice, s));
    return CANS_OK;
  }
  void release() {
    if (mem) cudaFree(mem);
    mem = nullptr;
    cap = 0;
  }
};

// Scratch of the non-resident drop-in calls: state buffers and metrics,
// reused while the sizes stay the same.
struct Scratch {
  double *A = nullptr, *B = nullptr;
  size_t cap = 0;  // doubles per buffer
  DevAxis ax, ay, az;
  unsigned long long *bits = nullptr;
  int ensure(size_t ndoubles) {
    if (cap < ndoubles) {
      if (A) cudaFree(A);
      if (B) cudaFree(B);
      A = B = nullptr;
      cap = 0;
      CK(cudaMalloc(&A, sizeof(double) * ndoubles));
      CK(cudaMalloc(&B, sizeof(double) * ndoubles));
      cap = ndoubles;
    }
    if (!bits) CK(cudaMalloc(&bits, sizeof(unsigned long long) * 2));
    return CANS_OK;
  }
  // stage scratch of the Roe step (half-step primitives and face fluxes)
  double *roe = nullptr;
  size_t roe_cap = 0;
  int ensure_roe(size_t ndoubles) {
    if (roe_cap < ndoubles) {
      if (roe) cudaFree(roe);
      roe = nullptr;
      roe_cap = 0;
      CK(cudaMalloc(&roe, sizeof(double) * ndoubles));
      roe_cap = ndoubles;
    }
    return CANS_OK;
  }
  // gravity fields of the steps with gravity: gx, gxm, gy, gym (2-D), and
  // gz, gzm (3-D)
  double *grav = nullptr;
  size_t grav_cap = 0;
  int upload_grav(const double *const *g, size_t n, cudaStream_t s, int nf = 4) {
    if (grav_cap < nf * n) {
      if (grav) cudaFree(grav);
      grav = nullptr;
      grav_cap = 0;
      CK(cudaMalloc(&grav, sizeof(double) * nf * n));
      grav_cap = nf * n;
    }
    for (int k = 0; k < nf; k++)
      CK(cudaMemcpyAsync(grav + k * n, g[k], sizeof(double) * n, cudaMemcpyHostToDevice, s));
    return CANS_OK;
  }
  // resistivity (et, then etm) of the resistive 2-D steps, and their eta*J
  // fields (nres doubles)
  double *eta = nullptr, *res = nullptr;
  size_t eta_cap = 0, res_cap = 0;
  int upload_eta(const double *const *e, int k, size_t n, size_t nres, cudaStream_t s) {
    if (eta_cap < 2 * n) {
      if (eta) cudaFree(eta);
      eta = nullptr;
      eta_cap = 0;
      CK(cudaMalloc(&eta, sizeof(double) * 2 * n));
      eta_cap = 2 * n;
    }
    if (res_cap < nres) {
      if (res) cudaFree(res);
      res = nullptr;
      res_cap = 0;
      CK(cudaMalloc(&res, sizeof(double) * nres));
      res_cap = nres;
    }
    for (int q = 0; q < k; q++)
      CK(cudaMemcpyAsync(eta + q * n, e[q], sizeof(double) * n, cudaMemcpyHostToDevice, s));
    return CANS_OK;
  }
};
Scratch g_scratch;

// Registered host-array sets and their device mirrors.
struct MirrorSet {
  int n0 = 1, n1 = 1, n2 = 1, narr = 0;
  size_t n = 0;
  std::vector<double *> host;
  double *buf[2] = {nullptr, nullptr};
  int cur = 0;
  DevAxis ax, ay, az;
  unsigned long long *bits = nullptr;
  double *arr(int v) { return buf[cur] + (size_t)v * n; }
};
std::unordered_map<const double *, std::pair<MirrorSet *, int>> g_registry;

MirrorSet *find_set(const double *p, int *var) {
  auto it = g_registry.find(p);
  if (it == g_registry.end()) return nullptr;
  if (var) *var = it->second.second;
  return it->second.first;
}

// The step's arrays are resident if they are the first nvar arrays of one
// set, in order.
MirrorSet *resident_step_set(double *const *arrs, int nvar) {
  int v0 = -1;
  MirrorSet *m = find_set(arrs[0], &v0);
  if (!m || v0 != 0 || m->narr < nvar) return nullptr;
  for (int v = 1; v < nvar; v++) {
    int vv = -1;
    if (find_set(arrs[v], &vv) != m || vv != v) return nullptr;
  }
  return m;
}

double bits_to_double(unsigned long long b) {
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
}

// ---- generic 2-D step (drop-in) -------------------------------------------
// One 2-D step on host arrays or on their registered mirrors; with grav (gx,
// gxm, gy, gym host arrays of ix*jx) the step with gravity, with eta (et,
// etm) the resistive step.
int step2d(int solver, double *const *arrs, int nvar, double dt, double qav,
           double gm, const double *dx, const double *dxm, int ix,
           const double *dy, const double *dym, int jx,
           const double *const *grav = nullptr, const double *const *eta = nullptr) {
  NvtxRange nvtx("mLW 2-D drop-in step");
  if (ix < 3 || jx < 3) return CANS_ERR_ARG;
  if (grav)
    for (int k = 0; k < 4; k++)
      if (!grav[k]) return CANS_ERR_ARG;
  if (eta && (!eta[0] || !eta[1])) return CANS_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  const Phys ph = make_phys(gm, qav);
  const size_t n = (size_t)ix * jx;
  Box3 box{};
  if (grav && (rc = g_scratch.upload_grav(grav, n, s))) return rc;
  if (eta && (rc = g_scratch.upload_eta(eta, 2, n, mlw2d_e_scratch_doubles(solver, ix, jx),
                                        s)))
    return rc;
  auto step = [&](const double *A, double *B, const Axis &ax, const Axis &ay) {
    if (eta)
      return launch_mlw2d_e(solver, exact_mode(), A, B, ix, jx, ax, ay, ph,
                            grav ? g_scratch.grav : nullptr, g_scratch.eta, g_scratch.res,
                            dt, nullptr, box, s);
    return grav ? launch_mlw2d_g(solver, exact_mode(), 0, A, B, ix, jx, ax, ay, ph,
                                 g_scratch.grav, dt, nullptr, box, s)
                : launch_mlw2d(solver, exact_mode(), 0, A, B, ix, jx, ax, ay, ph, dt,
                               nullptr, box, s);
  };
  MirrorSet *m = resident_step_set(arrs, nvar);
  if (m) {
    if ((rc = m->ax.upload(ix, dx, dxm, s))) return rc;
    if ((rc = m->ay.upload(jx, dy, dym, s))) return rc;
    CK(step(m->buf[m->cur], m->buf[m->cur ^ 1], m->ax.a, m->ay.a));
    m->cur ^= 1;
    return CANS_OK;
  }
  if ((rc = g_scratch.ensure((size_t)nvar * n))) return rc;
  for (int v = 0; v < nvar; v++)
    CK(cudaMemcpyAsync(g_scratch.A + v * n, arrs[v], sizeof(double) * n,
                       cudaMemcpyHostToDevice, s));
  if ((rc = g_scratch.ax.upload(ix, dx, dxm, s))) return rc;
  if ((rc = g_scratch.ay.upload(jx, dy, dym, s))) return rc;
  CK(step(g_scratch.A, g_scratch.B, g_scratch.ax.a, g_scratch.ay.a));
  for (int v = 0; v < nvar; v++)
    CK(cudaMemcpyAsync(arrs[v], g_scratch.B + v * n, sizeof(double) * n,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return CANS_OK;
}

// cfl_m3 / cfl_m; with et (host, ix*jx) cfl_m3_e / cfl_m_e.
int cfl2d(int solver, double *dt, double safety, double dtmin, int *merr,
          double gm, const double *const *arrs, int nvar, const double *dx,
          int ix, const double *dy, int jx, const double *et = nullptr) {
  NvtxRange nvtx("2-D drop-in CFL");
  if (ix < 1 || jx < 1) return CANS_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  const Phys ph = make_phys(gm, 0.0);
  const size_t n = (size_t)ix * jx;
  // cfl reads only d (dx, dy); dm is passed as the same array for the
  // derived metrics, which the CFL never reads.
  const double *base = nullptr;
  Axis ax, ay;
  unsigned long long *bits = nullptr;
  MirrorSet *m = resident_step_set(const_cast<double *const *>(arrs), nvar);
  if (m) {
    if ((rc = m->ax.upload(ix, dx, dx, s))) return rc;
    if ((rc = m->ay.upload(jx, dy, dy, s))) return rc;
    if (!m->bits) CK(cudaMalloc(&m->bits, sizeof(unsigned long long)));
    base = m->buf[m->cur];
    ax = m->ax.a;
    ay = m->ay.a;
    bits = m->bits;
  } else {
    if ((rc = g_scratch.ensure((size_t)nvar * n))) return rc;
    for (int v = 0; v < nvar; v++)
      CK(cudaMemcpyAsync(g_scratch.A + v * n, arrs[v], sizeof(double) * n,
                         cudaMemcpyHostToDevice, s));
    if ((rc = g_scratch.ax.upload(ix, dx, dx, s))) return rc;
    if ((rc = g_scratch.ay.upload(jx, dy, dy, s))) return rc;
    base = g_scratch.A;
    ax = g_scratch.ax.a;
    ay = g_scratch.ay.a;
    bits = g_scratch.bits;
  }
  // dt = 1.e20 (real*4) is the starting minimum of the reference scan
  const unsigned long long init = [] {
    double d = (double)1.e20f;
    unsigned long long b;
    std::memcpy(&b, &d, sizeof b);
    return b;
  }();
  CK(cudaMemcpyAsync(bits, &init, sizeof init, cudaMemcpyHostToDevice, s));
  if (et) {
    if ((rc = g_scratch.upload_eta(&et, 1, n, 0, s))) return rc;
    CK(launch_cfl2d_e(solver, exact_mode(), base, ix, jx, ax, ay, ph, g_scratch.eta, safety,
                      1, bits, s));
  } else {
    CK(launch_cfl2d_full(solver, exact_mode(), base, ix, jx, ax, ay, ph, safety,
                         bits, s));
  }
  unsigned long long out = 0;
  CK(cudaMemcpyAsync(&out, bits, sizeof out, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  *dt = bits_to_double(out);
  *merr = (*dt < dtmin) ? 9001 : 0;
  return CANS_OK;
}

// One reference bd* call.  dims = (n0, n1, n2).
int bd_call(int kind, int axis, int mbnd, int m0, int m1, double *qq,
            double q0, const double *dxm, int n0, int n1, int n2) {
  if (n0 < 1 || n1 < 1 || n2 < 1) return CANS_ERR_ARG;
  const int dims[3] = {n0, n1, n2};
  if (m0 < 0 || m1 < 0 || m0 + m1 > dims[axis]) return CANS_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  const size_t n = (size_t)n0 * n1 * n2;
  const double *ddxm = nullptr;
  int var = -1;
  MirrorSet *m = find_set(qq, &var);
  DevAxis *dax = nullptr;
  if (m) dax = axis == 0 ? &m->ax : (axis == 1 ? &m->ay : &m->az);
  else dax = axis == 0 ? &g_scratch.ax : (axis == 1 ? &g_scratch.ay : &g_scratch.az);
  if (kind == BD_FRD) {
    if ((rc = dax->upload(dims[axis], dxm, dxm, s))) return rc;
    ddxm = dax->a.dm;
  }
  if (m) {
    CK(launch_bd_one(kind, axis, mbnd, m0, m1, m->arr(var), q0, ddxm, n0, n1,
                     n2, s));
    return CANS_OK;
  }
  if ((rc = g_scratch.ensure(n))) return rc;
  CK(cudaMemcpyAsync(g_scratch.A, qq, sizeof(double) * n,
                     cudaMemcpyHostToDevice, s));
  CK(launch_bd_one(kind, axis, mbnd, m0, m1, g_scratch.A, q0, ddxm, n0, n1, n2,
                   s));
  CK(cudaMemcpyAsync(qq, g_scratch.A, sizeof(double) * n,
                     cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return CANS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// Settings
extern "C" int cans_set_exact(int exact) {
  g_exact = exact ? 1 : 0;
  return CANS_OK;
}
extern "C" int cans_get_exact(void) { return exact_mode(); }
extern "C" int cans_set_stream(void *stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_stream = (cudaStream_t)stream;
  g_stream_user = (stream != nullptr);
  return CANS_OK;
}
extern "C" const char *cans_last_error(void) { return g_last_error.c_str(); }
cudaStream_t cans::configured_stream() {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_stream;
}
extern "C" unsigned long long cans_launch_count(void) { return launch_count(); }
extern "C" int cans_device_ok(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return 0;
  return (p.major == 10 && p.minor == 3) ? 1 : 0;
}

// ---------------------------------------------------------------------------
// 2-D drop-in entry points
extern "C" int cans_mlw_m3_2d(double *ro, double *pr, double *vx, double *vy,
                              double *vz, double *bx, double *by, double *bz,
                              double *az, const double *dt, const double *qav,
                              const double *gm, const double *dx,
                              const double *dxm, const int *ix,
                              const double *dy, const double *dym,
                              const int *jx) {
  double *arrs[9] = {ro, pr, vx, vy, vz, bx, by, bz, az};
  return step2d(1, arrs, 9, *dt, *qav, *gm, dx, dxm, *ix, dy, dym, *jx);
}

// mlw_m3_g (cans2d/hdmlw/mlw_m3_g.f:1): mlw_m3 with gravity
extern "C" int cans_mlw_m3_g_2d(double *ro, double *pr, double *vx, double *vy,
                                double *vz, double *bx, double *by, double *bz,
                                double *az, const double *dt, const double *qav,
                                const double *gm, const double *gx,
                                const double *gxm, const double *gy,
                                const double *gym, const double *dx,
                                const double *dxm, const int *ix,
                                const double *dy, const double *dym,
                                const int *jx) {
  double *arrs[9] = {ro, pr, vx, vy, vz, bx, by, bz, az};
  const double *grav[4] = {gx, gxm, gy, gym};
  return step2d(1, arrs, 9, *dt, *qav, *gm, dx, dxm, *ix, dy, dym, *jx, grav);
}

// mlw_m_g (cans2d/hdmlw/mlw_m_g.f:1): mlw_m with gravity
extern "C" int cans_mlw_m_g_2d(double *ro, double *pr, double *vx, double *vy,
                               double *bx, double *by, double *az,
                               const double *dt, const double *qav,
                               const double *gm, const double *gx,
                               const double *gxm, const double *gy,
                               const double *gym, const double *dx,
                               const double *dxm, const int *ix,
                               const double *dy, const double *dym,
                               const int *jx) {
  double *arrs[7] = {ro, pr, vx, vy, bx, by, az};
  const double *grav[4] = {gx, gxm, gy, gym};
  return step2d(0, arrs, 7, *dt, *qav, *gm, dx, dxm, *ix, dy, dym, *jx, grav);
}

// mlw_m3_e (cans2d/hdmlw/mlw_m3_e.f:2): mlw_m3 with resistivity
extern "C" int cans_mlw_m3_e_2d(double *ro, double *pr, double *vx, double *vy,
                                double *vz, double *bx, double *by, double *bz,
                                double *az, const double *dt, const double *qav,
                                const double *gm, const double *et,
                                const double *etm, const double *dx,
                                const double *dxm, const int *ix,
                                const double *dy, const double *dym,
                                const int *jx) {
  double *arrs[9] = {ro, pr, vx, vy, vz, bx, by, bz, az};
  const double *eta[2] = {et, etm};
  return step2d(1, arrs, 9, *dt, *qav, *gm, dx, dxm, *ix, dy, dym, *jx, nullptr, eta);
}

// mlw_m_e (cans2d/hdmlw/mlw_m_e.f:2): mlw_m with resistivity
extern "C" int cans_mlw_m_e_2d(double *ro, double *pr, double *vx, double *vy,
                               double *bx, double *by, double *az,
                               const double *dt, const double *qav,
                               const double *gm, const double *et,
                               const double *etm, const double *dx,
                               const double *dxm, const int *ix,
                               const double *dy, const double *dym,
                               const int *jx) {
  double *arrs[7] = {ro, pr, vx, vy, bx, by, az};
  const double *eta[2] = {et, etm};
  return step2d(0, arrs, 7, *dt, *qav, *gm, dx, dxm, *ix, dy, dym, *jx, nullptr, eta);
}

// mlw_m3_ge (cans2d/hdmlw/mlw_m3_ge.f:2): mlw_m3 with gravity and resistivity
extern "C" int cans_mlw_m3_ge_2d(double *ro, double *pr, double *vx, double *vy,
                                 double *vz, double *bx, double *by, double *bz,
                                 double *az, const double *dt, const double *qav,
                                 const double *gm, const double *gx,
                                 const double *gxm, const double *gy,
                                 const double *gym, const double *et,
                                 const double *etm, const double *dx,
                                 const double *dxm, const int *ix,
                                 const double *dy, const double *dym,
                                 const int *jx) {
  double *arrs[9] = {ro, pr, vx, vy, vz, bx, by, bz, az};
  const double *grav[4] = {gx, gxm, gy, gym};
  const double *eta[2] = {et, etm};
  return step2d(1, arrs, 9, *dt, *qav, *gm, dx, dxm, *ix, dy, dym, *jx, grav, eta);
}

// mlw_m_ge (cans2d/hdmlw/mlw_m_ge.f:2): mlw_m with gravity and resistivity
extern "C" int cans_mlw_m_ge_2d(double *ro, double *pr, double *vx, double *vy,
                                double *bx, double *by, double *az,
                                const double *dt, const double *qav,
                                const double *gm, const double *gx,
                                const double *gxm, const double *gy,
                                const double *gym, const double *et,
                                const double *etm, const double *dx,
                                const double *dxm, const int *ix,
                                const double *dy, const double *dym,
                                const int *jx) {
  double *arrs[7] = {ro, pr, vx, vy, bx, by, az};
  const double *grav[4] = {gx, gxm, gy, gym};
  const double *eta[2] = {et, etm};
  return step2d(0, arrs, 7, *dt, *qav, *gm, dx, dxm, *ix, dy, dym, *jx, grav, eta);
}

// cfl_m3_e (cans2d/common/cfl_m3_e.f:2)
extern "C" int cans_cfl_m3_e_2d(double *dt, const double *safety,
                                const double *dtmin, int *merr,
                                const double *gm, const double *ro,
                                const double *pr, const double *vx,
                                const double *vy, const double *vz,
                                const double *bx, const double *by,
                                const double *bz, const double *et,
                                const double *dx, const int *ix,
                                const double *dy, const int *jx) {
  if (!et) return CANS_ERR_ARG;
  const double *arrs[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  return cfl2d(1, dt, *safety, *dtmin, merr, *gm, arrs, 8, dx, *ix, dy, *jx, et);
}

// cfl_m_e (cans2d/common/cfl_m_e.f:2)
extern "C" int cans_cfl_m_e_2d(double *dt, const double *safety,
                               const double *dtmin, int *merr, const double *gm,
                               const double *ro, const double *pr,
                               const double *vx, const double *vy,
                               const double *bx, const double *by,
                               const double *et, const double *dx,
                               const int *ix, const double *dy, const int *jx) {
  if (!et) return CANS_ERR_ARG;
  const double *arrs[6] = {ro, pr, vx, vy, bx, by};
  return cfl2d(0, dt, *safety, *dtmin, merr, *gm, arrs, 6, dx, *ix, dy, *jx, et);
}

extern "C" int cans_mlw_m_2d(double *ro, double *pr, double *vx, double *vy,
                             double *bx, double *by, double *az,
                             const double *dt, const double *qav,
                             const double *gm, const double *dx,
                             const double *dxm, const int *ix,
                             const double *dy, const double *dym,
                             const int *jx) {
  double *arrs[7] = {ro, pr, vx, vy, bx, by, az};
  return step2d(0, arrs, 7, *dt, *qav, *gm, dx, dxm, *ix, dy, dym, *jx);
}

extern "C" int cans_cfl_m3_2d(double *dt, const double *safety,
                              const double *dtmin, int *merr,
                              const double *gm, const double *ro,
                              const double *pr, const double *vx,
                              const double *vy, const double *vz,
                              const double *bx, const double *by,
                              const double *bz, const double *dx,
                              const int *ix, const double *dy,
                              const int *jx) {
  const double *arrs[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  return cfl2d(1, dt, *safety, *dtmin, merr, *gm, arrs, 8, dx, *ix, dy, *jx);
}

extern "C" int cans_cfl_m_2d(double *dt, const double *safety,
                             const double *dtmin, int *merr, const double *gm,
                             const double *ro, const double *pr,
                             const double *vx, const double *vy,
                             const double *bx, const double *by,
                             const double *dx, const int *ix,
                             const double *dy, const int *jx) {
  const double *arrs[6] = {ro, pr, vx, vy, bx, by};
  return cfl2d(0, dt, *safety, *dtmin, merr, *gm, arrs, 6, dx, *ix, dy, *jx);
}

#define CANS_BD2(NAME, KIND, AXIS)                                              \
  extern "C" int NAME(const int *mbnd, const int *margin, double *qq,           \
                      const int *ix, const int *jx) {                           \
    return bd_call(KIND, AXIS, *mbnd, *margin, *margin, qq, 0.0, nullptr, *ix,  \
                   *jx, 1);                                                      \
  }
CANS_BD2(cans_bdsppx_2d, BD_SPP, 0)
CANS_BD2(cans_bdsppy_2d, BD_SPP, 1)
CANS_BD2(cans_bdspnx_2d, BD_SPN, 0)
CANS_BD2(cans_bdspny_2d, BD_SPN, 1)
CANS_BD2(cans_bdsmpx_2d, BD_SMP, 0)
CANS_BD2(cans_bdsmpy_2d, BD_SMP, 1)
CANS_BD2(cans_bdsmnx_2d, BD_SMN, 0)
CANS_BD2(cans_bdsmny_2d, BD_SMN, 1)
CANS_BD2(cans_bdfrex_2d, BD_FRE, 0)
CANS_BD2(cans_bdfrey_2d, BD_FRE, 1)
#undef CANS_BD2

extern "C" int cans_bdperx_2d(const int *margin0, const int *margin1,
                              double *qq, const int *ix, const int *jx) {
  int rc = bd_call(BD_PER, 0, 0, *margin0, *margin1, qq, 0.0, nullptr, *ix, *jx, 1);
  if (rc) return rc;
  return bd_call(BD_PER, 0, 1, *margin0, *margin1, qq, 0.0, nullptr, *ix, *jx, 1);
}
extern "C" int cans_bdpery_2d(const int *margin0, const int *margin1,
                              double *qq, const int *ix, const int *jx) {
  int rc = bd_call(BD_PER, 1, 0, *margin0, *margin1, qq, 0.0, nullptr, *ix, *jx, 1);
  if (rc) return rc;
  return bd_call(BD_PER, 1, 1, *margin0, *margin1, qq, 0.0, nullptr, *ix, *jx, 1);
}
extern "C" int cans_bdcnsx_2d(const int *mbnd, const int *margin, double *qq,
                              const double *q0, const int *ix, const int *jx) {
  return bd_call(BD_CNS, 0, *mbnd, *margin, *margin, qq, *q0, nullptr, *ix, *jx, 1);
}
extern "C" int cans_bdcnsy_2d(const int *mbnd, const int *margin, double *qq,
                              const double *q0, const int *ix, const int *jx) {
  return bd_call(BD_CNS, 1, *mbnd, *margin, *margin, qq, *q0, nullptr, *ix, *jx, 1);
}
extern "C" int cans_bdfrdx_2d(const int *mbnd, const int *margin, double *qq,
                              const double *dxm, const int *ix, const int *jx) {
  return bd_call(BD_FRD, 0, *mbnd, *margin, *margin, qq, 0.0, dxm, *ix, *jx, 1);
}
extern "C" int cans_bdfrdy_2d(const int *mbnd, const int *margin, double *qq,
                              const double *dym, const int *ix, const int *jx) {
  return bd_call(BD_FRD, 1, *mbnd, *margin, *margin, qq, 0.0, dym, *ix, *jx, 1);
}

// ---------------------------------------------------------------------------
// 1-D drop-in entry points
namespace {
// device copies of the constant arrays of the 1-D steps: bx, bxm and, for
// mlw_m_bg, the ten profiles gx gxm sc scm dsc dscm rr rrm drr drrm
struct Dev1D {
  double *bx = nullptr;
  int cap = 0;
  int upload(int ix, const double *hbx, const double *hbxm, cudaStream_t s,
             const double *const *prof = nullptr) {
    if (cap < ix) {
      if (bx) cudaFree(bx);
      bx = nullptr;
      cap = 0;
      CK(cudaMalloc(&bx, sizeof(double) * 12 * (size_t)ix));
      cap = ix;
    }
    CK(cudaMemcpyAsync(bx, hbx, sizeof(double) * ix, cudaMemcpyHostToDevice, s));
    if (hbxm)
      CK(cudaMemcpyAsync(bx + ix, hbxm, sizeof(double) * ix, cudaMemcpyHostToDevice, s));
    if (prof)
      for (int k = 0; k < 10; k++)
        CK(cudaMemcpyAsync(bg() + (size_t)k * ix, prof[k], sizeof(double) * ix,
                           cudaMemcpyHostToDevice, s));
    return CANS_OK;
  }
  double *bg() const { return bx + 2 * (size_t)cap; }
};
Dev1D g_dev1d;
}  // namespace

extern "C" int cans_mlw_m_1d(double *ro, double *pr, double *vx, double *vy,
                             double *by, const double *bx, const double *bxm,
                             const double *dt, const double *qav,
                             const double *gm, const double *dx,
                             const double *dxm, const int *ix) {
  const int n = *ix;
  if (n < mlw1d_min_cells()) return CANS_ERR_ARG;
  double *arrs[5] = {ro, pr, vx, vy, by};
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  const Phys ph = make_phys(*gm, *qav);
  BcTable bc{};
  bc.margin = 1;
  MirrorSet *m = resident_step_set(arrs, 5);
  DevAxis *dax = m ? &m->ax : &g_scratch.ax;
  if ((rc = dax->upload(n, dx, dxm, s))) return rc;
  if ((rc = g_dev1d.upload(n, bx, bxm, s))) return rc;
  double *S;
  if (m) {
    S = m->buf[m->cur];  // the 1-D kernel updates its state in place
  } else {
    if ((rc = g_scratch.ensure(5 * (size_t)n))) return rc;
    for (int v = 0; v < 5; v++)
      CK(cudaMemcpyAsync(g_scratch.A + (size_t)v * n, arrs[v], sizeof(double) * n,
                         cudaMemcpyHostToDevice, s));
    S = g_scratch.A;
  }
  CK(launch_mlw1d(exact_mode(), S, g_dev1d.bx, g_dev1d.bx + n, Loop1D{}, n, dax->a, ph,
                  bc, nullptr, 1, 1, *dt, 0, s));
  if (m) return CANS_OK;
  for (int v = 0; v < 5; v++)
    CK(cudaMemcpyAsync(arrs[v], g_scratch.A + (size_t)v * n, sizeof(double) * n,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return CANS_OK;
}

extern "C" int cans_mlw_m_bg(double *ro, double *pr, double *vx, double *vy,
                             double *by, const double *bx, const double *bxm,
                             const double *dt, const double *qav,
                             const double *gm, const double *gx,
                             const double *gxm, const double *sc,
                             const double *dsc, const double *scm,
                             const double *dscm, const double *rr,
                             const double *rrm, const double *drr,
                             const double *drrm, const double *dx,
                             const double *dxm, const int *ix) {
  const int n = *ix;
  if (n < mlw1d_min_cells()) return CANS_ERR_ARG;
  double *arrs[5] = {ro, pr, vx, vy, by};
  const double *prof[10] = {gx, gxm, sc, scm, dsc, dscm, rr, rrm, drr, drrm};
  for (const double *q : prof)
    if (!q) return CANS_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  const Phys ph = make_phys(*gm, *qav);
  BcTable bc{};
  bc.margin = 1;
  MirrorSet *m = resident_step_set(arrs, 5);
  DevAxis *dax = m ? &m->ax : &g_scratch.ax;
  if ((rc = dax->upload(n, dx, dxm, s))) return rc;
  if ((rc = g_dev1d.upload(n, bx, bxm, s, prof))) return rc;
  double *S;
  if (m) {
    S = m->buf[m->cur];
  } else {
    if ((rc = g_scratch.ensure(5 * (size_t)n))) return rc;
    for (int v = 0; v < 5; v++)
      CK(cudaMemcpyAsync(g_scratch.A + (size_t)v * n, arrs[v], sizeof(double) * n,
                         cudaMemcpyHostToDevice, s));
    S = g_scratch.A;
  }
  Loop1D opt;
  opt.bg = g_dev1d.bg();
  CK(launch_mlw1d(exact_mode(), S, g_dev1d.bx, g_dev1d.bx + n, opt, n, dax->a, ph, bc,
                  nullptr, 1, 1, *dt, 0, s));
  if (m) return CANS_OK;
  for (int v = 0; v < 5; v++)
    CK(cudaMemcpyAsync(arrs[v], g_scratch.A + (size_t)v * n, sizeof(double) * n,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return CANS_OK;
}

// roe_m (cans1d/hdroe/roe_m.f:2): one 1-D Roe-MUSCL step, on the registered
// mirrors when the five arrays are a resident set.
extern "C" int cans_roe_m_1d(double *ro, double *pr, double *vx, double *vy,
                             double *by, const double *bx, const double *bxm,
                             const double *dt, const double *gm,
                             const double *dx, const int *ix) {
  if (!ro || !pr || !vx || !vy || !by || !bx || !bxm || !dt || !gm || !dx || !ix)
    return CANS_ERR_ARG;
  const int n = *ix;
  if (n < 5) return CANS_ERR_ARG;
  double *arrs[5] = {ro, pr, vx, vy, by};
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  MirrorSet *m = resident_step_set(arrs, 5);
  DevAxis *dax = m ? &m->ax : &g_scratch.ax;
  if ((rc = dax->upload(n, dx, dx, s))) return rc;  // roe_m reads dx only
  if ((rc = g_dev1d.upload(n, bx, bxm, s))) return rc;
  if ((rc = g_scratch.ensure_roe(roe1d_scratch_doubles(n)))) return rc;
  const double *dbx = g_dev1d.bx, *dbxm = g_dev1d.bx + n;
  if (m) {
    CK(launch_roe1d(exact_mode(), m->buf[m->cur], m->buf[m->cur ^ 1], g_scratch.roe, dbx,
                    dbxm, dax->a.d, n, *gm, *dt, s));
    m->cur ^= 1;
    return CANS_OK;
  }
  if ((rc = g_scratch.ensure(5 * (size_t)n))) return rc;
  for (int v = 0; v < 5; v++)
    CK(cudaMemcpyAsync(g_scratch.A + (size_t)v * n, arrs[v], sizeof(double) * n,
                       cudaMemcpyHostToDevice, s));
  CK(launch_roe1d(exact_mode(), g_scratch.A, g_scratch.B, g_scratch.roe, dbx, dbxm,
                  dax->a.d, n, *gm, *dt, s));
  for (int v = 0; v < 5; v++)
    CK(cudaMemcpyAsync(arrs[v], g_scratch.B + (size_t)v * n, sizeof(double) * n,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return CANS_OK;
}

extern "C" int cans_chkdav(int *n_events, double *da, double *vx,
                           const double *floor, const int *ix) {
  if (!n_events || !da || !vx || !floor || *ix < 0) return CANS_ERR_ARG;
  const size_t n = (size_t)*ix;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  if ((rc = g_scratch.ensure(2 * n + 1))) return rc;
  double *dd = g_scratch.A, *dv = g_scratch.A + n;
  unsigned long long *cnt = g_scratch.bits;
  CK(cudaMemcpyAsync(dd, da, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dv, vx, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(cnt, 0, sizeof *cnt, s));
  CK(launch_chkdav(dd, dv, *floor, n, cnt, s));
  unsigned long long out = 0;
  CK(cudaMemcpyAsync(da, dd, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(vx, dv, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&out, cnt, sizeof out, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  *n_events = (int)out;
  return CANS_OK;
}

namespace {
// chkdav of a 2-D / 3-D array and its nv velocity components, on their
// registered mirrors (velocities in consecutive slots of one set) or on host
// copies.
int chkdav_nd(int *n_events, double *da, double *const *vel, int nv, double floor,
              size_t n) {
  if (!n_events || !da || !vel) return CANS_ERR_ARG;
  for (int v = 0; v < nv; v++)
    if (!vel[v]) return CANS_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  if ((rc = g_scratch.ensure((size_t)(nv + 1) * n))) return rc;
  unsigned long long *cnt = g_scratch.bits;
  CK(cudaMemsetAsync(cnt, 0, sizeof *cnt, s));
  int va = -1, v0 = -1;
  MirrorSet *m = find_set(da, &va);
  bool resident = m != nullptr && find_set(vel[0], &v0) == m;
  for (int v = 1; resident && v < nv; v++) {
    int vv = -1;
    resident = find_set(vel[v], &vv) == m && vv == v0 + v;
  }
  if (resident && m->n == n) {
    CK(launch_chkdav_nd(m->buf[m->cur], n, 1, va, va, nv, v0, floor, nullptr, cnt, s));
  } else {
    double *S = g_scratch.A;
    CK(cudaMemcpyAsync(S, da, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    for (int v = 0; v < nv; v++)
      CK(cudaMemcpyAsync(S + (1 + v) * n, vel[v], sizeof(double) * n,
                         cudaMemcpyHostToDevice, s));
    CK(launch_chkdav_nd(S, n, 1, 0, 0, nv, 1, floor, nullptr, cnt, s));
    CK(cudaMemcpyAsync(da, S, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    for (int v = 0; v < nv; v++)
      CK(cudaMemcpyAsync(vel[v], S + (1 + v) * n, sizeof(double) * n,
                         cudaMemcpyDeviceToHost, s));
  }
  unsigned long long out = 0;
  CK(cudaMemcpyAsync(&out, cnt, sizeof out, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  *n_events = (int)out;
  return CANS_OK;
}
}  // namespace

// chkdav (cans2d/common/chkdav.f:2): da below floor raised to it, vx and vy
// set to zero there
extern "C" int cans_chkdav_2d(int *n_events, double *da, double *vx, double *vy,
                              const double *floor, const int *ix, const int *jx) {
  if (!floor || !ix || !jx || *ix < 0 || *jx < 0) return CANS_ERR_ARG;
  double *vel[2] = {vx, vy};
  return chkdav_nd(n_events, da, vel, 2, *floor, (size_t)*ix * *jx);
}

// chkdav (cans3d/common/chkdav.f:2): the same with vx, vy and vz
extern "C" int cans_chkdav_3d(int *n_events, double *da, double *vx, double *vy,
                              double *vz, const double *floor, const int *ix,
                              const int *jx, const int *kx) {
  if (!floor || !ix || !jx || !kx || *ix < 0 || *jx < 0 || *kx < 0) return CANS_ERR_ARG;
  double *vel[3] = {vx, vy, vz};
  return chkdav_nd(n_events, da, vel, 3, *floor, (size_t)*ix * *jx * *kx);
}

extern "C" int cans_cfl_m_1d(double *dt, const double *safety,
                             const double *dtmin, int *merr, const double *gm,
                             const double *bx, const double *ro,
                             const double *pr, const double *vx,
                             const double *vy, const double *by,
                             const double *dx, const int *ix) {
  const int n = *ix;
  if (n < 3) return CANS_ERR_ARG;
  const double *arrs[5] = {ro, pr, vx, vy, by};
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  const Phys ph = make_phys(*gm, 0.0);
  MirrorSet *m = resident_step_set(const_cast<double *const *>(arrs), 5);
  DevAxis *dax = m ? &m->ax : &g_scratch.ax;
  if ((rc = dax->upload(n, dx, dx, s))) return rc;
  if ((rc = g_dev1d.upload(n, bx, nullptr, s))) return rc;
  if ((rc = g_scratch.ensure(5 * (size_t)n))) return rc;
  const double *S;
  if (m) {
    S = m->buf[m->cur];
  } else {
    for (int v = 0; v < 5; v++)
      CK(cudaMemcpyAsync(g_scratch.A + (size_t)v * n, arrs[v], sizeof(double) * n,
                         cudaMemcpyHostToDevice, s));
    S = g_scratch.A;
  }
  const double d0 = (double)1.e20f;
  unsigned long long init;
  std::memcpy(&init, &d0, sizeof init);
  CK(cudaMemcpyAsync(g_scratch.bits, &init, sizeof init, cudaMemcpyHostToDevice, s));
  CK(launch_cfl1d(exact_mode(), S, g_dev1d.bx, n, dax->a, ph, *safety,
                  g_scratch.bits, s));
  unsigned long long out = 0;
  CK(cudaMemcpyAsync(&out, g_scratch.bits, sizeof out, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  *dt = bits_to_double(out);
  *merr = (*dt < *dtmin) ? 9001 : 0;
  return CANS_OK;
}

#define CANS_BD1(NAME, KIND)                                                    \
  extern "C" int NAME(const int *mbnd, const int *margin, double *qq,           \
                      const int *ix) {                                           \
    return bd_call(KIND, 0, *mbnd, *margin, *margin, qq, 0.0, nullptr, *ix, 1,  \
                   1);                                                           \
  }
CANS_BD1(cans_bdsppx_1d, BD_SPP)
CANS_BD1(cans_bdspnx_1d, BD_SPN)
CANS_BD1(cans_bdsmpx_1d, BD_SMP)
CANS_BD1(cans_bdsmnx_1d, BD_SMN)
CANS_BD1(cans_bdfrex_1d, BD_FRE)
#undef CANS_BD1
extern "C" int cans_bdperx_1d(const int *margin0, const int *margin1,
                              double *qq, const int *ix) {
  int rc = bd_call(BD_PER, 0, 0, *margin0, *margin1, qq, 0.0, nullptr, *ix, 1, 1);
  if (rc) return rc;
  return bd_call(BD_PER, 0, 1, *margin0, *margin1, qq, 0.0, nullptr, *ix, 1, 1);
}
extern "C" int cans_bdcnsx_1d(const int *mbnd, const int *margin, double *qq,
                              const double *q0, const int *ix) {
  return bd_call(BD_CNS, 0, *mbnd, *margin, *margin, qq, *q0, nullptr, *ix, 1, 1);
}
extern "C" int cans_bdfrdx_1d(const int *mbnd, const int *margin, double *qq,
                              const double *dxm, const int *ix) {
  return bd_call(BD_FRD, 0, *mbnd, *margin, *margin, qq, 0.0, dxm, *ix, 1, 1);
}

// ---------------------------------------------------------------------------
// 3-D drop-in entry points
namespace {
// One 3-D mLW step on host arrays or their registered mirrors; with grav
// (gx, gxm, gy, gym, gz, gzm host arrays) the step with gravity, with eta
// (et, etm host arrays) the resistive step.
int step3d(double *const *arrs, double dt, double qav, double gm, const double *dx,
           const double *dxm, int nx, const double *dy, const double *dym, int ny,
           const double *dz, const double *dzm, int nz,
           const double *const *grav = nullptr, const double *const *eta = nullptr) {
  NvtxRange nvtx("mLW 3-D drop-in step");
  if (nx < 3 || ny < 3 || nz < 3) return CANS_ERR_ARG;
  if (grav)
    for (int k = 0; k < 6; k++)
      if (!grav[k]) return CANS_ERR_ARG;
  if (eta && (!eta[0] || !eta[1])) return CANS_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  const Phys ph = make_phys(gm, qav);
  const size_t n = (size_t)nx * ny * nz;
  MirrorSet *m = resident_step_set(arrs, 8);
  Scratch &sc = g_scratch;
  DevAxis *dax = m ? &m->ax : &sc.ax, *day = m ? &m->ay : &sc.ay,
          *daz = m ? &m->az : &sc.az;
  if ((rc = dax->upload(nx, dx, dxm, s))) return rc;
  if ((rc = day->upload(ny, dy, dym, s))) return rc;
  if ((rc = daz->upload(nz, dz, dzm, s))) return rc;
  if (grav && (rc = sc.upload_grav(grav, n, s, 6))) return rc;
  if (eta && (rc = sc.upload_eta(eta, 2, n, mlw3d_e_scratch_doubles(nx, ny, nz), s)))
    return rc;
  auto step = [&](const double *A, double *B) {
    if (eta)
      return launch_mlw3d_e(exact_mode(), 0, A, B, nx, ny, nz, dax->a, day->a, daz->a, ph,
                            sc.eta, sc.res, dt, nullptr, Box3{}, s);
    return grav ? launch_mlw3d_g(exact_mode(), 0, A, B, nx, ny, nz, dax->a, day->a, daz->a,
                                 ph, sc.grav, dt, nullptr, Box3{}, s)
                : launch_mlw3d(exact_mode(), 0, A, B, nx, ny, nz, dax->a, day->a, daz->a,
                               ph, dt, nullptr, Box3{}, s);
  };
  if (m) {
    CK(step(m->buf[m->cur], m->buf[m->cur ^ 1]));
    m->cur ^= 1;
    return CANS_OK;
  }
  if ((rc = sc.ensure(8 * n))) return rc;
  for (int v = 0; v < 8; v++)
    CK(cudaMemcpyAsync(sc.A + v * n, arrs[v], sizeof(double) * n,
                       cudaMemcpyHostToDevice, s));
  CK(step(sc.A, sc.B));
  for (int v = 0; v < 8; v++)
    CK(cudaMemcpyAsync(arrs[v], sc.B + v * n, sizeof(double) * n,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return CANS_OK;
}
}  // namespace

extern "C" int cans_mlw_m_3d(double *ro, double *pr, double *vx, double *vy,
                             double *vz, double *bx, double *by, double *bz,
                             const double *dt, const double *qav,
                             const double *gm, const double *dx,
                             const double *dxm, const int *ix,
                             const double *dy, const double *dym,
                             const int *jx, const double *dz,
                             const double *dzm, const int *kx) {
  double *arrs[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  return step3d(arrs, *dt, *qav, *gm, dx, dxm, *ix, dy, dym, *jx, dz, dzm, *kx);
}

// mlw_m_g (cans3d/hdmlw/mlw_m_g.f:2-4): the 3-D step with gravity
extern "C" int cans_mlw_m_g_3d(double *ro, double *pr, double *vx, double *vy,
                               double *vz, double *bx, double *by, double *bz,
                               const double *dt, const double *qav,
                               const double *gm, const double *gx,
                               const double *gxm, const double *gy,
                               const double *gym, const double *gz,
                               const double *gzm, const double *dx,
                               const double *dxm, const int *ix,
                               const double *dy, const double *dym,
                               const int *jx, const double *dz,
                               const double *dzm, const int *kx) {
  double *arrs[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  const double *grav[6] = {gx, gxm, gy, gym, gz, gzm};
  return step3d(arrs, *dt, *qav, *gm, dx, dxm, *ix, dy, dym, *jx, dz, dzm, *kx, grav);
}

// mlw_m_e (cans3d/hdmlw/mlw_m_e.f:2-3): the 3-D resistive step
extern "C" int cans_mlw_m_e_3d(double *ro, double *pr, double *vx, double *vy,
                               double *vz, double *bx, double *by, double *bz,
                               const double *dt, const double *qav,
                               const double *gm, const double *et,
                               const double *etm, const double *dx,
                               const double *dxm, const int *ix,
                               const double *dy, const double *dym,
                               const int *jx, const double *dz,
                               const double *dzm, const int *kx) {
  double *arrs[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  const double *eta[2] = {et, etm};
  return step3d(arrs, *dt, *qav, *gm, dx, dxm, *ix, dy, dym, *jx, dz, dzm, *kx, nullptr,
                eta);
}

namespace {
// cfl_m (et == nullptr) and cfl_m_e 3-D on host arrays or their mirrors
int cfl3d(double *dt, double safety, double dtmin, int *merr, double gm,
          const double *const *arrs, const double *et, const double *dx, int nx,
          const double *dy, int ny, const double *dz, int nz) {
  if (nx < 1 || ny < 1 || nz < 1) return CANS_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  const Phys ph = make_phys(gm, 0.0);
  const size_t n = (size_t)nx * ny * nz;
  MirrorSet *m = resident_step_set(const_cast<double *const *>(arrs), 8);
  Scratch &sc = g_scratch;
  DevAxis *dax = m ? &m->ax : &sc.ax, *day = m ? &m->ay : &sc.ay,
          *daz = m ? &m->az : &sc.az;
  if ((rc = dax->upload(nx, dx, dx, s))) return rc;
  if ((rc = day->upload(ny, dy, dy, s))) return rc;
  if ((rc = daz->upload(nz, dz, dz, s))) return rc;
  if (et && (rc = sc.upload_eta(&et, 1, n, 0, s))) return rc;
  const double *base;
  unsigned long long *bits;
  if (m) {
    if (!m->bits) CK(cudaMalloc(&m->bits, sizeof(unsigned long long)));
    base = m->buf[m->cur];
    bits = m->bits;
  } else {
    if ((rc = sc.ensure(8 * n))) return rc;
    for (int v = 0; v < 8; v++)
      CK(cudaMemcpyAsync(sc.A + v * n, arrs[v], sizeof(double) * n,
                         cudaMemcpyHostToDevice, s));
    base = sc.A;
    bits = sc.bits;
  }
  const double d0 = (double)1.e20f;
  unsigned long long init;
  std::memcpy(&init, &d0, sizeof init);
  CK(cudaMemcpyAsync(bits, &init, sizeof init, cudaMemcpyHostToDevice, s));
  if (et)
    CK(launch_cfl3d_e(exact_mode(), base, nx, ny, nz, dax->a, day->a, daz->a, ph,
                      g_scratch.eta, safety, 1, bits, s));
  else
    CK(launch_cfl3d_full(exact_mode(), base, nx, ny, nz, dax->a, day->a, daz->a,
                         ph, safety, bits, s));
  unsigned long long out = 0;
  CK(cudaMemcpyAsync(&out, bits, sizeof out, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  *dt = bits_to_double(out);
  *merr = (*dt < dtmin) ? 9001 : 0;
  return CANS_OK;
}
}  // namespace

extern "C" int cans_cfl_m_3d(double *dt, const double *safety,
                             const double *dtmin, int *merr, const double *gm,
                             const double *ro, const double *pr,
                             const double *vx, const double *vy,
                             const double *vz, const double *bx,
                             const double *by, const double *bz,
                             const double *dx, const int *ix,
                             const double *dy, const int *jx,
                             const double *dz, const int *kx) {
  const double *arrs[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  return cfl3d(dt, *safety, *dtmin, merr, *gm, arrs, nullptr, dx, *ix, dy, *jx, dz, *kx);
}

// cfl_m_e (cans3d/common/cfl_m_e.f:2-4): the 3-D time step with the
// diffusion limit of the resistivity et
extern "C" int cans_cfl_m_e_3d(double *dt, const double *safety,
                               const double *dtmin, int *merr, const double *gm,
                               const double *ro, const double *pr,
                               const double *vx, const double *vy,
                               const double *vz, const double *bx,
                               const double *by, const double *bz,
                               const double *et, const double *dx, const int *ix,
                               const double *dy, const int *jx,
                               const double *dz, const int *kx) {
  if (!et) return CANS_ERR_ARG;
  const double *arrs[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  return cfl3d(dt, *safety, *dtmin, merr, *gm, arrs, et, dx, *ix, dy, *jx, dz, *kx);
}

// roe_m (cans3d/hdroe/roe_m.f:2): one Roe-MUSCL step, on the registered
// mirrors when the 8 arrays are a resident set, else through the scratch.
extern "C" int cans_roe_m_3d(double *ro, double *pr, double *vx, double *vy,
                             double *vz, double *bx, double *by, double *bz,
                             const double *dt, const double *gm,
                             const double *dx, const int *ix,
                             const double *dy, const int *jx,
                             const double *dz, const int *kx) {
  if (!ro || !pr || !vx || !vy || !vz || !bx || !by || !bz || !dt || !gm ||
      !dx || !dy || !dz || !ix || !jx || !kx)
    return CANS_ERR_ARG;
  const int nx = *ix, ny = *jx, nz = *kx;
  if (nx < 5 || ny < 5 || nz < 5) return CANS_ERR_ARG;
  double *arrs[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  const Phys ph = make_phys(*gm, 0.0);
  const size_t n = (size_t)nx * ny * nz;
  MirrorSet *m = resident_step_set(arrs, 8);
  Scratch &sc = g_scratch;
  DevAxis *dax = m ? &m->ax : &sc.ax, *day = m ? &m->ay : &sc.ay,
          *daz = m ? &m->az : &sc.az;
  // roe_m reads dx, dy, dz only
  if ((rc = dax->upload(nx, dx, dx, s))) return rc;
  if ((rc = day->upload(ny, dy, dy, s))) return rc;
  if ((rc = daz->upload(nz, dz, dz, s))) return rc;
  if ((rc = sc.ensure_roe(roe3d_scratch_doubles(n)))) return rc;
  if (m) {
    CK(launch_roe3d(exact_mode(), m->buf[m->cur], m->buf[m->cur ^ 1], sc.roe, nx,
                    ny, nz, dax->a, day->a, daz->a, ph, *dt, nullptr, Box3{}, s));
    m->cur ^= 1;
    return CANS_OK;
  }
  if ((rc = sc.ensure(8 * n))) return rc;
  for (int v = 0; v < 8; v++)
    CK(cudaMemcpyAsync(sc.A + v * n, arrs[v], sizeof(double) * n,
                       cudaMemcpyHostToDevice, s));
  CK(launch_roe3d(exact_mode(), sc.A, sc.B, sc.roe, nx, ny, nz, dax->a, day->a,
                  daz->a, ph, *dt, nullptr, Box3{}, s));
  for (int v = 0; v < 8; v++)
    CK(cudaMemcpyAsync(arrs[v], sc.B + v * n, sizeof(double) * n,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return CANS_OK;
}

// roe_m3 (cans2d/hdroe/roe_m3.f:1): one 2-D Roe-MUSCL step on the nine
// arrays, on the registered mirrors when they are a resident set.
extern "C" int cans_roe_m3_2d(double *ro, double *pr, double *vx, double *vy,
                              double *vz, double *bx, double *by, double *bz,
                              double *az, const double *dt, const double *gm,
                              const double *dx, const int *ix,
                              const double *dy, const int *jx) {
  if (!ro || !pr || !vx || !vy || !vz || !bx || !by || !bz || !az || !dt || !gm ||
      !dx || !dy || !ix || !jx)
    return CANS_ERR_ARG;
  const int nx = *ix, ny = *jx;
  if (nx < 5 || ny < 5) return CANS_ERR_ARG;
  double *arrs[9] = {ro, pr, vx, vy, vz, bx, by, bz, az};
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  const Phys ph = make_phys(*gm, 0.0);
  const size_t n = (size_t)nx * ny;
  MirrorSet *m = resident_step_set(arrs, 9);
  Scratch &sc = g_scratch;
  DevAxis *dax = m ? &m->ax : &sc.ax, *day = m ? &m->ay : &sc.ay;
  // roe_m3 reads dx, dy only
  if ((rc = dax->upload(nx, dx, dx, s))) return rc;
  if ((rc = day->upload(ny, dy, dy, s))) return rc;
  if ((rc = sc.ensure_roe(roe3d_scratch_doubles(n)))) return rc;
  if (m) {
    CK(launch_roe2d(exact_mode(), m->buf[m->cur], m->buf[m->cur ^ 1], sc.roe, nx, ny,
                    dax->a, day->a, ph, *dt, nullptr, Box3{}, s));
    m->cur ^= 1;
    return CANS_OK;
  }
  if ((rc = sc.ensure(9 * n))) return rc;
  for (int v = 0; v < 9; v++)
    CK(cudaMemcpyAsync(sc.A + v * n, arrs[v], sizeof(double) * n,
                       cudaMemcpyHostToDevice, s));
  CK(launch_roe2d(exact_mode(), sc.A, sc.B, sc.roe, nx, ny, dax->a, day->a, ph, *dt,
                  nullptr, Box3{}, s));
  for (int v = 0; v < 9; v++)
    CK(cudaMemcpyAsync(arrs[v], sc.B + v * n, sizeof(double) * n,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return CANS_OK;
}

// engine (cansxx-nosupport/md_mhdshktb/hdhlld-x/engine.f:2): one HLLD step,
// on the registered mirrors when the 8 arrays are a resident set.
extern "C" int cans_hlld_engine_3d(double *ro, double *pr, double *vx,
                                   double *vy, double *vz, double *bx,
                                   double *by, double *bz, const double *gm,
                                   const double *mu, const double *dt,
                                   const double *dx, const double *dxm,
                                   const double *dy, const double *dym,
                                   const double *dz, const double *dzm,
                                   const int *ix, const int *jx, const int *kx,
                                   const int *mfdim) {
  (void)dxm;
  (void)dym;
  (void)dzm;
  if (!ro || !pr || !vx || !vy || !vz || !bx || !by || !bz || !gm || !mu ||
      !dt || !dx || !dy || !dz || !ix || !jx || !kx || !mfdim)
    return CANS_ERR_ARG;
  const int nn[3] = {*ix, *jx, *kx};
  for (int a = 0; a < 3; a++) {
    if (nn[a] < 1 || (mfdim[a] == 1 && nn[a] < 4)) return CANS_ERR_ARG;
  }
  double *arrs[8] = {ro, pr, vx, vy, vz, bx, by, bz};
  std::lock_guard<std::mutex> lk(g_mu);
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  const size_t n = (size_t)nn[0] * nn[1] * nn[2];
  MirrorSet *m = resident_step_set(arrs, 8);
  Scratch &sc = g_scratch;
  DevAxis *dax = m ? &m->ax : &sc.ax, *day = m ? &m->ay : &sc.ay,
          *daz = m ? &m->az : &sc.az;
  // adddfdx reads dx, dy, dz only
  if ((rc = dax->upload(nn[0], dx, dx, s))) return rc;
  if ((rc = day->upload(nn[1], dy, dy, s))) return rc;
  if ((rc = daz->upload(nn[2], dz, dz, s))) return rc;
  if ((rc = sc.ensure_roe(hlld3d_scratch_doubles(n)))) return rc;
  if (m) {
    CK(launch_hlld3d(exact_mode(), m->buf[m->cur], m->buf[m->cur ^ 1], sc.roe,
                     nn[0], nn[1], nn[2], mfdim, dax->a, day->a, daz->a, *gm, *mu,
                     *dt, nullptr, s));
    m->cur ^= 1;
    return CANS_OK;
  }
  if ((rc = sc.ensure(8 * n))) return rc;
  for (int v = 0; v < 8; v++)
    CK(cudaMemcpyAsync(sc.A + v * n, arrs[v], sizeof(double) * n,
                       cudaMemcpyHostToDevice, s));
  CK(launch_hlld3d(exact_mode(), sc.A, sc.B, sc.roe, nn[0], nn[1], nn[2], mfdim,
                   dax->a, day->a, daz->a, *gm, *mu, *dt, nullptr, s));
  for (int v = 0; v < 8; v++)
    CK(cudaMemcpyAsync(arrs[v], sc.B + v * n, sizeof(double) * n,
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return CANS_OK;
}

#define CANS_BD3(NAME, KIND, AXIS)                                              \
  extern "C" int NAME(const int *mbnd, const int *margin, double *qq,           \
                      const int *ix, const int *jx, const int *kx) {            \
    return bd_call(KIND, AXIS, *mbnd, *margin, *margin, qq, 0.0, nullptr, *ix,  \
                   *jx, *kx);                                                    \
  }
CANS_BD3(cans_bdsppx_3d, BD_SPP, 0)
CANS_BD3(cans_bdsppy_3d, BD_SPP, 1)
CANS_BD3(cans_bdsppz_3d, BD_SPP, 2)
CANS_BD3(cans_bdspnx_3d, BD_SPN, 0)
CANS_BD3(cans_bdspny_3d, BD_SPN, 1)
CANS_BD3(cans_bdspnz_3d, BD_SPN, 2)
CANS_BD3(cans_bdsmpx_3d, BD_SMP, 0)
CANS_BD3(cans_bdsmpy_3d, BD_SMP, 1)
CANS_BD3(cans_bdsmpz_3d, BD_SMP, 2)
CANS_BD3(cans_bdsmnx_3d, BD_SMN, 0)
CANS_BD3(cans_bdsmny_3d, BD_SMN, 1)
CANS_BD3(cans_bdsmnz_3d, BD_SMN, 2)
CANS_BD3(cans_bdfrex_3d, BD_FRE, 0)
CANS_BD3(cans_bdfrey_3d, BD_FRE, 1)
CANS_BD3(cans_bdfrez_3d, BD_FRE, 2)
#undef CANS_BD3

#define CANS_BDPER3(NAME, AXIS)                                                 \
  extern "C" int NAME(const int *margin0, const int *margin1, double *qq,       \
                      const int *ix, const int *jx, const int *kx) {            \
    int rc = bd_call(BD_PER, AXIS, 0, *margin0, *margin1, qq, 0.0, nullptr,     \
                     *ix, *jx, *kx);                                             \
    if (rc) return rc;                                                          \
    return bd_call(BD_PER, AXIS, 1, *margin0, *margin1, qq, 0.0, nullptr, *ix,  \
                   *jx, *kx);                                                    \
  }
CANS_BDPER3(cans_bdperx_3d, 0)
CANS_BDPER3(cans_bdpery_3d, 1)
CANS_BDPER3(cans_bdperz_3d, 2)
#undef CANS_BDPER3

#define CANS_BDQ3(NAME, KIND, AXIS, ARG)                                        \
  extern "C" int NAME(const int *mbnd, const int *margin, double *qq,           \
                      const double *ARG, const int *ix, const int *jx,          \
                      const int *kx) {                                           \
    return KIND == BD_CNS                                                        \
               ? bd_call(KIND, AXIS, *mbnd, *margin, *margin, qq, *ARG,         \
                         nullptr, *ix, *jx, *kx)                                 \
               : bd_call(KIND, AXIS, *mbnd, *margin, *margin, qq, 0.0, ARG,     \
                         *ix, *jx, *kx);                                         \
  }
CANS_BDQ3(cans_bdcnsx_3d, BD_CNS, 0, q0)
CANS_BDQ3(cans_bdcnsy_3d, BD_CNS, 1, q0)
CANS_BDQ3(cans_bdcnsz_3d, BD_CNS, 2, q0)
CANS_BDQ3(cans_bdfrdx_3d, BD_FRD, 0, dxm)
CANS_BDQ3(cans_bdfrdy_3d, BD_FRD, 1, dym)
CANS_BDQ3(cans_bdfrdz_3d, BD_FRD, 2, dzm)
#undef CANS_BDQ3

// ---------------------------------------------------------------------------
// Residency registry
extern "C" int cans_gpu_register(double *const *arrays, const int *narr,
                                 const int *ix, const int *jx, const int *kx) {
  if (!arrays || *narr < 1 || *ix < 1 || *jx < 1 || *kx < 1) return CANS_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  for (int v = 0; v < *narr; v++)
    if (!arrays[v] || g_registry.count(arrays[v])) return CANS_ERR_ARG;
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  auto *m = new MirrorSet();
  m->n0 = *ix;
  m->n1 = *jx;
  m->n2 = *kx;
  m->narr = *narr;
  m->n = (size_t)*ix * *jx * *kx;
  m->host.assign(arrays, arrays + *narr);
  for (int b = 0; b < 2; b++) {
    cudaError_t e = cudaMalloc(&m->buf[b], sizeof(double) * m->n * m->narr);
    if (e != cudaSuccess) {
      if (m->buf[0]) cudaFree(m->buf[0]);
      delete m;
      return fail_cuda(e, "cudaMalloc(mirror)");
    }
  }
  for (int v = 0; v < m->narr; v++) {
    CK(cudaMemcpyAsync(m->buf[0] + v * m->n, arrays[v], sizeof(double) * m->n,
                       cudaMemcpyHostToDevice, s));
    g_registry[arrays[v]] = {m, v};
  }
  CK(cudaStreamSynchronize(s));
  return CANS_OK;
}

static int mirror_copy(const double *any, bool to_host) {
  std::lock_guard<std::mutex> lk(g_mu);
  MirrorSet *m = find_set(any, nullptr);
  if (!m) return CANS_ERR_ARG;
  cudaStream_t s;
  int rc = lib_stream(&s);
  if (rc) return rc;
  for (int v = 0; v < m->narr; v++) {
    if (to_host)
      CK(cudaMemcpyAsync(m->host[v], m->arr(v), sizeof(double) * m->n,
                         cudaMemcpyDeviceToHost, s));
    else
      CK(cudaMemcpyAsync(m->arr(v), m->host[v], sizeof(double) * m->n,
                         cudaMemcpyHostToDevice, s));
  }
  CK(cudaStreamSynchronize(s));
  return CANS_OK;
}
extern "C" int cans_gpu_pull(const double *any) { return mirror_copy(any, true); }
extern "C" int cans_gpu_push(const double *any) { return mirror_copy(any, false); }

extern "C" int cans_gpu_release(const double *any) {
  std::lock_guard<std::mutex> lk(g_mu);
  MirrorSet *m = find_set(any, nullptr);
  if (!m) return CANS_ERR_ARG;
  if (g_stream) cudaStreamSynchronize(g_stream);
  for (double *h : m->host) g_registry.erase(h);
  cudaFree(m->buf[0]);
  cudaFree(m->buf[1]);
  if (m->bits) cudaFree(m->bits);
  m->ax.release();
  m->ay.release();
  m->az.release();
  delete m;
  return CANS_OK;
}

// ---------------------------------------------------------------------------
// Device-resident run handle
struct cans_run {
  cans_run_desc d{};
  int ndim = 2;
  int nvar = 0;
  size_t n = 0;
  Phys ph{};
  BcTable bc{};
  DevAxis ax, ay, az;
  double *buf[2] = {nullptr, nullptr};
  Ctl *ctl = nullptr;          // device control block
  Ctl host_ctl{};              // last copy read back
  cudaStream_t s = nullptr;
  bool own_stream = false;
  int tile = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_iters = 0;
  int graph_nodes = 0;
  double *bx1 = nullptr;       // 1-D: device bx, bxm, then (mlw_m_bg) the ten
                               // profiles and the torque profile, ix each
  Loop1D loop1d{};             // 1-D loop options (device pointers into bx1)
  double *roe = nullptr;       // Roe / HLLD: stage scratch
  double *grav = nullptr;      // mLW with gravity: gx gxm gy gym (gz gzm), n each
  double *eta = nullptr;       // mLW with resistivity: et, etm (n each)
  double *res = nullptr;       //   and the eta*J fields of each step
  int mfdim[3] = {1, 1, 1};    // HLLD: active axes
  double mu = 1.0;             // HLLD: permeability
  bool use_graph = true;       // replay iterations as a CUDA graph
  bool df = false;             // double-float policy of the step
  bool adj_df = true;          // reverse sweep of the adjoint in double-float
  unsigned char *avb = nullptr;  // adjoint check: recorded viscosity branches,
  long long avb_steps = 0;       //   2*ix*jx bytes per step
};

namespace {

int solver_nvar(int solver) {
  switch (solver) {
    case CANS_SOLVER_MLW_M_2D: return 7;
    case CANS_SOLVER_MLW_M3_2D: return 9;
    case CANS_SOLVER_MLW_M_3D: return 8;
    case CANS_SOLVER_MLW_M_1D: return 5;
    case CANS_SOLVER_ROE_M_3D: return 8;
    case CANS_SOLVER_HLLD_3D: return 8;
    case CANS_SOLVER_MLW_M_BG_1D: return 5;
    case CANS_SOLVER_ROE_M3_2D: return 9;
    default: return 0;
  }
}
int solver_ndim(int solver) {
  if (solver == CANS_SOLVER_MLW_M_3D || solver == CANS_SOLVER_ROE_M_3D ||
      solver == CANS_SOLVER_HLLD_3D)
    return 3;
  return (solver == CANS_SOLVER_MLW_M_1D || solver == CANS_SOLVER_MLW_M_BG_1D) ? 1 : 2;
}
bool is_roe(const cans_run *h) {
  return h->d.solver == CANS_SOLVER_ROE_M_3D || h->d.solver == CANS_SOLVER_ROE_M3_2D;
}
// the 2-D kernels other than the step take the mlw_m3 layout (9 arrays,
// cfl_m3): the Roe 2-D state is the same
int layout2d(const cans_run *h) {
  return h->d.solver == CANS_SOLVER_ROE_M3_2D ? CANS_SOLVER_MLW_M3_2D : h->d.solver;
}
bool is_hlld(const cans_run *h) { return h->d.solver == CANS_SOLVER_HLLD_3D; }
int tile_count(const cans_run *h) {
  if (h->ndim == 1) return 1;
  if (h->df && !is_roe(h) && !is_hlld(h))
    return h->ndim == 3 ? mlw3d_df_tile_count() : mlw2d_df_tile_count();
  if (is_roe(h) || is_hlld(h) || h->ndim == 1) return 1;
  if (h->eta) return h->ndim == 3 ? mlw3d_tile_count() : 1;
  if (h->grav) return h->ndim == 3 ? mlw3d_g_tile_count() : mlw2d_g_tile_count();
  return h->ndim == 3 ? mlw3d_tile_count() : mlw2d_tile_count();
}
// 1-D: the whole loop (or one fixed step) as one cluster launch, in place
cudaError_t launch_1d(cans_run *h, int max_steps, int fixed, double dt,
                      int start) {
  return launch_mlw1d(h->d.exact != 0, h->buf[0], h->bx1, h->bx1 + h->d.ix, h->loop1d,
                      h->d.ix, h->ax.a, h->ph, h->bc, fixed ? nullptr : h->ctl,
                      max_steps, fixed, dt, start, h->s, h->df);
}

// cells whose CFL the step kernel reduces: all but the frame of width
// margin+1 that the boundary program may rewrite; none when chkdav may
// change cells after the fill (the frame kernel then reduces every cell)
Box3 inner_box(const cans_run *h) {
  const int w = h->bc.margin + 1;
  Box3 b{};
  if (h->d.chkdav && h->ndim >= 2) {
    for (int a = 0; a < 3; a++) {
      b.lo[a] = 1;
      b.hi[a] = 0;
    }
    return b;
  }
  b.lo[0] = w;
  b.hi[0] = h->d.ix - 1 - w;
  b.lo[1] = w;
  b.hi[1] = h->d.jx - 1 - w;
  b.lo[2] = h->ndim == 3 ? w : 0;
  b.hi[2] = h->ndim == 3 ? h->d.kx - 1 - w : 0;
  return b;
}

cudaError_t step_kernel(cans_run *h, int tile, const double *A, double *B,
                        double dt, Ctl *ctl, Box3 box) {
  if (is_hlld(h))
    return launch_hlld3d(h->d.exact != 0, A, B, h->roe, h->d.ix, h->d.jx, h->d.kx,
                         h->mfdim, h->ax.a, h->ay.a, h->az.a, h->ph.gm, h->mu, dt,
                         ctl, h->s, h->df);
  if (is_roe(h) && h->ndim == 2)
    return launch_roe2d(h->d.exact != 0, A, B, h->roe, h->d.ix, h->d.jx, h->ax.a,
                        h->ay.a, h->ph, dt, ctl, box, h->s, h->df);
  if (is_roe(h))
    return launch_roe3d(h->d.exact != 0, A, B, h->roe, h->d.ix, h->d.jx, h->d.kx,
                        h->ax.a, h->ay.a, h->az.a, h->ph, dt, ctl, box, h->s, h->df);
  if (h->ndim == 3 && h->eta)
    return launch_mlw3d_e(h->d.exact != 0, tile, A, B, h->d.ix, h->d.jx, h->d.kx, h->ax.a,
                          h->ay.a, h->az.a, h->ph, h->eta, h->res, dt, ctl, box, h->s);
  if (h->ndim == 3 && h->grav)
    return launch_mlw3d_g(h->d.exact != 0, tile, A, B, h->d.ix, h->d.jx, h->d.kx, h->ax.a,
                          h->ay.a, h->az.a, h->ph, h->grav, dt, ctl, box, h->s);
  if (h->ndim == 3 && h->df)
    return launch_mlw3d_df(tile, A, B, h->d.ix, h->d.jx, h->d.kx, h->ax.a, h->ay.a, h->az.a,
                           h->ph, dt, ctl, box, h->s);
  if (h->ndim == 3)
    return launch_mlw3d(h->d.exact != 0, tile, A, B, h->d.ix, h->d.jx, h->d.kx,
                        h->ax.a, h->ay.a, h->az.a, h->ph, dt, ctl, box, h->s);
  if (h->eta)
    return launch_mlw2d_e(h->d.solver, h->d.exact != 0, A, B, h->d.ix, h->d.jx, h->ax.a,
                          h->ay.a, h->ph, h->grav, h->eta, h->res, dt, ctl, box, h->s);
  if (h->grav)
    return launch_mlw2d_g(h->d.solver, h->d.exact != 0, tile, A, B, h->d.ix, h->d.jx,
                          h->ax.a, h->ay.a, h->ph, h->grav, dt, ctl, box, h->s);
  if (h->df)
    return launch_mlw2d_df(tile, A, B, h->d.ix, h->d.jx, h->ax.a, h->ay.a, h->ph, dt, ctl,
                           box, h->s);
  return launch_mlw2d(h->d.solver, h->d.exact != 0, tile, A, B, h->d.ix,
                      h->d.jx, h->ax.a, h->ay.a, h->ph, dt, ctl, box, h->s);
}
cudaError_t bc_kernels(cans_run *h, double *S, const Ctl *ctl) {
  if (h->ndim == 3)
    return launch_bc3d(h->nvar, S, h->d.ix, h->d.jx, h->d.kx, h->ax.a, h->ay.a,
                       h->az.a, h->bc, ctl, h->s);
  return launch_bc2d(h->nvar, S, h->d.ix, h->d.jx, h->ax.a, h->ay.a, h->bc, ctl,
                     h->s);
}
cudaError_t frame_kernel(cans_run *h) {
  if (is_hlld(h))  // the step reduces no CFL: every cell after the fill
    return launch_hlld3d_finish(h->d.exact != 0, h->d.ix, h->d.jx, h->d.kx,
                                h->ax.a, h->ay.a, h->az.a, h->ph, h->ctl, h->s);
  if (h->ndim == 3)
    return launch_frame3d(h->d.exact != 0, h->d.ix, h->d.jx, h->d.kx, h->ax.a,
                          h->ay.a, h->az.a, h->ph, h->bc.margin, h->ctl, h->s,
                          h->d.chkdav ? 1 : 0);
  return launch_frame2d(layout2d(h), h->d.exact != 0, nullptr, h->d.ix, h->d.jx,
                        h->ax.a, h->ay.a, h->ph, h->bc.margin, h->ctl, h->s,
                        h->d.chkdav ? 1 : 0);
}
cudaError_t cfl_full_kernel(cans_run *h, const double *S, double safety,
                            unsigned long long *bits) {
  if (h->ndim == 3 && h->eta)
    return launch_cfl3d_e(h->d.exact != 0, S, h->d.ix, h->d.jx, h->d.kx, h->ax.a, h->ay.a,
                          h->az.a, h->ph, h->eta, safety, 1, bits, h->s);
  if (h->ndim == 3)
    return launch_cfl3d_full(h->d.exact != 0, S, h->d.ix, h->d.jx, h->d.kx,
                             h->ax.a, h->ay.a, h->az.a, h->ph, safety, bits, h->s);
  if (h->eta)
    return launch_cfl2d_e(h->d.solver, h->d.exact != 0, S, h->d.ix, h->d.jx, h->ax.a,
                          h->ay.a, h->ph, h->eta, safety, 1, bits, h->s);
  return launch_cfl2d_full(layout2d(h), h->d.exact != 0, S, h->d.ix, h->d.jx,
                           h->ax.a, h->ay.a, h->ph, safety, bits, h->s);
}

// Kernels of one loop iteration on the device: step, boundary program,
// frame CFL (+ start of the next iteration).
int enqueue_iteration(cans_run *h) {
  CK(step_kernel(h, h->tile, nullptr, nullptr, 0.0, h->ctl, inner_box(h)));
  if (h->ndim == 2 && !h->d.chkdav && h->nvar == (layout2d(h) == 1 ? 9 : 7) &&
      h->d.ix >= 2 * h->bc.margin + 3 && h->d.jx >= 2 * h->bc.margin + 3) {
    // boundary program, frame CFL and loop end in one launch
    CK(launch_bcframe2d(layout2d(h), h->d.exact != 0, h->nvar, h->d.ix, h->d.jx, h->ax.a,
                        h->ay.a, h->ph, h->bc, h->ctl, h->s));
    return CANS_OK;
  }
  CK(bc_kernels(h, nullptr, h->ctl));
  // chkdav of ro, then pr, after the boundary fill (cans2d/md_efr/hdmlw/
  // main.f:183-185): velocities zeroed where a floor applies (vx, vy in 2-D,
  // also vz in 3-D)
  if (h->d.chkdav)
    CK(launch_chkdav_nd(nullptr, h->n, 2, 0, 1, h->ndim == 3 ? 3 : 2, 2, h->d.floor, h->ctl,
                        &h->ctl->nfloor, h->s));
  CK(frame_kernel(h));
  return CANS_OK;
}

void drop_graph(cans_run *h) {
  if (h->graph) cudaGraphExecDestroy(h->graph);
  h->graph = nullptr;
  h->graph_iters = 0;
}

int build_graph(cans_run *h, int iters) {
  drop_graph(h);
  cudaGraph_t g = nullptr;
  const unsigned long long before = launch_count();
  CK(cudaStreamBeginCapture(h->s, cudaStreamCaptureModeThreadLocal));
  int rc = CANS_OK;
  for (int k = 0; k < iters && rc == CANS_OK; k++) rc = enqueue_iteration(h);
  cudaError_t e = cudaStreamEndCapture(h->s, &g);
  // captured launches are counted when the graph is replayed
  g_launches -= (launch_count() - before);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return fail_cuda(e, "cudaStreamEndCapture");
  size_t nn = 0;
  cudaGraphGetNodes(g, nullptr, &nn);
  e = cudaGraphInstantiate(&h->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail_cuda(e, "cudaGraphInstantiate");
  h->graph_iters = iters;
  h->graph_nodes = (int)nn;
  return CANS_OK;
}

int read_ctl(cans_run *h) {
  CK(cudaMemcpyAsync(&h->host_ctl, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost,
                     h->s));
  CK(cudaStreamSynchronize(h->s));
  return CANS_OK;
}

unsigned long long r4_1e20_bits() {
  const double d = (double)1.e20f;  // the reference's starting minimum
  unsigned long long b;
  std::memcpy(&b, &d, sizeof b);
  return b;
}

}  // namespace

extern "C" int cans_run_create(cans_run **out, const cans_run_desc *d) {
  NvtxRange nvtx("cans_run_create");
  if (!out || !d) return CANS_ERR_ARG;
  const int nvar = solver_nvar(d->solver);
  if (nvar == 0 || d->margin < 1) return CANS_ERR_ARG;
  // the Roe step updates 3..n-2 and its stencil reaches three cells, so the
  // boundary program must rewrite three layers (hdroe/main.f:5)
  if (d->solver == CANS_SOLVER_ROE_M_3D && d->margin < 3) return CANS_ERR_ARG;
  // the 2-D roe_m3 updates 3..n-2: the md_mhdkh Roe package uses margin 2
  if (d->solver == CANS_SOLVER_ROE_M3_2D && d->margin < 2) return CANS_ERR_ARG;
  const int ndim = solver_ndim(d->solver);
  // HLLD: active axes from mfdim (all 0: every axis longer than one cell);
  // an inactive axis may have any extent, an active one needs the stencil
  int mfdim[3] = {d->mfdim[0], d->mfdim[1], d->mfdim[2]};
  if (d->solver == CANS_SOLVER_HLLD_3D) {
    const int nn[3] = {d->ix, d->jx, d->kx};
    if (!mfdim[0] && !mfdim[1] && !mfdim[2])
      for (int a = 0; a < 3; a++) mfdim[a] = nn[a] > 1 ? 1 : 0;
    for (int a = 0; a < 3; a++) {
      if (nn[a] < 1 || (mfdim[a] == 1 && nn[a] < 2 * d->margin + 2)) return CANS_ERR_ARG;
      if (mfdim[a] != 0 && mfdim[a] != 1) return CANS_ERR_ARG;
    }
    if (!d->dx || !d->dy || !d->dz || !d->dxm || !d->dym || !d->dzm) return CANS_ERR_ARG;
  }
  if (d->chkdav != 0 && d->chkdav != 1) return CANS_ERR_ARG;
  const bool bgv = d->solver == CANS_SOLVER_MLW_M_BG_1D;
  // 2-D mLW with gx set: the steps with gravity (mlw_m_g / mlw_m3_g)
  const bool mlw2d = d->solver == CANS_SOLVER_MLW_M_2D || d->solver == CANS_SOLVER_MLW_M3_2D;
  // every extent must hold the two frames of margin+1 cells that the
  // boundary program and the frame CFL work on; the mLW steps need nothing
  // between them (an axis of exactly two frames, as the thin y axis of the
  // md_efr model, leaves the whole CFL to the frame kernel), the Roe and
  // HLLD stencils one more cell
  const int wmin = 2 * (d->margin + 1) +
                   ((mlw2d || d->solver == CANS_SOLVER_MLW_M_3D) ? 0 : 1);
  const bool grav2d = mlw2d && d->gx != nullptr;
  // 3-D mLW with gx set: mlw_m_g (six fields)
  const bool grav3d = d->solver == CANS_SOLVER_MLW_M_3D && d->gx != nullptr;
  if ((d->gz || d->gzm) && !grav3d) return CANS_ERR_ARG;
  if (grav3d && (!d->gxm || !d->gy || !d->gym || !d->gz || !d->gzm)) return CANS_ERR_ARG;
  // a solver without a gravity step refuses the fields instead of ignoring them
  if ((d->gx || d->gy) && !(grav2d || grav3d || bgv)) return CANS_ERR_ARG;
  // mLW with et set: the resistive steps (2-D mlw_m_e / mlw_m3_e, with or
  // without gravity; 3-D mlw_m_e, which has no gravity variant)
  const bool eta2d = mlw2d && d->et != nullptr;
  const bool eta3d = d->solver == CANS_SOLVER_MLW_M_3D && d->et != nullptr;
  if ((d->et || d->etm) && !((eta2d || eta3d) && d->etm)) return CANS_ERR_ARG;
  if (eta3d && grav3d) return CANS_ERR_ARG;
  const double *prof[10] = {d->gx, d->gxm, d->sc, d->scm, d->dsc,
                            d->dscm, d->rr, d->rrm, d->drr, d->drrm};
  if (ndim == 1) {
    if (d->ix < mlw1d_min_cells() || d->jx != 1 || d->kx != 1 ||
        !d->dx || !d->dxm || !d->bx || !d->bxm)
      return CANS_ERR_ARG;
    if (bgv)
      for (const double *q : prof)
        if (!q) return CANS_ERR_ARG;
    // the torque source reads the rr profile of mlw_m_bg
    if (d->trq && !bgv) return CANS_ERR_ARG;
  } else if (d->solver == CANS_SOLVER_HLLD_3D) {
    // checked above
  } else {
    if (grav2d && (!d->gxm || !d->gy || !d->gym)) return CANS_ERR_ARG;
    if (d->ix < wmin || d->jx < wmin) return CANS_ERR_ARG;
    if (ndim == 2 && d->kx != 1) return CANS_ERR_ARG;
    if (ndim == 3 && (d->kx < wmin || !d->dz || !d->dzm)) return CANS_ERR_ARG;
    if (!d->dx || !d->dxm || !d->dy || !d->dym) return CANS_ERR_ARG;
  }
  auto *h = new cans_run();
  h->d = *d;
  h->ndim = ndim;
  h->nvar = nvar;
  h->n = (size_t)d->ix * (ndim >= 2 ? d->jx : 1) * (ndim == 3 ? d->kx : 1);
  h->ph = make_phys(d->gm, d->qav);
  h->tile = d->tile >= 0 && d->tile < tile_count(h) ? d->tile : 0;
  h->bc.margin = d->margin;
  for (int v = 0; v < kMaxVar; v++)
    for (int f = 0; f < 6; f++) {
      h->bc.kind[v][f] = BD_NONE;
      h->bc.q0[v][f] = 0.0;
    }
  int rc = CANS_OK;
  auto bail = [&](int code) {
    cans_run_destroy(h);
    return code;
  };
  if (d->stream) {
    h->s = (cudaStream_t)d->stream;
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(fail_cuda(e, "cudaStreamCreate"));
    h->own_stream = true;
  }
  for (int b = 0; b < 2; b++) {
    cudaError_t e = cudaMalloc(&h->buf[b], sizeof(double) * h->n * nvar);
    if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMalloc(state)"));
    e = cudaMemsetAsync(h->buf[b], 0, sizeof(double) * h->n * nvar, h->s);
    if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMemset(state)"));
  }
  cudaError_t e = cudaMalloc(&h->ctl, sizeof(Ctl));
  if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMalloc(ctl)"));
  if ((rc = h->ax.upload(d->ix, d->dx, d->dxm, h->s))) return bail(rc);
  if (ndim >= 2 && (rc = h->ay.upload(d->jx, d->dy, d->dym, h->s))) return bail(rc);
  if (ndim == 3 && (rc = h->az.upload(d->kx, d->dz, d->dzm, h->s))) return bail(rc);
  if (ndim == 1) {
    const size_t nx = (size_t)d->ix;
    e = cudaMalloc(&h->bx1, sizeof(double) * 13 * nx);
    if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMalloc(bx)"));
    e = cudaMemcpyAsync(h->bx1, d->bx, sizeof(double) * nx, cudaMemcpyHostToDevice, h->s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h->bx1 + nx, d->bxm, sizeof(double) * nx,
                          cudaMemcpyHostToDevice, h->s);
    for (int k = 0; bgv && k < 10 && e == cudaSuccess; k++)
      e = cudaMemcpyAsync(h->bx1 + (2 + k) * nx, prof[k], sizeof(double) * nx,
                          cudaMemcpyHostToDevice, h->s);
    if (e == cudaSuccess && d->trq)
      e = cudaMemcpyAsync(h->bx1 + 12 * nx, d->trq, sizeof(double) * nx,
                          cudaMemcpyHostToDevice, h->s);
    if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMemcpy(bx)"));
    if (bgv) h->loop1d.bg = h->bx1 + 2 * nx;
    if (d->trq) {
      h->loop1d.trq = h->bx1 + 12 * nx;
      h->loop1d.trq0 = d->trq0;
      h->loop1d.seed = d->seed;
    }
    h->loop1d.chk = d->chkdav;
    h->loop1d.floor = d->floor;
  }
  if (is_roe(h) || is_hlld(h)) {
    const size_t nd = is_roe(h) ? roe3d_scratch_doubles(h->n) : hlld3d_scratch_doubles(h->n);
    e = cudaMalloc(&h->roe, sizeof(double) * nd);
    if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMalloc(stage scratch)"));
  }
  if (grav2d || grav3d) {  // mlw_m_g / mlw_m3_g: four gravity fields, 3-D six
    const double *g[6] = {d->gx, d->gxm, d->gy, d->gym, d->gz, d->gzm};
    const int nf = grav3d ? 6 : 4;
    e = cudaMalloc(&h->grav, sizeof(double) * nf * h->n);
    for (int k = 0; k < nf && e == cudaSuccess; k++)
      e = cudaMemcpyAsync(h->grav + k * h->n, g[k], sizeof(double) * h->n,
                          cudaMemcpyHostToDevice, h->s);
    if (e != cudaSuccess) return bail(fail_cuda(e, "gravity fields"));
    h->tile = d->tile >= 0 && d->tile < tile_count(h) ? d->tile : 0;
  }
  if (eta2d || eta3d) {  // mlw_m_e / mlw_m3_e: et, etm and the eta*J scratch
    const size_t nres = eta3d ? mlw3d_e_scratch_doubles(d->ix, d->jx, d->kx)
                              : mlw2d_e_scratch_doubles(d->solver, d->ix, d->jx);
    e = cudaMalloc(&h->eta, sizeof(double) * 2 * h->n);
    if (e == cudaSuccess) e = cudaMalloc(&h->res, sizeof(double) * nres);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h->eta, d->et, sizeof(double) * h->n, cudaMemcpyHostToDevice, h->s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h->eta + h->n, d->etm, sizeof(double) * h->n,
                          cudaMemcpyHostToDevice, h->s);
    if (e != cudaSuccess) return bail(fail_cuda(e, "resistivity fields"));
    h->tile = d->tile >= 0 && d->tile < tile_count(h) ? d->tile : 0;
  }
  for (int a = 0; a < 3; a++) h->mfdim[a] = mfdim[a];
  h->mu = d->mu > 0.0 ? d->mu : 1.0;
  std::memset(&h->host_ctl, 0, sizeof(Ctl));
  h->host_ctl.done = 1;
  h->host_ctl.buf[0] = h->buf[0];
  h->host_ctl.buf[1] = h->buf[1];
  e = cudaMemcpyAsync(h->ctl, &h->host_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, h->s);
  if (e != cudaSuccess) return bail(fail_cuda(e, "cudaMemcpy(ctl)"));
  e = cudaStreamSynchronize(h->s);
  if (e != cudaSuccess) return bail(fail_cuda(e, "cudaStreamSynchronize"));
  *out = h;
  return CANS_OK;
}

extern "C" int cans_run_destroy(cans_run *h) {
  if (!h) return CANS_ERR_ARG;
  if (h->s) cudaStreamSynchronize(h->s);
  drop_graph(h);
  for (int b = 0; b < 2; b++)
    if (h->buf[b]) cudaFree(h->buf[b]);
  if (h->ctl) cudaFree(h->ctl);
  if (h->bx1) cudaFree(h->bx1);
  if (h->roe) cudaFree(h->roe);
  if (h->grav) cudaFree(h->grav);
  if (h->eta) cudaFree(h->eta);
  if (h->res) cudaFree(h->res);
  if (h->avb) cudaFree(h->avb);
  h->ax.release();
  h->ay.release();
  h->az.release();
  if (h->own_stream && h->s) cudaStreamDestroy(h->s);
  delete h;
  return CANS_OK;
}

extern "C" int cans_run_set_bc(cans_run *h, int var, int face, int kind,
                               double q0) {
  if (!h || var < 0 || var >= h->nvar || face < 0 || face >= 2 * h->ndim ||
      kind < CANS_BD_NONE || kind > CANS_BD_FRD)
    return CANS_ERR_ARG;
  // a boundary rule reads and writes `margin` layers on both sides of the
  // axis, so the axis must hold both frames and a cell between them
  const int ext[3] = {h->d.ix, h->d.jx, h->d.kx};
  if (kind != CANS_BD_NONE && ext[face / 2] < 2 * h->bc.margin + 1) return CANS_ERR_ARG;
  h->bc.kind[var][face] = kind;
  h->bc.q0[var][face] = q0;
  drop_graph(h);
  return CANS_OK;
}

extern "C" int cans_run_push(cans_run *h, double *const *host) {
  NvtxRange nvtx("cans_run_push");
  if (!h || !host) return CANS_ERR_ARG;
  int rc = read_ctl(h);  // learn which buffer is current
  if (rc) return rc;
  const int cur = h->host_ctl.cur;
  for (int v = 0; v < h->nvar; v++)
    CK(cudaMemcpyAsync(h->buf[cur] + v * h->n, host[v], sizeof(double) * h->n,
                       cudaMemcpyHostToDevice, h->s));
  return CANS_OK;
}

extern "C" int cans_run_pull(cans_run *h, double *const *host) {
  NvtxRange nvtx("cans_run_pull");
  if (!h || !host) return CANS_ERR_ARG;
  int rc = read_ctl(h);  // learn which buffer is current
  if (rc) return rc;
  const int cur = h->host_ctl.cur;
  for (int v = 0; v < h->nvar; v++)
    CK(cudaMemcpyAsync(host[v], h->buf[cur] + v * h->n, sizeof(double) * h->n,
                       cudaMemcpyDeviceToHost, h->s));
  CK(cudaStreamSynchronize(h->s));
  return CANS_OK;
}

extern "C" int cans_run_device_state(cans_run *h, double **dev) {
  if (!h || !dev) return CANS_ERR_ARG;
  int rc = read_ctl(h);
  if (rc) return rc;
  for (int v = 0; v < h->nvar; v++)
    dev[v] = h->buf[h->host_ctl.cur] + v * h->n;
  return CANS_OK;
}

extern "C" int cans_run_start(cans_run *h, double t0, double tend,
                              long long nstop, double safety, double dtmin,
                              double dtout, int pause_on_output) {
  NvtxRange nvtx("cans_run_start");
  if (!h) return CANS_ERR_ARG;
  int rc = read_ctl(h);
  if (rc) return rc;
  Ctl c = h->host_ctl;
  c.t = t0;
  c.tp = t0;
  c.tend = tend;
  c.nstop = nstop;
  c.safety = safety;
  c.dtmin = dtmin;
  c.dtout = dtout;
  c.pause_on_output = pause_on_output;
  c.ns = 0;
  c.nexec = 0;
  c.merr = 0;
  c.done = 0;
  c.pause = 0;
  c.frame_blocks_done = 0;
  c.nonfinite = 0;
  c.stop_on_bad = h->d.stop_on_bad ? 1 : 0;
  c.nfloor = 0;
  c.cfl_bits = r4_1e20_bits();
  c.dtdif_bits = h->eta ? 0x7ff0000000000000ull : 0ull;
  h->host_ctl = c;
  CK(cudaMemcpyAsync(h->ctl, &h->host_ctl, sizeof(Ctl), cudaMemcpyHostToDevice,
                     h->s));
  if (h->eta && h->ndim == 3)  // the diffusion limit: et, the mesh and safety only
    CK(launch_cfl3d_e(h->d.exact != 0, h->buf[c.cur], h->d.ix, h->d.jx, h->d.kx, h->ax.a,
                      h->ay.a, h->az.a, h->ph, h->eta, safety, 0, &h->ctl->dtdif_bits,
                      h->s));
  else if (h->eta)
    CK(launch_cfl2d_e(h->d.solver, h->d.exact != 0, h->buf[c.cur], h->d.ix, h->d.jx,
                      h->ax.a, h->ay.a, h->ph, h->eta, safety, 0, &h->ctl->dtdif_bits,
                      h->s));
  if (h->ndim == 1) {  // first CFL and loop start inside the cluster kernel
    CK(launch_1d(h, 0, 0, 0.0, 1));
    return CANS_OK;
  }
  CK(cfl_full_kernel(h, h->buf[c.cur], safety, &h->ctl->cfl_bits));
  CK(launch_prepare(h->ctl, h->s));
  return CANS_OK;
}

extern "C" int cans_run_advance(cans_run *h, int iters) {
  NvtxRange nvtx("cans_run_advance");
  if (!h || iters < 0) return CANS_ERR_ARG;
  if (iters == 0) return CANS_OK;
  if (h->ndim == 1) {
    CK(launch_1d(h, iters, 0, 0.0, 0));
    return CANS_OK;
  }
  if (!h->use_graph) {
    for (int k = 0; k < iters; k++) {
      int rc = enqueue_iteration(h);
      if (rc) return rc;
    }
    return CANS_OK;
  }
  const int chunk = iters < 32 ? iters : 32;
  if (!h->graph || h->graph_iters != chunk) {
    int rc = build_graph(h, chunk);
    if (rc) return rc;
  }
  int done = 0;
  while (done + chunk <= iters) {
    CK(cudaGraphLaunch(h->graph, h->s));
    count_launch(h->graph_nodes);
    done += chunk;
  }
  for (; done < iters; done++) {
    int rc = enqueue_iteration(h);
    if (rc) return rc;
  }
  return CANS_OK;
}

// No counterpart in the reference, whose studies (cans_beta_one,
// cans_beta_vary: the md_spicule model at several plasma betas) run each 1-D
// model as its own process: many started 1-D runs advanced together, one
// cluster per run in one launch, on the first run's stream (the others'
// streams are ordered before and after it with events).
extern "C" int cans_run_advance_group(cans_run *const *runs, int nruns, int iters) {
  NvtxRange nvtx("cans_run_advance_group");
  if (!runs || nruns < 1 || iters < 0) return CANS_ERR_ARG;
  for (int k = 0; k < nruns; k++) {
    const cans_run *h = runs[k];
    if (!h || h->ndim != 1 || !h->ctl) return CANS_ERR_ARG;
    if ((h->d.exact != 0) != (runs[0]->d.exact != 0)) return CANS_ERR_ARG;
    if ((h->loop1d.bg != nullptr) != (runs[0]->loop1d.bg != nullptr)) return CANS_ERR_ARG;
    if (h->df != runs[0]->df) return CANS_ERR_ARG;
  }
  {  // a run once: two clusters on one state would race
    std::vector<const cans_run *> sorted(runs, runs + nruns);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) return CANS_ERR_ARG;
  }
  if (iters == 0) return CANS_OK;
  std::vector<Run1DArgs> args((size_t)nruns);
  for (int k = 0; k < nruns; k++) {
    cans_run *h = runs[k];
    args[k] = Run1DArgs{h->buf[0], h->bx1, h->bx1 + h->d.ix, h->loop1d, h->d.ix,
                        h->ax.a,    h->ph,  h->bc,           h->ctl};
  }
  const cudaStream_t s0 = runs[0]->s;
  std::vector<cudaEvent_t> evs;
  auto cleanup = [&]() {
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
  };
  // the work already queued on every run's stream comes first
  for (int k = 1; k < nruns; k++) {
    if (runs[k]->s == s0) continue;
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      cleanup();
      return CANS_ERR_CUDA;
    }
    evs.push_back(e);
    if (cudaEventRecord(e, runs[k]->s) != cudaSuccess ||
        cudaStreamWaitEvent(s0, e, 0) != cudaSuccess) {
      cleanup();
      return CANS_ERR_CUDA;
    }
  }
  cudaError_t err = launch_mlw1d_group(runs[0]->d.exact != 0, runs[0]->loop1d.bg != nullptr,
                                       args.data(), nruns, iters, s0, runs[0]->df);
  if (err != cudaSuccess) {
    cleanup();
    return err == cudaErrorInvalidValue ? CANS_ERR_ARG : CANS_ERR_CUDA;
  }
  // and every run's later work waits for the group
  cudaEvent_t done;
  if (cudaEventCreateWithFlags(&done, cudaEventDisableTiming) != cudaSuccess) {
    cleanup();
    return CANS_ERR_CUDA;
  }
  evs.push_back(done);
  if (cudaEventRecord(done, s0) != cudaSuccess) {
    cleanup();
    return CANS_ERR_CUDA;
  }
  for (int k = 1; k < nruns; k++)
    if (runs[k]->s != s0 && cudaStreamWaitEvent(runs[k]->s, done, 0) != cudaSuccess) {
      cleanup();
      return CANS_ERR_CUDA;
    }
  cleanup();
  return CANS_OK;
}

extern "C" int cans_run_set_graph(cans_run *h, int use_graph) {
  if (!h) return CANS_ERR_ARG;
  h->use_graph = use_graph != 0;
  return CANS_OK;
}

extern "C" int cans_run_set_adjoint_df64(cans_run *h, int on) {
  if (!h) return CANS_ERR_ARG;
  h->adj_df = on != 0;
  return CANS_OK;
}

extern "C" int cans_run_set_tile(cans_run *h, int tile) {
  if (!h || tile < 0 || tile >= tile_count(h)) return CANS_ERR_ARG;
  if (h->tile != tile) {
    if (h->s) cudaStreamSynchronize(h->s);
    drop_graph(h);
    h->tile = tile;
  }
  return CANS_OK;
}

extern "C" int cans_run_set_df64(cans_run *h, int on) {
  if (!h) return CANS_ERR_ARG;
  if (on && ((h->d.solver != CANS_SOLVER_MLW_M3_2D && h->d.solver != CANS_SOLVER_MLW_M_3D &&
              h->d.solver != CANS_SOLVER_MLW_M_1D && h->d.solver != CANS_SOLVER_MLW_M_BG_1D &&
              !is_roe(h) && !is_hlld(h)) ||
             h->d.exact || h->grav || h->eta))
    return CANS_ERR_ARG;
  if (h->df != (on != 0)) {
    if (h->s) cudaStreamSynchronize(h->s);
    drop_graph(h);
    h->df = on != 0;
    h->tile = 0;
  }
  return CANS_OK;
}

extern "C" int cans_run_query(cans_run *h, cans_run_state *st) {
  if (!h || !st) return CANS_ERR_ARG;
  int rc = read_ctl(h);
  if (rc) return rc;
  const Ctl &c = h->host_ctl;
  st->t = c.t;
  st->dt = c.dt;
  st->ns = c.ns;
  st->nexec = c.nexec;
  st->merr = c.merr;
  st->done = c.done;
  st->pause = c.pause;
  st->n_floor = (long long)c.nfloor;
  st->n_bad = c.nonfinite;
  return c.merr ? c.merr : CANS_OK;
}

extern "C" int cans_run_resume(cans_run *h) {
  if (!h) return CANS_ERR_ARG;
  int zero = 0;
  CK(cudaMemcpyAsync(&h->ctl->pause, &zero, sizeof zero, cudaMemcpyHostToDevice,
                     h->s));
  // the iteration after the output starts now (a no-op when the loop ended)
  CK(launch_prepare(h->ctl, h->s));
  CK(cudaStreamSynchronize(h->s));
  return CANS_OK;
}

extern "C" int cans_run_step(cans_run *h, const double *dt, int apply_bc) {
  NvtxRange nvtx("cans_run_step");
  if (!h || !dt) return CANS_ERR_ARG;
  int rc = read_ctl(h);
  if (rc) return rc;
  if (h->ndim == 1) {  // in place; the boundary program needs the loop kernel
    if (apply_bc) return CANS_ERR_ARG;
    CK(launch_1d(h, 1, 1, *dt, 0));
    CK(cudaStreamSynchronize(h->s));
    return CANS_OK;
  }
  const int cur = h->host_ctl.cur;
  CK(step_kernel(h, h->tile, h->buf[cur], h->buf[cur ^ 1], *dt, nullptr, Box3{}));
  if (apply_bc) CK(bc_kernels(h, h->buf[cur ^ 1], nullptr));
  // flip the current buffer on the device copy of the control block
  const int nc = cur ^ 1;
  CK(cudaMemcpyAsync(&h->ctl->cur, &nc, sizeof nc, cudaMemcpyHostToDevice,
                     h->s));
  h->host_ctl.cur = nc;
  CK(cudaStreamSynchronize(h->s));
  return CANS_OK;
}

extern "C" int cans_run_cfl(cans_run *h, double safety, double *dt) {
  NvtxRange nvtx("cans_run_cfl");
  if (!h || !dt) return CANS_ERR_ARG;
  int rc = read_ctl(h);
  if (rc) return rc;
  unsigned long long *bits = &h->ctl->cfl_bits;
  const unsigned long long save = h->host_ctl.cfl_bits;
  const unsigned long long init = r4_1e20_bits();
  CK(cudaMemcpyAsync(bits, &init, sizeof init, cudaMemcpyHostToDevice, h->s));
  if (h->ndim == 1)
    CK(launch_cfl1d(h->d.exact != 0, h->buf[0], h->bx1, h->d.ix, h->ax.a, h->ph,
                    safety, bits, h->s));
  else
    CK(cfl_full_kernel(h, h->buf[h->host_ctl.cur], safety, bits));
  unsigned long long out = 0;
  CK(cudaMemcpyAsync(&out, bits, sizeof out, cudaMemcpyDeviceToHost, h->s));
  CK(cudaMemcpyAsync(bits, &save, sizeof save, cudaMemcpyHostToDevice, h->s));
  CK(cudaStreamSynchronize(h->s));
  *dt = bits_to_double(out);
  return CANS_OK;
}

extern "C" int cans_run_profile(cans_run *h, int iters, double *step_ms,
                                double *iter_ms) {
  if (!h || iters < 1 || !step_ms || !iter_ms) return CANS_ERR_ARG;
  if (h->ndim == 1) {  // one launch runs every iteration
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, h->s));
    CK(launch_1d(h, iters, 0, 0.0, 0));
    CK(cudaEventRecord(b, h->s));
    CK(cudaEventSynchronize(b));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *step_ms = ms;
    *iter_ms = ms;
    return CANS_OK;
  }
  std::vector<cudaEvent_t> ev(3 * (size_t)iters);
  for (auto &e : ev) CK(cudaEventCreate(&e));
  const Box3 box = inner_box(h);
  for (int k = 0; k < iters; k++) {
    CK(cudaEventRecord(ev[3 * k], h->s));
    CK(step_kernel(h, h->tile, nullptr, nullptr, 0.0, h->ctl, box));
    CK(cudaEventRecord(ev[3 * k + 1], h->s));
    CK(bc_kernels(h, nullptr, h->ctl));
    CK(frame_kernel(h));
    CK(cudaEventRecord(ev[3 * k + 2], h->s));
  }
  CK(cudaStreamSynchronize(h->s));
  double s1 = 0.0, s2 = 0.0;
  for (int k = 0; k < iters; k++) {
    float a = 0.f, b = 0.f;
    CK(cudaEventElapsedTime(&a, ev[3 * k], ev[3 * k + 1]));
    CK(cudaEventElapsedTime(&b, ev[3 * k], ev[3 * k + 2]));
    s1 += a;
    s2 += b;
  }
  for (auto &e : ev) cudaEventDestroy(e);
  *step_ms = s1;
  *iter_ms = s2;
  return CANS_OK;
}

extern "C" int cans_run_autotune(cans_run *h, int trial_steps, int *tile) {
  NvtxRange nvtx("cans_run_autotune");
  if (!h || trial_steps < 1) return CANS_ERR_ARG;
  if (h->ndim == 1) {  // a single configuration
    if (tile) *tile = 0;
    return CANS_OK;
  }
  int rc = read_ctl(h);
  if (rc) return rc;
  const int cur = h->host_ctl.cur;
  // the timing steps write only the other buffer, so the current state
  // is left as it is
  double dt = 0.0;
  if ((rc = cans_run_cfl(h, 0.4, &dt))) return rc;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_tile = h->tile;
  for (int t = 0; t < tile_count(h); t++) {
    CK(step_kernel(h, t, h->buf[cur], h->buf[cur ^ 1], dt, nullptr, Box3{}));
    CK(cudaEventRecord(e0, h->s));
    for (int k = 0; k < trial_steps; k++)
      CK(step_kernel(h, t, h->buf[cur], h->buf[cur ^ 1], dt, nullptr, Box3{}));
    CK(cudaEventRecord(e1, h->s));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) {
      best = ms;
      best_tile = t;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best_tile != h->tile) {
    h->tile = best_tile;
    drop_graph(h);
  }
  if (tile) *tile = best_tile;
  return CANS_OK;
}

// ---------------------------------------------------------------------------
// Reverse sweep of the 2-D mlw_m3 run (discrete adjoint) with binomial
// checkpointing.  The state of step k+1 is BC(step(P_k, dt_k)); dt is the
// frozen sequence of the forward run.  The run's current state is P_0 and is
// left unchanged.

namespace {

struct AdjWork {
  size_t n9 = 0;
  double *w[2] = {nullptr, nullptr};  // forward ping-pong buffers
  double *R = nullptr;                // raw output of the recorded step
  double *next = nullptr;             // filled state after the step being reversed
  long long next_k = -1;              // its step index (-1: none)
  double *lam[2] = {nullptr, nullptr};
  double *snap = nullptr;             // nsnap states
  double *scr = nullptr;              // adjoint-kernel scratch
  double *J = nullptr;                // objective (device)
  unsigned long long *bits = nullptr;
  int nsnap = 0;
  std::vector<void *> owned;
  ~AdjWork() {
    for (void *p : owned) cudaFree(p);
  }
  int alloc(double **p, size_t nd) {
    CK(cudaMalloc(p, sizeof(double) * nd));
    owned.push_back(*p);
    return CANS_OK;
  }
};

// the adjoint is that of the plain mlw_m3 step and boundary fill: no
// gravity, no resistivity, no chkdav floor
bool adj_supported(const cans_run *h) {
  return h->d.solver == CANS_SOLVER_MLW_M3_2D && !h->grav && !h->eta && !h->d.chkdav &&
         !h->df;
}

int adj_setup(cans_run *h, AdjWork &W, int nsnap) {
  W.n9 = h->n * (size_t)h->nvar;
  W.nsnap = nsnap;
  int rc;
  for (int b = 0; b < 2; b++) {
    if ((rc = W.alloc(&W.w[b], W.n9))) return rc;
    if ((rc = W.alloc(&W.lam[b], W.n9))) return rc;
  }
  if ((rc = W.alloc(&W.R, W.n9))) return rc;
  if (nsnap > 0 && (rc = W.alloc(&W.next, W.n9))) return rc;
  if (nsnap > 0 && (rc = W.alloc(&W.snap, W.n9 * (size_t)nsnap))) return rc;
  if ((rc = W.alloc(&W.scr, adj2d_scratch_doubles(h->n)))) return rc;
  if ((rc = W.alloc(&W.J, 1))) return rc;
  double *b = nullptr;
  if ((rc = W.alloc(&b, 1))) return rc;
  W.bits = reinterpret_cast<unsigned long long *>(b);
  return CANS_OK;
}

// Advance `steps` steps from the state A (not modified) starting at step k0;
// the result ends in W.w[*which].
int adj_advance(cans_run *h, AdjWork &W, const double *A, long long k0,
                long long steps, const double *dts, int *which,
                long long *nfwd) {
  const double *src = A;
  int cur = 0;
  for (long long k = 0; k < steps; k++) {
    double *dst = W.w[cur];
    CK(step_kernel(h, h->tile, src, dst, dts[k0 + k], nullptr, Box3{}));
    CK(bc_kernels(h, dst, nullptr));
    src = dst;
    cur ^= 1;
    (*nfwd)++;
  }
  *which = steps > 0 ? (cur ^ 1) : -1;
  return CANS_OK;
}

// Optimal binomial schedule: F(l, c) = minimal forward steps to reverse l
// steps from a stored start with c free snapshots (Griewank's treeverse
// recursion, solved by dynamic programming), and the first split of each.
// `leaf` is the forward cost of reversing one step from its stored input: 1
// when the step is re-run for its raw output, 0 when that output is rebuilt
// from the state after it.
struct Plan {
  int L = 0, C = 0, leaf = -1;
  std::vector<long long> F;
  std::vector<int> split;
  long long &f(int l, int c) { return F[(size_t)l * (C + 1) + c]; }
  int &s(int l, int c) { return split[(size_t)l * (C + 1) + c]; }
  void build(int L_, int C_, int leaf_) {
    L = L_;
    C = C_;
    leaf = leaf_;
    F.assign((size_t)(L + 1) * (C + 1), 0);
    split.assign((size_t)(L + 1) * (C + 1), 0);
    for (int l = 1; l <= L; l++) f(l, 0) = (long long)l * (l - 1) / 2 + (long long)l * leaf;
    for (int c = 1; c <= C; c++) {
      f(1, c) = leaf;
      for (int l = 2; l <= L; l++) {
        long long best = -1;
        int bm = 1;
        for (int m = 1; m < l; m++) {
          const long long v = m + f(l - m, c - 1) + f(m, c);
          if (best < 0 || v < best) {
            best = v;
            bm = m;
          }
        }
        f(l, c) = best;
        s(l, c) = bm;
      }
    }
  }
};

struct AdjRun {
  cans_run *h;
  AdjWork &W;
  Plan &P;
  const double *dts;
  long long L;
  long long nfwd = 0;
  bool have_J = false;
  bool merge = false;  // raw outputs from consecutive states (no re-run)
};

// The raw output of step k is the next filled state inside and the state k
// on the outer layer when the boundary program only rewrites that layer:
// margin 1 and no bdsmn* rule (which also zeroes the boundary cell).
bool adj_can_merge(const cans_run *h) {
  if (h->bc.margin != 1) return false;
  for (int v = 0; v < h->nvar; v++)
    for (int f = 0; f < 4; f++)
      if (h->bc.kind[v][f] == BD_SMN) return false;
  return true;
}

// Reverse steps [a, b): on entry W.lam[0] is the adjoint of the filled state
// b, on exit that of state a.  The state a is in snapshot `slot`.
int adj_reverse(AdjRun &r, long long a, long long b, int slot, int free_snaps) {
  cans_run *h = r.h;
  AdjWork &W = r.W;
  const size_t n9 = W.n9;
  const double *Sa = W.snap + n9 * (size_t)slot;
  const long long l = b - a;
  if (l == 1) {
    // raw output R of step a: rebuilt from the states a and a+1 when the
    // reverse sweep has just left state a+1, else by re-running the step
    if (r.merge && W.next_k == b) {
      CK(launch_adj2d_merge(W.next, Sa, W.R, h->nvar, h->d.ix, h->d.jx, h->s));
    } else {
      CK(step_kernel(h, h->tile, Sa, W.R, r.dts[a], nullptr, Box3{}));
      r.nfwd++;
    }
    if (b == r.L && !r.have_J) {  // J and its gradient on the final state
      CK(launch_adj2d_objective(W.R, W.lam[0], W.J, W.scr, h->d.ix, h->d.jx, h->ax.a,
                                h->ay.a, h->ph, h->s));
      r.have_J = true;
    }
    CK(launch_bc2d_transpose(h->nvar, W.lam[0], h->d.ix, h->d.jx, h->ax.a, h->ay.a,
                             h->bc, h->s));
    CK(launch_adj2d_step(Sa, W.R, W.lam[0], W.lam[1], W.scr, h->d.ix, h->d.jx, h->ax.a,
                         h->ay.a, h->ph, r.dts[a], h->adj_df, h->s));
    std::swap(W.lam[0], W.lam[1]);
    if (r.merge) {  // state a is the next one of the step reversed after this
      CK(cudaMemcpyAsync(W.next, Sa, sizeof(double) * n9, cudaMemcpyDeviceToDevice, h->s));
      W.next_k = a;
    }
    return CANS_OK;
  }
  if (free_snaps == 0) {  // recompute from a for every step, last first
    for (long long k = b - 1; k >= a; k--) {
      if (k == a) {
        int rc = adj_reverse(r, a, a + 1, slot, 0);
        if (rc) return rc;
        break;
      }
      // place state k in the scratch slot past the stored ones
      int which = -1;
      int rc = adj_advance(h, W, Sa, a, k - a, r.dts, &which, &r.nfwd);
      if (rc) return rc;
      const int tmp = W.nsnap - 1;
      CK(cudaMemcpyAsync(W.snap + n9 * (size_t)tmp, W.w[which], sizeof(double) * n9,
                         cudaMemcpyDeviceToDevice, h->s));
      rc = adj_reverse(r, k, k + 1, tmp, 0);
      if (rc) return rc;
    }
    return CANS_OK;
  }
  const int m = r.P.s((int)l, free_snaps);
  int which = -1;
  int rc = adj_advance(h, W, Sa, a, m, r.dts, &which, &r.nfwd);
  if (rc) return rc;
  const int ns = slot + 1;  // snapshots are used as a stack
  CK(cudaMemcpyAsync(W.snap + n9 * (size_t)ns, W.w[which], sizeof(double) * n9,
                     cudaMemcpyDeviceToDevice, h->s));
  if ((rc = adj_reverse(r, a + m, b, ns, free_snaps - 1))) return rc;
  return adj_reverse(r, a, a + m, slot, free_snaps);
}

}  // namespace

extern "C" int cans_run_record_dts(cans_run *h, long long nsteps, double safety,
                                   double *dts, double *J) {
  NvtxRange nvtx("cans_run_record_dts");
  if (!h || nsteps < 1 || !dts || !adj_supported(h)) return CANS_ERR_ARG;
  int rc = read_ctl(h);
  if (rc) return rc;
  AdjWork W;
  if ((rc = adj_setup(h, W, 0))) return rc;
  const double *src = h->buf[h->host_ctl.cur];
  int cur = 0;
  const unsigned long long init = r4_1e20_bits();
  for (long long k = 0; k < nsteps; k++) {
    CK(cudaMemcpyAsync(W.bits, &init, sizeof init, cudaMemcpyHostToDevice, h->s));
    CK(cfl_full_kernel(h, src, safety, W.bits));
    unsigned long long out = 0;
    CK(cudaMemcpyAsync(&out, W.bits, sizeof out, cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    dts[k] = bits_to_double(out);
    CK(step_kernel(h, h->tile, src, W.w[cur], dts[k], nullptr, Box3{}));
    CK(bc_kernels(h, W.w[cur], nullptr));
    src = W.w[cur];
    cur ^= 1;
  }
  if (J) {
    CK(launch_adj2d_objective(src, nullptr, W.J, W.scr, h->d.ix, h->d.jx, h->ax.a,
                              h->ay.a, h->ph, h->s));
    CK(cudaMemcpyAsync(J, W.J, sizeof(double), cudaMemcpyDeviceToHost, h->s));
  }
  CK(cudaStreamSynchronize(h->s));
  return CANS_OK;
}

extern "C" int cans_run_objective(cans_run *h, long long nsteps, const double *dts,
                                  double *J) {
  NvtxRange nvtx("cans_run_objective");
  if (!h || nsteps < 1 || !dts || !J || !adj_supported(h)) return CANS_ERR_ARG;
  int rc = read_ctl(h);
  if (rc) return rc;
  AdjWork W;
  if ((rc = adj_setup(h, W, 0))) return rc;
  int which = -1;
  long long nf = 0;
  if ((rc = adj_advance(h, W, h->buf[h->host_ctl.cur], 0, nsteps, dts, &which, &nf)))
    return rc;
  CK(launch_adj2d_objective(W.w[which], nullptr, W.J, W.scr, h->d.ix, h->d.jx, h->ax.a,
                            h->ay.a, h->ph, h->s));
  CK(cudaMemcpyAsync(J, W.J, sizeof(double), cudaMemcpyDeviceToHost, h->s));
  CK(cudaStreamSynchronize(h->s));
  return CANS_OK;
}

extern "C" int cans_run_av_record(cans_run *h, long long nsteps, const double *dts) {
  NvtxRange nvtx("cans_run_av_record");
  if (!h || nsteps < 1 || !dts || !adj_supported(h)) return CANS_ERR_ARG;
  const size_t per = 2 * h->n;
  if ((double)per * (double)nsteps > 64.0 * (1ull << 30)) return CANS_ERR_ARG;
  int rc = read_ctl(h);
  if (rc) return rc;
  if (h->avb_steps != nsteps) {
    CK(cudaStreamSynchronize(h->s));
    if (h->avb) cudaFree(h->avb);
    h->avb = nullptr;
    h->avb_steps = 0;
    CK(cudaMalloc(&h->avb, per * (size_t)nsteps));
  }
  AdjWork W;
  if ((rc = adj_setup(h, W, 0))) return rc;
  const double *src = h->buf[h->host_ctl.cur];
  int cur = 0;
  for (long long k = 0; k < nsteps; k++) {
    CK(launch_mlw2d_av(h->d.exact != 0, 1, src, W.w[cur], h->d.ix, h->d.jx, h->ax.a, h->ay.a,
                       h->ph, dts[k], h->avb + per * (size_t)k, nullptr, h->s));
    CK(bc_kernels(h, W.w[cur], nullptr));
    src = W.w[cur];
    cur ^= 1;
  }
  CK(cudaStreamSynchronize(h->s));
  h->avb_steps = nsteps;
  return CANS_OK;
}

extern "C" int cans_run_av_branches(cans_run *h, long long step, unsigned char *out) {
  if (!h || !out || !h->avb || step < 0 || step >= h->avb_steps) return CANS_ERR_ARG;
  const size_t per = 2 * h->n;
  CK(cudaMemcpyAsync(out, h->avb + per * (size_t)step, per, cudaMemcpyDeviceToHost, h->s));
  CK(cudaStreamSynchronize(h->s));
  return CANS_OK;
}

extern "C" int cans_run_objective_frozen_av(cans_run *h, long long nsteps, const double *dts,
                                            double *J, long long *nflip) {
  NvtxRange nvtx("cans_run_objective_frozen_av");
  if (!h || nsteps < 1 || !dts || !J || !adj_supported(h)) return CANS_ERR_ARG;
  if (!h->avb || nsteps > h->avb_steps) return CANS_ERR_ARG;
  int rc = read_ctl(h);
  if (rc) return rc;
  AdjWork W;
  if ((rc = adj_setup(h, W, 0))) return rc;
  const size_t per = 2 * h->n;
  CK(cudaMemsetAsync(W.bits, 0, sizeof(unsigned long long), h->s));
  const double *src = h->buf[h->host_ctl.cur];
  int cur = 0;
  for (long long k = 0; k < nsteps; k++) {
    CK(launch_mlw2d_av(h->d.exact != 0, 2, src, W.w[cur], h->d.ix, h->d.jx, h->ax.a, h->ay.a,
                       h->ph, dts[k], h->avb + per * (size_t)k, W.bits, h->s));
    CK(bc_kernels(h, W.w[cur], nullptr));
    src = W.w[cur];
    cur ^= 1;
  }
  CK(launch_adj2d_objective(src, nullptr, W.J, W.scr, h->d.ix, h->d.jx, h->ax.a, h->ay.a,
                            h->ph, h->s));
  unsigned long long flips = 0;
  CK(cudaMemcpyAsync(J, W.J, sizeof(double), cudaMemcpyDeviceToHost, h->s));
  CK(cudaMemcpyAsync(&flips, W.bits, sizeof flips, cudaMemcpyDeviceToHost, h->s));
  CK(cudaStreamSynchronize(h->s));
  if (nflip) *nflip = (long long)flips;
  return CANS_OK;
}

extern "C" int cans_run_adjoint(cans_run *h, long long nsteps, const double *dts,
                                int nsnap, double *J, double *const *grad,
                                long long *nfwd) {
  NvtxRange nvtx("cans_run_adjoint");
  if (!h || nsteps < 1 || !dts || nsnap < 2 || !adj_supported(h)) return CANS_ERR_ARG;
  if (nsteps > (1LL << 20)) return CANS_ERR_ARG;
  int rc = read_ctl(h);
  if (rc) return rc;
  AdjWork W;
  // nsnap stored states: the start plus nsnap-2 free ones, and one scratch
  // slot for the no-free-snapshot case
  if ((rc = adj_setup(h, W, nsnap))) return rc;
  CK(cudaMemcpyAsync(W.snap, h->buf[h->host_ctl.cur], sizeof(double) * W.n9,
                     cudaMemcpyDeviceToDevice, h->s));
  static Plan plan;  // reused while (nsteps, nsnap) repeat
  const int free_snaps = nsnap - 2;
  const bool merge = adj_can_merge(h);
  if (plan.L != (int)nsteps || plan.C != free_snaps || plan.leaf != (merge ? 0 : 1))
    plan.build((int)nsteps, free_snaps, merge ? 0 : 1);
  AdjRun r{h, W, plan, dts, nsteps};
  r.merge = merge;
  if ((rc = adj_reverse(r, 0, nsteps, 0, free_snaps))) return rc;
  if (J) CK(cudaMemcpyAsync(J, W.J, sizeof(double), cudaMemcpyDeviceToHost, h->s));
  if (grad)
    for (int v = 0; v < h->nvar; v++)
      if (grad[v])
        CK(cudaMemcpyAsync(grad[v], W.lam[0] + v * h->n, sizeof(double) * h->n,
                           cudaMemcpyDeviceToHost, h->s));
  CK(cudaStreamSynchronize(h->s));
  if (nfwd) *nfwd = r.nfwd;
  return CANS_OK;
}

extern "C" int cans_run_bc_transpose(cans_run *h, double *const *arrays) {
  if (!h || !arrays || h->ndim != 2) return CANS_ERR_ARG;
  const size_t n = h->n;
  double *d = nullptr;
  CK(cudaMalloc(&d, sizeof(double) * n * h->nvar));
  for (int v = 0; v < h->nvar; v++)
    CK(cudaMemcpyAsync(d + v * n, arrays[v], sizeof(double) * n, cudaMemcpyHostToDevice,
                       h->s));
  cudaError_t e = launch_bc2d_transpose(h->nvar, d, h->d.ix, h->d.jx, h->ax.a, h->ay.a,
                                        h->bc, h->s);
  for (int v = 0; v < h->nvar && e == cudaSuccess; v++)
    e = cudaMemcpyAsync(arrays[v], d + v * n, sizeof(double) * n, cudaMemcpyDeviceToHost,
                        h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  cudaFree(d);
  if (e != cudaSuccess) return fail_cuda(e, "cans_run_bc_transpose");
  return CANS_OK;
}
