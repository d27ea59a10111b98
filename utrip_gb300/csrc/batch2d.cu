// Many independent 2-D runs advanced together (sm_103a, FP64).
//
// A parameter sweep runs the same 2-D model (for example the magnetised shear
// layer of cans2d/md_mhdkh/hdmlw/model.f) for many grid sizes and plasma
// betas.  Run one at a time, a small grid fills a fraction of the 152 SMs and
// every step pays the launch latency of its kernels.  Here one loop iteration
// of every run is four launches in total:
//   1. a persistent step kernel: one block per resident slot; each block pulls
//      (run, tile) work items from a device work queue and applies the same
//      fused tile step as the single-run kernel (mlw2d_tile.cuh), with the
//      run's own arrays, metrics, dt and CFL accumulator;
//   2.-3. the boundary programs of all runs, x faces then y faces;
//   4. the frame CFL of each run (one block per run), the loop bookkeeping of
//      each run (finish_iteration), and the reset of the work queue.
// Each run keeps its own dt, t, ns and termination exactly as if it ran
// alone, so the results equal single-run results bit for bit.  The four
// launches are captured in a CUDA graph; the tile shape and the cells per
// thread are picked by timing (cans_batch_autotune).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "bc_line.cuh"
#include "cans_common.cuh"
#include "cans_gpu.h"
#include "cans_internal.h"
#include "mlw2d_tile.cuh"

namespace cans {

// Device description of one run of the batch.
struct BatchGrid {
  Ctl *ctl;
  Axis ax, ay;
  Phys ph;
  Box3 box;       // cells whose CFL the step kernel reduces
  int ix, jx;
  int ntx, nty;   // tiles of the current configuration
  int tile0;      // first work item of this run
};

// Step of every run: persistent blocks pull work items until the queue is
// exhausted.
template <bool E, bool M3, int TX, int TY, int RPT>
__global__ void __launch_bounds__(TX *TY / RPT, 1)
    k_mlw2d_batch(const BatchGrid *__restrict__ grids, int ngrids, int nitems,
                  unsigned int *queue) {
  extern __shared__ double smem[];
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(queue, 1u);
    __syncthreads();
    const int item = s_item;
    __syncthreads();  // every thread has read s_item before it is rewritten
    if (item >= nitems) break;
    int lo = 0, hi = ngrids - 1;  // last run whose first item <= item
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (grids[mid].tile0 <= item) lo = mid;
      else hi = mid - 1;
    }
    const BatchGrid &G = grids[lo];
    Ctl *ctl = G.ctl;
    if (ctl->done | ctl->pause) continue;
    const int t = item - G.tile0;
    tile_step<E, M3, TX, TY, RPT>(ctl->buf[ctl->cur], ctl->buf[ctl->cur ^ 1], G.ix,
                                  G.jx, G.ax, G.ay, G.ph, ctl->dt, ctl->safety,
                                  &ctl->cfl_bits, G.box, t % G.ntx, t / G.ntx,
                                  G.ntx, G.nty, smem, nullptr, nullptr, &ctl->nonfinite);
  }
}

// Boundary program of one axis for every run: blockIdx.y is the run.
__global__ void k_bc_batch(const BatchGrid *__restrict__ grids,
                           const BcTable *__restrict__ tables, int nvar,
                           int axis) {
  const BatchGrid &G = grids[blockIdx.y];
  const Ctl *ctl = G.ctl;
  if (ctl->done | ctl->pause) return;
  double *S = ctl->buf[ctl->cur ^ 1];
  const BcTable &bc = tables[blockIdx.y];
  const int n0 = G.ix, n1 = G.jx;
  const int n = axis == 0 ? n0 : n1;
  const size_t stride = axis == 0 ? 1 : (size_t)n0;
  const long long nlines = (long long)n0 * n1 / n;
  const size_t nall = (size_t)n0 * n1;
  const double *dxm = axis == 0 ? G.ax.dm : G.ay.dm;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       t < nlines * nvar; t += (long long)gridDim.x * blockDim.x) {
    const int v = (int)(t / nlines);
    const long long line = t % nlines;
    double *q = S + (size_t)v * nall + line_base(axis, line, n0, n1);
    const int klo = bc.kind[v][2 * axis], khi = bc.kind[v][2 * axis + 1];
    if (klo >= 0) bd_line(klo, 0, bc.margin, bc.margin, q, n, stride, bc.q0[v][2 * axis], dxm);
    if (khi >= 0)
      bd_line(khi, 1, bc.margin, bc.margin, q, n, stride, bc.q0[v][2 * axis + 1], dxm);
  }
}

// Frame CFL and loop bookkeeping of every run (one block per run), then the
// reset of the work queue for the next step.
template <bool E, bool M3>
__global__ void k_frame_batch(const BatchGrid *__restrict__ grids, int margin,
                              unsigned int *queue) {
  using FT = F<E>;
  using P = Prim<M3>;
  __shared__ double red[32];
  if (blockIdx.x == 0 && threadIdx.x == 0) *queue = 0u;
  const BatchGrid &G = grids[blockIdx.x];
  Ctl *ctl = G.ctl;
  if (ctl->done | ctl->pause) return;
  const double *S = ctl->buf[ctl->cur ^ 1];
  const int ix = G.ix, jx = G.jx, w = margin + 1;
  const size_t n = (size_t)ix * jx;
  const long long nrow = 2LL * w * ix;
  const long long total = nrow + (jx - 2LL * w) * 2LL * w;
  const FT gm(G.ph.gm), pi4i(G.ph.pi4i), safety(ctl->safety);
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  bool bad = false;
  for (long long f = threadIdx.x; f < total; f += blockDim.x) {
    int i, j;
    if (f < nrow) {
      const long long r = f / ix;
      i = (int)(f % ix);
      j = (r < w) ? (int)r : (int)(jx - 2 * w + r);
    } else {
      const long long q = f - nrow;
      j = (int)(w + q / (2 * w));
      const int c = (int)(q % (2 * w));
      i = (c < w) ? c : (ix - 2 * w + c);
    }
    const size_t g = (size_t)i + (size_t)j * ix;
    const FT ro(S[P::RO * n + g]), pr(S[P::PR * n + g]);
    const FT vx(S[P::VX * n + g]), vy(S[P::VY * n + g]);
    const FT bx(S[P::BX * n + g]), by(S[P::BY * n + g]);
    FT b2, v2;
    if constexpr (M3) {
      const FT vz(S[P::VZ * n + g]), bz(S[P::BZ * n + g]);
      b2 = bx * bx + by * by + bz * bz;
      v2 = vx * vx + vy * vy + vz * vz;
    } else {
      b2 = bx * bx + by * by;
      v2 = vx * vx + vy * vy;
    }
    const FT ca2 = b2 * pi4i / ro;
    const FT cs2 = gm * pr / ro;
    const FT dtcfl = fmin_(FT(G.ax.d[i]), FT(G.ay.d[j])) / fsqrt(v2 + cs2 + ca2);
    const double dtq = (safety * dtcfl).v;
    if (dtq < dmin) dmin = dtq;
    bad |= bad_cell(ro.v, pr.v, dtq);
  }
  count_bad_block(bad, &ctl->nonfinite, threadIdx.x);
  block_min_to(&ctl->cfl_bits, dmin, red, threadIdx.x, blockDim.x);
  __syncthreads();
  if (threadIdx.x == 0) finish_iteration(ctl);
}

// Start of every run (the first CFL is reduced into cfl_bits beforehand).
__global__ void k_prepare_batch(const BatchGrid *__restrict__ grids, int ngrids) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngrids) return;
  Ctl *ctl = grids[g].ctl;
  if (ctl->done || ctl->pause) return;
  start_iteration(ctl);
}

// ---------------------------------------------------------------------------
// Configurations the autotuner chooses from: tile shape and cells per thread.
struct BatchConfig {
  int tx, ty, rpt;
};
static const BatchConfig kConfigs[] = {
    {32, 8, 2}, {32, 8, 1}, {32, 16, 2}, {16, 16, 2}, {32, 16, 4}, {64, 8, 2}};
constexpr int kNumConfigs = sizeof(kConfigs) / sizeof(kConfigs[0]);

template <bool E, bool M3, int TX, int TY, int RPT>
static cudaError_t launch_batch_cfg(const BatchGrid *grids, int ngrids, int nitems,
                                    unsigned int *queue, cudaStream_t s) {
  using T = Tile<TX, TY, M3, RPT>;
  static int resident = 0;  // per template instance
  auto kern = k_mlw2d_batch<E, M3, TX, TY, RPT>;
  if (resident == 0) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)T::smem_bytes);
    if (e != cudaSuccess) return e;
    int per_sm = 0, dev = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, T::NT, T::smem_bytes);
    if (e != cudaSuccess) return e;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    resident = (per_sm > 0 ? per_sm : 1) * sms;
  }
  const int blocks = resident < nitems ? resident : nitems;
  kern<<<blocks > 0 ? blocks : 1, T::NT, T::smem_bytes, s>>>(grids, ngrids, nitems, queue);
  count_launch();
  return cudaGetLastError();
}

template <bool E, bool M3>
static cudaError_t launch_batch(int cfg, const BatchGrid *grids, int ngrids,
                                int nitems, unsigned int *queue, cudaStream_t s) {
  switch (cfg) {
    case 1: return launch_batch_cfg<E, M3, 32, 8, 1>(grids, ngrids, nitems, queue, s);
    case 2: return launch_batch_cfg<E, M3, 32, 16, 2>(grids, ngrids, nitems, queue, s);
    case 3: return launch_batch_cfg<E, M3, 16, 16, 2>(grids, ngrids, nitems, queue, s);
    case 4: return launch_batch_cfg<E, M3, 32, 16, 4>(grids, ngrids, nitems, queue, s);
    case 5: return launch_batch_cfg<E, M3, 64, 8, 2>(grids, ngrids, nitems, queue, s);
    default: return launch_batch_cfg<E, M3, 32, 8, 2>(grids, ngrids, nitems, queue, s);
  }
}

}  // namespace cans

using namespace cans;

namespace {

thread_local std::string g_batch_error;
int bfail(cudaError_t e, const char *where) {
  g_batch_error = std::string(where) + ": " + cudaGetErrorString(e);
  return CANS_ERR_CUDA;
}
#define BK(call)                                            \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return bfail(_e, #call);         \
  } while (0)

unsigned long long r4_1e20() {
  const double d = (double)1.e20f;
  unsigned long long b;
  std::memcpy(&b, &d, sizeof b);
  return b;
}

}  // namespace

struct cans_batch {
  int ngrids = 0, solver = 1, nvar = 9, exact = 0, config = 0, margin = 1;
  cudaStream_t s = nullptr;
  bool own_stream = false;
  struct Grid {
    int ix = 0, jx = 0;
    size_t n = 0;
    double *buf[2] = {nullptr, nullptr};
    double *metrics = nullptr;  // d, dm, di, dim, u0, u1 of x then of y
    Ctl *ctl = nullptr;
    BcTable bc{};
    Phys ph{};
    Axis ax, ay;
    int stop_on_bad = 0;
  };
  std::vector<Grid> g;
  std::vector<BatchGrid> hgrids;
  BatchGrid *d_grids = nullptr;
  BcTable *d_bc = nullptr;
  unsigned int *d_queue = nullptr;
  int nitems = 0, max_lines = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_iters = 0, graph_nodes = 0;
};

namespace {

void drop_graph(cans_batch *b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_iters = 0;
}

// Tiles of every run under the current configuration, uploaded with the
// run descriptions and boundary tables.
int sync_tables(cans_batch *b) {
  const BatchConfig c = kConfigs[b->config];
  int item = 0, maxl = 0;
  b->hgrids.resize(b->ngrids);
  for (int r = 0; r < b->ngrids; r++) {
    auto &G = b->g[r];
    BatchGrid &H = b->hgrids[r];
    H.ctl = G.ctl;
    H.ax = G.ax;
    H.ay = G.ay;
    H.ph = G.ph;
    const int w = b->margin + 1;
    H.box = Box3{{w, w, 0}, {G.ix - 1 - w, G.jx - 1 - w, 0}};
    H.ix = G.ix;
    H.jx = G.jx;
    H.ntx = (G.ix - 2 + c.tx - 1) / c.tx;
    H.nty = (G.jx - 2 + c.ty - 1) / c.ty;
    H.tile0 = item;
    item += H.ntx * H.nty;
    maxl = std::max(maxl, std::max(G.ix, G.jx) * b->nvar);
  }
  b->nitems = item;
  b->max_lines = maxl;
  std::vector<BcTable> bcs(b->ngrids);
  for (int r = 0; r < b->ngrids; r++) bcs[r] = b->g[r].bc;
  BK(cudaMemcpyAsync(b->d_grids, b->hgrids.data(), sizeof(BatchGrid) * b->ngrids,
                     cudaMemcpyHostToDevice, b->s));
  BK(cudaMemcpyAsync(b->d_bc, bcs.data(), sizeof(BcTable) * b->ngrids,
                     cudaMemcpyHostToDevice, b->s));
  BK(cudaStreamSynchronize(b->s));
  drop_graph(b);
  return CANS_OK;
}

int step_launch(cans_batch *b, int cfg) {
  const bool m3 = b->solver == CANS_SOLVER_MLW_M3_2D;
  cudaError_t e;
  if (b->exact)
    e = m3 ? launch_batch<true, true>(cfg, b->d_grids, b->ngrids, b->nitems, b->d_queue, b->s)
           : launch_batch<true, false>(cfg, b->d_grids, b->ngrids, b->nitems, b->d_queue, b->s);
  else
    e = m3 ? launch_batch<false, true>(cfg, b->d_grids, b->ngrids, b->nitems, b->d_queue, b->s)
           : launch_batch<false, false>(cfg, b->d_grids, b->ngrids, b->nitems, b->d_queue, b->s);
  BK(e);
  return CANS_OK;
}

int enqueue_batch_iteration(cans_batch *b) {
  int rc = step_launch(b, b->config);
  if (rc) return rc;
  const int bx = (b->max_lines + 255) / 256;
  for (int axis = 0; axis < 2; axis++) {
    k_bc_batch<<<dim3(bx, b->ngrids), 256, 0, b->s>>>(b->d_grids, b->d_bc, b->nvar, axis);
    count_launch();
    BK(cudaGetLastError());
  }
  const bool m3 = b->solver == CANS_SOLVER_MLW_M3_2D;
  if (b->exact) {
    if (m3) k_frame_batch<true, true><<<b->ngrids, 256, 0, b->s>>>(b->d_grids, b->margin, b->d_queue);
    else k_frame_batch<true, false><<<b->ngrids, 256, 0, b->s>>>(b->d_grids, b->margin, b->d_queue);
  } else {
    if (m3) k_frame_batch<false, true><<<b->ngrids, 256, 0, b->s>>>(b->d_grids, b->margin, b->d_queue);
    else k_frame_batch<false, false><<<b->ngrids, 256, 0, b->s>>>(b->d_grids, b->margin, b->d_queue);
  }
  count_launch();
  BK(cudaGetLastError());
  return CANS_OK;
}

int read_ctl(cans_batch *b, int r, Ctl *out) {
  BK(cudaMemcpyAsync(out, b->g[r].ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, b->s));
  BK(cudaStreamSynchronize(b->s));
  return CANS_OK;
}

}  // namespace

extern "C" int cans_batch_destroy(cans_batch *b) {
  if (!b) return CANS_ERR_ARG;
  if (b->s) cudaStreamSynchronize(b->s);
  drop_graph(b);
  for (auto &G : b->g) {
    for (int k = 0; k < 2; k++)
      if (G.buf[k]) cudaFree(G.buf[k]);
    if (G.metrics) cudaFree(G.metrics);
    if (G.ctl) cudaFree(G.ctl);
  }
  if (b->d_grids) cudaFree(b->d_grids);
  if (b->d_bc) cudaFree(b->d_bc);
  if (b->d_queue) cudaFree(b->d_queue);
  if (b->own_stream && b->s) cudaStreamDestroy(b->s);
  delete b;
  return CANS_OK;
}

extern "C" int cans_batch_create(cans_batch **out, int ngrids,
                                 const cans_run_desc *descs) {
  if (!out || ngrids < 1 || ngrids > 65535 || !descs) return CANS_ERR_ARG;
  const int solver = descs[0].solver;
  if (solver != CANS_SOLVER_MLW_M_2D && solver != CANS_SOLVER_MLW_M3_2D) return CANS_ERR_ARG;
  for (int r = 0; r < ngrids; r++) {
    const cans_run_desc &d = descs[r];
    const int wmin = 2 * (d.margin + 1) + 1;
    if (d.solver != solver || d.margin != descs[0].margin || d.exact != descs[0].exact ||
        d.ix < wmin || d.jx < wmin || d.kx != 1 || !d.dx || !d.dxm || !d.dy || !d.dym)
      return CANS_ERR_ARG;
    // the batch runs the plain mlw_m / mlw_m3 step: no source-term variant
    if (d.gx || d.et || d.etm) return CANS_ERR_ARG;
  }
  auto *b = new cans_batch();
  b->ngrids = ngrids;
  b->solver = solver;
  b->nvar = solver == CANS_SOLVER_MLW_M3_2D ? 9 : 7;
  b->exact = descs[0].exact;
  b->margin = descs[0].margin;
  b->g.resize(ngrids);
  auto bail = [&](int rc) {
    cans_batch_destroy(b);
    return rc;
  };
  cudaError_t e;
  if (descs[0].stream) {
    b->s = (cudaStream_t)descs[0].stream;
  } else {
    e = cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(bfail(e, "cudaStreamCreate"));
    b->own_stream = true;
  }
  std::vector<double> h;
  for (int r = 0; r < ngrids; r++) {
    const cans_run_desc &d = descs[r];
    auto &G = b->g[r];
    G.ix = d.ix;
    G.stop_on_bad = d.stop_on_bad ? 1 : 0;
    G.jx = d.jx;
    G.n = (size_t)d.ix * d.jx;
    G.ph = make_phys(d.gm, d.qav);
    G.bc.margin = d.margin;
    for (int v = 0; v < kMaxVar; v++)
      for (int f = 0; f < 6; f++) {
        G.bc.kind[v][f] = BD_NONE;
        G.bc.q0[v][f] = 0.0;
      }
    for (int k = 0; k < 2; k++) {
      e = cudaMalloc(&G.buf[k], sizeof(double) * G.n * b->nvar);
      if (e != cudaSuccess) return bail(bfail(e, "cudaMalloc(state)"));
      e = cudaMemsetAsync(G.buf[k], 0, sizeof(double) * G.n * b->nvar, b->s);
      if (e != cudaSuccess) return bail(bfail(e, "cudaMemset(state)"));
    }
    const size_t nm = 6 * (size_t)(d.ix + d.jx);
    e = cudaMalloc(&G.metrics, sizeof(double) * nm);
    if (e != cudaSuccess) return bail(bfail(e, "cudaMalloc(metrics)"));
    h.assign(nm, 0.0);
    double *hx = h.data(), *hy = h.data() + 6 * (size_t)d.ix;
    std::memcpy(hx, d.dx, sizeof(double) * d.ix);
    std::memcpy(hx + d.ix, d.dxm, sizeof(double) * d.ix);
    build_axis_host(d.ix, d.dx, d.dxm, hx + 2 * d.ix, hx + 3 * d.ix, hx + 4 * d.ix, hx + 5 * d.ix);
    std::memcpy(hy, d.dy, sizeof(double) * d.jx);
    std::memcpy(hy + d.jx, d.dym, sizeof(double) * d.jx);
    build_axis_host(d.jx, d.dy, d.dym, hy + 2 * d.jx, hy + 3 * d.jx, hy + 4 * d.jx, hy + 5 * d.jx);
    e = cudaMemcpyAsync(G.metrics, h.data(), sizeof(double) * nm, cudaMemcpyHostToDevice, b->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->s);
    if (e != cudaSuccess) return bail(bfail(e, "cudaMemcpy(metrics)"));
    double *mx = G.metrics, *my = G.metrics + 6 * (size_t)d.ix;
    G.ax.n = d.ix;
    G.ax.d = mx; G.ax.dm = mx + d.ix; G.ax.di = mx + 2 * d.ix; G.ax.dim = mx + 3 * d.ix;
    G.ax.u0 = mx + 4 * d.ix; G.ax.u1 = mx + 5 * d.ix;
    G.ay.n = d.jx;
    G.ay.d = my; G.ay.dm = my + d.jx; G.ay.di = my + 2 * d.jx; G.ay.dim = my + 3 * d.jx;
    G.ay.u0 = my + 4 * d.jx; G.ay.u1 = my + 5 * d.jx;
    e = cudaMalloc(&G.ctl, sizeof(Ctl));
    if (e != cudaSuccess) return bail(bfail(e, "cudaMalloc(ctl)"));
    Ctl c;
    std::memset(&c, 0, sizeof c);
    c.done = 1;
    c.buf[0] = G.buf[0];
    c.buf[1] = G.buf[1];
    e = cudaMemcpyAsync(G.ctl, &c, sizeof c, cudaMemcpyHostToDevice, b->s);
    if (e != cudaSuccess) return bail(bfail(e, "cudaMemcpy(ctl)"));
  }
  e = cudaMalloc(&b->d_grids, sizeof(BatchGrid) * ngrids);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_bc, sizeof(BcTable) * ngrids);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_queue, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned int), b->s);
  if (e != cudaSuccess) return bail(bfail(e, "cudaMalloc(batch tables)"));
  int rc = sync_tables(b);
  if (rc) return bail(rc);
  *out = b;
  return CANS_OK;
}

extern "C" int cans_batch_set_bc(cans_batch *b, int grid, int var, int face, int kind,
                                 double q0) {
  if (!b || grid < 0 || grid >= b->ngrids || var < 0 || var >= b->nvar || face < 0 ||
      face >= 4 || kind < CANS_BD_NONE || kind > CANS_BD_FRD)
    return CANS_ERR_ARG;
  b->g[grid].bc.kind[var][face] = kind;
  b->g[grid].bc.q0[var][face] = q0;
  return sync_tables(b);
}

extern "C" int cans_batch_push(cans_batch *b, int grid, double *const *host) {
  if (!b || grid < 0 || grid >= b->ngrids || !host) return CANS_ERR_ARG;
  Ctl c;
  int rc = read_ctl(b, grid, &c);
  if (rc) return rc;
  auto &G = b->g[grid];
  for (int v = 0; v < b->nvar; v++)
    BK(cudaMemcpyAsync(G.buf[c.cur] + v * G.n, host[v], sizeof(double) * G.n,
                       cudaMemcpyHostToDevice, b->s));
  BK(cudaStreamSynchronize(b->s));
  return CANS_OK;
}

extern "C" int cans_batch_pull(cans_batch *b, int grid, double *const *host) {
  if (!b || grid < 0 || grid >= b->ngrids || !host) return CANS_ERR_ARG;
  Ctl c;
  int rc = read_ctl(b, grid, &c);
  if (rc) return rc;
  auto &G = b->g[grid];
  for (int v = 0; v < b->nvar; v++)
    BK(cudaMemcpyAsync(host[v], G.buf[c.cur] + v * G.n, sizeof(double) * G.n,
                       cudaMemcpyDeviceToHost, b->s));
  BK(cudaStreamSynchronize(b->s));
  return CANS_OK;
}

extern "C" int cans_batch_start(cans_batch *b, double t0, double tend, long long nstop,
                                double safety, double dtmin) {
  NvtxRange nvtx("cans_batch_start");
  if (!b) return CANS_ERR_ARG;
  for (int r = 0; r < b->ngrids; r++) {
    auto &G = b->g[r];
    Ctl c;
    int rc = read_ctl(b, r, &c);
    if (rc) return rc;
    c.t = t0;
    c.tp = t0;
    c.tend = tend;
    c.nstop = nstop;
    c.safety = safety;
    c.dtmin = dtmin;
    c.dtout = 0.0;
    c.pause_on_output = 0;
    c.ns = 0;
    c.nexec = 0;
    c.merr = 0;
    c.done = 0;
    c.pause = 0;
    c.frame_blocks_done = 0;
    c.nonfinite = 0;
    c.nfloor = 0;
    c.stop_on_bad = G.stop_on_bad;
    c.cfl_bits = r4_1e20();
    BK(cudaMemcpyAsync(G.ctl, &c, sizeof c, cudaMemcpyHostToDevice, b->s));
    BK(launch_cfl2d_full(b->solver, b->exact != 0, G.buf[c.cur], G.ix, G.jx, G.ax, G.ay,
                         G.ph, safety, &G.ctl->cfl_bits, b->s));
  }
  k_prepare_batch<<<(b->ngrids + 127) / 128, 128, 0, b->s>>>(b->d_grids, b->ngrids);
  count_launch();
  BK(cudaGetLastError());
  BK(cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned int), b->s));
  BK(cudaStreamSynchronize(b->s));
  return CANS_OK;
}

extern "C" int cans_batch_advance(cans_batch *b, int iters, int use_graph) {
  NvtxRange nvtx("cans_batch_advance");
  if (!b || iters < 0) return CANS_ERR_ARG;
  if (!use_graph) {
    for (int k = 0; k < iters; k++) {
      int rc = enqueue_batch_iteration(b);
      if (rc) return rc;
    }
    return CANS_OK;
  }
  const int chunk = iters < 16 ? iters : 16;
  if (chunk == 0) return CANS_OK;
  if (!b->graph || b->graph_iters != chunk) {
    drop_graph(b);
    cudaGraph_t g = nullptr;
    const unsigned long long before = launch_count();
    BK(cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal));
    int rc = CANS_OK;
    for (int k = 0; k < chunk && rc == CANS_OK; k++) rc = enqueue_batch_iteration(b);
    cudaError_t e = cudaStreamEndCapture(b->s, &g);
    count_launch(-(int)(launch_count() - before));  // counted at replay
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return bfail(e, "cudaStreamEndCapture");
    size_t nn = 0;
    cudaGraphGetNodes(g, nullptr, &nn);
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(e, "cudaGraphInstantiate");
    b->graph_iters = chunk;
    b->graph_nodes = (int)nn;
  }
  int done = 0;
  while (done + chunk <= iters) {
    BK(cudaGraphLaunch(b->graph, b->s));
    count_launch(b->graph_nodes);
    done += chunk;
  }
  for (; done < iters; done++) {
    int rc = enqueue_batch_iteration(b);
    if (rc) return rc;
  }
  return CANS_OK;
}

extern "C" int cans_batch_query(cans_batch *b, int grid, cans_run_state *st) {
  if (!b || grid < 0 || grid >= b->ngrids || !st) return CANS_ERR_ARG;
  Ctl c;
  int rc = read_ctl(b, grid, &c);
  if (rc) return rc;
  st->t = c.t;
  st->dt = c.dt;
  st->ns = c.ns;
  st->nexec = c.nexec;
  st->merr = c.merr;
  st->done = c.done;
  st->pause = c.pause;
  st->n_floor = 0;
  st->n_bad = c.nonfinite;
  return CANS_OK;
}

extern "C" int cans_batch_configs(void) { return kNumConfigs; }

extern "C" int cans_batch_set_config(cans_batch *b, int config) {
  if (!b || config < 0 || config >= kNumConfigs) return CANS_ERR_ARG;
  b->config = config;
  return sync_tables(b);
}

extern "C" int cans_batch_autotune(cans_batch *b, int trial_steps, int *config) {
  if (!b || trial_steps < 1) return CANS_ERR_ARG;
  // Time the step kernel alone: it writes only each run's other buffer and
  // leaves the current states, times and dt unchanged.  Call after
  // cans_batch_start.
  cudaEvent_t e0, e1;
  BK(cudaEventCreate(&e0));
  BK(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_cfg = b->config;
  for (int c = 0; c < kNumConfigs; c++) {
    b->config = c;
    int rc = sync_tables(b);
    if (rc) return rc;
    BK(cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned int), b->s));
    if ((rc = step_launch(b, c))) return rc;  // warm-up
    BK(cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned int), b->s));
    BK(cudaEventRecord(e0, b->s));
    for (int k = 0; k < trial_steps; k++) {
      if ((rc = step_launch(b, c))) return rc;
      BK(cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned int), b->s));
    }
    BK(cudaEventRecord(e1, b->s));
    BK(cudaEventSynchronize(e1));
    float ms = 0.f;
    BK(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) {
      best = ms;
      best_cfg = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // the trial steps reduced the CFL of the state they wrote, which is the
  // state the first real step writes again: the minimum is unchanged
  b->config = best_cfg;
  int rc = sync_tables(b);
  if (rc) return rc;
  if (config) *config = best_cfg;
  return CANS_OK;
}
