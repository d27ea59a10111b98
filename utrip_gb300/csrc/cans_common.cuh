// Shared device-side definitions for the CANS mLW GPU library (sm_103a).
//
// Two arithmetic policies are compiled from one source:
//   exact (E=true)  every + - * / and sqrt is an explicitly rounded intrinsic
//                   (__dadd_rn, __dmul_rn, ...), so nothing is contracted into
//                   an FMA and the order written is the order executed.  With
//                   the expressions written as in the reference Fortran this
//                   reproduces a -ffp-contract=off CPU build bit for bit.
//   fast  (E=false) plain double operators: the compiler contracts into FMA,
//                   and the kernels replace divisions by one reciprocal per
//                   cell where the reference divides several times.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cans {

template <bool E> struct F {
  double v;
  __device__ __forceinline__ F() {}
  __device__ __forceinline__ F(double x) : v(x) {}
};

#define CANS_BINOP(OP, RN)                                                     \
  template <bool E> __device__ __forceinline__ F<E> operator OP(F<E> a, F<E> b) { \
    if constexpr (E) return F<E>(RN(a.v, b.v));                                \
    else return F<E>(a.v OP b.v);                                              \
  }                                                                            \
  template <bool E> __device__ __forceinline__ F<E> operator OP(double a, F<E> b) { \
    return F<E>(a) OP b;                                                       \
  }                                                                            \
  template <bool E> __device__ __forceinline__ F<E> operator OP(F<E> a, double b) { \
    return a OP F<E>(b);                                                       \
  }
CANS_BINOP(+, __dadd_rn)
CANS_BINOP(-, __dsub_rn)
CANS_BINOP(*, __dmul_rn)
CANS_BINOP(/, __ddiv_rn)
#undef CANS_BINOP

template <bool E> __device__ __forceinline__ F<E> operator-(F<E> a) {
  return F<E>(-a.v);
}
template <bool E> __device__ __forceinline__ F<E> fsqrt(F<E> a) {
  if constexpr (E) return F<E>(__dsqrt_rn(a.v));
  else return F<E>(sqrt(a.v));
}
template <bool E> __device__ __forceinline__ F<E> fabs_(F<E> a) {
  return F<E>(fabs(a.v));
}
// Fortran max(zero, a) on finite values
template <bool E> __device__ __forceinline__ F<E> max0(F<E> a) {
  return F<E>(a.v > 0.0 ? a.v : 0.0);
}
template <bool E> __device__ __forceinline__ F<E> fmin_(F<E> a, F<E> b) {
  return F<E>(a.v < b.v ? a.v : b.v);
}

// 1.0e-4 as the single-precision literal of the reference artificial
// viscosity threshold, widened to double.
#define CANS_AV_EPS ((double)1.0e-4f)

// Device control block of a resident run: the time-loop state of the
// reference driver (ns, t, dt, merr) lives here so that no per-step host
// round trip is needed.
struct Ctl {
  double dt;        // time step used by the next step kernel
  double t;         // current time (after the step that dt belongs to)
  double tp;        // time before that step
  double tend;      // loop ends when t >= tend
  double dtmin;     // merr=9001 when dt < dtmin
  double safety;    // CFL safety factor
  double dtout;     // pause for output when int(tp/dtout) < int(t/dtout)
  unsigned long long cfl_bits;  // running CFL minimum (bit pattern, >= 0)
  long long ns;     // steps taken
  long long nstop;  // loop ends when ns >= nstop
  int merr;         // 0, or 9001 (dt < dtmin)
  int done;         // 1: loop finished (tend/nstop/merr); kernels are no-ops
  int pause;        // 1: an output time was crossed; host clears it
  int pause_on_output;
  unsigned int frame_blocks_done;  // last-block detection in the frame kernel
  int nonfinite;    // warps whose CFL saw a bad cell (below) since the start
  int stop_on_bad;  // 1: a bad cell ends the loop with merr = 9100
  // Double-buffered state: a step reads buf[cur] and writes buf[cur^1]; the
  // frame kernel flips cur once the boundary fill and CFL are done, so the
  // same captured graph serves every iteration.
  double *buf[2];
  int cur;
  long long nexec;  // steps executed since the run started
  unsigned long long nfloor;  // chkdav events since the run started
  // resistive runs: the smallest diffusion limit of the time step over the
  // cells (cfl_m_e.f:61), a constant of the run; 0 = none
  unsigned long long dtdif_bits;
};

// Positive doubles order like their unsigned bit patterns.
__device__ __forceinline__ void atomic_min_pos(unsigned long long *addr,
                                               double v) {
  // NaN never compares below the running minimum, as in the reference
  // `if (dtq .lt. dt)`.
  if (!(v >= 0.0)) return;
  atomicMin(addr, (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w < v || v != v) ? w : v;   // a NaN never survives a finite value
  }
  return v;
}

// Start of a loop iteration (main.f:161-173): ns+=1, dt = CFL minimum held in
// cfl_bits, the dtmin test, tp = t, t += dt.
__device__ __forceinline__ void start_iteration(Ctl *ctl) {
  if (ctl->stop_on_bad && ctl->nonfinite) {  // the state just written is bad
    ctl->merr = 9100;  // CANS_ERR_NONFINITE
    ctl->done = 1;
    return;
  }
  ctl->ns += 1;
  const unsigned long long bits = atomicAdd(&ctl->cfl_bits, 0ull);  // coherent read
  double dt = __longlong_as_double((long long)bits);
  if (ctl->dtdif_bits) {  // min over cells of min(dtwav, dtdif)
    const double dd = __longlong_as_double((long long)ctl->dtdif_bits);
    if (dd < dt) dt = dd;
  }
  ctl->dt = dt;
  ctl->cfl_bits = 0x7ff0000000000000ull;
  if (dt < ctl->dtmin) {
    ctl->merr = 9001;
    ctl->done = 1;
    return;
  }
  ctl->tp = ctl->t;
  ctl->t = ctl->t + dt;
}

// End of one loop iteration (main.f:191-219), run by one thread once the
// step, the boundary fill and the CFL reduction of the new state are
// complete: flip the state buffers, the output test, the loop test, then the
// start of the next iteration -- unless an output time was crossed, in which
// case the loop pauses with t still the time of the state just written and
// the next iteration starts when the host resumes it.
__device__ __forceinline__ void finish_iteration(Ctl *ctl) {
  ctl->frame_blocks_done = 0;
  ctl->cur ^= 1;
  ctl->nexec += 1;
  if (ctl->pause_on_output && ctl->dtout > 0.0) {
    const long long nt1 = (long long)(ctl->tp / ctl->dtout);
    const long long nt2 = (long long)(ctl->t / ctl->dtout);
    if (nt1 < nt2) ctl->pause = 1;
  }
  if (!(ctl->ns < ctl->nstop && ctl->t < ctl->tend)) {
    ctl->done = 1;
    return;
  }
  if (ctl->pause) return;
  start_iteration(ctl);
}

// A cell the CFL cannot use: density or pressure not positive, or a time
// step that is not a number (a non-finite value anywhere in the cell).  The
// reference scan skips such a cell (`dtq .lt. dt` is false for a NaN); here
// it is also counted.
// The tests are integer compares of the bit patterns, kept off the FP64
// pipe that bounds the step kernels: x > 0 (NaN excluded, +inf included)
// is 0 < bits <= bits(+inf) as a signed integer, and x is a NaN when its
// magnitude bits exceed those of +inf.
__device__ __forceinline__ bool bad_cell(double ro, double pr, double dtq) {
  constexpr long long kInf = 0x7ff0000000000000LL;
  const long long a = __double_as_longlong(ro), b = __double_as_longlong(pr);
  const long long c = __double_as_longlong(dtq) & 0x7fffffffffffffffLL;
  return a <= 0 || a > kInf || b <= 0 || b > kInf || c > kInf;
}
// One count per warp that saw a bad cell (a vote, no block barrier).  All
// 32 threads of the warp must call it; tid is the linear thread index.
__device__ __forceinline__ void count_bad_block(bool bad, int *count, int tid) {
  if (__ballot_sync(0xffffffffu, bad) != 0u && (tid & 31) == 0) atomicAdd(count, 1);
}

// Block-wide minimum, valid on thread 0.  All threads of the block must call
// it; the block size must be a multiple of 32.
__device__ __forceinline__ double block_min(double v, double *red, int tid,
                                            int nthreads) {
  v = warp_min(v);
  const int lane = tid & 31, w = tid >> 5;
  const int nw = (nthreads + 31) >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  double x = __longlong_as_double(0x7ff0000000000000LL);
  if (w == 0) {
    x = (lane < nw) ? red[lane] : x;
    x = warp_min(x);
  }
  return x;
}

// Block-wide minimum reduced into one atomicMin.  All threads of the block
// must call it; tid is the linear thread index, nthreads the block size.
__device__ __forceinline__ void block_min_to(unsigned long long *addr,
                                             double v, double *red, int tid,
                                             int nthreads) {
  v = warp_min(v);
  const int lane = tid & 31, w = tid >> 5;
  const int nw = (nthreads + 31) >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    double x = (lane < nw) ? red[lane] : __longlong_as_double(0x7ff0000000000000LL);
    x = warp_min(x);
    if (lane == 0) atomic_min_pos(addr, x);
  }
}

}  // namespace cans
