// Double-float ("df64") arithmetic on the FP32 pipes (sm_103a).
//
// GB300 executes FP64 at 2 lanes per SM per clock and FP32 at 128; the mLW
// step, which needs several hundred FP64 operations per zone, is bound by the
// FP64 pipe.  A double-float value is an unevaluated sum h + l of two floats
// with |l| <= ulp(h)/2: 48 significant bits, the exponent range of float.
// The operations below are written from the published error-free
// transformations:
//   two_sum       Knuth, TAOCP vol. 2 (Moller 1965): s + e == a + b exactly
//   fast_two_sum  Dekker 1971, for |a| >= |b|
//   two_prod      with one FMA: p + e == a * b exactly
// and the double-word algorithms of Joldes, Muller and Popescu, "Tight and
// rigorous error bounds for basic building blocks of double-word arithmetic"
// (ACM TOMS 44, 2017): the sloppy sum (their Alg. 5; absolute error of order
// u^2 (|x| + |y|), u = 2^-24, which is all a difference of nearby values
// needs), the product with FMA (Alg. 10, relative error below 7 u^2), the
// product by a float (Alg. 9), and the sum with a float (Alg. 4).  The
// reciprocal is one Newton step on the correctly rounded float reciprocal,
// with the residual 1 - y r formed in double-float (about 2^-46).
//
// Every float operation is an explicitly rounded intrinsic, so nothing is
// contracted or reassociated: the error-free transformations stay exact.
//
// Conversions between double and double-float use integer operations only
// (on GB300 a double <-> float conversion instruction runs at the FP64 rate):
// the head takes the top 24 significand bits, the tail the remaining 29
// rounded to 24, so the value is kept to 2^-48 for 2^-74 <= |x| < 2^128.
// Outside that range the tail is dropped down to 2^-126, smaller values
// flush to zero, larger ones are infinite.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cans {
namespace df {

struct D {
  float h, l;
};

__device__ __forceinline__ D two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ D fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ D mk(float a) { return {a, 0.0f}; }
__device__ __forceinline__ D neg(D x) { return {-x.h, -x.l}; }
// multiplication by a power of two is exact
__device__ __forceinline__ D scale(D x, float p2) {
  return {__fmul_rn(x.h, p2), __fmul_rn(x.l, p2)};
}

// x + y, sloppy (JMP Alg. 5)
__device__ __forceinline__ D add(D x, D y) {
  const D s = two_sum(x.h, y.h);
  const float v = __fadd_rn(x.l, y.l);
  const float w = __fadd_rn(s.l, v);
  return fast_two_sum(s.h, w);
}
__device__ __forceinline__ D sub(D x, D y) { return add(x, neg(y)); }
// x + y for a float y (JMP Alg. 4)
__device__ __forceinline__ D addf(D x, float y) {
  const D s = two_sum(x.h, y);
  const float v = __fadd_rn(x.l, s.l);
  return fast_two_sum(s.h, v);
}

// x * y (JMP Alg. 10)
__device__ __forceinline__ D mul(D x, D y) {
  const float ch = __fmul_rn(x.h, y.h);
  const float cl1 = __fmaf_rn(x.h, y.h, -ch);
  const float tl = __fmul_rn(x.h, y.l);
  const float cl2 = __fmaf_rn(x.l, y.h, tl);
  return fast_two_sum(ch, __fadd_rn(cl1, cl2));
}
// x * y for a float y (JMP Alg. 9)
__device__ __forceinline__ D mulf(D x, float y) {
  const float ch = __fmul_rn(x.h, y);
  const float cl1 = __fmaf_rn(x.h, y, -ch);
  return fast_two_sum(ch, __fmaf_rn(x.l, y, cl1));
}
// x * y + z: the product's head and tail are added to z before one
// normalisation (the error terms of mul and add, without the intermediate
// fast_two_sum).
__device__ __forceinline__ D mad(D x, D y, D z) {
  const float ch = __fmul_rn(x.h, y.h);
  const float cl1 = __fmaf_rn(x.h, y.h, -ch);
  const float cl2 = __fmaf_rn(x.l, y.h, __fmul_rn(x.h, y.l));
  const D s = two_sum(ch, z.h);
  const float t = __fadd_rn(__fadd_rn(cl1, cl2), z.l);
  return fast_two_sum(s.h, __fadd_rn(s.l, t));
}
__device__ __forceinline__ D sqr(D x) { return mul(x, x); }

// 1 / y: r = rn(1/y.h), then r + r (1 - y r) with 1 - y r in double-float
__device__ __forceinline__ D rcp(D y) {
  const float r = __frcp_rn(y.h);
  const D p = mulf(y, r);
  const float e = __fsub_rn(__fsub_rn(1.0f, p.h), p.l);  // 1 - p.h is exact
  return fast_two_sum(r, __fmul_rn(r, e));
}

// sign tests of a normalised value: its head carries the sign (or is 0 with
// a zero tail)
__device__ __forceinline__ bool pos(D x) { return x.h > 0.0f; }
__device__ __forceinline__ bool gt(D a, D b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }
__device__ __forceinline__ D absd(D x) { return x.h < 0.0f ? neg(x) : x; }

// double -> double-float (see the file comment), with integer operations
// only: a head whose exponent fits a float (2^-126 <= |x| < 2^128) keeps the
// top 24 significand bits; the tail, the low 29 bits rounded to 24, is kept
// while it is a normal float (|x| >= 2^-74) and dropped below; smaller
// values flush to zero, larger ones become infinities, and NaN stays NaN.
__device__ __forceinline__ D from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const int e = (int)((hi >> 20) & 0x7ffu);
  const unsigned sgn = hi & 0x80000000u;
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 stored bits
  if (e >= 897 && e <= 1150) {
    const float h = __uint_as_float(sgn | ((unsigned)(e - 896) << 23) | mant);
    if (e < 949) return {h, 0.0f};
    // tail: the low 29 bits times 2^(e - 1075), a normal float for e >= 949
    const float t = __fmul_rn(__uint2float_rn(lo & 0x1fffffffu),
                              __uint_as_float((unsigned)(e - 948) << 23));
    return fast_two_sum(h, sgn ? -t : t);
  }
  if (e < 897) return {__uint_as_float(sgn), 0.0f};
  // overflow to infinity; NaN keeps a non-zero significand
  const bool nan = e == 2047 && ((hi & 0xfffffu) | lo) != 0u;
  return {__uint_as_float(sgn | 0x7f800000u | (nan ? 0x400000u : 0u)), 0.0f};
}

// double-float -> double, rounded once: the two floats are widened exactly
// with integer operations (a subnormal float, below 2^-126, widens to zero)
// and added in FP64
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ef = (u >> 23) & 0xffu;
  const unsigned long long sg = (unsigned long long)(u & 0x80000000u) << 32;
  if (ef == 0u) return __longlong_as_double((long long)sg);
  const unsigned long long ed = ef == 0xffu ? 0x7ffull : (unsigned long long)(ef + 896u);
  return __longlong_as_double(
      (long long)(sg | (ed << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}
__device__ __forceinline__ double to_double(D x) { return __dadd_rn(widen(x.h), widen(x.l)); }

// A double-float number with the arithmetic operators, so that code written
// once for a number type R runs as R = double (FP64 pipe) or R = DF (FP32
// pipes).  Literal constants in such code are floats (0.5f, 2.0f): exact in
// both, and a float operand takes the cheaper mixed operations here.
struct DF {
  D d;
  DF() = default;
  __device__ __forceinline__ DF(float f) : d{f, 0.0f} {}
  __device__ __forceinline__ explicit DF(D x) : d(x) {}
};
__device__ __forceinline__ DF operator+(DF a, DF b) { return DF(add(a.d, b.d)); }
__device__ __forceinline__ DF operator+(DF a, float b) { return DF(addf(a.d, b)); }
__device__ __forceinline__ DF operator+(float a, DF b) { return DF(addf(b.d, a)); }
__device__ __forceinline__ DF operator-(DF a, DF b) { return DF(sub(a.d, b.d)); }
__device__ __forceinline__ DF operator-(DF a, float b) { return DF(addf(a.d, -b)); }
__device__ __forceinline__ DF operator-(float a, DF b) { return DF(addf(neg(b.d), a)); }
__device__ __forceinline__ DF operator-(DF a) { return DF(neg(a.d)); }
__device__ __forceinline__ DF operator*(DF a, DF b) { return DF(mul(a.d, b.d)); }
__device__ __forceinline__ DF operator*(DF a, float b) { return DF(mulf(a.d, b)); }
__device__ __forceinline__ DF operator*(float a, DF b) { return DF(mulf(b.d, a)); }
__device__ __forceinline__ DF operator/(DF a, DF b) { return DF(mul(a.d, rcp(b.d))); }
__device__ __forceinline__ DF &operator+=(DF &a, DF b) { return a = a + b; }
__device__ __forceinline__ DF &operator-=(DF &a, DF b) { return a = a - b; }
__device__ __forceinline__ bool operator>(DF a, float b) {
  return a.d.h > b || (a.d.h == b && a.d.l > 0.0f);
}
__device__ __forceinline__ bool operator!=(DF a, float b) {
  return a.d.h != b || a.d.l != 0.0f;
}
__device__ __forceinline__ DF fma(DF a, DF b, DF c) { return DF(mad(a.d, b.d, c.d)); }
__device__ __forceinline__ DF fabs(DF a) { return DF(absd(a.d)); }

}  // namespace df

// Loads and stores for code templated on its number type R.
//   num_in<R>(x)   a double of the caller's data (state, metrics) as R
//   num_out(v)     R back to a double for the caller's data
//   num_ld / num_st  R through scratch of 8 bytes per value that only this
//                  code reads back: a double-float is stored as its two
//                  floats, with no conversion
template <class R> __device__ __forceinline__ R num_in(double x);
template <> __device__ __forceinline__ double num_in<double>(double x) { return x; }
template <> __device__ __forceinline__ df::DF num_in<df::DF>(double x) {
  return df::DF(df::from_double(x));
}
__device__ __forceinline__ double num_out(double v) { return v; }
__device__ __forceinline__ double num_out(df::DF v) { return df::to_double(v.d); }
template <class R> __device__ __forceinline__ R num_ld(const double *p);
template <> __device__ __forceinline__ double num_ld<double>(const double *p) { return *p; }
template <> __device__ __forceinline__ df::DF num_ld<df::DF>(const double *p) {
  const float2 f = *reinterpret_cast<const float2 *>(p);
  return df::DF(df::D{f.x, f.y});
}
__device__ __forceinline__ void num_st(double *p, double v) { *p = v; }
__device__ __forceinline__ void num_st(double *p, df::DF v) {
  *reinterpret_cast<float2 *>(p) = make_float2(v.d.h, v.d.l);
}

}  // namespace cans
