// Floating-point operation count of the reference mLW step -- TEST
// INFRASTRUCTURE ONLY.
//
// The oracle's restatement of mlw_m3 (cans2d/hdmlw/mlw_m3.f:64-374) and
// cfl_m3 (cans2d/common/cfl_m3.f:38-65), compiled with its double replaced by
// a counting type: every add or subtract, multiply, divide, square root and
// comparison the reference algorithm performs is counted.  This is the
// algorithm's own arithmetic per zone-update, the numerator of an FP64
// roofline for it (the GPU's fast policy reaches the same results with a
// different algebra and fewer operations).  Single-threaded (no OpenMP), so
// the counters are plain statics.
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>

namespace opcount {
struct Counts {
  unsigned long long add = 0, mul = 0, div = 0, sqrt = 0, cmp = 0;
};
static Counts c;

struct CD {
  double v;
  CD() = default;
  CD(double x) : v(x) {}  // literals and integers enter as doubles, uncounted
};
inline CD operator+(CD a, CD b) { c.add++; return CD(a.v + b.v); }
inline CD operator-(CD a, CD b) { c.add++; return CD(a.v - b.v); }
inline CD operator*(CD a, CD b) { c.mul++; return CD(a.v * b.v); }
inline CD operator/(CD a, CD b) { c.div++; return CD(a.v / b.v); }
inline CD operator-(CD a) { return CD(-a.v); }  // a sign flip, not an operation
inline bool operator<(CD a, CD b) { c.cmp++; return a.v < b.v; }
inline bool operator>(CD a, CD b) { c.cmp++; return a.v > b.v; }
inline bool operator<=(CD a, CD b) { c.cmp++; return a.v <= b.v; }
inline bool operator>=(CD a, CD b) { c.cmp++; return a.v >= b.v; }
inline bool operator==(CD a, CD b) { c.cmp++; return a.v == b.v; }
inline bool operator!=(CD a, CD b) { c.cmp++; return a.v != b.v; }
inline CD fabs(CD a) { return CD(std::fabs(a.v)); }  // a sign clear, not counted
inline CD sqrt(CD a) { c.sqrt++; return CD(std::sqrt(a.v)); }
}  // namespace opcount

using opcount::CD;
using opcount::fabs;
using opcount::sqrt;

// the restatement, with every double counted (its C entry points become
// C++ functions of CD arrays in this translation unit)
#define double CD
#undef _OPENMP
#define oracle_set_av_branch opcount_set_av_branch
#define oracle_mlw_m3_2d opcount_mlw_m3_2d
#define oracle_mlw_m3_g_2d opcount_mlw_m3_g_2d
#define oracle_mlw_m_2d opcount_mlw_m_2d
#define oracle_mlw_m_g_2d opcount_mlw_m_g_2d
#define oracle_mlw_m3_ge_2d opcount_mlw_m3_ge_2d
#define oracle_mlw_m_ge_2d opcount_mlw_m_ge_2d
#define oracle_cfl_m3_e_2d opcount_cfl_m3_e_2d
#define oracle_cfl_m3_2d opcount_cfl_m3_2d
#define oracle_cfl_m_2d opcount_cfl_m_2d
#define oracle_bbtoaa_2d opcount_bbtoaa_2d
#define oracle_roe_face opcount_roe_face_unused
#include "mlw2d.c"
#undef double

// One mlw_m3 step (qav, gm, dt given) and one cfl_m3 of the state in st
// (9 arrays of ix*jx, column-major; updated in place) on the grid dx, dxm,
// dy, dym; out receives the counts of each: out[0..4] the step's adds,
// multiplies, divides, square roots, comparisons, out[5..9] the CFL's.
extern "C" void oracle_opcount_mlw_m3_2d(double *const *st, double dt, double qav, double gm,
                                         const double *dx, const double *dxm, int ix,
                                         const double *dy, const double *dym, int jx,
                                         double *out) {
  const size_t n = (size_t)ix * (size_t)jx;
  CD *a[9];
  for (int v = 0; v < 9; v++) {
    a[v] = (CD *)std::calloc(n, sizeof(CD));
    for (size_t k = 0; k < n; k++) a[v][k] = CD(st[v][k]);
  }
  CD *g[4];
  const double *src[4] = {dx, dxm, dy, dym};
  const int len[4] = {ix, ix, jx, jx};
  for (int q = 0; q < 4; q++) {
    g[q] = (CD *)std::calloc((size_t)len[q], sizeof(CD));
    for (int k = 0; k < len[q]; k++) g[q][k] = CD(src[q][k]);
  }
  opcount::c = opcount::Counts{};
  opcount_mlw_m3_2d(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], CD(dt), CD(qav),
                    CD(gm), g[0], g[1], ix, g[2], g[3], jx);
  const opcount::Counts step = opcount::c;
  opcount::c = opcount::Counts{};
  CD dtc(0.0);
  int merr = 0;
  opcount_cfl_m3_2d(&dtc, CD(0.4), CD(1e-10), &merr, CD(gm), a[0], a[1], a[2], a[3], a[4],
                    a[5], a[6], a[7], g[0], ix, g[2], jx);
  const opcount::Counts cfl = opcount::c;
  const opcount::Counts *both[2] = {&step, &cfl};
  for (int b = 0; b < 2; b++) {
    out[5 * b + 0] = (double)both[b]->add;
    out[5 * b + 1] = (double)both[b]->mul;
    out[5 * b + 2] = (double)both[b]->div;
    out[5 * b + 3] = (double)both[b]->sqrt;
    out[5 * b + 4] = (double)both[b]->cmp;
  }
  for (int v = 0; v < 9; v++) {
    for (size_t k = 0; k < n; k++) st[v][k] = a[v][k].v;
    std::free(a[v]);
  }
  for (int q = 0; q < 4; q++) std::free(g[q]);
}
