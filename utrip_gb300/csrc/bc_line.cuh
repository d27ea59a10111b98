// One reference bd* rule on one grid line, and the mapping of line indices
// to array offsets; shared by every boundary-fill kernel.
//
// Every bd* routine applies one rule to each grid line that runs along its
// axis (cans2d/bc/bdperx.f:33-46, bdsppx.f:31-47, bdsmnx.f:31-55, bdfrex.f,
// bdcnsx.f, bdfrdx.f and their y/z and 1-D/3-D twins).
#pragma once
#include "cans_common.cuh"
#include "cans_internal.h"

namespace cans {

// One rule on one line: q(l), l = 1..n, at stride `stride`.
__device__ __forceinline__ void bd_line(int kind, int mbnd, int m0, int m1,
                                        double *q, int n, size_t stride,
                                        double q0, const double *dxm) {
#define QL(l) q[(size_t)((l)-1) * stride]
  if (kind == BD_PER) {  // bdperx(margin0, margin1)
    const int b0 = 1 + m0, b1 = n - m1;
    if (mbnd == 0)
      for (int i = 1; i <= m0; i++) QL(b0 - i) = QL(b1 + 1 - i);
    else
      for (int i = 1; i <= m1; i++) QL(b1 + i) = QL(b0 - 1 + i);
    return;
  }
  const int m = (mbnd == 0) ? m0 : m1;
  if (mbnd == 0) {
    const int b = 1 + m;
    switch (kind) {
      case BD_SPP: for (int i = 1; i <= m; i++) QL(b - i) = QL(b - 1 + i); break;
      case BD_SPN: for (int i = 1; i <= m; i++) QL(b - i) = -QL(b - 1 + i); break;
      case BD_SMP: for (int i = 1; i <= m; i++) QL(b - i) = QL(b + i); break;
      case BD_SMN:
        for (int i = 1; i <= m; i++) QL(b - i) = -QL(b + i);
        QL(b) = 0.;
        break;
      case BD_FRE: for (int i = 1; i <= m; i++) QL(b - i) = QL(b); break;
      case BD_CNS: for (int i = 1; i <= m; i++) QL(b - i) = q0; break;
      case BD_FRD:
        for (int i = 1; i <= m; i++) {
          const double dqq = __ddiv_rn(__dsub_rn(QL(b + 1), QL(b)), dxm[b - 1]);
          QL(b - i) = __dsub_rn(QL(b - i + 1), __dmul_rn(dqq, dxm[b - i - 1]));
        }
        break;
      default: break;
    }
  } else {
    const int b = n - m;
    switch (kind) {
      case BD_SPP: for (int i = 1; i <= m; i++) QL(b + i) = QL(b + 1 - i); break;
      case BD_SPN: for (int i = 1; i <= m; i++) QL(b + i) = -QL(b + 1 - i); break;
      case BD_SMP: for (int i = 1; i <= m; i++) QL(b + i) = QL(b - i); break;
      case BD_SMN:
        for (int i = 1; i <= m; i++) QL(b + i) = -QL(b - i);
        QL(b) = 0.;
        break;
      case BD_FRE: for (int i = 1; i <= m; i++) QL(b + i) = QL(b); break;
      case BD_CNS: for (int i = 1; i <= m; i++) QL(b + i) = q0; break;
      case BD_FRD:
        for (int i = 1; i <= m; i++) {
          const double dqq = __ddiv_rn(__dsub_rn(QL(b), QL(b - 1)), dxm[b - 2]);
          QL(b + i) = __dadd_rn(QL(b + i - 1), __dmul_rn(dqq, dxm[b + i - 2]));
        }
        break;
      default: break;
    }
  }
#undef QL
}

// The value at position l (1-based) of a line of n values after bd_line's
// lower-face rule and then its upper-face rule, with margin m on both faces,
// computed without writing: get(l') supplies the line's values at positions
// that neither rule changes.  The operations (the only arithmetic is bdfrd's)
// are those of bd_line in the same order, so the value is the same bits.
__device__ __forceinline__ bool bd_changes(int klo, int khi, int m, int n, int l) {
  return (klo >= 0 && (l <= m || (klo == BD_SMN && l == 1 + m))) ||
         (khi >= 0 && (l > n - m || (khi == BD_SMN && l == n - m)));
}
template <class G>
__device__ __forceinline__ double bd_value(int klo, int khi, int m, int n, double q0lo,
                                           double q0hi, const double *dxm, int l, G get) {
  // after the lower-face rule
  auto vlo = [&](int p) -> double {
    const int b = 1 + m;
    if (klo >= 0 && p <= m) {
      const int i = b - p;
      switch (klo) {
        case BD_PER: return get(p + n - 2 * m);
        case BD_SPP: return get(b - 1 + i);
        case BD_SPN: return -get(b - 1 + i);
        case BD_SMP: return get(b + i);
        case BD_SMN: return -get(b + i);
        case BD_FRE: return get(b);
        case BD_CNS: return q0lo;
        case BD_FRD: {
          const double qb = get(b);
          const double dqq = __ddiv_rn(__dsub_rn(get(b + 1), qb), dxm[b - 1]);
          double v = qb;
          for (int k = 1; k <= i; k++) v = __dsub_rn(v, __dmul_rn(dqq, dxm[b - k - 1]));
          return v;
        }
        default: break;
      }
    }
    if (klo == BD_SMN && p == b) return 0.0;
    return get(p);
  };
  const int b = n - m;
  if (khi >= 0 && l > b) {
    const int i = l - b;
    switch (khi) {
      case BD_PER: return vlo(l - (n - 2 * m));
      case BD_SPP: return vlo(b + 1 - i);
      case BD_SPN: return -vlo(b + 1 - i);
      case BD_SMP: return vlo(b - i);
      case BD_SMN: return -vlo(b - i);
      case BD_FRE: return vlo(b);
      case BD_CNS: return q0hi;
      case BD_FRD: {
        const double qb = vlo(b);
        const double dqq = __ddiv_rn(__dsub_rn(qb, vlo(b - 1)), dxm[b - 2]);
        double v = qb;
        for (int k = 1; k <= i; k++) v = __dadd_rn(v, __dmul_rn(dqq, dxm[b + k - 2]));
        return v;
      }
      default: break;
    }
  }
  if (khi == BD_SMN && l == b) return 0.0;
  return vlo(l);
}

// Lines along `axis` of an (n0, n1, n2) array: line index -> base offset.
__device__ __forceinline__ size_t line_base(int axis, long long line, int n0,
                                            int n1) {
  if (axis == 0) return (size_t)line * n0;                 // (j,k) -> j*n0 + k*n0*n1
  if (axis == 1) {
    const long long i = line % n0, k = line / n0;
    return (size_t)i + (size_t)k * n0 * n1;
  }
  return (size_t)line;                                     // (i,j) plane index
}

}  // namespace cans
