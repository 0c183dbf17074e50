// Truncation rule of a two-site split, shared by the single-CTA and the
// wide path.
#pragma once
#include <math.h>

#include "mps_common.cuh"

namespace gbmps {

// Kept dimension for descending eigenvalues lam[0..mm) (squared singular
// values): ExaTN's absolute per-index cutoff (truncateSvdTensors,
// ExaTnMpsVisitor.cpp:2366-2536) or ITensor's relative truncate
// (decomp.cc:307-463, mindim 1), both capped at chi.
__host__ __device__ inline int keep_rule(const double* lam, int mm, int mode, double cutoff, int cap) {
  int k = mm;
  if (mode == TRUNC_EXATN) {
    // first index whose partial norms (= singular value) are below the cutoff, keep it too
    for (int i = 0; i < mm; ++i) {
      const double v = lam[i];
      const double sv = v > 0.0 ? sqrt(v) : 0.0;
      if (sv < cutoff) {
        k = i + 1;
        break;
      }
    }
    if (k > cap) k = cap;
  } else {
    const double p0 = lam[0];
    if (!(p0 > 0.0) || mm == 1) {
      k = 1;
    } else {
      double scale = 0.0;
      for (int i = 0; i < mm; ++i) {
        const double v = lam[i] / p0;
        scale += v > 0.0 ? v : 0.0;
      }
      int n = mm - 1;
      double err = 0.0;
      while (n >= cap) {
        const double v = lam[n] / p0;
        err += v > 0.0 ? v : 0.0;
        --n;
      }
      if (scale == 0.0) scale = 1.0;
      while (n >= 1) {
        const double v = lam[n] / p0;
        const double pv = v > 0.0 ? v : 0.0;
        if (err + pv > cutoff * scale) break;
        err += pv;
        --n;
      }
      k = n + 1;
    }
  }
  return k < 1 ? 1 : k;
}

}  // namespace gbmps
