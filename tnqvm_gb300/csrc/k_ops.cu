// Fused single-CTA MPS update kernels (sm_103a).
//
// One CTA executes one program's op list in order: single-site gates
// (ExaTnMpsVisitor.cpp:1185-1292, ITensorMPSVisitor.cpp:288-299), two-site
// gates with SVD split and truncation (ExaTnMpsVisitor.cpp:1387-1730 +
// truncateSvdTensors :2366-2536; ITensorMPSVisitor.cpp:312-331 + ITensor
// truncate decomp.cc:307-463), and orthogonality-centre moves (ITensor
// MPS::position, ITensorMPSVisitor.cpp:294,317).  The persistent launch pulls
// programs from an atomic queue, so a batch of circuits of any size runs in
// one launch with no inter-CTA waits.
//
// Two-site split: theta = gate . (A . B) is formed in per-CTA scratch, its
// Gram matrix on the isometric side is reduced to real tridiagonal form by
// Householder reflections, every eigenvalue (squared singular value) is found
// by multisection bisection and ranked, the kept dimension is chosen with
// FP64 sums, the kept eigenvectors come from twisted factorisations and the
// back-transform, and the other side is the projection W_k^H X (no division
// by singular values).
#include <math.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "expect_sweep.cuh"
#include "keep.cuh"
#include "mps_common.cuh"

namespace gbmps {

// Program statistics are updated by one thread per op.  Atomics, because a
// program run site-parallel (k_run_ops_sites) has ops of several CTAs in
// flight; in a sequential run the order of the additions is unchanged.
__device__ __forceinline__ void stat_add(double* slot, double v) { atomicAdd(slot, v); }
__device__ __forceinline__ void stat_max(double* slot, double v) {
  unsigned long long* a = reinterpret_cast<unsigned long long*>(slot);
  unsigned long long old = *(volatile unsigned long long*)a;
  while (__longlong_as_double((long long)old) < v) {
    const unsigned long long prev = atomicCAS(a, old, (unsigned long long)__double_as_longlong(v));
    if (prev == old) break;
    old = prev;
  }
}

template <typename T>
struct Prec;
// u_in_smem: the m x m work matrix of the eigensolver (and the staged X)
// fits next to the packed Gram in shared memory (FP32), else it lives in the
// CTA's global scratch (FP64, L2-resident).  refine: the FP32-only accuracy
// steps of the split.  bisect_rounds: 5-section rounds, each shrinking the
// bracket 5x (5^-16 = 7e-12 of the span in FP32; 5^-24 = 1.7e-17 in FP64,
// below eps: Sturm counts resolve an eigenvalue no more finely); with eight
// lanes per eigenvalue (bisect_rounds9 9-section rounds, FP64 with m <= 64)
// the bracket ends at least as narrow.
template <>
struct Prec<float> {
  static constexpr double eps = 1.1920929e-07;
  static constexpr bool u_in_smem = true;
  static constexpr bool refine = true;
  static constexpr int bisect_rounds = 16;
  static constexpr double ns_stop = 1e-4;  // last Newton-Schulz step leaves ~1.5 ns_stop^2 < eps
  static constexpr double tri_flush = 1e-30;  // relative |column|^2 flushed in the tridiagonalisation
  static constexpr double tiny = 1e-36;       // absolute |column|^2 below which no reflector is formed
};
template <>
struct Prec<double> {
  static constexpr double eps = 2.220446049250313e-16;
  static constexpr bool u_in_smem = false;
  static constexpr bool refine = false;
  static constexpr int bisect_rounds = 24;
  static constexpr int bisect_rounds9 = 18;  // 9^18 = 1.5e17 >= 5^24 = 6.0e16
  static constexpr double ns_stop = 1e-8;
  static constexpr double tri_flush = 1e-60;
  static constexpr double tiny = 1e-280;
};

__device__ __forceinline__ int pidx(int i, int j, int m) {  // i <= j
  return i * m - ((i * (i - 1)) >> 1) + (j - i);
}

template <typename T>
__device__ __forceinline__ cx<T> gget(const cx<T>* Gp, int i, int j, int m) {
  return i <= j ? Gp[pidx(i, j, m)] : conj(Gp[pidx(j, i, m)]);
}
template <typename T>
__device__ __forceinline__ void gset(cx<T>* Gp, int i, int j, int m, cx<T> v) {
  if (i <= j)
    Gp[pidx(i, j, m)] = v;
  else
    Gp[pidx(j, i, m)] = conj(v);
}

// Block-wide sum in R (float or double); `red` holds >= 32 doubles of shared
// memory.  FP64 runs at a small fraction of the FP32 rate on this part, so the
// FP32 kernels sum in float.
template <typename R>
__device__ R block_sum(R v, double* red_d) {
  R* red = reinterpret_cast<R*>(red_d);
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  R s = R(0);
  const int nw = blockDim.x >> 5;
  for (int i = 0; i < nw; ++i) s += red[i];
  __syncthreads();
  return s;
}

// Small per-CTA shared state that lives after the large arrays.
template <typename T>
struct SmallSmem {
  T lam[kMaxM];      // eigenvalues (working precision, from bisection)
  int perm[kMaxM];
  T iso[kMaxM];
  T oth[kMaxM];
  cx<T> g[16];
  cx<T> tau[kChiLimit];
  // tridiagonal eigensolver
  cx<T> ttau[kMaxM];     // Householder scalars of the tridiagonalisation
  cx<T> tv[kMaxM];       // current reflector v
  cx<T> tv2[kMaxM];      // the next one (the tridiagonalisation alternates buffers)
  cx<T> tp[kMaxM];       // p = tau A v, then w
  cx<T> twv[kMaxM];      // v^H W during the back-transform
  T td[kMaxM], te[kMaxM];  // tridiagonal: diagonal, off-diagonal
  int bs[kMaxM], bt[kMaxM];  // unreduced block [bs, bt] containing each row
  double lk[kMaxM];  // eigenvalues of the kept-column order (head, then refined tail)
  double red[32];
  int ival[8];
  double dval[8];
};

static_assert((kOpThreads / 32) * sizeof(cx<double>) <= sizeof(double) * 32,
              "per-warp complex partials must fit in SmallSmem::red");

template <typename T>
struct Layout {
  // Large shared region: Gram (packed upper) [+ U for FP32], or the QR matrix + R.
  static constexpr size_t gram_bytes = sizeof(cx<T>) * (kMaxM * (kMaxM + 1) / 2);
  // U (m x m), or X staged for the Gram with a padded stride (m x (m+1))
  // (the eigensolver's row stride is at most kMaxM + 4, see eig_ld)
  static constexpr size_t u_bytes = Prec<T>::u_in_smem ? sizeof(cx<T>) * kMaxM * (kMaxM + 4) : 0;
  // QR of a centre move: M (<= kMaxM x kChiLimit, odd row stride <= kChiLimit + 1), then R
  static constexpr size_t qr_bytes = sizeof(cx<T>) * (kMaxM * (kChiLimit + 1) + kChiLimit * kChiLimit);
  static constexpr size_t big = (gram_bytes + u_bytes) > qr_bytes ? (gram_bytes + u_bytes) : qr_bytes;
  static constexpr size_t smem = big + sizeof(SmallSmem<T>);
  // Global scratch per CTA: theta, then the eigensolver's work matrix for
  // FP64, or for FP32 two m x chi blocks (the refinement's head vectors, then
  // the subspace step's X^H W).
  static constexpr size_t scratch =
      sizeof(cx<T>) * (kMaxM * kMaxM + (Prec<T>::u_in_smem ? 2 * kMaxM * kChiLimit : kMaxM * kMaxM));
};

static_assert(Layout<float>::smem <= 232448 && Layout<double>::smem <= 232448,
              "the fused kernel's shared memory must fit one CTA's 227 KB");

// FP32 refinement threshold: eigenvalues below this fraction of the largest
// form the tail that is re-solved (singular-value ratio 1e-2; the FP32 Gram's
// absolute error is ~1e-7 of the trace).
constexpr double kRefineRatio = 1e-4;

// ---------------------------------------------------------- Householder QR
// M (mr x nc, row stride ld >= nc) -> Q in the first k = min(mr,nc) columns
// of M, R (k x nc, ld = nc) in Rb.  Same reflector convention as LAPACK
// zgeqr2/zung2r.  Lanes walk a column's rows, so an odd ld keeps those
// shared-memory loads free of bank conflicts (an ld that is a multiple of 16
// puts all 32 lanes on one bank).
template <typename T>
__device__ void householder_qr(cx<T>* M, int mr, int nc, int ld, cx<T>* Rb, SmallSmem<T>* sm) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  const int k = mr < nc ? mr : nc;
  // warp 0: reflector of column jj (norm, scalars in working precision, the
  // scaled column); tau[jj] = 0 when the column is left as is
  auto reflector = [&](int jj) {
    T s = T(0);
    for (int i = jj + 1 + lane; i < mr; i += 32) s += abs2(M[i * ld + jj]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const cx<T> alpha = M[jj * ld + jj];
    __syncwarp();  // every lane has read alpha before lane 0 overwrites it with beta
    const T ar = alpha.re, ai = alpha.im;
    const T nrm2 = ar * ar + ai * ai + s;
    // a column below ~sqrt(tiny) is left as is (its reflector scale would overflow)
    const bool refl = !(s == T(0) && ai == T(0)) && nrm2 > T(Prec<T>::tiny);
    if (refl) {
      const T beta = -copysign(sqrt(nrm2), ar);
      const T dr = ar - beta, di = ai, den = dr * dr + di * di;
      const T ir = dr / den, ii = -di / den;
      if (lane == 0) {
        // real part 1 - ar / beta >= 1: a reflector always has tau != 0
        sm->tau[jj] = mk<T>((beta - ar) / beta, -ai / beta);
        M[jj * ld + jj] = mk<T>(beta, T(0));
      }
      for (int i = jj + 1 + lane; i < mr; i += 32) {
        const cx<T> x = M[i * ld + jj];
        M[i * ld + jj] = mk<T>(x.re * ir - x.im * ii, x.re * ii + x.im * ir);
      }
    } else if (lane == 0) {
      sm->tau[jj] = mk<T>(0, 0);
    }
  };
  // column c <- H_j^H column c (one warp, lanes over rows)
  auto apply = [&](int j, int c, cx<T> ctau) {
    cx<T> w = mk<T>(0, 0);
    for (int i = j + 1 + lane; i < mr; i += 32) fma_cj(w, M[i * ld + j], M[i * ld + c]);
    for (int o = 16; o > 0; o >>= 1) {
      w.re += __shfl_xor_sync(0xffffffffu, w.re, o);
      w.im += __shfl_xor_sync(0xffffffffu, w.im, o);
    }
    w = w + M[j * ld + c];
    const cx<T> tw = ctau * w;
    for (int i = j + 1 + lane; i < mr; i += 32) M[i * ld + c] = M[i * ld + c] - M[i * ld + j] * tw;
    __syncwarp();
    if (lane == 0) M[j * ld + c] = M[j * ld + c] - tw;
  };
  // One barrier per column: warp 0 applies reflector j to column j+1 and
  // forms reflector j+1 from it while warps 1.. apply reflector j to the
  // columns after it.
  if (k > 0 && warp == 0) reflector(0);
  __syncthreads();
  for (int j = 0; j < k; ++j) {
    const cx<T> tj = sm->tau[j];
    const bool has = tj.re != T(0) || tj.im != T(0);
    const cx<T> ctau = conj(tj);
    if (warp == 0) {
      if (has && j + 1 < nc) apply(j, j + 1, ctau);
      __syncwarp();
      if (j + 1 < k) reflector(j + 1);
    } else if (has) {
      for (int c = j + 2 + (warp - 1); c < nc; c += nw - 1) apply(j, c, ctau);
    }
    __syncthreads();
  }
  for (int t = tid; t < k * nc; t += nt) {
    const int i = t / nc, c = t - i * nc;
    Rb[t] = c >= i ? M[i * ld + c] : mk<T>(0, 0);
  }
  __syncthreads();
  for (int j = k - 1; j >= 0; --j) {
    const cx<T> tj = sm->tau[j];
    if (j < k - 1 && (tj.re != T(0) || tj.im != T(0))) {
      for (int c = j + 1 + warp; c < k; c += nw) {
        cx<T> w = mk<T>(0, 0);
        for (int i = j + 1 + lane; i < mr; i += 32) fma_cj(w, M[i * ld + j], M[i * ld + c]);
        for (int o = 16; o > 0; o >>= 1) {
          w.re += __shfl_xor_sync(0xffffffffu, w.re, o);
          w.im += __shfl_xor_sync(0xffffffffu, w.im, o);
        }
        w = w + M[j * ld + c];
        const cx<T> tw = tj * w;
        for (int i = j + 1 + lane; i < mr; i += 32) M[i * ld + c] = M[i * ld + c] - M[i * ld + j] * tw;
        __syncwarp();
        if (lane == 0) M[j * ld + c] = M[j * ld + c] - tw;
      }
    }
    __syncthreads();
    for (int i = tid; i < mr; i += nt) {
      if (i > j)
        M[i * ld + j] = mk<T>(T(0), T(0)) - tj * M[i * ld + j];
      else if (i == j)
        M[i * ld + j] = mk<T>(T(1) - tj.re, -tj.im);
      else
        M[i * ld + j] = mk<T>(0, 0);
    }
    __syncthreads();
  }
}

// ------------------------------------------------- tridiagonal eigensolver
// Gram eigen-decomposition (both precisions), ~10x fewer flops than Jacobi:
// Householder reduction to real symmetric tridiagonal form, eigenvalues of
// each unreduced block by multisection bisection (Sturm counts), the kept
// eigenvectors by one twisted factorisation each (Dhillon-Parlett), and the
// back-transform by the stored reflectors.

// Row stride of the eigensolver's m x m work matrix.  In shared memory (FP32)
// it is the smallest value >= m that is 4 mod 16 (at most kMaxM + 4): the
// tridiagonalisation's p = A v has four lanes per row and eight rows per
// warp, and with that stride a half-warp's sixteen 8-byte loads fall on
// sixteen distinct bank pairs.  In global memory (FP64) it is m, as the
// scratch holds exactly m x m.
template <typename T>
__device__ __forceinline__ int eig_ld(int m) {
  return Prec<T>::u_in_smem ? ((m + 11) & ~15) + 4 : m;
}

// A: full Hermitian m x m (row stride eig_ld(m)) in shared memory.  On return td/te hold the
// tridiagonal T = Q^H A Q, Q = H_0 ... H_{m-2}, H_j = I - ttau[j] v_j v_j^H with
// v_j[j+1] = 1 and v_j[i] (i > j+1) stored in A[i][j] (LAPACK zhetd2, lower).
//
// Two CTA barriers per column.  Warp 0 forms the reflector of column j+1
// while the other warps apply step j's rank-2 update to columns j+2..: it
// updates column j+1 (the trailing matrix's first column, which no other
// warp touches) itself, then reduces it.  The reflectors alternate between two buffers, since the
// other warps still read v_j while warp 0 writes v_{j+1}.
template <typename T>
__device__ void tridiagonalize(cx<T>* A, int m, double trace, SmallSmem<T>* sm) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int lda = eig_ld<T>(m);
  // columns this small relative to the trace carry eigen-weight below the
  // working precision; they are flushed to zero so 1/(alpha - beta) stays finite
  const T flush2 = T(Prec<T>::tri_flush * trace * trace + Prec<T>::tiny);
  cx<T>* tvb[2] = {sm->tv, sm->tv2};
  // warp 0: reflector of column jj (x = A[jj+1:m, jj]) into tvb[b], its
  // scalars into ttau[jj] / te[jj], and column jj rewritten as (beta, v)
  auto reflector = [&](int jj, int b) {
    const int L = m - jj - 1;
    cx<T>* tv = tvb[b];
    T s = T(0);
    for (int i = 1 + lane; i < L; i += 32) s += abs2(A[(jj + 1 + i) * lda + jj]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const cx<T> alpha = A[(jj + 1) * lda + jj];
    const T ar = alpha.re, ai = alpha.im;
    const T nrm2 = ar * ar + ai * ai + s;
    const bool flush = nrm2 <= flush2;
    const bool refl = !flush && !(s == T(0) && ai == T(0));
    T beta = flush ? T(0) : ar, tr = T(0), ti = T(0), ir = T(0), ii = T(0);
    if (refl) {
      beta = -copysign(sqrt(nrm2), ar);
      tr = (beta - ar) / beta;
      ti = -ai / beta;
      const T dr = ar - beta, di = ai, den = dr * dr + di * di;
      ir = dr / den;
      ii = -di / den;
    }
    for (int i = lane; i < L; i += 32) {
      cx<T> v = mk<T>(T(i == 0), T(0));
      if (i > 0 && refl) {
        const cx<T> x = A[(jj + 1 + i) * lda + jj];
        v = mk<T>(x.re * ir - x.im * ii, x.re * ii + x.im * ir);
      }
      tv[i] = v;
      A[(jj + 1 + i) * lda + jj] = i == 0 ? mk<T>(beta, 0) : v;
    }
    if (lane == 0) {
      sm->ttau[jj] = mk<T>(tr, ti);
      sm->te[jj] = beta;
    }
  };
  if (m > 1 && warp == 0) reflector(0, 0);
  __syncthreads();
  for (int j = 0; j + 1 < m; ++j) {
    const int L = m - j - 1;  // trailing matrix At = A[j+1:m, j+1:m]
    const int b = j & 1;
    const cx<T>* tv = tvb[b];
    const bool next = j + 2 < m;  // column j+1 still has a reflector to form
    const cx<T> tau = sm->ttau[j];
    if (tau.re == T(0) && tau.im == T(0)) {
      if (next && warp == 0) reflector(j + 1, b ^ 1);
      __syncthreads();
      continue;
    }
    // p = tau At v (four lanes per row) and d = p^H v
    {
      const int r = tid >> 2, q = tid & 3;
      cx<T> acc = mk<T>(0, 0);
      if (r < L) {
        const cx<T>* row = A + (j + 1 + r) * lda + (j + 1);
        for (int c = q; c < L; c += 4) fma_c(acc, row[c], tv[c]);
      }
      acc.re += __shfl_xor_sync(0xffffffffu, acc.re, 1);
      acc.im += __shfl_xor_sync(0xffffffffu, acc.im, 1);
      acc.re += __shfl_xor_sync(0xffffffffu, acc.re, 2);
      acc.im += __shfl_xor_sync(0xffffffffu, acc.im, 2);
      cx<T> dpart = mk<T>(0, 0);
      if (r < L && q == 0) {
        const cx<T> p = tau * acc;
        sm->tp[r] = p;
        fma_cj(dpart, p, tv[r]);
      }
      for (int o = 16; o > 0; o >>= 1) {
        dpart.re += __shfl_xor_sync(0xffffffffu, dpart.re, o);
        dpart.im += __shfl_xor_sync(0xffffffffu, dpart.im, o);
      }
      // per-warp partials, summed below in a fixed order (reproducible results)
      if (lane == 0) reinterpret_cast<cx<T>*>(sm->red)[warp] = dpart;
    }
    __syncthreads();
    // At -= v w^H + w v^H with w = p - 1/2 tau (p^H v) v formed on the fly;
    // column 0 of At (column j+1 of A) by warp 0, then its reflector
    {
      cx<T> d = mk<T>(0, 0);
      const cx<T>* part = reinterpret_cast<const cx<T>*>(sm->red);
      for (int w = 0; w < (nt >> 5); ++w) d = d + part[w];
      const cx<T> a2 = scl(tau * d, T(-0.5));
      if (warp == 0) {
        const cx<T> v0 = tv[0];
        const cx<T> w0 = sm->tp[0] + a2 * v0;
        for (int r = lane; r < L; r += 32) {
          const cx<T> vr = tv[r];
          const cx<T> wr = sm->tp[r] + a2 * vr;
          cx<T>& a = A[(j + 1 + r) * lda + (j + 1)];
          a = a - (vr * conj(w0) + wr * conj(v0));
        }
        __syncwarp();
        if (next) reflector(j + 1, b ^ 1);
      }
      if (L >= 32) {
        // warps 1.. one row each, lanes over its columns 1..L-1 (warp 0 is
        // busy with column 0 and the next reflector): no index division per
        // element, and the row's v and w are loaded once
        const int nw = (nt >> 5) - 1;
        for (int r = warp - 1; warp > 0 && r < L; r += nw) {
          const cx<T> vr = tv[r];
          const cx<T> wr = sm->tp[r] + a2 * vr;
          cx<T>* arow = A + (j + 1 + r) * lda + (j + 1);
          for (int c = 1 + lane; c < L; c += 32) {
            const cx<T> vc = tv[c];
            const cx<T> wc = sm->tp[c] + a2 * vc;
            arow[c] = arow[c] - (vr * conj(wc) + wr * conj(vc));
          }
        }
      } else {
        const int Lc = L - 1;
        for (int t = tid - 32; tid >= 32 && t < L * Lc; t += nt - 32) {
          const int r = t / Lc, c = 1 + (t - r * Lc);
          const cx<T> vr = tv[r], vc = tv[c];
          const cx<T> wr = sm->tp[r] + a2 * vr, wc = sm->tp[c] + a2 * vc;
          cx<T>& a = A[(j + 1 + r) * lda + (j + 1 + c)];
          a = a - (vr * conj(wc) + wr * conj(vc));
        }
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < m; i += nt) sm->td[i] = A[i * lda + i].re;
  __syncthreads();
}

// Number of eigenvalues below x of the unreduced block [s, t] of (td, te),
// FP64, without a division per step.  The pivots q_i = (d_i - x) - e_{i-1}^2
// / q_{i-1} of the usual count are ratios p_i / p_{i-1} of the leading
// principal minors p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2}, so a negative
// pivot is a sign change between consecutive minors.  A pivot below pivmin
// in magnitude is set to -pivmin, as in the division form (p_i = -pivmin
// p_{i-1}).  The pair (p_{i-1}, p_i) is rescaled by a power of two whenever
// p_i leaves [2^-500, 2^500], which keeps the ratios exact.  FP64 division
// is a long sequence on a pipe with 1/63 of the FP32 rate; this count uses
// three multiply-adds per step.
__device__ __forceinline__ int sturm_count_minors(const double* td, const double* te, int s, int t, double x,
                                                  double pivmin) {
  int cnt = 0;
  double pm = 1.0, pc = td[s] - x;  // p_{i-1}, p_i
  if (fabs(pc) < pivmin) pc = -pivmin;
  cnt += pc < 0.0;
  for (int i = s + 1; i <= t; ++i) {
    const double e = te[i - 1];
    double pn = fma(td[i] - x, pc, -(e * e) * pm);
    if (fabs(pn) < pivmin * fabs(pc)) pn = -pivmin * pc;
    cnt += (pn < 0.0) != (pc < 0.0);
    pm = pc;
    pc = pn;
    const int ex = (__double2hiint(pc) >> 20) & 0x7ff;  // biased exponent of p_i
    if (ex > 1023 + 500 || ex < 1023 - 500) {
      const double sc = __hiloint2double((2046 - ex) << 20, 0);  // ~1 / |p_i|, a power of two
      pc *= sc;
      pm *= sc;
    }
  }
  return cnt;
}

// All eigenvalues of T (td, te): split into unreduced blocks, then each row j
// finds the (j - block start)-th smallest eigenvalue of its block with L
// lanes multisecting the interval: L Sturm counts per round, the bracket
// shrinks (L+1)-fold.  L = 4 (512 threads cover m = 128), or L = 8 when m <=
// 64, where four lanes per eigenvalue would leave half the block idle.
// Results: sm->lam[j] and the block bounds sm->bs[j], sm->bt[j].
template <typename T, int L>
__device__ void tri_multisect(int m, SmallSmem<T>* sm, int rounds) {
  const int tid = threadIdx.x;
  const T eps = T(Prec<T>::eps);
  const int j = tid / L, q = tid % L;
  const bool live = j < m;
  const int s = live ? sm->bs[j] : 0, t = live ? sm->bt[j] : -1;
  const int local = j - s;
  T lo = T(0), hi = T(0), maxe2 = T(1);
  for (int i = s; i <= t; ++i) {
    const T el = i > s ? fabs(sm->te[i - 1]) : T(0), er = i < t ? fabs(sm->te[i]) : T(0);
    const T d = sm->td[i];
    if (i == s) {
      lo = d - el - er;
      hi = d + el + er;
    } else {
      lo = fmin(lo, d - el - er);
      hi = fmax(hi, d + el + er);
    }
    maxe2 = fmax(maxe2, er * er);
  }
  const T pivmin = T(1.2e-38) * maxe2;
  const T pad = T(4) * eps * fmax(fabs(lo), fabs(hi)) + pivmin;
  T a = lo - pad, b = hi + pad;
  const int base = threadIdx.x & 31 & ~(L - 1);
  const unsigned gmask = ((1u << L) - 1u) << base;
  for (int round = 0; round < rounds; ++round) {
    const T w = (b - a) / T(L + 1);
    const T x = a + w * T(q + 1);
    int cnt = 0;
    if constexpr (sizeof(T) == 8) {
      cnt = sturm_count_minors(sm->td, sm->te, s, t, x, pivmin);
    } else {
      // FP32 keeps the division form: a division-free count from the
      // leading minors was 1.6 % faster over the batched-VQE workload but
      // moved four of its 1024 energies past 1e-6 (max 1.8e-6)
      T qv = T(1);
      for (int i = s; i <= t; ++i) {
        const T e2 = i > s ? sm->te[i - 1] * sm->te[i - 1] : T(0);
        qv = (sm->td[i] - x) - (i > s ? e2 / qv : T(0));
        if (fabs(qv) < pivmin) qv = -pivmin;
        cnt += qv < T(0);
      }
    }
    // the new bracket ends at the first point whose count exceeds `local`
    int first = L;
#pragma unroll
    for (int u = L - 1; u >= 0; --u)
      if (__shfl_sync(gmask, cnt, base + u) > local) first = u;
    const T na = first == 0 ? a : a + w * T(first);
    const T nb = first == L ? b : a + w * T(first + 1);
    // a bracket that no longer moves never moves again (the same points,
    // the same counts): the warp stops once all of its brackets are stuck,
    // with the results of the full round count
    const bool stuck = !live || (na == a && nb == b);
    a = na;
    b = nb;
    if (__all_sync(0xffffffffu, stuck)) break;
  }
  if (live && q == 0) sm->lam[j] = T(0.5) * (a + b);
}

template <typename T>
__device__ void tri_bisect(int m, SmallSmem<T>* sm) {
  const int tid = threadIdx.x;
  const T eps = T(Prec<T>::eps);
  if (tid == 0) {
    int s = 0;
    for (int i = 0; i < m; ++i) {
      bool split = i == m - 1;
      if (!split) {
        const T e = fabs(sm->te[i]);
        if (e <= eps * (fabs(sm->td[i]) + fabs(sm->td[i + 1]))) {
          split = true;
          sm->te[i] = T(0);
        }
      }
      if (split) {
        for (int r = s; r <= i; ++r) {
          sm->bs[r] = s;
          sm->bt[r] = i;
        }
        s = i + 1;
      }
    }
  }
  __syncthreads();
  // eight lanes only in FP64, where each Sturm step's division is costly;
  // FP32 keeps four lanes and its 5-section brackets (the complex64 results
  // stay those the accuracy figures were measured with)
  bool eight = false;
  if constexpr (sizeof(T) == 8) {
    eight = 8 * m <= (int)blockDim.x;
    if (eight) tri_multisect<T, 8>(m, sm, Prec<T>::bisect_rounds9);
  }
  if (!eight) tri_multisect<T, 4>(m, sm, Prec<T>::bisect_rounds);
  __syncthreads();
}

// Twisted-factorisation eigenvector of T for eigenvalue lam on block [s, t],
// written into column c of W (m x k, ld k); real parts first hold D+ and
// imaginary parts D- of the two factorisations, then the vector.
template <typename T>
__device__ void tri_twisted(cx<T>* W, int m, int k, int c, T lam, int s, int t, SmallSmem<T>* sm) {
  // Pivots are kept at least eps*|T| (block scale) away from zero, so one
  // step of the vector recurrence grows a component by at most ~1/eps^2; the
  // partial vector is rescaled whenever a component passes 1e15, so neither
  // the components nor their squared norm overflow.
  T scale = T(0);
  for (int i = s; i <= t; ++i) scale = fmax(scale, fabs(sm->td[i] - lam) + (i < t ? fabs(sm->te[i]) : T(0)));
  const T tiny = fmax(T(Prec<T>::eps) * T(Prec<T>::eps) * scale, T(1e-35));
  auto guard = [&](T v) { return fabs(v) < tiny ? -tiny : v; };
  W[s * k + c].re = sm->td[s] - lam;
  for (int i = s + 1; i <= t; ++i) {
    const T e = sm->te[i - 1];
    W[i * k + c].re = (sm->td[i] - lam) - e * e / guard(W[(i - 1) * k + c].re);
  }
  W[t * k + c].im = sm->td[t] - lam;
  for (int i = t - 1; i >= s; --i) {
    const T e = sm->te[i];
    W[i * k + c].im = (sm->td[i] - lam) - e * e / guard(W[(i + 1) * k + c].im);
  }
  int r = s;
  T best = T(3.0e38);
  for (int i = s; i <= t; ++i) {
    const T g = fabs(W[i * k + c].re + W[i * k + c].im - (sm->td[i] - lam));
    if (g < best) {
      best = g;
      r = i;
    }
  }
  const T big = T(1e15), shrink = T(1e-15);
  T nrm = T(1);
  W[r * k + c].re = T(1);
  int lo_done = r;
  for (int i = r - 1; i >= s; --i) {
    T z = -(sm->te[i] / guard(W[i * k + c].re)) * W[(i + 1) * k + c].re;
    if (fabs(z) > big) {  // rescale what is computed so far: rows i+1..r
      for (int u = i + 1; u <= r; ++u) W[u * k + c].re *= shrink;
      nrm *= shrink * shrink;
      z *= shrink;
    }
    W[i * k + c].re = z;
    nrm += z * z;
    lo_done = i;
  }
  for (int i = r + 1; i <= t; ++i) {
    T z = -(sm->te[i - 1] / guard(W[i * k + c].im)) * W[(i - 1) * k + c].re;
    if (fabs(z) > big) {  // rows lo_done..i-1
      for (int u = lo_done; u < i; ++u) W[u * k + c].re *= shrink;
      nrm *= shrink * shrink;
      z *= shrink;
    }
    W[i * k + c].re = z;
    nrm += z * z;
  }
  const T inv = T(1) / sqrt(nrm);
  for (int i = 0; i < m; ++i) {
    const bool in = i >= s && i <= t;
    W[i * k + c] = mk<T>(in ? W[i * k + c].re * inv : T(0), T(0));
  }
}

// W <- Q W with the reflectors left in A by tridiagonalize (W: m x k, ld ld).
template <typename T>
__device__ void tri_backtransform(const cx<T>* A, cx<T>* W, int m, int k, int ld, SmallSmem<T>* sm) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lda = eig_ld<T>(m);
  for (int j = m - 2; j >= 0; --j) {
    const cx<T> tau = sm->ttau[j];
    if (tau.re == T(0) && tau.im == T(0)) continue;
    const int L = m - j - 1;
    // v^H W for each column: serial over rows, one thread per column (k <= 64)
    for (int c = tid; c < k; c += nt) {
      cx<T> acc = W[(j + 1) * ld + c];
      for (int i = 1; i < L; ++i) fma_cj(acc, A[(j + 1 + i) * lda + j], W[(j + 1 + i) * ld + c]);
      sm->twv[c] = tau * acc;
    }
    __syncthreads();
    if (k >= 32) {
      // a warp per row of W, lanes over its columns (no index division)
      const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
      for (int i = warp; i < L; i += nw) {
        const cx<T> v = i == 0 ? mk<T>(1, 0) : A[(j + 1 + i) * lda + j];
        cx<T>* wrow = W + (j + 1 + i) * ld;
        for (int c = lane; c < k; c += 32) wrow[c] = wrow[c] - v * sm->twv[c];
      }
    } else {
      for (int t = tid; t < L * k; t += nt) {
        const int i = t / k, c = t - i * k;
        const cx<T> v = i == 0 ? mk<T>(1, 0) : A[(j + 1 + i) * lda + j];
        W[(j + 1 + i) * ld + c] = W[(j + 1 + i) * ld + c] - v * sm->twv[c];
      }
    }
    __syncthreads();
  }
}

// C (R x Q) = A B with A(r, l), B(l, q) given by functors, in register
// tiles of TR consecutive rows x TQ columns strided by the tile count (threads
// take tiles with q fastest, so a warp reads B contiguously and A as a
// broadcast).  Each output sums l = 0 ..
// K-1 in order with fma_c, as the untiled loops do; store(r, q, value).
template <typename T, int TR, int TQ, typename FA, typename FB, typename FS>
__device__ __forceinline__ void tiled_product(int R, int Q, int K, FA fa, FB fb, FS store) {
  const int nr = (R + TR - 1) / TR, nq = (Q + TQ - 1) / TQ;
  for (int tt = threadIdx.x; tt < nr * nq; tt += blockDim.x) {
    const int tr = tt / nq, tq = tt - tr * nq;
    int rr[TR], qq[TQ];
#pragma unroll
    for (int a = 0; a < TR; ++a) rr[a] = min(TR * tr + a, R - 1);
#pragma unroll
    for (int b = 0; b < TQ; ++b) qq[b] = min(tq + b * nq, Q - 1);
    cx<T> acc[TR][TQ];
#pragma unroll
    for (int a = 0; a < TR; ++a)
#pragma unroll
      for (int b = 0; b < TQ; ++b) acc[a][b] = mk<T>(0, 0);
    for (int l = 0; l < K; ++l) {
      cx<T> x[TR], y[TQ];
#pragma unroll
      for (int a = 0; a < TR; ++a) x[a] = fa(rr[a], l);
#pragma unroll
      for (int b = 0; b < TQ; ++b) y[b] = fb(l, qq[b]);
#pragma unroll
      for (int a = 0; a < TR; ++a)
#pragma unroll
        for (int b = 0; b < TQ; ++b) fma_c(acc[a][b], x[a], y[b]);
    }
#pragma unroll
    for (int a = 0; a < TR; ++a)
#pragma unroll
      for (int b = 0; b < TQ; ++b) {
        const int r = TR * tr + a, q = tq + b * nq;
        if (r < R && q < Q) store(r, q, acc[a][b]);
      }
  }
}

// Orthonormalise the columns of Wc (m x k, ld k).  Newton-Schulz steps
// W <- W - 1/2 W (W^H W - I) remove rounding from the orthonormality (each
// step squares the defect; W W^H is a projector only to that defect, so steps
// repeat until the step taken from |W^H W - I|_F < ns_stop leaves ~eps, at
// most five); vectors from a near-degenerate cluster can be far from
// orthogonal (|W^H W - I|_F > 0.1), and then a Householder QR of W (leading
// columns kept) replaces the steps.  U is workspace
// (>= k*k + m*k entries).  Returns where the result lies.
template <typename T>
__device__ const cx<T>* orthonormalize(cx<T>* Wc, int m, int k, cx<T>* U, SmallSmem<T>* sm) {
  const int tid = threadIdx.x, nt = blockDim.x;
  cx<T>* E = U;
  cx<T>* cur = Wc;
  cx<T>* nxt = U + k * k;
  for (int it = 0; it < 5; ++it) {
    __syncthreads();
    T f2 = T(0);
    {
      // E = W^H W - I in 2 x 4 register tiles (each entry sums over rows in order)
      const int nta = (k + 1) >> 1, ntb = (k + 3) >> 2;
      for (int tt = tid; tt < nta * ntb; tt += nt) {
        const int ta = tt / ntb, tb = tt - ta * ntb;
        int ca[2], cb[4];
#pragma unroll
        for (int a = 0; a < 2; ++a) ca[a] = min(2 * ta + a, k - 1);
#pragma unroll
        for (int b = 0; b < 4; ++b) cb[b] = min(tb + b * ntb, k - 1);  // strided: conflict-free loads
        cx<T> acc[2][4];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] = mk<T>(0, 0);
        for (int i = 0; i < m; ++i) {
          const cx<T>* row = cur + i * k;
          cx<T> xa[2], xb[4];
#pragma unroll
          for (int a = 0; a < 2; ++a) xa[a] = row[ca[a]];
#pragma unroll
          for (int b = 0; b < 4; ++b) xb[b] = row[cb[b]];
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) fma_cj(acc[a][b], xa[a], xb[b]);
        }
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int ea = 2 * ta + a, eb = tb + b * ntb;
            if (ea < k && eb < k) {
              cx<T> v = acc[a][b];
              if (ea == eb) v.re -= T(1);
              E[ea * k + eb] = v;
              f2 += abs2(v);
            }
          }
      }
    }
    // |E|_2 <= |E|_F: below 0.1 the steps converge quadratically
    const double fro = sqrt((double)block_sum<T>(f2, sm->red));
    if (it == 0 && fro > 0.1) {
      householder_qr<T>(Wc, m, k, k, U, sm);
      if (tid == 0) sm->ival[5] = 1;  // QR taken: vectors of a degenerate cluster
      __syncthreads();
      return Wc;
    }
    {
      // W - 1/2 W E in UR x 4 register tiles (each entry sums over l in order)
      constexpr int UR = sizeof(T) == 4 ? 4 : 2;
      const int nti = (m + UR - 1) / UR, ntj = (k + 3) >> 2;
      for (int tt = tid; tt < nti * ntj; tt += nt) {
        const int ti = tt / ntj, tj = tt - ti * ntj;
        int ri[UR], cj[4];
#pragma unroll
        for (int a = 0; a < UR; ++a) ri[a] = min(UR * ti + a, m - 1) * k;
#pragma unroll
        for (int b = 0; b < 4; ++b) cj[b] = min(tj + b * ntj, k - 1);  // strided: conflict-free loads
        cx<T> corr[UR][4];
#pragma unroll
        for (int a = 0; a < UR; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) corr[a][b] = mk<T>(0, 0);
        for (int l = 0; l < k; ++l) {
          cx<T> xa[UR], eb[4];
#pragma unroll
          for (int a = 0; a < UR; ++a) xa[a] = cur[ri[a] + l];
#pragma unroll
          for (int b = 0; b < 4; ++b) eb[b] = E[l * k + cj[b]];
#pragma unroll
          for (int a = 0; a < UR; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) fma_c(corr[a][b], xa[a], eb[b]);
        }
#pragma unroll
        for (int a = 0; a < UR; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int i = UR * ti + a, j = tj + b * ntj;
            if (i < m && j < k) nxt[i * k + j] = cur[i * k + j] - scl(corr[a][b], T(0.5));
          }
      }
    }
    __syncthreads();
    cx<T>* tmp = cur;
    cur = nxt;
    nxt = tmp;
    if (fro < Prec<T>::ns_stop) break;
  }
  if (tid == 0) sm->ival[5] = 0;
  __syncthreads();
  return cur;
}

// Packed upper Gram G = X X^H of the staged X (m x nn, row stride ld) in 4x4
// register tiles; returns the trace (block-wide).
template <typename T>
__device__ double gram_staged(const cx<T>* Xs, int m, int nn, int ld, cx<T>* Gp, SmallSmem<T>* sm) {
  const int tid = threadIdx.x, nt = blockDim.x;
  T tr_part = T(0);
  const int nb = (m + 3) >> 2;
  const int ntiles = nb * (nb + 1) / 2;
  for (int tt = tid; tt < ntiles; tt += nt) {
    int bi = 0, rem = tt;
    while (rem >= nb - bi) {
      rem -= nb - bi;
      ++bi;
    }
    const int bj = bi + rem;
    int ri[4], rj[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      ri[a] = min(4 * bi + a, m - 1) * ld;
      rj[a] = min(4 * bj + a, m - 1) * ld;
    }
    cx<T> acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = mk<T>(0, 0);
    for (int c = 0; c < nn; ++c) {
      cx<T> xi[4], xj[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        xi[a] = Xs[ri[a] + c];
        xj[a] = Xs[rj[a] + c];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) fma_c(acc[a][b], xi[a], conj(xj[b]));
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int i = 4 * bi + a, j = 4 * bj + b;
        if (i < m && j < m && i <= j) {
          cx<T> v = acc[a][b];
          if (i == j) {
            v.im = T(0);
            tr_part += v.re;
          }
          Gp[pidx(i, j, m)] = v;
        }
      }
  }
  return (double)block_sum<T>(tr_part, sm->red);
}

// Eigenvalues of the packed Hermitian Gp (FP32 path): expanded into Af, reduced
// to tridiagonal form (reflectors stay in Af), all eigenvalues by bisection
// into sm->lam, and sm->perm ordering them descending.
template <typename T>
__device__ void eigvals_sorted(const cx<T>* Gp, cx<T>* Af, int m, double trace, SmallSmem<T>* sm,
                               long long& cyc_trid, long long& cyc_bisect) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const long long t0 = clock64();
  const int lda = eig_ld<T>(m);
  for (int t = tid; t < m * m; t += nt) {
    const int i = t / m, j = t - i * m;
    Af[i * lda + j] = gget(Gp, i, j, m);
  }
  __syncthreads();
  tridiagonalize<T>(Af, m, trace, sm);
  const long long t1 = clock64();
  tri_bisect<T>(m, sm);
  for (int i = tid; i < m; i += nt) {
    const T li = sm->lam[i];
    int rank = 0;
    for (int j = 0; j < m; ++j) {
      const T lj = sm->lam[j];
      rank += (lj > li) || (lj == li && j < i);
    }
    sm->perm[rank] = i;
  }
  __syncthreads();
  cyc_trid += t1 - t0;
  cyc_bisect += clock64() - t1;
}

// Kept dimension of a two-site split (keep_rule in keep.cuh) for this program.
__device__ int decide_keep(const double* lam, int mm, const ProgDesc& P) {
  return keep_rule(lam, mm, P.mode, P.cutoff, P.chi_cap);
}

// ------------------------------------------------------------------- ops
template <typename T>
__device__ void op_gate1(const ProgDesc& P, const DevOp& op, SmallSmem<T>* sm) {
  const int s = op.site;
  cx<T>* A = reinterpret_cast<cx<T>*>(P.sites) + P.site_off[s];
  const int dl = P.bond[s], dr = P.bond[s + 1];
  const cx<T> g00 = mk<T>(T(op.m[0]), T(op.m[1])), g01 = mk<T>(T(op.m[2]), T(op.m[3]));
  const cx<T> g10 = mk<T>(T(op.m[4]), T(op.m[5])), g11 = mk<T>(T(op.m[6]), T(op.m[7]));
  for (int idx = threadIdx.x; idx < dl * dr; idx += blockDim.x) {
    const int l = idx / dr, r = idx - l * dr;
    const cx<T> a0 = A[(l * 2) * dr + r], a1 = A[(l * 2 + 1) * dr + r];
    A[(l * 2) * dr + r] = g00 * a0 + g01 * a1;
    A[(l * 2 + 1) * dr + r] = g10 * a0 + g11 * a1;
  }
}

template <typename T>
__device__ void op_gate2(const ProgDesc& P, const DevOp& op, char* big, SmallSmem<T>* sm, char* scratch) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lo = op.site;
  const int dl = P.bond[lo], dm = P.bond[lo + 1], dr = P.bond[lo + 2];
  if (dl > kChiLimit || dm > kChiLimit || dr > kChiLimit) {
    if (tid == 0) atomicOr(P.err, ERR_DIMS);
    return;
  }
  cx<T>* sites = reinterpret_cast<cx<T>*>(P.sites);
  cx<T>* A = sites + P.site_off[lo];
  cx<T>* B = sites + P.site_off[lo + 1];
  const int R = 2 * dl, Cc = 2 * dr;
  cx<T>* Th = reinterpret_cast<cx<T>*>(scratch);
  const long long c_start = clock64();
  if (tid < 16) sm->g[tid] = mk<T>(T(op.m[2 * tid]), T(op.m[2 * tid + 1]));
  __syncthreads();
  // theta[(l,p1),(p2,r)] = sum_{q1,q2} G[2p1+p2][2q1+q2] sum_m A[l,q1,m] B[m,q2,r]
  for (int idx = tid; idx < dl * dr; idx += nt) {
    const int l = idx / dr, r = idx - l * dr;
    cx<T> t[4] = {mk<T>(0, 0), mk<T>(0, 0), mk<T>(0, 0), mk<T>(0, 0)};
    const cx<T>* a0 = A + (l * 2) * dm;
    const cx<T>* a1 = a0 + dm;
    for (int mm = 0; mm < dm; ++mm) {
      const cx<T> x0 = a0[mm], x1 = a1[mm];
      const cx<T> y0 = B[(mm * 2) * dr + r], y1 = B[(mm * 2 + 1) * dr + r];
      fma_c(t[0], x0, y0);
      fma_c(t[1], x0, y1);
      fma_c(t[2], x1, y0);
      fma_c(t[3], x1, y1);
    }
#pragma unroll
    for (int row = 0; row < 4; ++row) {
      cx<T> acc = mk<T>(0, 0);
#pragma unroll
      for (int col = 0; col < 4; ++col) fma_c(acc, sm->g[row * 4 + col], t[col]);
      // exatn semantics: entries of modulus below 1e-100 are set to zero
      // before the split (stabilizeTensorBody, ExaTnMpsVisitor.cpp:141-161);
      // no complex64 value is that small, so only complex128 checks
      if (sizeof(T) == 8 && P.mode == TRUNC_EXATN && (double)abs2(acc) < 1e-200) acc = mk<T>(0, 0);
      Th[(l * 2 + (row >> 1)) * Cc + (row & 1) * dr + r] = acc;
    }
  }
  __syncthreads();
  // Isometric side: rows of theta (tr = false) or its columns (tr = true).
  bool tr;
  if (op.orient == ORIENT_TO_HI)
    tr = false;
  else if (op.orient == ORIENT_TO_LO)
    tr = true;
  else
    tr = R > Cc;
  const int m = tr ? Cc : R, nn = tr ? R : Cc;
  auto X = [&](int i, int c) -> cx<T> { return tr ? Th[c * Cc + i] : Th[i * Cc + c]; };
  cx<T>* Gp = reinterpret_cast<cx<T>*>(big);
  cx<T>* U = Prec<T>::u_in_smem ? reinterpret_cast<cx<T>*>(big + Layout<T>::gram_bytes)
                                : reinterpret_cast<cx<T>*>(scratch + sizeof(cx<T>) * kMaxM * kMaxM);
  const long long c_theta = clock64();
  double trace;
  if (Prec<T>::u_in_smem) {
    // Stage X (m x nn) in the U region with a padded row stride, then form
    // the upper triangle of G = X X^H in 4x4 register tiles.
    cx<T>* Xs = U;
    const int ld = nn + 1;
    for (int t = tid; t < m * nn; t += nt) {
      if (!tr) {
        const int i = t / nn, c = t - i * nn;
        Xs[i * ld + c] = Th[i * Cc + c];
      } else {
        const int c = t / m, i = t - c * m;
        Xs[i * ld + c] = Th[c * Cc + i];
      }
    }
    __syncthreads();
    trace = gram_staged<T>(Xs, m, nn, ld, Gp, sm);
  } else {
    double tr_part = 0.0;
    for (int t = tid; t < m * m; t += nt) {
      const int i = t / m, j = t - i * m;
      if (i > j) continue;
      cx<T> acc = mk<T>(0, 0);
      for (int c = 0; c < nn; ++c) fma_c(acc, X(i, c), conj(X(j, c)));
      if (i == j) {
        acc.im = T(0);
        tr_part += (double)acc.re;
      }
      Gp[pidx(i, j, m)] = acc;
    }
    trace = block_sum(tr_part, sm->red);
  }
  const long long c_gram = clock64();
  const int mm = R < Cc ? R : Cc;  // number of singular values (min(vol) in ExaTnMpsVisitor.cpp:1594)
  // reduce G (expanded into the U work matrix) to tridiagonal form
  long long cyc_trid = 0, cyc_bisect = 0, cyc_vec = 0, cyc_orth = 0;
  eigvals_sorted<T>(Gp, U, m, trace, sm, cyc_trid, cyc_bisect);
  for (int r = tid; r < m; r += nt) sm->lk[r] = sm->lam[sm->perm[r]];
  __syncthreads();
  // FP32 small-eigenvalue refinement.  An FP32 Gram resolves eigenvalues only
  // down to ~eps * trace, so when the cut falls among eigenvalues below
  // kRefineRatio * lambda_max the kept subspace is re-chosen in the
  // complement of the head (the eigenvectors above that ratio): Z = X -
  // W_h (W_h^H X) has norm ~ the tail's, its own Gram resolves the tail to
  // ~eps * |Z|^2, and the kept tail vectors are its leading eigenvectors.
  // This is ITensor's recursive SVD refinement (SVDRefImpl, tensor/algs.cc:
  // 510-579, checkSVDDone :486-507) in a deflated form, one level deep.
  cx<T>* Wc = reinterpret_cast<cx<T>*>(big);
  cx<T>* Wg = reinterpret_cast<cx<T>*>(scratch) + kMaxM * kMaxM;  // head vectors (m x s)
  double refine_flops = 0.0;
  if (Prec<T>::refine) {
    if (tid == 0) {
      const int k0 = decide_keep(sm->lk, mm, P);
      const double l0 = sm->lk[0];
      int s = 0;
      while (s < m && sm->lk[s] >= kRefineRatio * l0) ++s;
      sm->ival[6] = s;
      sm->ival[7] = (l0 > 0.0 && s < k0 && k0 < m) ? 1 : 0;
    }
    __syncthreads();
    const int s = sm->ival[6];
    if (sm->ival[7]) {
      const long long v0 = clock64();
      for (int c = tid; c < s; c += nt) {
        const int ev = sm->perm[c];
        tri_twisted<T>(Wc, m, s, c, T(sm->lam[ev]), sm->bs[ev], sm->bt[ev], sm);
      }
      __syncthreads();
      tri_backtransform<T>(U, Wc, m, s, s, sm);
      const long long v1 = clock64();
      const cx<T>* Wh = orthonormalize<T>(Wc, m, s, U, sm);
      cyc_vec += v1 - v0;
      cyc_orth += clock64() - v1;
      for (int t = tid; t < m * s; t += nt) Wg[t] = Wh[t];
      __syncthreads();
      // Y_h = W_h^H X (s x nn) in the Gram region
      cx<T>* Yh = Gp;
      for (int t = tid; t < s * nn; t += nt) {
        const int j = t / nn, c = t - j * nn;
        cx<T> acc = mk<T>(0, 0);
        for (int i = 0; i < m; ++i) fma_cj(acc, Wg[i * s + j], X(i, c));
        Yh[t] = acc;
      }
      __syncthreads();
      // Z = X - W_h Y_h, staged like X
      cx<T>* Zs = U;
      const int ld = nn + 1;
      for (int t = tid; t < m * nn; t += nt) {
        const int i = t / nn, c = t - i * nn;
        cx<T> acc = X(i, c);
        for (int j = 0; j < s; ++j) acc = acc - Wg[i * s + j] * Yh[j * nn + c];
        Zs[i * ld + c] = acc;
      }
      __syncthreads();
      const double trz = gram_staged<T>(Zs, m, nn, ld, Gp, sm);
      eigvals_sorted<T>(Gp, U, m, trz, sm, cyc_trid, cyc_bisect);
      for (int r = s + tid; r < m; r += nt) sm->lk[r] = sm->lam[sm->perm[r - s]];
      __syncthreads();
      refine_flops = 16.0 * m * s * nn + 8.0 * m * m * nn;
    }
  }
  const long long c_eig = clock64();
  if (tid == 0) {
    double total = 0.0;
    int bad = 0;
    for (int i = 0; i < mm; ++i) {
      const double v = sm->lk[i];
      if (!(v == v) || isinf(v)) bad = 1;
      total += v > 0.0 ? v : 0.0;
    }
    const int k = decide_keep(sm->lk, mm, P);
    double kept = 0.0;
    for (int i = 0; i < k; ++i) {
      const double v = sm->lk[i];
      kept += v > 0.0 ? v : 0.0;
    }
    const double frac = total > 0.0 ? (total - kept) / total : 0.0;
    double rn = 1.0;
    if ((P.flags & 1) && kept > 0.0) rn = sqrt(total / kept);
    sm->ival[2] = k;
    sm->dval[2] = rn;
    stat_add(P.stats + ST_LOG_FID, log1p(-(frac < 1.0 ? frac : 0.0)));
    stat_max(P.stats + ST_MAX_DISC, frac);
    stat_add(P.stats + ST_N_GATE2, 1.0);
    // algorithmic flops (complex MAC = 8): merge, gate, Gram, split
    stat_add(P.stats + ST_FLOPS, 32.0 * dl * dm * dr + 128.0 * dl * dr + 8.0 * m * m * nn + 8.0 * k * nn * m +
                                     16.0 * m * k * k + refine_flops +
                                     (Prec<T>::refine && k < m ? 16.0 * m * nn * k + 16.0 * m * k * k : 0.0));
    // Householder tridiagonalisation (complex, both sides) and the back-transform
    stat_add(P.stats + ST_EIG_FLOPS, (32.0 / 3.0) * m * m * m * (refine_flops > 0.0 ? 2.0 : 1.0) + 8.0 * m * m * k);
    if (refine_flops > 0.0) stat_add(P.stats + ST_N_REFINE, 1.0);
    if (bad) atomicOr(P.err, ERR_NAN);
  }
  __syncthreads();
  const int k = sm->ival[2];
  const double rn = sm->dval[2];
  for (int j = tid; j < k; j += nt) {
    const double v = sm->lk[j];
    const double sv = v > 0.0 ? sqrt(v) : 0.0;
    if (op.orient == ORIENT_SQRT) {
      const double h = sqrt(sv);
      sm->iso[j] = T(h);
      sm->oth[j] = T(h > 0.0 ? rn / h : 0.0);
    } else {
      sm->iso[j] = T(1);
      sm->oth[j] = T(rn);
    }
  }
  __syncthreads();
  // Kept eigenvectors W_k (m x k, ld k) in the Gram region.
  const cx<T>* W;
  const long long c_vec = clock64();
  long long c_orth = 0;
  {
    // twisted-factorisation vectors of the tridiagonal matrix, back-transformed
    // by the reflectors still held in the U work matrix; with the refinement,
    // the head columns come from W_h and the rest from Z.
    if (Prec<T>::refine && sm->ival[7]) {
      const int s = sm->ival[6];
      const int ks = k < s ? k : s, kt = k - ks;
      for (int c = tid; c < kt; c += nt) {
        const int ev = sm->perm[c];
        tri_twisted<T>(Wc + ks, m, k, c, T(sm->lam[ev]), sm->bs[ev], sm->bt[ev], sm);
      }
      __syncthreads();
      if (kt > 0) {
        tri_backtransform<T>(U, Wc + ks, m, kt, k, sm);
        // Gram-Schmidt the tail columns against the head (kt > 0 means ks == s):
        // Z's rounding leaves components along W_h that a symmetric
        // orthonormalisation would otherwise spread into the head.
        cx<T>* Pr = U;  // W_h^H W_t (s x kt)
        for (int t = tid; t < s * kt; t += nt) {
          const int a = t / kt, c = t - a * kt;
          cx<T> acc = mk<T>(0, 0);
          for (int i = 0; i < m; ++i) fma_cj(acc, Wg[i * s + a], Wc[i * k + ks + c]);
          Pr[t] = acc;
        }
        __syncthreads();
        for (int t = tid; t < m * kt; t += nt) {
          const int i = t / kt, c = t - i * kt;
          cx<T> acc = Wc[i * k + ks + c];
          for (int a = 0; a < s; ++a) acc = acc - Wg[i * s + a] * Pr[a * kt + c];
          Wc[i * k + ks + c] = acc;
        }
        __syncthreads();
      }
      for (int t = tid; t < m * ks; t += nt) {
        const int i = t / ks, j = t - i * ks;
        Wc[i * k + j] = Wg[i * s + j];
      }
    } else {
      for (int c = tid; c < k; c += nt) {
        const int ev = sm->perm[c];
        tri_twisted<T>(Wc, m, k, c, T(sm->lam[ev]), sm->bs[ev], sm->bt[ev], sm);
      }
      __syncthreads();
      tri_backtransform<T>(U, Wc, m, k, k, sm);
    }
    c_orth = clock64();
    W = orthonormalize<T>(Wc, m, k, U, sm);
    if ((Prec<T>::refine || sm->ival[5]) && k < m) {
      // One subspace-iteration step W <- orth(X (X^H W)) with X itself, not
      // the FP32 Gram: the Gram's rounding (~eps * trace) tilts a kept
      // eigenvector into the discarded space by ~eps * trace / lambda, while
      // the product's rounding is ~eps * sigma_max / sigma relative, so the
      // weight lost to the cut drops from ~eps^2 trace^2 / lambda to
      // ~eps^2 sigma_max^2 (the accuracy of a backward-stable SVD).  FP64
      // takes the step only after the QR fallback: twisted vectors of an
      // (exactly) degenerate cluster in one unreduced block can coincide, and
      // the QR then fills the deficient columns with rounding-noise
      // directions, which X X^H maps back onto the dominant subspace.
      cx<T>* Wk = Wg;                     // W copied out (m x k)
      cx<T>* Yv = Wg + kMaxM * kChiLimit;  // X^H W (nn x k)
      for (int t = tid; t < m * k; t += nt) Wk[t] = W[t];
      __syncthreads();
      constexpr int TR = sizeof(T) == 4 ? 4 : 2;
      tiled_product<T, TR, 4>(
          nn, k, m, [&](int c, int i) { return conj(X(i, c)); }, [&](int i, int j) { return Wk[i * k + j]; },
          [&](int c, int j, cx<T> v) { Yv[c * k + j] = v; });
      __syncthreads();
      tiled_product<T, TR, 4>(
          m, k, nn, [&](int i, int c) { return X(i, c); }, [&](int c, int j) { return Yv[c * k + j]; },
          [&](int i, int j, cx<T> v) { Wc[i * k + j] = v; });
      __syncthreads();
      for (int j = tid; j < k; j += nt) {
        T s2 = T(0);
        for (int i = 0; i < m; ++i) s2 += abs2(Wc[i * k + j]);
        // inverse column norm, 0 for a column that vanished (keep W's column)
        sm->twv[j].re = s2 > T(Prec<T>::tiny) ? T(1) / sqrt(s2) : T(0);
      }
      __syncthreads();
      for (int t = tid; t < m * k; t += nt) {
        const int j = t - (t / k) * k;
        const T inv = sm->twv[j].re;
        Wc[t] = inv > T(0) ? scl(Wc[t], inv) : Wk[t];
      }
      W = orthonormalize<T>(Wc, m, k, U, sm);
    }
  }
  cyc_vec += c_orth - c_vec;
  cyc_orth += clock64() - c_orth;
  // other side: Z = W_k^H X (k x nn)
  const bool sqrt_split = op.orient == ORIENT_SQRT;
  {
    constexpr int TR = sizeof(T) == 4 ? 4 : 2;
    tiled_product<T, TR, 4>(
        k, nn, m, [&](int j, int i) { return conj(W[i * k + j]); }, [&](int i, int c) { return X(i, c); },
        [&](int j, int c, cx<T> v) {
          const cx<T> acc = sqrt_split ? v : scl(v, sm->oth[j]);
          if (!tr)
            B[j * Cc + c] = acc;  // hi site (k, 2, dr)
          else
            A[c * k + j] = acc;   // lo site (dl, 2, k)
        });
  }
  if (sqrt_split) {
    // sqrt(S) on both sides needs each kept singular value to its own
    // relative accuracy.  sqrt(lambda) of the Gram eigenvalue carries an
    // absolute error ~eps * lambda_max, i.e. ~eps * (sigma_max / sigma)^2
    // relative, and that error moves the gauge of both sites and with it
    // every later truncation.  The row norm |w_j^H X| is accurate to ~eps *
    // sigma_max / sigma, as ITensor's singular values from the QR of M^H U
    // are (SVDRefImpl, tensor/algs.cc:541-548).  Columns whose eigenvalue
    // counts as zero stay zero on both sides.
    __syncthreads();
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    for (int j = warp; j < k; j += nw) {
      double s2 = 0.0;
      for (int c = lane; c < nn; c += 32) s2 += (double)abs2(!tr ? B[j * Cc + c] : A[c * k + j]);
      for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      if (lane == 0) {
        const double h = sm->lk[j] > 0.0 ? sqrt(sqrt(s2)) : 0.0;
        sm->iso[j] = T(h);
        sm->oth[j] = T(h > 0.0 ? rn / h : 0.0);
      }
    }
    __syncthreads();
    for (int t = tid; t < k * nn; t += nt) {
      if (!tr) {
        const int j = t / nn;
        B[t] = scl(B[t], sm->oth[j]);  // rows j of the hi site, (k, 2, dr) = k x nn
      } else {
        const int j = t - (t / k) * k;
        A[t] = scl(A[t], sm->oth[j]);  // lo site (dl, 2, k) = nn x k
      }
    }
  }
  // isometric side: W_k
  for (int t = tid; t < m * k; t += nt) {
    const int i = t / k, j = t - i * k;
    const cx<T> w = scl(W[i * k + j], sm->iso[j]);
    if (!tr)
      A[i * k + j] = w;   // lo site (dl, 2, k)
    else
      B[j * Cc + i] = w;  // hi site (k, 2, dr)
  }
  __syncthreads();
  if (tid == 0) {
    P.bond[lo + 1] = k;
    const long long c_end = clock64();
    stat_add(P.stats + ST_CYC_THETA, (double)(c_theta - c_start));
    stat_add(P.stats + ST_CYC_GRAM, (double)(c_gram - c_theta));
    stat_add(P.stats + ST_CYC_EIG, (double)(c_eig - c_gram));
    stat_add(P.stats + ST_CYC_SPLIT, (double)(c_end - c_eig));
    stat_add(P.stats + ST_CYC_TRID, (double)cyc_trid);
    stat_add(P.stats + ST_CYC_BISECT, (double)cyc_bisect);
    stat_add(P.stats + ST_CYC_VEC, (double)cyc_vec);
    stat_add(P.stats + ST_CYC_ORTH, (double)cyc_orth);
  }
}

// Centre move to the right: A_c = Q R (rows (l,p)), A_{c+1} <- R A_{c+1}.
template <typename T>
__device__ void op_move_r(const ProgDesc& P, const DevOp& op, char* big, SmallSmem<T>* sm, char* scratch) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int c = op.site;
  const long long c_start = clock64();
  const int dl = P.bond[c], dr = P.bond[c + 1], dr2 = P.bond[c + 2];
  if (2 * dl > kMaxM || dr > kChiLimit) {
    if (tid == 0) atomicOr(P.err, ERR_DIMS);
    return;
  }
  cx<T>* sites = reinterpret_cast<cx<T>*>(P.sites);
  cx<T>* A = sites + P.site_off[c];
  cx<T>* B = sites + P.site_off[c + 1];
  cx<T>* M = reinterpret_cast<cx<T>*>(big);
  cx<T>* Rb = M + kMaxM * (kChiLimit + 1);
  const int mr = 2 * dl, nc = dr, ld = nc | 1;  // odd row stride: conflict-free column walks
  for (int t = tid; t < mr * nc; t += nt) {
    const int i = t / nc, j = t - i * nc;
    M[i * ld + j] = A[t];
  }
  __syncthreads();
  householder_qr<T>(M, mr, nc, ld, Rb, sm);
  const int k = mr < nc ? mr : nc;
  for (int t = tid; t < mr * k; t += nt) {
    const int i = t / k, j = t - i * k;
    A[t] = M[i * ld + j];
  }
  cx<T>* out = reinterpret_cast<cx<T>*>(scratch);
  const int w = 2 * dr2;
  for (int t = tid; t < k * w; t += nt) {
    const int i = t / w, x = t - i * w;
    cx<T> acc = mk<T>(0, 0);
    for (int j = i; j < nc; ++j) fma_c(acc, Rb[i * nc + j], B[j * w + x]);
    out[t] = acc;
  }
  __syncthreads();
  for (int t = tid; t < k * w; t += nt) B[t] = out[t];
  __syncthreads();
  if (tid == 0) {
    P.bond[c + 1] = k;
    stat_add(P.stats + ST_FLOPS, 4.0 * k * nc * w);
    stat_add(P.stats + ST_EIG_FLOPS, 32.0 * mr * nc * nc);
    stat_add(P.stats + ST_CYC_MOVE, (double)(clock64() - c_start));
  }
}

// Centre move to the left: A_c^H = Q R, A_c <- Q^H, A_{c-1} <- A_{c-1} R^H.
template <typename T>
__device__ void op_move_l(const ProgDesc& P, const DevOp& op, char* big, SmallSmem<T>* sm, char* scratch) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int c = op.site;
  const long long c_start = clock64();
  const int dl = P.bond[c], dr = P.bond[c + 1], dl2 = P.bond[c - 1];
  if (2 * dr > kMaxM || dl > kChiLimit) {
    if (tid == 0) atomicOr(P.err, ERR_DIMS);
    return;
  }
  cx<T>* sites = reinterpret_cast<cx<T>*>(P.sites);
  cx<T>* A = sites + P.site_off[c];
  cx<T>* L = sites + P.site_off[c - 1];
  cx<T>* M = reinterpret_cast<cx<T>*>(big);
  cx<T>* Rb = M + kMaxM * (kChiLimit + 1);
  const int mr = 2 * dr, nc = dl, ld = nc | 1;  // odd row stride: conflict-free column walks
  for (int t = tid; t < mr * nc; t += nt) {
    const int j = t / mr, i = t - j * mr;  // lanes walk A's rows (contiguous loads)
    M[i * ld + j] = conj(A[t]);
  }
  __syncthreads();
  householder_qr<T>(M, mr, nc, ld, Rb, sm);
  const int k = mr < nc ? mr : nc;
  for (int t = tid; t < k * mr; t += nt) {
    const int j = t / mr, i = t - j * mr;
    A[t] = conj(M[i * ld + j]);
  }
  cx<T>* out = reinterpret_cast<cx<T>*>(scratch);
  const int h = 2 * dl2;
  for (int t = tid; t < h * k; t += nt) {
    const int x = t / k, j = t - x * k;
    cx<T> acc = mk<T>(0, 0);
    for (int i = j; i < nc; ++i) fma_cj(acc, Rb[j * nc + i], L[x * nc + i]);  // sum_i L[x,i] conj(R[j,i])
    out[t] = acc;
  }
  __syncthreads();
  for (int t = tid; t < h * k; t += nt) L[t] = out[t];
  __syncthreads();
  if (tid == 0) {
    P.bond[c] = k;
    stat_add(P.stats + ST_FLOPS, 4.0 * k * nc * h);
    stat_add(P.stats + ST_EIG_FLOPS, 32.0 * mr * nc * nc);
    stat_add(P.stats + ST_CYC_MOVE, (double)(clock64() - c_start));
  }
}

// One program on this CTA, in its own precision: its ops in order, then its
// attached observables, then the completion flag of the serve loop.
// One op of a program on this CTA.  Each precision's op body is one
// non-inlined function that both the persistent kernel (program order) and
// the site-parallel kernel call, so the two runs execute the same machine
// code for every op and give bit-identical results.
template <typename T>
__device__ __forceinline__ void run_one_op(const ProgDesc& P, const DevOp& op, char* smem, char* scratch) {
  char* big = smem;
  SmallSmem<T>* sm = reinterpret_cast<SmallSmem<T>*>(smem + Layout<T>::big);
  switch (op.kind) {
    case OP_GATE1:
      op_gate1<T>(P, op, sm);
      break;
    case OP_GATE2:
      op_gate2<T>(P, op, big, sm, scratch);
      break;
    case OP_MOVE_R:
      op_move_r<T>(P, op, big, sm, scratch);
      break;
    case OP_MOVE_L:
      op_move_l<T>(P, op, big, sm, scratch);
      break;
    default:
      break;
  }
}
__device__ __noinline__ void run_one_op_f64(const ProgDesc& P, const DevOp& op, char* smem, char* scratch) {
  run_one_op<double>(P, op, smem, scratch);
}
__device__ __noinline__ void run_one_op_f32(const ProgDesc& P, const DevOp& op, char* smem, char* scratch) {
  run_one_op<float>(P, op, smem, scratch);
}
template <typename T>
__device__ __forceinline__ void run_op(const ProgDesc& P, const DevOp& op, char* smem, char* scratch) {
  if (sizeof(T) == 8)
    run_one_op_f64(P, op, smem, scratch);
  else
    run_one_op_f32(P, op, smem, scratch);
}

template <typename T>
__device__ void run_program(const ProgDesc& P, char* smem, char* scratch) {
  const long long c_begin = clock64();
  char* big = smem;
  for (int o = 0; o < P.n_ops; ++o) {
    run_op<T>(P, P.ops[o], smem, scratch);
    __syncthreads();
  }
  if (threadIdx.x == 0) stat_add(P.stats + ST_N_OPS, (double)P.n_ops);
  if (P.n_obs > 0) {
    // the program's observables on this CTA (the shared memory of the
    // update is free now): per-request completion for the serve loop
    using EL = ExpLayout<T>;
    static_assert(EL::smem <= Layout<T>::big, "expectation work space must fit the update's shared memory");
    static_assert(EL::scratch <= Layout<T>::scratch, "expectation scratch must fit the update's scratch");
    cx<T>* E = reinterpret_cast<cx<T>*>(big);
    cx<T>* As = E + EL::e_elems;
    cx<T>* X = EL::staged ? As + EL::a_elems : reinterpret_cast<cx<T>*>(scratch);
    ExpTask tk;
    tk.sites = P.sites;
    tk.site_off = P.site_off;
    tk.bond = P.bond;
    tk.n = P.n;
    tk.pad = 0;
    const long long c_obs = clock64();
    for (int t = 0; t < P.n_obs; ++t) {
      tk.codes = P.obs_codes + (size_t)t * P.n;
      expect_sweep<T>(tk, E, As, X, P.obs_out + 2 * t);
    }
    if (threadIdx.x == 0) stat_add(P.stats + ST_CYC_OBS, (double)(clock64() - c_obs));
  }
  if (P.cycles_out != nullptr && threadIdx.x == 0) *P.cycles_out = (double)(clock64() - c_begin);
  if (P.done != nullptr) {
    __syncthreads();
    if (threadIdx.x == 0) {
      P.done[1] = *(volatile int*)P.err;
      __threadfence_system();
      *(volatile int*)P.done = 1;
    }
  }
}

// The complex128 body is a separate call: its register allocation (which
// spills) stays out of the complex64 body's.
__device__ __noinline__ void run_program_f64(const ProgDesc& P, char* smem, char* scratch) {
  run_program<double>(P, smem, scratch);
}


// Dynamic shared memory and global scratch per CTA of the persistent kernel:
// enough for a program of either precision.
constexpr size_t kOpsSmem = Layout<float>::smem > Layout<double>::smem ? Layout<float>::smem : Layout<double>::smem;
constexpr size_t kOpsScratch =
    Layout<float>::scratch > Layout<double>::scratch ? Layout<float>::scratch : Layout<double>::scratch;

// Persistent: CTAs take programs from an atomic queue (longest first) until
// it runs dry; each program runs in its own precision (ProgDesc::prec), so a
// batch may mix complex64 and complex128 programs.
__global__ void __launch_bounds__(kOpThreads, 1)
k_run_ops(const ProgDesc* __restrict__ progs, int n_progs, int* queue, char* scratch_base, size_t scratch_stride) {
  extern __shared__ __align__(16) char smem[];
  __shared__ int next;
  char* scratch = scratch_base + scratch_stride * blockIdx.x;
  int pi = blockIdx.x;
  while (true) {
    if (queue != nullptr) {
      if (threadIdx.x == 0) next = atomicAdd(queue, 1);
      __syncthreads();
      pi = next;
      __syncthreads();
    }
    if (pi >= n_progs) break;
    const ProgDesc P = progs[pi];
    if (P.prec == 0)
      run_program_f64(P, smem, scratch);
    else
      run_program<float>(P, smem, scratch);
    if (queue == nullptr) break;
  }
}

// Site-parallel run of ONE program: its two-site updates on disjoint sites
// run on different SMs at once.  Ops are claimed in program order from an
// atomic counter; op o waits until every earlier op on its sites has
// finished: deps[o] = (earlier ops on its first site, on its second site or
// -1), and done[s] counts the finished ops on site s.  Each op reads its
// sites and the bonds around them only (bond[lo] and bond[lo+2] belong to
// the ops on sites lo and lo+1), so every op computes exactly what it
// computes in program order.  No deadlock: an op only waits for ops claimed
// before it by CTAs that are already running, and the earliest unfinished
// op waits for nothing.  A wait is bounded (kDepWaitNs): past it the CTA sets
// ERR_TIMEOUT in the program's error word and every CTA leaves.
constexpr long long kDepWaitNs = 2000000000LL;

__device__ __forceinline__ long long dag_timer() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__global__ void __launch_bounds__(kOpThreads, 1)
k_run_ops_sites(const ProgDesc* __restrict__ progs, const int2* __restrict__ deps, int* ctr, char* scratch_base,
                size_t scratch_stride) {
  extern __shared__ __align__(16) char smem[];
  __shared__ int s_op, s_ok;
  const ProgDesc P = progs[0];
  int* next = ctr;      // op counter
  int* done = ctr + 1;  // finished ops per site
  char* scratch = scratch_base + scratch_stride * blockIdx.x;
  for (;;) {
    if (threadIdx.x == 0) {
      const int o = atomicAdd(next, 1);
      int ok = 1;
      if (o < P.n_ops) {
        const DevOp& op = P.ops[o];
        const int2 d = deps[o];
        const int s0 = op.kind == OP_MOVE_L ? op.site - 1 : op.site;
        const bool two = op.kind != OP_GATE1;
        long long t0 = -1;
        for (unsigned int polls = 1;; ++polls) {
          if (ld_acquire(done + s0) >= d.x && (!two || ld_acquire(done + s0 + 1) >= d.y)) break;
          if ((polls & 255u) == 0u) {
            if (*(volatile int*)P.err & ERR_TIMEOUT) {
              ok = 0;
              break;
            }
            const long long t = dag_timer();
            if (t0 < 0) {
              t0 = t;
            } else if (t - t0 > kDepWaitNs) {
              atomicOr(P.err, ERR_TIMEOUT);
              ok = 0;
              break;
            }
          }
        }
      }
      s_op = o;
      s_ok = ok;
    }
    __syncthreads();
    const int o = s_op;
    if (o >= P.n_ops || !s_ok) break;
    const DevOp& op = P.ops[o];
    if (P.prec == 0)
      run_one_op_f64(P, op, smem, scratch);
    else
      run_one_op_f32(P, op, smem, scratch);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      const int s0 = op.kind == OP_MOVE_L ? op.site - 1 : op.site;
      asm volatile("red.release.gpu.global.add.s32 [%0], 1;" ::"l"(done + s0) : "memory");
      if (op.kind != OP_GATE1) asm volatile("red.release.gpu.global.add.s32 [%0], 1;" ::"l"(done + s0 + 1) : "memory");
    }
  }
  if (threadIdx.x == 0 && blockIdx.x == 0) stat_add(P.stats + ST_N_OPS, (double)P.n_ops);
}

// ------------------------------------------------------------- launchers
// Opt in to the large dynamic shared memory once per device (outside any capture).
cudaError_t configure_ops() {
  cudaError_t e = cudaFuncSetAttribute(k_run_ops, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kOpsSmem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_run_ops_sites, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kOpsSmem);
}

size_t op_scratch_bytes() { return kOpsScratch; }
size_t op_smem_bytes() { return kOpsSmem; }

cudaError_t launch_ops(const ProgDesc* d_progs, int n_progs, int grid, int* d_queue, char* scratch,
                       cudaStream_t st) {
  k_run_ops<<<grid, kOpThreads, kOpsSmem, st>>>(d_progs, n_progs, d_queue, scratch, kOpsScratch);
  return cudaGetLastError();
}

cudaError_t launch_ops_sites(const ProgDesc* d_prog, const int2* d_deps, int* d_ctr, int grid, char* scratch,
                             cudaStream_t st) {
  k_run_ops_sites<<<grid, kOpThreads, kOpsSmem, st>>>(d_prog, d_deps, d_ctr, scratch, kOpsScratch);
  return cudaGetLastError();
}

// ------------------------------------------------- allocation-free variant
// Some callers cannot allocate device memory: a plugin loaded into a host
// application whose device memory belongs to that application's own pool
// allocator (every byte reserved up front, cudaMalloc forbidden or failing),
// or a process running under a fixed device-memory cap.  For them,
// mps_gate2_apply_noalloc runs one fused two-site update with all of its
// scratch (theta, the FP64 eigenvector matrix, the two site offsets,
// statistics and the error word) in the file-scope array below, which every
// GPU that loads this library holds until process exit.
constexpr size_t kNoAllocHeader = 256;  // two site offsets, stats, error word
constexpr size_t kNoAllocScratch = Layout<double>::scratch;  // largest per-CTA scratch (FP64)
constexpr size_t kNoAllocBytes = kNoAllocHeader + kNoAllocScratch;  // 256 B + 512 KiB
static __device__ __align__(256) char g_noalloc_scratch[kNoAllocBytes];
static_assert(64 + sizeof(double) * ST_COUNT <= 240, "stats must end before the error word at 240");

// The site offsets arrive by value and are written into the array's header
// by the kernel itself, so a call issues no host-to-device copy.
template <typename T>
__global__ void __launch_bounds__(kOpThreads, 1)
k_gate2_noalloc(ProgDesc P, DevOp op, char* scratch, int64_t* offs, int64_t hi_offset) {
  extern __shared__ __align__(16) char smem[];
  SmallSmem<T>* sm = reinterpret_cast<SmallSmem<T>*>(smem + Layout<T>::big);
  // the array keeps the previous call's contents: clear what must start at zero
  if (threadIdx.x < ST_COUNT) P.stats[threadIdx.x] = 0.0;
  if (threadIdx.x == 0) {
    *P.err = 0;
    offs[0] = 0;
    offs[1] = hi_offset;
  }
  __syncthreads();
  op_gate2<T>(P, op, smem, sm, scratch);
}

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
char* g_noalloc_ptr[kMaxDevices] = {nullptr};
}  // namespace

// Once per device, with that device current: the device address of the
// array (its name in host code is only a stand-in) and the shared-memory
// opt-in of the kernel.
static int noalloc_setup(int dev, char** out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    char* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return 1;
    e = cudaFuncSetAttribute(k_gate2_noalloc<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)Layout<float>::smem);
    if (e != cudaSuccess) return 1;
    e = cudaFuncSetAttribute(k_gate2_noalloc<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)Layout<double>::smem);
    if (e != cudaSuccess) return 1;
    g_noalloc_ptr[dev] = ptr;
  }
  *out = g_noalloc_ptr[dev];
  return 0;
}

}  // namespace gbmps

#include "../../include/gb300mps.h"

namespace gbmps {
int fail(int code, const std::string& msg);
}

extern "C" int mps_gate2_apply_noalloc(int precision, int trunc_mode, int chi_max, double cutoff, void* sites,
                                       int64_t hi_offset, int* d_bonds, const int* bonds, const double gate[32],
                                       void* cuda_stream) {
  using namespace gbmps;
  if (!sites || !d_bonds || !bonds || !gate) return fail(MPS_ERR_ARG, "NULL argument");
  if (precision != MPS_PREC_FP64 && precision != MPS_PREC_FP32) return fail(MPS_ERR_ARG, "bad precision");
  if (trunc_mode != MPS_TRUNC_EXATN && trunc_mode != MPS_TRUNC_ITENSOR) return fail(MPS_ERR_ARG, "bad trunc_mode");
  for (int i = 0; i < 3; ++i)
    if (bonds[i] < 1) return fail(MPS_ERR_ARG, "bond dimensions must be >= 1");
  if (bonds[0] > kChiLimit || bonds[1] > kChiLimit || bonds[2] > kChiLimit)
    return fail(MPS_ERR_UNSUPPORTED, "bond dimension above 64: the static scratch of the allocation-free "
                                     "entry point holds one 128 x 128 theta (512 KiB)");
  if (chi_max <= 0 || chi_max > kChiLimit) chi_max = kChiLimit;
  {
    // the hi site must start after the lo site, before and after the split
    // (dl x 2 x dm in, dl x 2 x k out with k <= min(2 dl, 2 dr, chi_max))
    const int kmax = std::min(std::min(2 * bonds[0], 2 * bonds[2]), chi_max);
    const int64_t lo_in = 2LL * bonds[0] * bonds[1], lo_out = 2LL * bonds[0] * kmax;
    if (hi_offset < std::max(lo_in, lo_out))
      return fail(MPS_ERR_ARG, "hi_offset overlaps the lo site (it must be >= 2*dl*max(dm, k_max))");
  }
  if (cutoff < 0.0) cutoff = trunc_mode == MPS_TRUNC_EXATN ? 2.2250738585072014e-308 : 1e-6;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(MPS_ERR_UNSUPPORTED, "device ordinal too large");
  char* base = nullptr;
  if (noalloc_setup(dev, &base)) {
    cudaGetLastError();
    return fail(MPS_ERR_CUDA, "cudaGetSymbolAddress / cudaFuncSetAttribute failed for the static scratch");
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(cuda_stream);
  // header: site offsets (2 x int64) at 0, stats (ST_COUNT doubles) at 64, error word at 240
  int64_t* offs = reinterpret_cast<int64_t*>(base);
  ProgDesc P;
  std::memset(&P, 0, sizeof(P));
  P.sites = sites;
  P.site_off = reinterpret_cast<const int64_t*>(base);
  P.bond = d_bonds;
  P.ops = nullptr;
  P.n_ops = 1;
  P.n = 2;
  P.chi_cap = chi_max;
  P.mode = trunc_mode;
  P.flags = 0;
  P.cutoff = cutoff;
  P.stats = reinterpret_cast<double*>(base + 64);
  P.err = reinterpret_cast<int*>(base + 240);
  DevOp op;
  std::memset(&op, 0, sizeof(op));
  op.kind = OP_GATE2;
  op.site = 0;
  op.orient = trunc_mode == MPS_TRUNC_EXATN ? ORIENT_SQRT : ORIENT_TO_HI;
  for (int i = 0; i < 32; ++i) op.m[i] = gate[i];
  char* scratch = base + kNoAllocHeader;
  if (precision == MPS_PREC_FP64)
    k_gate2_noalloc<double><<<1, kOpThreads, Layout<double>::smem, st>>>(P, op, scratch, offs, hi_offset);
  else
    k_gate2_noalloc<float><<<1, kOpThreads, Layout<float>::smem, st>>>(P, op, scratch, offs, hi_offset);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  int herr = 0;
  e = cudaMemcpyAsync(&herr, base + 240, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  if (herr & ERR_NAN) return fail(MPS_ERR_NUMERIC, "non-finite value in the two-site split");
  if (herr & ERR_DIMS) return fail(MPS_ERR_UNSUPPORTED, "bond dimension beyond the kernel limit");
  return MPS_OK;
}
