// Cooperative (grid-wide) kernels of the wide two-site path (sm_103a).
//
// k_wide_eig: eigen-decomposition of the m x m Gram matrix of a two-site
// theta (m up to 2048), the wide counterpart of the single-CTA tridiagonal
// eigensolver in k_ops.cu and of ITensor's Gram route (SVDRefImpl,
// tensor/algs.cc:509-580):
//   1. Householder reduction to real tridiagonal form (LAPACK zhetd2, lower).
//      Rows are owned cyclically by the CTAs.  Step j needs column j after
//      step j-1's rank-2 update; every CTA rebuilds it from a column buffer
//      that the row owners wrote during step j-1 and the (v, w) of step
//      j-1, so one grid barrier per column suffices: owners apply the
//      pending update to their rows and form p = tau A v in the same pass.
//   2. Every eigenvalue by 33-section bisection (Sturm counts), one warp per
//      eigenvalue on its unreduced block.
//   3. Ranking (descending), the keep rule (keep.cuh) on the sorted values.
//   4. Kept eigenvectors: one twisted factorisation per vector, then the
//      back-transform by the stored reflectors, 8 (FP32) or 4 (FP64)
//      columns per CTA staged in shared memory.
// k_wide_qr: Householder QR (LAPACK zgeqr2 + zung2r conventions) of a view,
// columns owned cyclically by the CTAs, one grid barrier per column.
//
// All CTAs of a launch are co-resident (cooperative launch, grid <= SMs x
// occupancy).  The grid barrier is a monotonic arrival counter with a 2 s
// bound on every wait: a CTA that gives up sets kCoopTimeout and all CTAs
// leave the kernel at their next barrier.  Data written by other CTAs during
// the launch is read with ld.global.cg (L2), never through L1.
#include <math.h>

#include "keep.cuh"
#include "wide.hpp"

namespace gbmps {

template <typename T>
struct CoopPrec;
template <>
struct CoopPrec<float> {
  static constexpr double eps = 1.1920929e-07;
  static constexpr int rounds = 7;            // 33^7 > 2^35
  static constexpr double tri_flush = 1e-30;  // relative |column|^2 flushed in the tridiagonalisation
  static constexpr double tiny = 1e-36;
  static constexpr int cb = 8;                // back-transform columns per CTA
};
template <>
struct CoopPrec<double> {
  static constexpr double eps = 2.220446049250313e-16;
  static constexpr int rounds = 12;  // 33^12 > 2^60
  static constexpr double tri_flush = 1e-60;
  static constexpr double tiny = 1e-280;
  static constexpr int cb = 4;
};

constexpr int kCoopThreads = 256;
constexpr int kCoopWarps = kCoopThreads / 32;
constexpr long long kBarrierNs = 2000000000LL;

struct GridBar {
  unsigned int count;  // arrivals so far (zeroed before each launch)
  unsigned int pad;
  int err;
  int k;
};

__device__ __forceinline__ long long coop_timer() {
  long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

template <typename T>
__device__ __forceinline__ cx<T> ldcg(const cx<T>* p) {
  cx<T> z;
  z.re = __ldcg(&p->re);
  z.im = __ldcg(&p->im);
  return z;
}
template <typename T>
__device__ __forceinline__ void stcg(cx<T>* p, cx<T> z) {
  __stcg(&p->re, z.re);
  __stcg(&p->im, z.im);
}

// Grid-wide barrier with a bounded wait.  The counter only grows: a CTA's
// arrival (release atomic) returns the count before it, which fixes the
// barrier's epoch and the count that marks everyone's arrival; the CTA then
// spins on acquire loads of the counter until it reaches that mark (later
// barriers only raise it further).  Every 256 polls it checks the 2 s bound
// and the error word another CTA may have set.  Returns false when any CTA
// timed out (the caller leaves the kernel).
__device__ bool grid_sync(GridBar* b) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned int old;
    asm volatile("atom.add.release.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(&b->count) : "memory");
    const unsigned int G = gridDim.x;
    const unsigned int target = (old / G + 1u) * G;
    unsigned int cur = old + 1u;
    long long t0 = -1;
    for (unsigned int polls = 1; cur < target; ++polls) {
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(&b->count) : "memory");
      if ((polls & 255u) == 0u) {
        if (*(volatile int*)&b->err) {
          ok = 0;
          break;
        }
        const long long t = coop_timer();
        if (t0 < 0) {
          t0 = t;
        } else if (t - t0 > kBarrierNs) {
          atomicOr(&b->err, kCoopTimeout);
          ok = 0;
          break;
        }
      }
    }
    s_ok = ok && *(volatile int*)&b->err == 0;
  }
  __syncthreads();
  return s_ok != 0;
}

// Block-wide sum in a fixed order (identical in every CTA); `red` holds
// kCoopWarps entries of R.
template <typename R>
__device__ R coop_sum(R v, R* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  R s = R(0);
  for (int w = 0; w < kCoopWarps; ++w) s += red[w];
  __syncthreads();
  return s;
}
template <typename T>
__device__ cx<T> coop_sum_c(cx<T> v, cx<T>* red) {
  for (int o = 16; o > 0; o >>= 1) {
    v.re += __shfl_xor_sync(0xffffffffu, v.re, o);
    v.im += __shfl_xor_sync(0xffffffffu, v.im, o);
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  cx<T> s = mk<T>(T(0), T(0));
  for (int w = 0; w < kCoopWarps; ++w) s = s + red[w];
  __syncthreads();
  return s;
}

// ------------------------------------------------------------ eigensolver
template <typename T>
struct EigWork {
  GridBar* bar;
  cx<T>* colbuf;  // [2][m]
  cx<T>* pvec;    // [2][m]
  cx<T>* part;    // [2][grid]
  T* td;
  T* te;
  cx<T>* ttau;
  T* lamj;        // eigenvalue of each tridiagonal index (block-local order)
  int* perm;      // rank -> index
};

__host__ __device__ inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

template <typename T>
__host__ __device__ inline size_t eig_work_bytes_t(int m, int grid) {
  const size_t c = sizeof(cx<T>);
  return al256(sizeof(GridBar)) + al256(2 * m * c) + al256(2 * m * c) + al256(2 * (size_t)grid * c) +
         2 * al256(m * sizeof(T)) + al256(m * c) + al256(m * sizeof(T)) + al256(m * sizeof(int));
}

template <typename T>
__device__ EigWork<T> eig_work(void* base, int m, int grid) {
  char* w = reinterpret_cast<char*>(base);
  const size_t c = sizeof(cx<T>);
  EigWork<T> e;
  e.bar = reinterpret_cast<GridBar*>(w);
  w += al256(sizeof(GridBar));
  e.colbuf = reinterpret_cast<cx<T>*>(w);
  w += al256(2 * m * c);
  e.pvec = reinterpret_cast<cx<T>*>(w);
  w += al256(2 * m * c);
  e.part = reinterpret_cast<cx<T>*>(w);
  w += al256(2 * (size_t)grid * c);
  e.td = reinterpret_cast<T*>(w);
  w += al256(m * sizeof(T));
  e.te = reinterpret_cast<T*>(w);
  w += al256(m * sizeof(T));
  e.ttau = reinterpret_cast<cx<T>*>(w);
  w += al256(m * c);
  e.lamj = reinterpret_cast<T*>(w);
  w += al256(m * sizeof(T));
  e.perm = reinterpret_cast<int*>(w);
  return e;
}

// Shared memory: [td te (T) | bs bt (int) | union: 4 vectors of m / W block
// (m x cb) and a staged reflector / m doubles | reduction scratch]
template <typename T>
__host__ __device__ inline size_t eig_smem_bytes(int m) {
  const size_t head = al256(2 * m * sizeof(T)) + al256(2 * m * sizeof(int));
  size_t u = 4 * (size_t)m * sizeof(cx<T>);
  const size_t wb = (size_t)m * (CoopPrec<T>::cb + 1) * sizeof(cx<T>);
  if (wb > u) u = wb;
  if ((size_t)m * sizeof(double) > u) u = (size_t)m * sizeof(double);
  return head + al256(u) + 4096;
}

// Twisted-factorisation eigenvector of the tridiagonal (sd, se) for eigenvalue
// lam on block [s, t], into column c of W (m x ld); real parts first hold D+
// and imaginary parts D- of the two factorisations, then the vector (the
// single-CTA tri_twisted of k_ops.cu on global memory).
template <typename T>
__device__ void coop_twisted(cx<T>* W, int m, int ld, int c, T lam, int s, int t, const T* sd, const T* se) {
  T scale = T(0);
  for (int i = s; i <= t; ++i) scale = fmax(scale, fabs(sd[i] - lam) + (i < t ? fabs(se[i]) : T(0)));
  const T tiny = fmax(T(CoopPrec<T>::eps) * T(CoopPrec<T>::eps) * scale, T(1e-35));
  auto guard = [&](T v) { return fabs(v) < tiny ? -tiny : v; };
  auto at = [&](int i) -> cx<T>& { return W[(int64_t)i * ld + c]; };
  at(s).re = sd[s] - lam;
  for (int i = s + 1; i <= t; ++i) {
    const T e = se[i - 1];
    at(i).re = (sd[i] - lam) - e * e / guard(at(i - 1).re);
  }
  at(t).im = sd[t] - lam;
  for (int i = t - 1; i >= s; --i) {
    const T e = se[i];
    at(i).im = (sd[i] - lam) - e * e / guard(at(i + 1).im);
  }
  int r = s;
  T best = T(3.0e38);
  for (int i = s; i <= t; ++i) {
    const T g = fabs(at(i).re + at(i).im - (sd[i] - lam));
    if (g < best) {
      best = g;
      r = i;
    }
  }
  const T big = T(1e15), shrink = T(1e-15);
  T nrm = T(1);
  at(r).re = T(1);
  int lo_done = r;
  for (int i = r - 1; i >= s; --i) {
    T z = -(se[i] / guard(at(i).re)) * at(i + 1).re;
    if (fabs(z) > big) {
      for (int u = i + 1; u <= r; ++u) at(u).re *= shrink;
      nrm *= shrink * shrink;
      z *= shrink;
    }
    at(i).re = z;
    nrm += z * z;
    lo_done = i;
  }
  for (int i = r + 1; i <= t; ++i) {
    T z = -(se[i - 1] / guard(at(i).im)) * at(i - 1).re;
    if (fabs(z) > big) {
      for (int u = lo_done; u < i; ++u) at(u).re *= shrink;
      nrm *= shrink * shrink;
      z *= shrink;
    }
    at(i).re = z;
    nrm += z * z;
  }
  const T inv = T(1) / sqrt(nrm);
  for (int i = 0; i < m; ++i) {
    const bool in = i >= s && i <= t;
    at(i) = mk<T>(in ? at(i).re * inv : T(0), T(0));
  }
}

template <typename T>
__global__ void __launch_bounds__(kCoopThreads, 1) k_wide_eig(WideEigArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int m = a.m, G = gridDim.x, cta = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  EigWork<T> wk = eig_work<T>(a.work, m, a.grid0);
  cx<T>* A = reinterpret_cast<cx<T>*>(a.G);
  T* sd = reinterpret_cast<T*>(smem);
  T* se = sd + m;
  int* sbs = reinterpret_cast<int*>(smem + al256(2 * m * sizeof(T)));
  int* sbt = sbs + m;
  unsigned char* uni = smem + al256(2 * m * sizeof(T)) + al256(2 * m * sizeof(int));
  size_t usz = 4 * (size_t)m * sizeof(cx<T>);
  {
    const size_t wb = (size_t)m * (CoopPrec<T>::cb + 1) * sizeof(cx<T>);
    if (wb > usz) usz = wb;
    if ((size_t)m * sizeof(double) > usz) usz = (size_t)m * sizeof(double);
  }
  unsigned char* redb = uni + al256(usz);
  T* red = reinterpret_cast<T*>(redb);
  cx<T>* redc = reinterpret_cast<cx<T>*>(redb + 256);
  double* redd = reinterpret_cast<double*>(redb + 1024);

  // ---- 1. tridiagonalisation
  cx<T>* vprev = reinterpret_cast<cx<T>*>(uni);
  cx<T>* wprev = vprev + m;
  cx<T>* vcur = wprev + m;
  double tr_part = 0.0;
  for (int i = tid; i < m; i += nt) tr_part += (double)ldcg(A + (int64_t)i * m + i).re;
  const double trace = coop_sum<double>(tr_part, redd);
  const T flush2 = T(CoopPrec<T>::tri_flush * trace * trace + CoopPrec<T>::tiny);
  for (int i = cta + G * tid; i < m; i += G * nt) stcg(wk.colbuf + i, A[(int64_t)i * m]);
  if (!grid_sync(wk.bar)) return;
  // After the barrier of step j-1 every CTA needs p_{j-1} (to form w_{j-1})
  // and column j's buffer; both were written before that barrier, so their
  // loads are issued together (one L2 round trip per column).
  cx<T>* craw = vcur + m;  // column j as the owners wrote it (before step j-1's update)
  bool hasprev = false;
  cx<T> tau_prev = mk<T>(T(0), T(0));
  for (int j = 0; j + 1 < m; ++j) {
    const int buf = j & 1;
    const cx<T>* cb_in = wk.colbuf + buf * m;
    cx<T>* cb_out = wk.colbuf + (buf ^ 1) * m;
    if (hasprev) {
      // (d) of step j-1: w = p - 1/2 tau (p^H v) v
      const int pb = buf ^ 1;
      if (warp == 0) {
        // fixed summation order: lane-strided partial sums, then a butterfly
        cx<T> d = mk<T>(T(0), T(0));
        for (int q = lane; q < G; q += 32) d = d + ldcg(wk.part + pb * G + q);
        for (int o = 16; o > 0; o >>= 1) {
          d.re += __shfl_xor_sync(0xffffffffu, d.re, o);
          d.im += __shfl_xor_sync(0xffffffffu, d.im, o);
        }
        if (lane == 0) redc[0] = d;
      }
      for (int i = j + tid; i < m; i += nt) {
        wprev[i] = ldcg(wk.pvec + pb * m + i);
        craw[i] = ldcg(cb_in + i);
      }
      __syncthreads();
      const cx<T> a2 = scl(tau_prev * redc[0], T(-0.5));
      for (int i = j + tid; i < m; i += nt) {
        const cx<T> v = vcur[i];
        wprev[i] = wprev[i] + a2 * v;
        vprev[i] = v;
      }
    } else {
      for (int i = j + tid; i < m; i += nt) craw[i] = ldcg(cb_in + i);
    }
    __syncthreads();
    // (a) column j of the current matrix (rows j..m-1), kept in vcur
    const cx<T> cwj = hasprev ? conj(wprev[j]) : mk<T>(T(0), T(0));
    const cx<T> cvj = hasprev ? conj(vprev[j]) : mk<T>(T(0), T(0));
    T s_part = T(0);
    for (int i = j + tid; i < m; i += nt) {
      cx<T> c = craw[i];
      if (hasprev) c = c - (vprev[i] * cwj + wprev[i] * cvj);
      vcur[i] = c;
      if (i >= j + 2) s_part += abs2(c);
    }
    const T s = coop_sum<T>(s_part, red);
    const T dj = vcur[j].re;
    const cx<T> alpha = vcur[j + 1];
    __syncthreads();  // every thread has read alpha before vcur is rewritten
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
    const cx<T> tau = mk<T>(tr, ti);
    for (int i = j + 2 + tid; i < m; i += nt) {
      const cx<T> x = vcur[i];
      vcur[i] = refl ? mk<T>(x.re * ir - x.im * ii, x.re * ii + x.im * ir) : mk<T>(T(0), T(0));
    }
    if (tid == 0) {
      vcur[j + 1] = mk<T>(T(1), T(0));
      if (cta == 0) {
        wk.td[j] = dj;
        wk.te[j] = beta;
        wk.ttau[j] = tau;
      }
    }
    __syncthreads();
    // (b) owned rows: pending update of step j-1, p = tau A v, next column
    cx<T> dpart = mk<T>(T(0), T(0));
    for (int li = warp;; li += kCoopWarps) {
      const int i = cta + G * li;
      if (i >= m) break;
      if (i < j) continue;
      cx<T>* Ai = A + (int64_t)i * m;
      if (i == j) {  // row j is finished: it stores the reflector v_j
        for (int c = j + 1 + lane; c < m; c += 32) Ai[c] = vcur[c];
        continue;
      }
      const cx<T> vpi = hasprev ? vprev[i] : mk<T>(T(0), T(0));
      const cx<T> wpi = hasprev ? wprev[i] : mk<T>(T(0), T(0));
      cx<T> acc = mk<T>(T(0), T(0));
      cx<T> first = mk<T>(T(0), T(0));
      for (int c = j + 1 + lane; c < m; c += 32) {
        cx<T> x = Ai[c];
        if (hasprev) {
          x = x - (vpi * conj(wprev[c]) + wpi * conj(vprev[c]));
          Ai[c] = x;
        }
        if (c == j + 1) first = x;
        fma_c(acc, x, vcur[c]);
      }
      for (int o = 16; o > 0; o >>= 1) {
        acc.re += __shfl_xor_sync(0xffffffffu, acc.re, o);
        acc.im += __shfl_xor_sync(0xffffffffu, acc.im, o);
      }
      if (lane == 0) {
        const cx<T> p = tau * acc;
        stcg(wk.pvec + buf * m + i, p);
        stcg(cb_out + i, first);
        fma_cj(dpart, p, vcur[i]);
      }
    }
    const cx<T> dsum_cta = coop_sum_c<T>(dpart, redc);
    if (tid == 0) stcg(wk.part + buf * G + cta, dsum_cta);
    if (!grid_sync(wk.bar)) return;
    hasprev = refl;
    tau_prev = tau;
  }
  if (cta == 0 && tid == 0) {
    // last diagonal entry: column m-1's buffer minus step m-2's rank-2 term
    cx<T> c = ldcg(wk.colbuf + ((m - 1) & 1) * m + (m - 1));
    if (hasprev) {
      const int pb = (m - 2) & 1;
      cx<T> d = mk<T>(T(0), T(0));
      for (int q = 0; q < G; ++q) d = d + ldcg(wk.part + pb * G + q);
      const cx<T> v = vcur[m - 1];
      const cx<T> w = ldcg(wk.pvec + pb * m + (m - 1)) + scl(tau_prev * d, T(-0.5)) * v;
      c = c - (v * conj(w) + w * conj(v));
    }
    wk.td[m - 1] = c.re;
    wk.te[m - 1] = T(0);
    if (m == 1) wk.ttau[0] = mk<T>(T(0), T(0));
  }
  if (!grid_sync(wk.bar)) return;

  // ---- 2. eigenvalues: unreduced blocks, 33-section bisection per eigenvalue
  const T eps = T(CoopPrec<T>::eps);
  for (int i = tid; i < m; i += nt) {
    sd[i] = __ldcg(wk.td + i);
    se[i] = __ldcg(wk.te + i);
  }
  __syncthreads();
  if (tid == 0) {
    int s0 = 0;
    for (int i = 0; i < m; ++i) {
      bool split = i == m - 1;
      if (!split && fabs(se[i]) <= eps * (fabs(sd[i]) + fabs(sd[i + 1]))) {
        split = true;
        se[i] = T(0);
      }
      if (split) {
        for (int r = s0; r <= i; ++r) {
          sbs[r] = s0;
          sbt[r] = i;
        }
        s0 = i + 1;
      }
    }
  }
  __syncthreads();
  for (int j = cta * kCoopWarps + warp; j < m; j += G * kCoopWarps) {
    const int s0 = sbs[j], t0 = sbt[j], local = j - s0;
    T lo = T(3.0e38), hi = T(-3.0e38), maxe2 = T(1);
    for (int i = s0 + lane; i <= t0; i += 32) {
      const T el = i > s0 ? fabs(se[i - 1]) : T(0), er = i < t0 ? fabs(se[i]) : T(0);
      lo = fmin(lo, sd[i] - el - er);
      hi = fmax(hi, sd[i] + el + er);
      maxe2 = fmax(maxe2, er * er);
    }
    for (int o = 16; o > 0; o >>= 1) {
      lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
      maxe2 = fmax(maxe2, __shfl_xor_sync(0xffffffffu, maxe2, o));
    }
    const T pivmin = T(sizeof(T) == 4 ? 1.2e-38 : 2.3e-308) * maxe2;
    const T pad = T(4) * eps * fmax(fabs(lo), fabs(hi)) + pivmin;
    T aa = lo - pad, bb = hi + pad;
    for (int round = 0; round < CoopPrec<T>::rounds; ++round) {
      const T w = (bb - aa) / T(33);
      const T x = aa + w * T(lane + 1);
      int cnt = 0;
      T qv = T(1);
      for (int i = s0; i <= t0; ++i) {
        const T e2 = i > s0 ? se[i - 1] * se[i - 1] : T(0);
        qv = (sd[i] - x) - (i > s0 ? e2 / qv : T(0));
        if (fabs(qv) < pivmin) qv = -pivmin;
        cnt += qv < T(0);
      }
      const unsigned ball = __ballot_sync(0xffffffffu, cnt > local);
      const int f = ball ? __ffs(ball) - 1 : 32;
      const T na = aa + w * T(f), nb = f == 32 ? bb : aa + w * T(f + 1);
      aa = na;
      bb = nb;
    }
    if (lane == 0) __stcg(wk.lamj + j, T(0.5) * (aa + bb));
  }
  if (!grid_sync(wk.bar)) return;

  // ---- 3. ranking (descending, ties by index)
  T* slam = reinterpret_cast<T*>(uni);
  for (int i = tid; i < m; i += nt) slam[i] = __ldcg(wk.lamj + i);
  __syncthreads();
  for (int j = cta * nt + tid; j < m; j += G * nt) {
    const T lj = slam[j];
    int r = 0;
    for (int i = 0; i < m; ++i) {
      const T li = slam[i];
      r += (li > lj) || (li == lj && i < j);
    }
    __stcg(wk.perm + r, j);
    __stcg(a.lam + r, (double)lj);
  }
  if (!grid_sync(wk.bar)) return;

  if (cta == 0 && tid == 0) a.status_err[0] = *(volatile int*)&wk.bar->err;
}

// Kept eigenvectors (phase 2 of the decomposition): columns 0..kv-1 of W
// (row stride ld) are the eigenvectors of ranks 0..kv-1, from the
// tridiagonal, ranks and reflectors that k_wide_eig left in G and the work
// buffer.
template <typename T>
__global__ void __launch_bounds__(kCoopThreads, 1) k_wide_eigvec(WideEigArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int m = a.m, G = gridDim.x, cta = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  EigWork<T> wk = eig_work<T>(a.work, m, a.grid0);
  const cx<T>* A = reinterpret_cast<const cx<T>*>(a.G);
  T* sd = reinterpret_cast<T*>(smem);
  T* se = sd + m;
  int* sbs = reinterpret_cast<int*>(smem + al256(2 * m * sizeof(T)));
  int* sbt = sbs + m;
  unsigned char* uni = smem + al256(2 * m * sizeof(T)) + al256(2 * m * sizeof(int));
  size_t usz = 4 * (size_t)m * sizeof(cx<T>);
  {
    const size_t wb = (size_t)m * (CoopPrec<T>::cb + 1) * sizeof(cx<T>);
    if (wb > usz) usz = wb;
    if ((size_t)m * sizeof(double) > usz) usz = (size_t)m * sizeof(double);
  }
  unsigned char* redb = uni + al256(usz);
  const T eps = T(CoopPrec<T>::eps);
  for (int i = tid; i < m; i += nt) {
    sd[i] = __ldcg(wk.td + i);
    se[i] = __ldcg(wk.te + i);
  }
  __syncthreads();
  if (tid == 0) {
    int s0 = 0;
    for (int i = 0; i < m; ++i) {
      bool split = i == m - 1;
      if (!split && fabs(se[i]) <= eps * (fabs(sd[i]) + fabs(sd[i + 1]))) {
        split = true;
        se[i] = T(0);
      }
      if (split) {
        for (int r = s0; r <= i; ++r) {
          sbs[r] = s0;
          sbt[r] = i;
        }
        s0 = i + 1;
      }
    }
  }
  __syncthreads();
  const int k = a.kv;
  // ---- twisted vectors of the kept eigenvalues
  cx<T>* W = reinterpret_cast<cx<T>*>(a.W);
  for (int c = cta * nt + tid; c < k; c += G * nt) {
    const int j = __ldcg(wk.perm + c);
    coop_twisted<T>(W, m, a.ld, c, __ldcg(wk.lamj + j), sbs[j], sbt[j], sd, se);
  }
  if (!grid_sync(wk.bar)) return;

  // ---- back-transform W <- Q W, CB columns per CTA in shared memory
  constexpr int CB = CoopPrec<T>::cb;
  constexpr int Q = kCoopThreads / CB;  // row chunks
  cx<T>* Ws = reinterpret_cast<cx<T>*>(uni);
  cx<T>* vb = Ws + (size_t)m * CB;                      // staged reflector (m entries)
  cx<T>* part = reinterpret_cast<cx<T>*>(redb + 1024);  // per-warp partial sums (CB each)
  const int ngroups = (k + CB - 1) / CB;
  for (int g = cta; g < ngroups; g += G) {
    const int c0 = g * CB;
    for (int t = tid; t < m * CB; t += nt) {
      const int i = t / CB, c = t - i * CB;
      Ws[t] = c0 + c < k ? ldcg(W + (int64_t)i * a.ld + c0 + c) : mk<T>(T(0), T(0));
    }
    __syncthreads();
    const int c = tid % CB, q = tid / CB;
    // reflector j (row j of A, v[0] = 1 stored) staged in vb for all threads;
    // the next one's loads are issued before this one's products
    constexpr int PF = kWideM / kCoopThreads;
    cx<T> pre[PF];
    auto fetch = [&](int j) {
      const cx<T>* v = A + (int64_t)j * m + (j + 1);
      const int L = m - j - 1;
#pragma unroll
      for (int u = 0; u < PF; ++u) {
        const int i = tid + u * kCoopThreads;
        pre[u] = i < L ? ldcg(v + i) : mk<T>(T(0), T(0));
      }
    };
    if (m >= 2) fetch(m - 2);
    for (int j = m - 2; j >= 0; --j) {
      const int L = m - j - 1;
#pragma unroll
      for (int u = 0; u < PF; ++u) {
        const int i = tid + u * kCoopThreads;
        if (i < L) vb[i] = pre[u];
      }
      const cx<T> tj = ldcg(wk.ttau + j);
      __syncthreads();
      if (j > 0) fetch(j - 1);
      if (tj.re == T(0) && tj.im == T(0)) {
        __syncthreads();  // vb is rewritten next
        continue;
      }
      cx<T> acc = mk<T>(T(0), T(0));
      for (int r = q; r < L; r += Q) fma_cj(acc, vb[r], Ws[(j + 1 + r) * CB + c]);
      // reduce over the Q row chunks: lanes q, q+32/CB, ... share c within a warp
      for (int o = 16; o >= CB; o >>= 1) {
        acc.re += __shfl_xor_sync(0xffffffffu, acc.re, o);
        acc.im += __shfl_xor_sync(0xffffffffu, acc.im, o);
      }
      if (lane < CB) part[warp * CB + lane] = acc;
      __syncthreads();
      cx<T> sc = mk<T>(T(0), T(0));
      for (int w = 0; w < kCoopWarps; ++w) sc = sc + part[w * CB + c];
      sc = tj * sc;
      for (int r = q; r < L; r += Q) {
        cx<T>& x = Ws[(j + 1 + r) * CB + c];
        x = x - vb[r] * sc;
      }
      __syncthreads();
    }
    for (int t = tid; t < m * CB; t += nt) {
      const int i = t / CB, cc = t - i * CB;
      if (c0 + cc < k) W[(int64_t)i * a.ld + c0 + cc] = Ws[t];
    }
    __syncthreads();
  }
  if (cta == 0 && tid == 0) a.status_err[0] = *(volatile int*)&wk.bar->err;
}

// ------------------------------------------------------------------- QR
template <typename T>
struct QrWork {
  GridBar* bar;
  cx<T>* MT;    // nc x mr: row c = column c of the input (then R above, reflectors below)
  cx<T>* QT;    // k x mr: row c = column c of Q
  cx<T>* tau;   // k
};
template <typename T>
__host__ __device__ inline size_t qr_work_bytes_t(int mr, int nc) {
  const int k = mr < nc ? mr : nc;
  const size_t c = sizeof(cx<T>);
  return al256(sizeof(GridBar)) + al256((size_t)nc * mr * c) + al256((size_t)k * mr * c) + al256((size_t)k * c);
}
template <typename T>
__device__ QrWork<T> qr_work(void* base, int mr, int nc) {
  const int k = mr < nc ? mr : nc;
  char* w = reinterpret_cast<char*>(base);
  const size_t c = sizeof(cx<T>);
  QrWork<T> q;
  q.bar = reinterpret_cast<GridBar*>(w);
  w += al256(sizeof(GridBar));
  q.MT = reinterpret_cast<cx<T>*>(w);
  w += al256((size_t)nc * mr * c);
  q.QT = reinterpret_cast<cx<T>*>(w);
  w += al256((size_t)k * mr * c);
  q.tau = reinterpret_cast<cx<T>*>(w);
  return q;
}

template <typename T>
struct QrArgsT {
  CMat<T> M;        // input view mr x nc
  CMatOut<T> Q;     // output view mr x k (element (i, c) = Q(i, c), conjugated if qconj)
  int qconj;
  int own_smem;     // the CTA's own columns live in shared memory during the factorisation
  cx<T>* R;         // k x nc row-major
  void* work;
  int* err;
};

// Copy rows [0, nr) x cols [0, nc) of src(i, j) into dst[j * ldd + i] (a
// transposing copy) or dst(i, j) through 32 x 32 shared tiles, tiles spread
// over the grid.
template <typename T, typename Src, typename Dst>
__device__ void grid_tile_copy(int nr, int nc, bool lanes_on_rows, Src src, Dst dst, cx<T> (*tile)[33]) {
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int tr = (nr + 31) / 32, tcn = (nc + 31) / 32;
  for (int t = blockIdx.x; t < tr * tcn; t += gridDim.x) {
    const int r0 = (t / tcn) * 32, c0 = (t % tcn) * 32;
    for (int q = ty; q < 32; q += kCoopWarps) {
      const int rr = lanes_on_rows ? tx : q, cc = lanes_on_rows ? q : tx;
      if (r0 + rr < nr && c0 + cc < nc) tile[rr][cc] = src(r0 + rr, c0 + cc);
    }
    __syncthreads();
    for (int q = ty; q < 32; q += kCoopWarps) {
      // lanes along rows: dst is written along its row index i
      const int rr = tx, cc = q;
      if (r0 + rr < nr && c0 + cc < nc) dst(r0 + rr, c0 + cc, tile[rr][cc]);
    }
    __syncthreads();
  }
}

// Dynamic shared memory of k_wide_qr: 32 x 33 tile, reduction scratch, two
// staged reflectors (2 x mr), then (own_smem) the CTA's own columns.
template <typename T>
__host__ __device__ inline size_t qr_smem_bytes(int mr, int nown, bool own) {
  return al256(sizeof(cx<T>) * 32 * 33) + 256 + al256(2 * (size_t)mr * sizeof(cx<T>)) +
         (own ? (size_t)nown * mr * sizeof(cx<T>) : 0);
}

template <typename T>
__global__ void __launch_bounds__(kCoopThreads, 1) k_wide_qr(QrArgsT<T> a) {
  extern __shared__ __align__(16) unsigned char qsm[];
  const int mr = a.M.rows, nc = a.M.cols, k = mr < nc ? mr : nc;
  const int G = gridDim.x, cta = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  QrWork<T> wk = qr_work<T>(a.work, mr, nc);
  cx<T>(*tile)[33] = reinterpret_cast<cx<T>(*)[33]>(qsm);
  T* s_sum = reinterpret_cast<T*>(qsm + al256(sizeof(cx<T>) * 32 * 33));
  cx<T>* vbuf = reinterpret_cast<cx<T>*>(qsm + al256(sizeof(cx<T>) * 32 * 33) + 256);
  cx<T>* own = vbuf + 2 * (size_t)mr;
  const bool osm = a.own_smem != 0;
  const int nown = cta < nc ? (nc - cta + G - 1) / G : 0;
  // own column li (global index cta + G li): shared memory, or its row of MT
  auto col = [&](int li) -> cx<T>* { return osm ? own + (size_t)li * mr : wk.MT + (int64_t)(cta + G * li) * mr; };
  auto ld = [&](const cx<T>* p) { return osm ? *p : ldcg(p); };
  auto st = [&](cx<T>* p, cx<T> z) {
    if (osm)
      *p = z;
    else
      stcg(p, z);
  };
  // 0. MT[c][i] = M(i, c)
  {
    const CMat<T> M = a.M;
    cx<T>* MT = wk.MT;
    auto src = [&](int i, int c) {
      cx<T> z = M.p[(int64_t)i * M.rs + (int64_t)c * M.cs];
      if (M.conj) z.im = -z.im;
      return z;
    };
    auto dst = [&](int i, int c, cx<T> z) { MT[(int64_t)c * mr + i] = z; };
    grid_tile_copy<T>(mr, nc, M.rs == 1, src, dst, tile);
  }
  if (!grid_sync(wk.bar)) return;
  if (osm)
    for (int li = 0; li < nown; ++li)
      for (int i = tid; i < mr; i += kCoopThreads) own[(size_t)li * mr + i] = ldcg(wk.MT + (int64_t)(cta + G * li) * mr + i);
  __syncthreads();
  const T tiny = T(CoopPrec<T>::tiny);
  // 1. reflectors; column c is owned by CTA c % G, one warp per owned column
  for (int j = 0; j < k; ++j) {
    if (j % G == cta) {
      // the whole owner CTA forms reflector j (block-wide norm) and
      // publishes it in MT (row j) for the other CTAs
      cx<T>* x = col(j / G);
      cx<T>* xg = wk.MT + (int64_t)j * mr;
      T s_part = T(0);
      for (int i = j + 1 + tid; i < mr; i += kCoopThreads) s_part += abs2(ld(x + i));
      const T s = coop_sum<T>(s_part, s_sum);
      const cx<T> alpha = ld(x + j);
      const T ar = alpha.re, ai = alpha.im;
      const T nrm2 = ar * ar + ai * ai + s;
      const bool refl = !(s == T(0) && ai == T(0)) && nrm2 > tiny;
      cx<T> tau = mk<T>(T(0), T(0));
      if (refl) {
        const T beta = -copysign(sqrt(nrm2), ar);
        const T dr = ar - beta, di = ai, den = dr * dr + di * di;
        const T ir = dr / den, ii = -di / den;
        tau = mk<T>((beta - ar) / beta, -ai / beta);
        for (int i = j + 1 + tid; i < mr; i += kCoopThreads) {
          const cx<T> v = ld(x + i);
          const cx<T> sv = mk<T>(v.re * ir - v.im * ii, v.re * ii + v.im * ir);
          st(x + i, sv);
          if (osm) stcg(xg + i, sv);
        }
        __syncthreads();  // every thread has read alpha
        if (tid == 0) {
          st(x + j, mk<T>(beta, T(0)));
          if (osm) stcg(xg + j, mk<T>(beta, T(0)));
        }
      }
      if (tid == 0) stcg(wk.tau + j, tau);
    }
    if (!grid_sync(wk.bar)) return;
    const cx<T> tj = ldcg(wk.tau + j);
    if (tj.re == T(0) && tj.im == T(0)) continue;
    const cx<T> ctau = conj(tj);
    const cx<T>* v = wk.MT + (int64_t)j * mr;
    for (int i = j + 1 + tid; i < mr; i += kCoopThreads) vbuf[i] = ldcg(v + i);
    __syncthreads();
    for (int li = warp; li < nown; li += kCoopWarps) {
      const int c = cta + G * li;
      if (c <= j) continue;
      cx<T>* y = col(li);
      cx<T> w = mk<T>(T(0), T(0));
      for (int i = j + 1 + lane; i < mr; i += 32) fma_cj(w, vbuf[i], ld(y + i));
      for (int o = 16; o > 0; o >>= 1) {
        w.re += __shfl_xor_sync(0xffffffffu, w.re, o);
        w.im += __shfl_xor_sync(0xffffffffu, w.im, o);
      }
      w = w + ld(y + j);
      const cx<T> tw = ctau * w;
      for (int i = j + 1 + lane; i < mr; i += 32) st(y + i, ld(y + i) - vbuf[i] * tw);
      __syncwarp();
      if (lane == 0) st(y + j, ld(y + j) - tw);
      __syncwarp();
    }
    __syncthreads();  // column j+1 is final before its owner forms the next reflector
  }
  if (osm) {
    for (int li = 0; li < nown; ++li)
      for (int i = tid; i < mr; i += kCoopThreads) stcg(wk.MT + (int64_t)(cta + G * li) * mr + i, own[(size_t)li * mr + i]);
  }
  if (!grid_sync(wk.bar)) return;
  // 2. R (k x nc): R[r][c] = MT[c][r] for r <= c
  {
    cx<T>* MT = wk.MT;
    cx<T>* R = a.R;
    auto src = [&](int c, int r) { return r <= c ? ldcg(MT + (int64_t)c * mr + r) : mk<T>(T(0), T(0)); };
    // rows of the copy = c (nc), cols = r (k); write R row-major along c
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int tr = (nc + 31) / 32, tcn = (k + 31) / 32;
    for (int t = blockIdx.x; t < tr * tcn; t += gridDim.x) {
      const int c0 = (t / tcn) * 32, r0 = (t % tcn) * 32;
      for (int q = ty; q < 32; q += kCoopWarps)
        if (c0 + q < nc && r0 + tx < k) tile[q][tx] = src(c0 + q, r0 + tx);
      __syncthreads();
      for (int q = ty; q < 32; q += kCoopWarps)
        if (r0 + q < k && c0 + tx < nc) R[(int64_t)(r0 + q) * nc + c0 + tx] = tile[tx][q];
      __syncthreads();
    }
  }
  // 3. Q columns: q_c = H_0 ... H_c e_c.  The CTA walks the reflectors from
  // its largest own column down to 0, each staged once in shared memory for
  // all its warps (double-buffered, the next one's loads issued before this
  // one's products); one warp per own column.
  const int nq = cta < k ? (k - cta + G - 1) / G : 0;
  for (int li = warp; li < nq; li += kCoopWarps) {
    cx<T>* q = wk.QT + (int64_t)(cta + G * li) * mr;
    for (int i = lane; i < mr; i += 32) q[i] = mk<T>(T(i == cta + G * li), T(0));
  }
  if (nq > 0) {
    const int cmax = cta + G * (nq - 1);
    constexpr int PF = 8;  // staged elements per thread (mr <= 2048)
    cx<T> pre[PF];
    auto fetch = [&](int j) {
#pragma unroll
      for (int u = 0; u < PF; ++u) {
        const int i = j + 1 + tid + u * kCoopThreads;
        pre[u] = i < mr ? ldcg(wk.MT + (int64_t)j * mr + i) : mk<T>(T(0), T(0));
      }
    };
    fetch(cmax);
    for (int j = cmax; j >= 0; --j) {
      cx<T>* vb = vbuf + (size_t)(j & 1) * mr;
#pragma unroll
      for (int u = 0; u < PF; ++u) {
        const int i = j + 1 + tid + u * kCoopThreads;
        if (i < mr) vb[i] = pre[u];
      }
      for (int i = j + 1 + PF * kCoopThreads + tid; i < mr; i += kCoopThreads) vb[i] = ldcg(wk.MT + (int64_t)j * mr + i);
      const cx<T> tj = ldcg(wk.tau + j);
      __syncthreads();
      if (j > 0) fetch(j - 1);
      if (tj.re == T(0) && tj.im == T(0)) continue;
      for (int li = warp; li < nq; li += kCoopWarps) {
        const int c = cta + G * li;
        if (c < j) continue;
        cx<T>* q = wk.QT + (int64_t)c * mr;
        cx<T> w = mk<T>(T(0), T(0));
        for (int i = j + 1 + lane; i < mr; i += 32) fma_cj(w, vb[i], q[i]);
        for (int o = 16; o > 0; o >>= 1) {
          w.re += __shfl_xor_sync(0xffffffffu, w.re, o);
          w.im += __shfl_xor_sync(0xffffffffu, w.im, o);
        }
        w = w + q[j];
        const cx<T> tw = tj * w;
        for (int i = j + 1 + lane; i < mr; i += 32) q[i] = q[i] - vb[i] * tw;
        __syncwarp();
        if (lane == 0) q[j] = q[j] - tw;
        __syncwarp();
      }
    }
  }
  if (!grid_sync(wk.bar)) return;
  // 4. Q out through the output view
  {
    const CMatOut<T> Qo = a.Q;
    const int cj = a.qconj;
    cx<T>* QT = wk.QT;
    auto src = [&](int i, int c) { return ldcg(QT + (int64_t)c * mr + i); };
    auto dst = [&](int i, int c, cx<T> z) {
      if (cj) z.im = -z.im;
      Qo.p[(int64_t)i * Qo.rs + (int64_t)c * Qo.cs] = z;
    };
    // read QT along i (lanes on rows), write along the view's unit stride
    grid_tile_copy<T>(mr, k, true, src, dst, tile);
  }
  if (cta == 0 && tid == 0 && a.err) atomicOr(a.err, *(volatile int*)&wk.bar->err);
}

// ---------------------------------------------------------------- host side
template <typename T>
static int coop_grid_t(int which) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (which == 0) {
    const size_t sm = eig_smem_bytes<T>(kWideM);
    cudaFuncSetAttribute(k_wide_eig<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_wide_eig<T>, kCoopThreads, sm);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_wide_qr<T>, kCoopThreads, 0);
  }
  if (per < 1) per = 1;
  return sms * (per > 1 ? 1 : per);
}

int coop_grid(int prec, int which) {
  static int cache[2][2] = {{0, 0}, {0, 0}};
  int& c = cache[prec][which];
  if (c == 0) c = prec == 0 ? coop_grid_t<double>(which) : coop_grid_t<float>(which);
  return c;
}

size_t wide_eig_work_bytes(int prec, int m) {
  const int g = 1024;  // any grid up to 1024 CTAs
  return prec == 0 ? eig_work_bytes_t<double>(m, g) : eig_work_bytes_t<float>(m, g);
}
size_t wide_qr_work_bytes(int prec, int mr, int nc) {
  return prec == 0 ? qr_work_bytes_t<double>(mr, nc) : qr_work_bytes_t<float>(mr, nc);
}

template <typename T>
static cudaError_t eig_launch(const WideEigArgs& a, int grid, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_wide_eig<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)eig_smem_bytes<T>(kWideM));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_wide_eigvec<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)eig_smem_bytes<T>(kWideM));
    if (e != cudaSuccess) return e;
    attr = true;
  }
  cudaError_t e = cudaMemsetAsync(a.work, 0, 256, st);
  if (e != cudaSuccess) return e;
  const size_t sm = eig_smem_bytes<T>(a.m);
  WideEigArgs arg = a;
  arg.grid0 = grid;
  void* params[] = {&arg};
  const void* fn = a.phase == 0 ? (const void*)k_wide_eig<T> : (const void*)k_wide_eigvec<T>;
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kCoopThreads), params, sm, st);
}

cudaError_t launch_wide_eig(int prec, const WideEigArgs& a, int grid, cudaStream_t st) {
  return prec == 0 ? eig_launch<double>(a, grid, st) : eig_launch<float>(a, grid, st);
}

template <typename T>
cudaError_t launch_wide_qr_t(const CMat<T>& M, const CMatOut<T>& Q, int qconj, void* R, void* work, int* err,
                             int grid, cudaStream_t st) {
  static bool attr = false;
  constexpr size_t kQrSmemMax = 200 * 1024;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_wide_qr<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kQrSmemMax);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  cudaError_t e = cudaMemsetAsync(work, 0, 256, st);
  if (e != cudaSuccess) return e;
  QrArgsT<T> a;
  a.M = M;
  a.Q = Q;
  a.qconj = qconj;
  a.R = reinterpret_cast<cx<T>*>(R);
  a.work = work;
  a.err = err;
  const int nown = (M.cols + grid - 1) / grid;
  size_t sm = qr_smem_bytes<T>(M.rows, nown, true);
  a.own_smem = sm <= kQrSmemMax ? 1 : 0;
  if (!a.own_smem) sm = qr_smem_bytes<T>(M.rows, nown, false);
  void* params[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)k_wide_qr<T>, dim3(grid), dim3(kCoopThreads), params, sm, st);
}
template cudaError_t launch_wide_qr_t<float>(const CMat<float>&, const CMatOut<float>&, int, void*, void*, int*,
                                             int, cudaStream_t);
template cudaError_t launch_wide_qr_t<double>(const CMat<double>&, const CMatOut<double>&, int, void*, void*, int*,
                                              int, cudaStream_t);

}  // namespace gbmps
