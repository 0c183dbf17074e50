// Host-driven executor of wide programs (bond cap above the single-CTA limit).
//
// A wide program runs its compiled ops (routing, 1-qubit fusion and gauge
// moves as for every program) one at a time on the lane's stream; the host
// mirrors the bond dimensions and reads the kept dimension back after each
// split (one small copy per two-qubit gate, negligible next to a split of a
// 2chi x 2chi theta).  Two-site update (ExaTnMpsVisitor.cpp:1387-1730 with
// truncateSvdTensors :2366-2536; ITensorMPSVisitor.cpp:312-331 with ITensor
// truncate decomp.cc:307-463):
//   T = A.B (GEMM), theta = gate(T), G = X X^H on the isometric side (GEMM),
//   eigen-decomposition + keep rule (k_wide_eig), [complex64: one subspace
//   step W <- X (X^H W)], orthonormalisation (Newton-Schulz GEMMs, or the
//   cooperative QR for a degenerate cluster), isometric site W_k, other site
//   W_k^H X (GEMM).
// Centre moves (ITensor MPS::position) use the cooperative QR plus one GEMM.
// Pauli expectations (ITensorMPSVisitor.cpp:173-250) and shot sampling
// (ExaTnMpsVisitor.cpp:2211-2364) are transfer-matrix sweeps of GEMMs.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gb300mps.h"
#include "engine_internal.hpp"
#include "keep.cuh"
#include "philox.cuh"
#include "wide.hpp"

namespace gbmps {

struct G16 {
  double m[32];
};

template <typename T>
__global__ void k_theta_gate(const cx<T>* __restrict__ Tb, cx<T>* __restrict__ Th, int dl, int dr, G16 g,
                             int trim) {
  const int Cc = 2 * dr;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)dl * dr;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int l = (int)(idx / dr), r = (int)(idx - (int64_t)l * dr);
    cx<T> t[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) t[q] = Tb[(int64_t)(2 * l + (q >> 1)) * Cc + (q & 1) * dr + r];
#pragma unroll
    for (int row = 0; row < 4; ++row) {
      cx<T> acc = mk<T>(T(0), T(0));
#pragma unroll
      for (int col = 0; col < 4; ++col)
        fma_c(acc, mk<T>(T(g.m[2 * (row * 4 + col)]), T(g.m[2 * (row * 4 + col) + 1])), t[col]);
      // exatn semantics: moduli below 1e-100 become zero before the split
      // (stabilizeTensorBody, ExaTnMpsVisitor.cpp:141-161); complex128 only
      if (sizeof(T) == 8 && trim && (double)abs2(acc) < 1e-200) acc = mk<T>(T(0), T(0));
      Th[(int64_t)(2 * l + (row >> 1)) * Cc + (row & 1) * dr + r] = acc;
    }
  }
}

template <typename T>
__global__ void k_wide_gate1(cx<T>* A, int dl, int dr, G16 g) {
  const cx<T> g00 = mk<T>(T(g.m[0]), T(g.m[1])), g01 = mk<T>(T(g.m[2]), T(g.m[3]));
  const cx<T> g10 = mk<T>(T(g.m[4]), T(g.m[5])), g11 = mk<T>(T(g.m[6]), T(g.m[7]));
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)dl * dr;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int l = (int)(idx / dr), r = (int)(idx - (int64_t)l * dr);
    const cx<T> a0 = A[(int64_t)(l * 2) * dr + r], a1 = A[(int64_t)(l * 2 + 1) * dr + r];
    A[(int64_t)(l * 2) * dr + r] = g00 * a0 + g01 * a1;
    A[(int64_t)(l * 2 + 1) * dr + r] = g10 * a0 + g11 * a1;
  }
}

// Split scales: exatn puts sqrt(S) on both sides, itensor leaves the
// isometric side as is; rn rescales the kept part to the pre-truncation norm
// (1 without renormalisation).
template <typename T>
__global__ void k_split_scales(const double* lam, int k, int sqrt_mode, double rn, T* iso, T* oth) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < k; j += gridDim.x * blockDim.x) {
    const double v = lam[j];
    const double sv = v > 0.0 ? sqrt(v) : 0.0;
    if (sqrt_mode) {
      const double h = sqrt(sv);
      iso[j] = T(h);
      oth[j] = T(h > 0.0 ? rn / h : 0.0);
    } else {
      iso[j] = T(1);
      oth[j] = T(rn);
    }
  }
}

// sqrt(S) on both sides (exatn semantics) from the unscaled other side O =
// W_k^H X: sigma_j = |row j of O| (rows contiguous in a k x nn O, or column j
// of an nn x k O^T), accurate to ~eps * sigma_max / sigma where sqrt of the
// Gram eigenvalue is only accurate to ~eps * (sigma_max / sigma)^2 (ITensor
// takes its singular values from the QR of M^H U, SVDRefImpl, tensor/
// algs.cc:541-548).  A column whose eigenvalue counts as zero gets 0 on both
// sides.  One block per kept column.
template <typename T>
__global__ void k_sqrt_scales(const cx<T>* O, int nn, int k, int transposed, const double* lam, double rn, T* iso,
                              T* oth) {
  __shared__ double red[32];
  const int j = blockIdx.x;
  double s2 = 0.0;
  for (int c = threadIdx.x; c < nn; c += blockDim.x)
    s2 += (double)abs2(transposed ? O[(int64_t)c * k + j] : O[(int64_t)j * nn + c]);
  for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    const double h = lam[j] > 0.0 ? sqrt(sqrt(tot)) : 0.0;
    iso[j] = T(h);
    oth[j] = T(h > 0.0 ? rn / h : 0.0);
  }
}

// Other side O scaled by oth per kept index (rows of k x nn, or columns of nn x k).
template <typename T>
__global__ void k_scale_other(cx<T>* O, int nn, int k, int transposed, const T* oth) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)k * nn;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int j = transposed ? (int)(t % k) : (int)(t / nn);
    O[t] = scl(O[t], oth[j]);
  }
}

// Isometric site from W (m x k): plain (dst[i*k + j]) or transposed
// (dst[j*m + i]); and Wo = W diag(oth) for the other side.
template <typename T>
__global__ void k_write_iso(const cx<T>* W, int m, int k, const T* iso, const T* oth, int transpose, cx<T>* dst,
                            cx<T>* Wo) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)m * k;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / k), j = (int)(t - (int64_t)i * k);
    const cx<T> w = W[t];
    if (transpose)
      dst[(int64_t)j * m + i] = scl(w, iso[j]);
    else
      dst[t] = scl(w, iso[j]);
    Wo[t] = scl(w, oth[j]);
  }
}

// |S - I|_F of a k x k matrix (one block).
template <typename T>
__global__ void k_defect(const cx<T>* S, int k, double* out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t t = threadIdx.x; t < (int64_t)k * k; t += blockDim.x) {
    const int a = (int)(t / k), b = (int)(t - (int64_t)a * k);
    cx<T> z = S[t];
    if (a == b) z.re -= T(1);
    s += (double)abs2(z);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    *out = sqrt(tot);
  }
}

// Column normalisation of W2 (m x k, ld k); a vanished column takes the
// column of Wf (ld ldf) instead.
template <typename T>
__global__ void k_colnorm(cx<T>* W2, int m, int k, int ld, const cx<T>* Wf, int ldf, T* inv) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  T s2 = T(0);
  for (int i = 0; i < m; ++i) s2 += abs2(W2[(int64_t)i * ld + j]);
  const T tiny = sizeof(T) == 4 ? T(1e-36) : T(1e-280);
  inv[j] = s2 > tiny ? T(1) / sqrt(s2) : T(0);
  if (!(s2 > tiny))
    for (int i = 0; i < m; ++i) W2[(int64_t)i * ld + j] = Wf[(int64_t)i * ldf + j];
}
template <typename T>
__global__ void k_colscale(cx<T>* W2, int m, int k, int ld, const T* inv) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)m * k;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / k), j = (int)(t - (int64_t)i * k);
    if (inv[j] > T(0)) W2[(int64_t)i * ld + j] = scl(W2[(int64_t)i * ld + j], inv[j]);
  }
}

// Statistics of a wide split (same slots as the single-CTA kernel) and the
// new bond dimension.
__global__ void k_wide_commit(double* stats, int* bond, int b, int k, double total, double kept, double flops,
                              double eig_flops) {
  const double frac = total > 0.0 ? (total - kept) / total : 0.0;
  stats[ST_LOG_FID] += log1p(-(frac < 1.0 ? frac : 0.0));
  if (frac > stats[ST_MAX_DISC]) stats[ST_MAX_DISC] = frac;
  stats[ST_N_GATE2] += 1.0;
  stats[ST_N_OPS] += 1.0;
  stats[ST_FLOPS] += flops;
  stats[ST_EIG_FLOPS] += eig_flops;
  bond[b] = k;
}
// Z = X (strided view) copied into a compact m x nn buffer.
template <typename T>
__global__ void k_copy_view(CMat<T> X, cx<T>* Z) {
  const int nn = X.cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)X.rows * nn;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / nn), c = (int)(t - (int64_t)i * nn);
    Z[t] = X.p[(int64_t)i * X.rs + (int64_t)c * X.cs];
  }
}
__global__ void k_set_bond(double* stats, int* bond, int b, int v, double flops) {
  if (b >= 0) bond[b] = v;
  stats[ST_N_OPS] += 1.0;
  stats[ST_FLOPS] += flops;
}

// H[l, s', r] = sum_s P[s'][s] F[l, s, r] for one Pauli (1 X, 2 Y, 3 Z).
template <typename T>
__global__ void k_pauli(const cx<T>* F, cx<T>* H, int dl, int dr, int code) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)dl * dr;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int l = (int)(idx / dr), r = (int)(idx - (int64_t)l * dr);
    const cx<T> f0 = F[(int64_t)(2 * l) * dr + r], f1 = F[(int64_t)(2 * l + 1) * dr + r];
    cx<T> h0, h1;
    if (code == 1) {
      h0 = f1;
      h1 = f0;
    } else if (code == 2) {  // Y = [[0, -i], [i, 0]]
      h0 = mk<T>(f1.im, -f1.re);
      h1 = mk<T>(-f0.im, f0.re);
    } else {
      h0 = f0;
      h1 = mk<T>(-f1.re, -f1.im);
    }
    H[(int64_t)(2 * l) * dr + r] = h0;
    H[(int64_t)(2 * l + 1) * dr + r] = h1;
  }
}

template <typename T>
__global__ void k_store_scalar(const cx<T>* E, double* out) {
  out[0] = (double)E[0].re;
  out[1] = (double)E[0].im;
}

// Philox4x32-10 uniform in [0, 1) for (shot, site), its own stream tag.
__device__ __forceinline__ double wide_uniform(uint64_t seed, uint32_t shot, uint32_t site) {
  return philox_uniform(seed, shot, site, 0x57494445u);
}

// One site of shot sampling: U (S x 2dr, cols (s, r)) = V A, Q = U R_{i+1}
// (rows (shot, s)); p_s = Re <U_s, Q_s>; bit 0 when u <= p0 / (p0 + p1)
// (ExaTnMpsVisitor.cpp:2342-2345); V <- U_bit / sqrt(p_bit).  One warp per shot.
template <typename T>
__global__ void k_wide_sample_step(const cx<T>* U, const cx<T>* Q, cx<T>* V, int shots, int dr, int site, int n,
                                   uint64_t seed, uint8_t* bits) {
  const int lane = threadIdx.x & 31;
  const int shot = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (shot >= shots) return;
  const cx<T>* u = U + (int64_t)shot * 2 * dr;
  const cx<T>* q = Q + (int64_t)shot * 2 * dr;
  double p[2] = {0.0, 0.0};
  for (int s = 0; s < 2; ++s) {
    double acc = 0.0;
    for (int r = lane; r < dr; r += 32) {
      const cx<T> a = u[s * dr + r], b = q[s * dr + r];
      acc += (double)a.re * b.re + (double)a.im * b.im;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    p[s] = acc > 0.0 ? acc : 0.0;
  }
  const double tot = p[0] + p[1];
  const double uu = wide_uniform(seed, (uint32_t)shot, (uint32_t)site);
  const int bit = (tot > 0.0 && uu > p[0] / tot) ? 1 : 0;
  const double inv = p[bit] > 0.0 ? 1.0 / sqrt(p[bit]) : 0.0;
  for (int r = lane; r < dr; r += 32) V[(int64_t)shot * dr + r] = scl(u[bit * dr + r], T(inv));
  if (lane == 0) bits[(int64_t)shot * n + site] = (uint8_t)bit;
}

// ------------------------------------------------------------ workspace
struct WideBufs {
  int prec = -1;
  int m = 0;  // sized for Gram side m
  void* theta = nullptr;
  void* tbuf = nullptr;
  void* gram = nullptr;
  void* W = nullptr;
  void* W2 = nullptr;
  void* W3 = nullptr;
  void* Y = nullptr;
  void* S = nullptr;
  void* R = nullptr;
  void* gram2 = nullptr;  // Gram of the deflated tail
  void* Z = nullptr;      // deflated X
  void* scal = nullptr;  // iso, oth, inv (3 m of T)
  double* lam = nullptr;
  void* eig_work = nullptr;
  void* eig_work2 = nullptr;
  void* qr_work = nullptr;
  int* d_status = nullptr;     // grid-barrier status of the cooperative launches
  double* d_scalar = nullptr;  // 2 doubles
  int* d_err = nullptr;
  char* h_pinned = nullptr;    // [0, 256): scalars; then 2 x kWideM doubles of eigenvalues
  GemmWs gemm;
};

struct WideAll {
  WideBufs b[2];
};

static void wide_bufs_free(WideBufs& B) {
  void* ptrs[] = {B.theta, B.tbuf, B.gram, B.W, B.W2, B.W3, B.Y, B.S, B.R, B.gram2, B.Z, B.scal, B.lam,
                  B.eig_work, B.eig_work2, B.qr_work, B.d_status, B.d_scalar, B.d_err};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (B.h_pinned) cudaFreeHost(B.h_pinned);
  gemm_ws_free(B.gemm);
  B = WideBufs();
}

void wide_ws_free(void** ws) {
  if (!*ws) return;
  WideAll* w = reinterpret_cast<WideAll*>(*ws);
  for (auto& b : w->b) wide_bufs_free(b);
  delete w;
  *ws = nullptr;
}

void wide_free(mps_ctx* c) { wide_ws_free(&c->wide); }

// Workspace `ws` (a WideAll, created on first use): the context's own, or
// the serve loop's, so the two never share buffers.
static int wide_bufs(void** ws, int prec, int chi, WideBufs** out) {
  if (!*ws) *ws = new WideAll();
  WideBufs& B = reinterpret_cast<WideAll*>(*ws)->b[prec];
  const int m = 2 * chi;
  if (B.prec == prec && B.m >= m) {
    *out = &B;
    return MPS_OK;
  }
  wide_bufs_free(B);
  const size_t eb = prec == MPS_PREC_FP64 ? 16 : 8;
  const size_t E = (size_t)m * m;
  void** big[] = {&B.theta, &B.tbuf, &B.gram, &B.W, &B.W2, &B.W3, &B.Y, &B.S, &B.R, &B.gram2, &B.Z};
  bool ok = true;
  for (void** q : big) ok = ok && cudaMalloc(q, E * eb) == cudaSuccess;
  ok = ok && cudaMalloc(&B.scal, 3 * (size_t)m * eb) == cudaSuccess;
  ok = ok && cudaMalloc(&B.lam, (size_t)m * sizeof(double)) == cudaSuccess;
  ok = ok && cudaMalloc(&B.eig_work, wide_eig_work_bytes(prec, m)) == cudaSuccess;
  ok = ok && cudaMalloc(&B.eig_work2, wide_eig_work_bytes(prec, m)) == cudaSuccess;
  ok = ok && cudaMalloc(&B.qr_work, wide_qr_work_bytes(prec, m, m)) == cudaSuccess;
  ok = ok && cudaMalloc(&B.d_status, 16) == cudaSuccess;
  ok = ok && cudaMalloc(&B.d_scalar, 4 * sizeof(double)) == cudaSuccess;
  ok = ok && cudaMalloc(&B.d_err, sizeof(int)) == cudaSuccess;
  ok = ok && cudaMallocHost(&B.h_pinned, 256 + 2 * sizeof(double) * (size_t)kWideM) == cudaSuccess;
  // tensor-core operands: A side up to m x 2m, B side up to 2m x 2m (padded)
  if (ok && prec == MPS_PREC_FP32) {
    const size_t pad = (size_t)(m + 128) * (2 * m + 128);
    ok = gemm_ws_init(B.gemm, pad, 2 * pad) == 0;
  } else if (ok) {
    ok = gemm_ws_init(B.gemm, 1, 1) == 0;
  }
  if (!ok) {
    cudaGetLastError();
    wide_bufs_free(B);
    return fail(MPS_ERR_OOM, "wide-path workspace allocation failed");
  }
  cudaMemset(B.d_err, 0, sizeof(int));
  B.prec = prec;
  B.m = m;
  *out = &B;
  return MPS_OK;
}

#define WCK(call)                                                             \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

static int blocks_for(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4096); }

// Grid of a cooperative launch over n rows (eigensolver) or columns (QR):
// one CTA per g_coop_rows rows (default 8, about one per warp), at most the
// co-resident maximum.  Fewer CTAs make each grid barrier cheaper when the
// matrix is small.
static std::atomic<int> g_coop_rows{8};
static int coop_grid_for(int prec, int which, int n) {
  const int g = coop_grid(prec, which);
  const int rows = g_coop_rows.load();
  const int want = std::max(8, (n + rows - 1) / rows);
  return std::min(g, want);
}

// ------------------------------------------------------------ two-site update
template <typename T>
static int orthonormalize_w(WideBufs& B, const CMat<T>& X, int m, int nn, int kk, int ld, cx<T>* Wc, int nsub,
                            cudaStream_t st, cx<T>** result, double* ortho_flops) {
  // Wc: m x kk (row stride ld).  Returns the orthonormal columns in *result
  // (m x kk, row stride ld); columns kk..ld-1 of the result are unspecified.
  // nsub: leading columns whose eigenvalue lies clearly above the Gram's
  // rounding floor; after a QR fallback only they take the subspace step
  // (a column at the floor must stay in X's null space).
  cx<T>* cur = Wc;
  cx<T>* nxt = reinterpret_cast<cx<T>*>(cur == B.W3 ? B.W2 : B.W3);
  cx<T>* S = reinterpret_cast<cx<T>*>(B.S);
  double* hs = reinterpret_cast<double*>(B.h_pinned + 128);
  const double ns_stop = sizeof(T) == 4 ? 1e-4 : 1e-8;
  bool qr_taken = false;
  auto view = [&](cx<T>* p) { return cmat<T>(p, m, kk, ld, 1); };
  auto oview = [&](cx<T>* p) { return cout_<T>(p, m, kk, ld, 1); };
  // The defect |W^H W - I|_F is read back once; each Newton-Schulz step
  // W <- W (3 I - W^H W) / 2 maps a defect e to at most 3/4 e^2 + 1/4 e^3,
  // so the number of steps follows from it without further round trips
  // (steps until the one taken from a defect below ns_stop, at most five).
  WCK(cgemm(adj(view(cur)), view(cur), cout_<T>(S, kk, kk, kk, 1), T(1), T(0), B.gemm, st));
  *ortho_flops += 8.0 * kk * kk * m;
  k_defect<T><<<1, 256, 0, st>>>(S, kk, B.d_scalar);
  WCK(cudaMemcpyAsync(hs, B.d_scalar, sizeof(double), cudaMemcpyDeviceToHost, st));
  WCK(cudaStreamSynchronize(st));
  double fro = hs[0];
  if (!(fro == fro)) return fail(MPS_ERR_NUMERIC, "non-finite value in a wide split");
  if (fro > 0.1) {
    qr_taken = true;
  } else {
    for (int it = 0; it < 5; ++it) {
      if (it > 0) {
        WCK(cgemm(adj(view(cur)), view(cur), cout_<T>(S, kk, kk, kk, 1), T(1), T(0), B.gemm, st));
        *ortho_flops += 8.0 * kk * kk * m;
      }
      WCK(cudaMemcpyAsync(nxt, cur, (size_t)m * ld * sizeof(cx<T>), cudaMemcpyDeviceToDevice, st));
      WCK(cgemm(view(cur), cmat<T>(S, kk, kk, kk, 1), oview(nxt), T(-0.5), T(1.5), B.gemm, st));
      *ortho_flops += 8.0 * kk * kk * m;
      std::swap(cur, nxt);
      if (fro < ns_stop) break;
      fro = 0.75 * fro * fro + 0.25 * fro * fro * fro;
    }
  }
  if (qr_taken) {
    // degenerate cluster: Householder QR, then (when vectors were completed
    // from rounding noise) one subspace step with X and a second QR
    const int grid = coop_grid_for(sizeof(T) == 8 ? 0 : 1, 1, kk);
    for (int pass = 0; pass < 2; ++pass) {
      WCK(launch_wide_qr_t<T>(view(cur), oview(nxt), 0, B.R, B.qr_work, B.d_err, grid, st));
      std::swap(cur, nxt);
      const int ns = std::min(nsub, kk);
      if (pass == 1 || kk >= m || ns <= 0) break;
      cx<T>* Y = reinterpret_cast<cx<T>*>(B.Y);
      WCK(cgemm(adj(X), cmat<T>(cur, m, ns, ld, 1), cout_<T>(Y, nn, ns, ns, 1), T(1), T(0), B.gemm, st));
      WCK(cudaMemcpyAsync(nxt, cur, (size_t)m * ld * sizeof(cx<T>), cudaMemcpyDeviceToDevice, st));
      WCK(cgemm(X, cmat<T>(Y, nn, ns, ns, 1), cout_<T>(nxt, m, ns, ld, 1), T(1), T(0), B.gemm, st));
      T* inv = reinterpret_cast<T*>(B.scal) + 2 * B.m;
      k_colnorm<T><<<(ns + 255) / 256, 256, 0, st>>>(nxt, m, ns, ld, cur, ld, inv);
      k_colscale<T><<<blocks_for((int64_t)m * ns), 256, 0, st>>>(nxt, m, ns, ld, inv);
      std::swap(cur, nxt);
      *ortho_flops += 16.0 * m * nn * ns;
    }
    int* herr = reinterpret_cast<int*>(B.h_pinned + 96);
    WCK(cudaMemcpyAsync(herr, B.d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    WCK(cudaStreamSynchronize(st));
    if (*herr) return fail(MPS_ERR_TIMEOUT, "cooperative QR gave up at a grid barrier");
  }
  *result = cur;
  return MPS_OK;
}

// Eigenvalues (descending) of the m x m Gram G into h_lam (host, pinned);
// the reflectors stay in G and the work buffer for eig_vectors.
template <typename T>
static int eig_values(WideBufs& B, void* G, void* work, int m, double* h_lam, cudaStream_t st) {
  const int prec = sizeof(T) == 8 ? 0 : 1;
  WideEigArgs ea;
  std::memset(&ea, 0, sizeof(ea));
  ea.G = G;
  ea.lam = B.lam;
  ea.m = m;
  ea.phase = 0;
  ea.work = work;
  ea.status_err = B.d_status;
  WCK(launch_wide_eig(prec, ea, coop_grid_for(prec, 0, m), st));
  int* herr = reinterpret_cast<int*>(B.h_pinned + 64);
  WCK(cudaMemcpyAsync(h_lam, B.lam, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
  WCK(cudaMemcpyAsync(herr, B.d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  WCK(cudaStreamSynchronize(st));
  if (*herr) return fail(MPS_ERR_TIMEOUT, "cooperative eigensolver gave up at a grid barrier");
  for (int i = 0; i < m; ++i)
    if (!std::isfinite(h_lam[i])) return fail(MPS_ERR_NUMERIC, "non-finite value in a wide split");
  return MPS_OK;
}

// Eigenvectors of ranks 0..kv-1 into W (m x kv, row stride ld).
template <typename T>
static int eig_vectors(WideBufs& B, void* G, void* work, int m, int kv, void* W, int ld, cudaStream_t st) {
  const int prec = sizeof(T) == 8 ? 0 : 1;
  WideEigArgs ea;
  std::memset(&ea, 0, sizeof(ea));
  ea.G = G;
  ea.W = W;
  ea.m = m;
  ea.phase = 1;
  ea.kv = kv;
  ea.ld = ld;
  ea.work = work;
  ea.status_err = B.d_status;
  WCK(launch_wide_eig(prec, ea, coop_grid_for(prec, 0, m), st));
  return MPS_OK;
}

template <typename T>
static int wide_gate2(mps_prog* p, WideBufs& B, cudaStream_t st, const DevOp& op) {
  const int lo = op.site;
  const int dl = p->hbond[lo], dm = p->hbond[lo + 1], dr = p->hbond[lo + 2];
  cx<T>* sites = reinterpret_cast<cx<T>*>(p->d_sites);
  cx<T>* A = sites + p->off[lo];
  cx<T>* Bs = sites + p->off[lo + 1];
  const int R = 2 * dl, Cc = 2 * dr;
  cx<T>* theta = reinterpret_cast<cx<T>*>(B.theta);
  cx<T>* tb = reinterpret_cast<cx<T>*>(B.tbuf);
  WCK(cgemm(cmat<T>(A, R, dm, dm, 1), cmat<T>(Bs, dm, Cc, Cc, 1), cout_<T>(tb, R, Cc, Cc, 1), T(1), T(0), B.gemm,
            st));
  G16 g;
  std::memcpy(g.m, op.m, sizeof(g.m));
  k_theta_gate<T><<<blocks_for((int64_t)dl * dr), 256, 0, st>>>(tb, theta, dl, dr, g,
                                                                 p->mode == TRUNC_EXATN ? 1 : 0);
  bool tr;
  if (op.orient == ORIENT_TO_HI)
    tr = false;
  else if (op.orient == ORIENT_TO_LO)
    tr = true;
  else
    tr = R > Cc;
  const int m = tr ? Cc : R, nn = tr ? R : Cc, mm = std::min(R, Cc);
  const CMat<T> X = tr ? cmat<T>(theta, Cc, R, 1, Cc) : cmat<T>(theta, R, Cc, Cc, 1);
  cx<T>* G = reinterpret_cast<cx<T>*>(B.gram);
  WCK(cgemm(X, adj(X), cout_<T>(G, m, m, m, 1), T(1), T(0), B.gemm, st));
  const int kcap = std::min(p->chi_cap, mm);
  double* hl = reinterpret_cast<double*>(B.h_pinned + 256);
  double* hl2 = hl + kWideM;
  int rc = eig_values<T>(B, G, B.eig_work, m, hl, st);
  if (rc) return rc;
  const bool fp32 = sizeof(T) == 4;
  double extra = 0.0, eig_flops = (32.0 / 3.0) * m * m * m;
  std::vector<double> lk(hl, hl + mm);
  int k = keep_rule(lk.data(), mm, p->mode, p->cutoff, kcap);
  cx<T>* Wk = reinterpret_cast<cx<T>*>(B.W2);  // kept vectors, m x k (row stride k)
  // FP32 refinement: an FP32 Gram resolves eigenvalues only down to ~eps *
  // lambda_max.  When the cut falls below kRefine * lambda_max, the tail is
  // re-solved in the complement of the head (the eigenvectors above that
  // ratio): Z = X - W_h (W_h^H X) has the size of the tail and its Gram
  // resolves it to ~eps * |Z|^2 (ITensor's recursive refinement of small
  // singular values, SVDRefImpl, tensor/algs.cc:510-579, one level deep).
  constexpr double kRefine = 1e-4;
  int s_head = 0;
  while (s_head < mm && hl[s_head] >= kRefine * hl[0]) ++s_head;
  const bool refine = fp32 && hl[0] > 0.0 && k > s_head && s_head < m;
  if (refine) {
    cx<T>* Wh = reinterpret_cast<cx<T>*>(B.W);
    rc = eig_vectors<T>(B, G, B.eig_work, m, s_head, Wh, s_head, st);
    if (rc) return rc;
    cx<T>* Who = nullptr;
    rc = orthonormalize_w<T>(B, X, m, nn, s_head, s_head, Wh, 0, st, &Who, &extra);
    if (rc) return rc;
    // keep W_h in B.W (the buffers W2/W3 serve the orthonormalisation)
    if (Who != Wh)
      WCK(cudaMemcpyAsync(Wh, Who, (size_t)m * s_head * sizeof(cx<T>), cudaMemcpyDeviceToDevice, st));
    cx<T>* Y = reinterpret_cast<cx<T>*>(B.Y);
    cx<T>* Z = reinterpret_cast<cx<T>*>(B.Z);
    WCK(cgemm(adj(cmat<T>(Wh, m, s_head, s_head, 1)), X, cout_<T>(Y, s_head, nn, nn, 1), T(1), T(0), B.gemm, st));
    k_copy_view<T><<<blocks_for((int64_t)m * nn), 256, 0, st>>>(X, Z);
    WCK(cgemm(cmat<T>(Wh, m, s_head, s_head, 1), cmat<T>(Y, s_head, nn, nn, 1), cout_<T>(Z, m, nn, nn, 1), T(-1),
              T(1), B.gemm, st));
    const CMat<T> Zv = cmat<T>(Z, m, nn, nn, 1);
    cx<T>* G2 = reinterpret_cast<cx<T>*>(B.gram2);
    WCK(cgemm(Zv, adj(Zv), cout_<T>(G2, m, m, m, 1), T(1), T(0), B.gemm, st));
    rc = eig_values<T>(B, G2, B.eig_work2, m, hl2, st);
    if (rc) return rc;
    extra += 16.0 * m * s_head * nn + 8.0 * m * m * nn;
    eig_flops *= 2.0;
    // combined spectrum: the head from G, the tail from the deflated Gram;
    // tail values below ~eps^2 * lambda_max are its rounding noise
    const double floor_t = 64.0 * 1.4210854715202004e-14 * hl[0];
    for (int i = s_head; i < mm; ++i) {
      const double v = hl2[i - s_head];
      lk[i] = v > floor_t ? v : 0.0;
    }
    k = keep_rule(lk.data(), mm, p->mode, p->cutoff, kcap);
    // kept vectors: head columns, then the tail's leading eigenvectors made
    // orthogonal to the head (Gram-Schmidt, as Z's rounding leaves small
    // components along W_h)
    const int ks = std::min(k, s_head), kt = k - ks;
    WCK(cudaMemcpy2DAsync(Wk, (size_t)k * sizeof(cx<T>), Wh, (size_t)s_head * sizeof(cx<T>),
                          (size_t)ks * sizeof(cx<T>), m, cudaMemcpyDeviceToDevice, st));
    if (kt > 0) {
      rc = eig_vectors<T>(B, G2, B.eig_work2, m, kt, Wk + ks, k, st);
      if (rc) return rc;
      cx<T>* P = reinterpret_cast<cx<T>*>(B.S);
      WCK(cgemm(adj(cmat<T>(Wh, m, s_head, s_head, 1)), cmat<T>(Wk + ks, m, kt, k, 1),
                cout_<T>(P, s_head, kt, kt, 1), T(1), T(0), B.gemm, st));
      WCK(cgemm(cmat<T>(Wh, m, s_head, s_head, 1), cmat<T>(P, s_head, kt, kt, 1), cout_<T>(Wk + ks, m, kt, k, 1),
                T(-1), T(1), B.gemm, st));
      extra += 16.0 * m * s_head * kt;
    }
  } else {
    rc = eig_vectors<T>(B, G, B.eig_work, m, k, Wk, k, st);
    if (rc) return rc;
  }
  eig_flops += 8.0 * m * m * k;
  double total = 0.0, kept = 0.0;
  int kpos = 0;
  for (int i = 0; i < mm; ++i) {
    const double v = lk[i] > 0.0 ? lk[i] : 0.0;
    total += v;
    if (i < k) {
      kept += v;
      kpos += v > 0.0;
    }
  }
  if (k < 1 || k > kcap) return fail(MPS_ERR_NUMERIC, "wide split returned an invalid bond dimension");
  // columns with zero weight are scaled by 0 (exatn) or never kept (itensor),
  // so only the first kk need to be orthonormal
  const int kk = std::max(1, std::min(k, kpos));
  // FP32: one subspace step W <- X (X^H W) with X itself on the head columns
  // (eigenvalues >= kRefine * lambda_max): the Gram's rounding tilts such an
  // eigenvector by ~eps * lambda_max / lambda, the product's only by ~eps *
  // sigma_max / sigma.  Tail columns come from the deflated Gram and are
  // accurate to their own scale; the step would magnify their residual head
  // components by lambda_head / lambda_tail.
  const int ksub = fp32 ? std::min(kk, s_head) : 0;
  if (ksub > 0 && ksub < m) {
    cx<T>* Y = reinterpret_cast<cx<T>*>(B.Y);
    cx<T>* W3 = reinterpret_cast<cx<T>*>(B.W3);
    WCK(cgemm(adj(X), cmat<T>(Wk, m, ksub, k, 1), cout_<T>(Y, nn, ksub, ksub, 1), T(1), T(0), B.gemm, st));
    WCK(cgemm(X, cmat<T>(Y, nn, ksub, ksub, 1), cout_<T>(W3, m, ksub, k, 1), T(1), T(0), B.gemm, st));
    T* inv = reinterpret_cast<T*>(B.scal) + 2 * B.m;
    k_colnorm<T><<<(ksub + 255) / 256, 256, 0, st>>>(W3, m, ksub, k, Wk, k, inv);
    k_colscale<T><<<blocks_for((int64_t)m * ksub), 256, 0, st>>>(W3, m, ksub, k, inv);
    if (ksub < k)  // tail and zero-weight columns carried over unchanged
      WCK(cudaMemcpy2DAsync(W3 + ksub, (size_t)k * sizeof(cx<T>), Wk + ksub, (size_t)k * sizeof(cx<T>),
                            (size_t)(k - ksub) * sizeof(cx<T>), m, cudaMemcpyDeviceToDevice, st));
    extra += 16.0 * m * nn * ksub;
    Wk = W3;
  }
  // columns eligible for a subspace step after a QR fallback: eigenvalue
  // above the Gram's rounding floor (FP32: the head; FP64: 1e-10 lambda_max)
  int nsub = 0;
  if (fp32) {
    nsub = refine ? 0 : std::min(kk, s_head);
  } else {
    while (nsub < kk && lk[nsub] >= 1e-10 * lk[0]) ++nsub;
  }
  cx<T>* Wf = nullptr;
  rc = orthonormalize_w<T>(B, X, m, nn, kk, k, Wk, nsub, st, &Wf, &extra);
  if (rc) return rc;
  if (Wf != Wk && kk < k)
    WCK(cudaMemcpy2DAsync(Wf + kk, (size_t)k * sizeof(cx<T>), Wk + kk, (size_t)k * sizeof(cx<T>),
                          (size_t)(k - kk) * sizeof(cx<T>), m, cudaMemcpyDeviceToDevice, st));
  // scales from the kept eigenvalues
  double* hk = reinterpret_cast<double*>(B.h_pinned + 256) + kWideM;
  for (int i = 0; i < k; ++i) hk[i] = lk[i] > 0.0 ? lk[i] : 0.0;
  WCK(cudaMemcpyAsync(B.lam, hk, sizeof(double) * k, cudaMemcpyHostToDevice, st));
  const double rn = ((p->flags & MPS_FLAG_RENORM) && kept > 0.0) ? std::sqrt(total / kept) : 1.0;
  T* iso = reinterpret_cast<T*>(B.scal);
  T* oth = iso + B.m;
  cx<T>* Wo = reinterpret_cast<cx<T>*>(Wf == reinterpret_cast<cx<T>*>(B.W2) ? B.W3 : B.W2);
  if (op.orient == ORIENT_SQRT) {
    // other side unscaled first, its row norms give the singular values
    if (!tr)
      WCK(cgemm(adj(cmat<T>(Wf, m, k, k, 1)), X, cout_<T>(Bs, k, Cc, Cc, 1), T(1), T(0), B.gemm, st));
    else
      WCK(cgemm(cmat<T>(theta, R, Cc, Cc, 1), cmat<T>(Wf, Cc, k, k, 1, 1), cout_<T>(A, R, k, k, 1), T(1), T(0),
                B.gemm, st));
    cx<T>* O = tr ? A : Bs;
    k_sqrt_scales<T><<<k, 256, 0, st>>>(O, nn, k, tr ? 1 : 0, B.lam, rn, iso, oth);
    k_scale_other<T><<<blocks_for((int64_t)k * nn), 256, 0, st>>>(O, nn, k, tr ? 1 : 0, oth);
    k_write_iso<T><<<blocks_for((int64_t)m * k), 256, 0, st>>>(Wf, m, k, iso, oth, tr ? 1 : 0, tr ? Bs : A, Wo);
  } else if (!tr) {
    k_split_scales<T><<<(k + 255) / 256, 256, 0, st>>>(B.lam, k, 0, rn, iso, oth);
    k_write_iso<T><<<blocks_for((int64_t)m * k), 256, 0, st>>>(Wf, m, k, iso, oth, 0, A, Wo);
    WCK(cgemm(adj(cmat<T>(Wo, m, k, k, 1)), X, cout_<T>(Bs, k, Cc, Cc, 1), T(1), T(0), B.gemm, st));
  } else {
    k_split_scales<T><<<(k + 255) / 256, 256, 0, st>>>(B.lam, k, 0, rn, iso, oth);
    k_write_iso<T><<<blocks_for((int64_t)m * k), 256, 0, st>>>(Wf, m, k, iso, oth, 1, Bs, Wo);
    WCK(cgemm(cmat<T>(theta, R, Cc, Cc, 1), cmat<T>(Wo, Cc, k, k, 1, 1), cout_<T>(A, R, k, k, 1), T(1), T(0),
              B.gemm, st));
  }
  const double flops = 32.0 * dl * dm * dr + 128.0 * dl * dr + 8.0 * m * m * nn + 8.0 * k * nn * m + extra;
  k_wide_commit<<<1, 1, 0, st>>>(p->d_stats, p->d_bond, lo + 1, k, total, kept, flops, eig_flops);
  WCK(cudaGetLastError());
  // the host buffer hk must outlive the copy above
  int* herr = reinterpret_cast<int*>(B.h_pinned + 64);
  WCK(cudaMemcpyAsync(herr, B.d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  WCK(cudaStreamSynchronize(st));
  if (*herr) return fail(MPS_ERR_TIMEOUT, "cooperative eigensolver gave up at a grid barrier");
  p->hbond[lo + 1] = k;
  return MPS_OK;
}

// Centre moves.  Right: A_c (2dl x dr) = Q R, A_{c+1} <- R A_{c+1}.  Left:
// A_c^H (2dr x dl) = Q R, A_c <- Q^H, A_{c-1} <- A_{c-1} R^H.
template <typename T>
static int wide_move(mps_prog* p, WideBufs& B, cudaStream_t st, const DevOp& op) {
  const int c = op.site;
  cx<T>* sites = reinterpret_cast<cx<T>*>(p->d_sites);
  const int prec = sizeof(T) == 8 ? 0 : 1;
  cx<T>* tmp = reinterpret_cast<cx<T>*>(B.tbuf);
  cx<T>* Rm = reinterpret_cast<cx<T>*>(B.R);
  if (op.kind == OP_MOVE_R) {
    const int dl = p->hbond[c], dr = p->hbond[c + 1], d2 = p->hbond[c + 2];
    const int mr = 2 * dl, k = std::min(mr, dr);
    const int grid = coop_grid_for(prec, 1, dr);
    cx<T>* Ac = sites + p->off[c];
    cx<T>* An = sites + p->off[c + 1];
    WCK(launch_wide_qr_t<T>(cmat<T>(Ac, mr, dr, dr, 1), cout_<T>(Ac, mr, k, k, 1), 0, Rm, B.qr_work, B.d_err, grid,
                            st));
    WCK(cgemm(cmat<T>(Rm, k, dr, dr, 1), cmat<T>(An, dr, 2 * d2, 2 * d2, 1), cout_<T>(tmp, k, 2 * d2, 2 * d2, 1),
              T(1), T(0), B.gemm, st));
    WCK(cudaMemcpyAsync(An, tmp, (size_t)k * 2 * d2 * sizeof(cx<T>), cudaMemcpyDeviceToDevice, st));
    k_set_bond<<<1, 1, 0, st>>>(p->d_stats, p->d_bond, c + 1, k, 8.0 * k * dr * 2 * d2);
    p->hbond[c + 1] = k;
  } else {
    const int dl = p->hbond[c], dr = p->hbond[c + 1], d0 = p->hbond[c - 1];
    const int mr = 2 * dr, k = std::min(mr, dl);
    const int grid = coop_grid_for(prec, 1, dl);
    cx<T>* Ac = sites + p->off[c];
    cx<T>* Ap = sites + p->off[c - 1];
    // M = A_c^H: M(i, j) = conj(A_c[j][i]) with A_c as dl x 2dr
    WCK(launch_wide_qr_t<T>(cmat<T>(Ac, mr, dl, 1, mr, 1), cout_<T>(Ac, mr, k, 1, mr), 1, Rm, B.qr_work, B.d_err,
                            grid, st));
    WCK(cgemm(cmat<T>(Ap, 2 * d0, dl, dl, 1), adj(cmat<T>(Rm, k, dl, dl, 1)), cout_<T>(tmp, 2 * d0, k, k, 1), T(1),
              T(0), B.gemm, st));
    WCK(cudaMemcpyAsync(Ap, tmp, (size_t)2 * d0 * k * sizeof(cx<T>), cudaMemcpyDeviceToDevice, st));
    k_set_bond<<<1, 1, 0, st>>>(p->d_stats, p->d_bond, c, k, 8.0 * k * dl * 2 * d0);
    p->hbond[c] = k;
  }
  WCK(cudaGetLastError());
  return MPS_OK;
}

template <typename T>
static int wide_run_t(mps_prog* p, WideBufs& B, cudaStream_t st, const std::vector<DevOp>& ops) {
  cx<T>* sites = reinterpret_cast<cx<T>*>(p->d_sites);
  for (const DevOp& op : ops) {
    int rc = MPS_OK;
    if (op.kind == OP_GATE1) {
      G16 g;
      std::memcpy(g.m, op.m, sizeof(g.m));
      const int dl = p->hbond[op.site], dr = p->hbond[op.site + 1];
      k_wide_gate1<T><<<blocks_for((int64_t)dl * dr), 256, 0, st>>>(sites + p->off[op.site], dl, dr, g);
      k_set_bond<<<1, 1, 0, st>>>(p->d_stats, p->d_bond, -1, 0, 0.0);
      WCK(cudaGetLastError());
    } else if (op.kind == OP_GATE2) {
      rc = wide_gate2<T>(p, B, st, op);
    } else {
      rc = wide_move<T>(p, B, st, op);
    }
    if (rc) return rc;
  }
  // time-out flags of the QR moves and of the tensor-core GEMMs
  int* hf = reinterpret_cast<int*>(B.h_pinned + 100);
  WCK(cudaMemcpyAsync(hf, B.d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  WCK(cudaMemcpyAsync(hf + 1, B.gemm.d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  WCK(cudaStreamSynchronize(st));
  if (hf[0]) return fail(MPS_ERR_TIMEOUT, "cooperative QR gave up at a grid barrier");
  if (hf[1]) return fail(MPS_ERR_TIMEOUT, "tensor-core GEMM gave up waiting on its pipeline");
  return MPS_OK;
}

bool prog_is_wide(const mps_prog* p) { return p->chi_cap > kChiLimit; }

int wide_run(mps_ctx* c, Lane& L, mps_prog* p, void** ws) {
  std::vector<DevOp> ops;
  compile_program(p, ops);
  WideBufs* B = nullptr;
  int rc = wide_bufs(ws ? ws : &c->wide, p->prec, p->chi_cap, &B);
  if (rc) return rc;
  B->gemm.split_bf16 = p->split_bf16;  // tensor-core products of this program
  rc = p->prec == MPS_PREC_FP64 ? wide_run_t<double>(p, *B, L.stream, ops) : wide_run_t<float>(p, *B, L.stream, ops);
  if (rc) return rc;
  WCK(cudaEventRecord(p->ev, L.stream));
  p->submitted = true;
  return MPS_OK;
}

// ------------------------------------------------------------ measurement
template <typename T>
static int wide_expect_t(mps_prog* p, WideBufs& B, cudaStream_t st, const uint8_t* codes, int n_terms, double* out) {
  cx<T>* sites = reinterpret_cast<cx<T>*>(p->d_sites);
  cx<T>* E = reinterpret_cast<cx<T>*>(B.gram);
  cx<T>* F = reinterpret_cast<cx<T>*>(B.theta);
  cx<T>* H = reinterpret_cast<cx<T>*>(B.tbuf);
  double* d_out = nullptr;
  WCK(cudaMalloc(&d_out, 2 * sizeof(double) * (size_t)std::max(1, n_terms)));
  const cx<T> one = mk<T>(T(1), T(0));
  for (int t = 0; t < n_terms; ++t) {
    WCK(cudaMemcpyAsync(E, &one, sizeof(one), cudaMemcpyHostToDevice, st));
    for (int i = 0; i < p->n; ++i) {
      const int dl = p->hbond[i], dr = p->hbond[i + 1];
      const cx<T>* Ai = sites + p->off[i];
      WCK(cgemm(cmat<T>(E, dl, dl, dl, 1), cmat<T>(Ai, dl, 2 * dr, 2 * dr, 1), cout_<T>(F, dl, 2 * dr, 2 * dr, 1),
                T(1), T(0), B.gemm, st));
      const int code = codes[(size_t)t * p->n + i];
      const cx<T>* Hs = F;
      if (code != 0) {
        k_pauli<T><<<blocks_for((int64_t)dl * dr), 256, 0, st>>>(F, H, dl, dr, code);
        Hs = H;
      }
      WCK(cgemm(adj(cmat<T>(Ai, 2 * dl, dr, dr, 1)), cmat<T>(Hs, 2 * dl, dr, dr, 1), cout_<T>(E, dr, dr, dr, 1), T(1),
                T(0), B.gemm, st));
    }
    k_store_scalar<T><<<1, 1, 0, st>>>(E, d_out + 2 * t);
  }
  cudaError_t e = cudaMemcpyAsync(out, d_out, 2 * sizeof(double) * n_terms, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_out);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  return MPS_OK;
}

int wide_expect(mps_prog* p, const uint8_t* codes, int n_terms, double* out, Lane* L, void** ws) {
  WideBufs* B = nullptr;
  int rc = wide_bufs(ws ? ws : &p->ctx->wide, p->prec, p->chi_cap, &B);
  if (rc) return rc;
  B->gemm.split_bf16 = p->split_bf16;  // tensor-core products of this program
  cudaStream_t st = L ? L->stream : p->ctx->lane0.stream;
  return p->prec == MPS_PREC_FP64 ? wide_expect_t<double>(p, *B, st, codes, n_terms, out)
                                  : wide_expect_t<float>(p, *B, st, codes, n_terms, out);
}

template <typename T>
static int wide_sample_t(mps_prog* p, WideBufs& B, cudaStream_t st, int shots, uint64_t seed, uint8_t* h_bits) {
  const int n = p->n;
  cx<T>* sites = reinterpret_cast<cx<T>*>(p->d_sites);
  std::vector<int64_t> eoff(n + 2, 0);
  int64_t tot = 0;
  for (int i = 1; i <= n; ++i) {
    eoff[i] = tot;
    tot += (int64_t)p->hbond[i] * p->hbond[i];
  }
  int maxd = 1;
  for (int i = 0; i <= n; ++i) maxd = std::max(maxd, p->hbond[i]);
  const size_t eb = sizeof(cx<T>);
  const size_t vbytes = (size_t)shots * maxd * eb, ubytes = (size_t)shots * 2 * maxd * eb;
  char* buf = nullptr;
  WCK(cudaMalloc(&buf, (size_t)tot * eb + vbytes + 2 * ubytes + (size_t)shots * n + 1024));
  cx<T>* env = reinterpret_cast<cx<T>*>(buf);
  cx<T>* V = reinterpret_cast<cx<T>*>(buf + (size_t)tot * eb);
  cx<T>* U = reinterpret_cast<cx<T>*>(buf + (size_t)tot * eb + vbytes);
  cx<T>* Q = reinterpret_cast<cx<T>*>(buf + (size_t)tot * eb + vbytes + ubytes);
  uint8_t* d_bits = reinterpret_cast<uint8_t*>(buf + (size_t)tot * eb + vbytes + 2 * ubytes);
  cx<T>* F = reinterpret_cast<cx<T>*>(B.theta);
  int rc = MPS_OK;
  auto run = [&]() -> int {
    // right environments: R_n = 1, R_i = sum_s A_i[:, s, :] R_{i+1} A_i[:, s, :]^H
    const cx<T> one = mk<T>(T(1), T(0));
    WCK(cudaMemcpyAsync(env + eoff[n], &one, sizeof(one), cudaMemcpyHostToDevice, st));
    for (int i = n - 1; i >= 1; --i) {
      const int dl = p->hbond[i], dr = p->hbond[i + 1];
      const cx<T>* Ai = sites + p->off[i];
      WCK(cgemm(cmat<T>(Ai, 2 * dl, dr, dr, 1), cmat<T>(env + eoff[i + 1], dr, dr, dr, 1),
                cout_<T>(F, 2 * dl, dr, dr, 1), T(1), T(0), B.gemm, st));
      WCK(cgemm(cmat<T>(F, dl, 2 * dr, 2 * dr, 1), adj(cmat<T>(Ai, dl, 2 * dr, 2 * dr, 1)),
                cout_<T>(env + eoff[i], dl, dl, dl, 1), T(1), T(0), B.gemm, st));
    }
    // shots: V (S x dl) starts at 1
    std::vector<cx<T>> ones((size_t)shots, one);
    WCK(cudaMemcpyAsync(V, ones.data(), (size_t)shots * eb, cudaMemcpyHostToDevice, st));
    for (int i = 0; i < n; ++i) {
      const int dl = p->hbond[i], dr = p->hbond[i + 1];
      const cx<T>* Ai = sites + p->off[i];
      WCK(cgemm(cmat<T>(V, shots, dl, dl, 1), cmat<T>(Ai, dl, 2 * dr, 2 * dr, 1), cout_<T>(U, shots, 2 * dr, 2 * dr, 1),
                T(1), T(0), B.gemm, st));
      const cx<T>* Rn = i + 1 < n ? env + eoff[i + 1] : nullptr;
      if (Rn)
        WCK(cgemm(cmat<T>(U, 2 * shots, dr, dr, 1), cmat<T>(Rn, dr, dr, dr, 1), cout_<T>(Q, 2 * shots, dr, dr, 1),
                  T(1), T(0), B.gemm, st));
      else
        WCK(cudaMemcpyAsync(Q, U, (size_t)shots * 2 * dr * eb, cudaMemcpyDeviceToDevice, st));
      k_wide_sample_step<T><<<(shots * 32 + 255) / 256, 256, 0, st>>>(U, Q, V, shots, dr, i, n, seed, d_bits);
      WCK(cudaGetLastError());
    }
    WCK(cudaMemcpyAsync(h_bits, d_bits, (size_t)shots * n, cudaMemcpyDeviceToHost, st));
    WCK(cudaStreamSynchronize(st));
    return MPS_OK;
  };
  rc = run();
  cudaFree(buf);
  return rc;
}

int wide_sample(mps_prog* p, int shots, uint64_t seed, uint8_t* h_all_bits, Lane* L, void** ws) {
  WideBufs* B = nullptr;
  int rc = wide_bufs(ws ? ws : &p->ctx->wide, p->prec, p->chi_cap, &B);
  if (rc) return rc;
  B->gemm.split_bf16 = p->split_bf16;  // tensor-core products of this program
  cudaStream_t st = L ? L->stream : p->ctx->lane0.stream;
  return p->prec == MPS_PREC_FP64 ? wide_sample_t<double>(p, *B, st, shots, seed, h_all_bits)
                                  : wide_sample_t<float>(p, *B, st, shots, seed, h_all_bits);
}

template <typename T>
static int wide_amp_one_t(mps_prog* p, WideBufs& B, cudaStream_t st, const int* bits, double* out) {
  cx<T>* sites = reinterpret_cast<cx<T>*>(p->d_sites);
  cx<T>* v0 = reinterpret_cast<cx<T>*>(B.theta);
  cx<T>* v1 = reinterpret_cast<cx<T>*>(B.tbuf);
  const cx<T> one = mk<T>(T(1), T(0));
  WCK(cudaMemcpyAsync(v0, &one, sizeof(one), cudaMemcpyHostToDevice, st));
  for (int i = 0; i < p->n; ++i) {
    const int dl = p->hbond[i], dr = p->hbond[i + 1];
    const cx<T>* Ai = sites + p->off[i] + (int64_t)bits[i] * dr;
    WCK(cgemm(cmat<T>(v0, 1, dl, dl, 1), cmat<T>(Ai, dl, dr, 2 * dr, 1), cout_<T>(v1, 1, dr, dr, 1), T(1), T(0),
              B.gemm, st));
    std::swap(v0, v1);
  }
  double* d = reinterpret_cast<double*>(B.d_scalar);
  k_store_scalar<T><<<1, 1, 0, st>>>(v0, d);
  WCK(cudaMemcpyAsync(out, d, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  WCK(cudaStreamSynchronize(st));
  return MPS_OK;
}

int wide_amp_one(mps_prog* p, const int* bits, double* out) {
  WideBufs* B = nullptr;
  int rc = wide_bufs(&p->ctx->wide, p->prec, p->chi_cap, &B);
  if (rc) return rc;
  B->gemm.split_bf16 = p->split_bf16;  // tensor-core products of this program
  cudaStream_t st = p->ctx->lane0.stream;
  return p->prec == MPS_PREC_FP64 ? wide_amp_one_t<double>(p, *B, st, bits, out)
                                  : wide_amp_one_t<float>(p, *B, st, bits, out);
}

int wide_gemm_counts(mps_ctx* c, int* tc, int* simt) {
  *tc = *simt = 0;
  if (!c->wide) return MPS_OK;
  for (auto& b : reinterpret_cast<WideAll*>(c->wide)->b) {
    *tc += b.gemm.tc_launches;
    *simt += b.gemm.simt_launches;
  }
  return MPS_OK;
}

// Cross-check entry of the tensor-core GEMM against the CUDA-core kernel.
int wide_diag_cgemm(mps_ctx* c, int M, int N, int K, const double* a, const double* b, double* out_tc,
                    double* out_simt) {
  WideBufs* B = nullptr;
  const int chi = std::max(std::max(M, N), std::max(K, 64));
  int rc = wide_bufs(&c->wide, MPS_PREC_FP32, (chi + 1) / 2 + 64, &B);
  if (rc) return rc;
  cudaStream_t st = c->lane0.stream;
  std::vector<cx<float>> ha((size_t)M * K), hb((size_t)K * N), hc((size_t)M * N);
  for (size_t i = 0; i < ha.size(); ++i) ha[i] = mk<float>((float)a[2 * i], (float)a[2 * i + 1]);
  for (size_t i = 0; i < hb.size(); ++i) hb[i] = mk<float>((float)b[2 * i], (float)b[2 * i + 1]);
  cx<float>* da = reinterpret_cast<cx<float>*>(B->theta);
  cx<float>* db = reinterpret_cast<cx<float>*>(B->tbuf);
  cx<float>* dc = reinterpret_cast<cx<float>*>(B->gram);
  WCK(cudaMemcpyAsync(da, ha.data(), ha.size() * 8, cudaMemcpyHostToDevice, st));
  WCK(cudaMemcpyAsync(db, hb.data(), hb.size() * 8, cudaMemcpyHostToDevice, st));
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 0) {
      // the tensor-core kernel wherever it takes the product (whatever the
      // autotuner would pick), else the CUDA-core kernel
      const cudaError_t e = cgemm_kind(GEMM_TC, cmat<float>(da, M, K, K, 1), cmat<float>(db, K, N, N, 1),
                                       cout_<float>(dc, M, N, N, 1), 1.0f, 0.0f, B->gemm, st);
      if (e == cudaErrorInvalidValue) {
        cudaGetLastError();
        WCK(cgemm_simt(cmat<float>(da, M, K, K, 1), cmat<float>(db, K, N, N, 1), cout_<float>(dc, M, N, N, 1), 1.0f,
                       0.0f, st));
      } else {
        WCK(e);
      }
    } else
      WCK(cgemm_simt(cmat<float>(da, M, K, K, 1), cmat<float>(db, K, N, N, 1), cout_<float>(dc, M, N, N, 1), 1.0f,
                     0.0f, st));
    WCK(cudaMemcpyAsync(hc.data(), dc, hc.size() * 8, cudaMemcpyDeviceToHost, st));
    WCK(cudaStreamSynchronize(st));
    double* o = pass == 0 ? out_tc : out_simt;
    for (size_t i = 0; i < hc.size(); ++i) {
      o[2 * i] = hc[i].re;
      o[2 * i + 1] = hc[i].im;
    }
  }
  int herr = 0;
  WCK(cudaMemcpy(&herr, B->gemm.d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) return fail(MPS_ERR_TIMEOUT, "tensor-core GEMM wait timed out");
  return MPS_OK;
}

// One complex product on a chosen GEMM kernel (GemmKind), for tests of
// every tile shape.  flags: bit 0 stores A column-major, bit 1 stores B
// column-major, bit 2 writes C column-major, so the kernels' strided loads
// and stores are exercised; host arrays stay row-major.
template <typename T>
static int wide_diag_cgemm_kind_t(mps_ctx* c, int kind, int flags, int M, int N, int K, const double* a,
                                  const double* b, double* out) {
  WideBufs* B = nullptr;
  const int chi = std::max(std::max(M, N), std::max(K, 64));
  int rc = wide_bufs(&c->wide, sizeof(T) == 8 ? MPS_PREC_FP64 : MPS_PREC_FP32, (chi + 1) / 2 + 64, &B);
  if (rc) return rc;
  cudaStream_t st = c->lane0.stream;
  const bool acm = flags & 1, bcm = flags & 2, ccm = flags & 4;
  B->gemm.split_bf16 = sizeof(T) == 4 && (flags & 8);
  std::vector<cx<T>> ha((size_t)M * K), hb((size_t)K * N), hc((size_t)M * N);
  for (int i = 0; i < M; ++i)
    for (int k = 0; k < K; ++k) {
      const size_t s0 = (size_t)i * K + k;
      ha[acm ? (size_t)k * M + i : s0] = mk<T>((T)a[2 * s0], (T)a[2 * s0 + 1]);
    }
  for (int k = 0; k < K; ++k)
    for (int j = 0; j < N; ++j) {
      const size_t s0 = (size_t)k * N + j;
      hb[bcm ? (size_t)j * K + k : s0] = mk<T>((T)b[2 * s0], (T)b[2 * s0 + 1]);
    }
  cx<T>* da = reinterpret_cast<cx<T>*>(B->theta);
  cx<T>* db = reinterpret_cast<cx<T>*>(B->tbuf);
  cx<T>* dc = reinterpret_cast<cx<T>*>(B->gram);
  WCK(cudaMemcpyAsync(da, ha.data(), ha.size() * sizeof(cx<T>), cudaMemcpyHostToDevice, st));
  WCK(cudaMemcpyAsync(db, hb.data(), hb.size() * sizeof(cx<T>), cudaMemcpyHostToDevice, st));
  const CMat<T> va = acm ? cmat<T>(da, M, K, 1, M) : cmat<T>(da, M, K, K, 1);
  const CMat<T> vb = bcm ? cmat<T>(db, K, N, 1, K) : cmat<T>(db, K, N, N, 1);
  const CMatOut<T> vc = ccm ? cout_<T>(dc, M, N, 1, M) : cout_<T>(dc, M, N, N, 1);
  const cudaError_t e = cgemm_kind(kind, va, vb, vc, T(1), T(0), B->gemm, st);
  if (e == cudaErrorInvalidValue) return fail(MPS_ERR_ARG, "this kernel does not take this product");
  WCK(e);
  WCK(cudaMemcpyAsync(hc.data(), dc, hc.size() * sizeof(cx<T>), cudaMemcpyDeviceToHost, st));
  WCK(cudaStreamSynchronize(st));
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < N; ++j) {
      const cx<T> z = hc[ccm ? (size_t)j * M + i : (size_t)i * N + j];
      out[2 * ((size_t)i * N + j)] = (double)z.re;
      out[2 * ((size_t)i * N + j) + 1] = (double)z.im;
    }
  if (sizeof(T) == 4) {
    int herr = 0;
    WCK(cudaMemcpy(&herr, B->gemm.d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) return fail(MPS_ERR_TIMEOUT, "tensor-core GEMM wait timed out");
  }
  return MPS_OK;
}

int wide_diag_cgemm_kind(mps_ctx* c, int prec, int kind, int flags, int M, int N, int K, const double* a,
                         const double* b, double* out) {
  return prec == MPS_PREC_FP64 ? wide_diag_cgemm_kind_t<double>(c, kind, flags, M, N, K, a, b, out)
                               : wide_diag_cgemm_kind_t<float>(c, kind, flags, M, N, K, a, b, out);
}

int wide_set_coop_rows(int rows) {
  if (rows < 0 || rows > 4096) return fail(MPS_ERR_ARG, "rows per CTA must be in 0..4096");
  g_coop_rows.store(rows == 0 ? 8 : rows);
  return MPS_OK;
}

int wide_gemm_tunings(mps_ctx* c) {
  int n = 0;
  if (!c->wide) return 0;
  for (auto& b : reinterpret_cast<WideAll*>(c->wide)->b) n += b.gemm.tunings;
  return n;
}

}  // namespace gbmps
