// Noisy circuits: the density matrix of n qubits held as a vectorised MPS on
// 2n sites (programs begun with MPS_FLAG_DENSITY).
//
// The reference's noisy MPS visitor (visitors/exatn-mpo/ExaTnPmpsVisitor.cpp)
// keeps a purified MPS: each site tensor carries an extra Kraus leg whose
// contraction with the conjugate network gives rho (buildInitialNetwork
// :544-656), a gate acts on the physical leg (:820-885) and a single-qubit
// channel widens and re-truncates the Kraus leg (applyLocalKrausOp
// :909-1130).  Here rho itself is the tensor train: site 2q carries the ket
// index of qubit q and site 2q+1 its bra index, so entry (ket i, bra j) of a
// qubit pair is rho_ij.  Every operation is then a one- or two-site update of
// the engine's existing split kernels:
//   gate U on q           U on site 2q, conj(U) on site 2q+1
//   gate U on (a, b)      U on (2a, 2b), conj(U) on (2a+1, 2b+1) (routed)
//   channel {K_k} on q    S = sum_k K_k (x) conj(K_k) on the adjacent pair
//                         (2q, 2q+1): rho -> sum_k K_k rho K_k^H
// Both representations are exact without truncation; they truncate
// differently (here: the bond singular values of vec(rho)).
//
// This file contracts the doubled chain into what finalize (:658-795) reads:
// Tr(rho P) for Pauli strings (many at once), the reduced density matrix of a
// few qubits, and its diagonal for shot sampling.  The contraction walks the
// chain left to right with a row vector per open index: at pair q the ket
// site opens the pair's ket index (k_dm_ket), then the bra site either
// closes it against a 2x2 weight (trace, or a Pauli letter), keeps the
// diagonal (i = j) or keeps both (k_dm_bra).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gb300mps.h"
#include "engine_internal.hpp"
#include "philox.cuh"

namespace gbmps {

// U[m][c + i W] = sum_l A[l][i][m] vin[l][c]   (A: dl x 2 x dr, vin: dl x W)
template <typename T>
__global__ void k_dm_ket(const cx<T>* __restrict__ A, int dl, int dr, int64_t W, const cx<double>* __restrict__ vin,
                         cx<double>* __restrict__ U) {
  const int64_t total = (int64_t)dr * 2 * W;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(t / (2 * W));
    const int64_t col = t - (int64_t)m * 2 * W;
    const int i = (int)(col / W);
    const int64_t c = col - (int64_t)i * W;
    cx<double> acc = mk<double>(0, 0);
    for (int l = 0; l < dl; ++l) {
      const cx<T> a = A[((int64_t)l * 2 + i) * dr + m];
      fma_c(acc, mk<double>((double)a.re, (double)a.im), vin[(int64_t)l * W + c]);
    }
    U[t] = acc;
  }
}

enum DmMode : int { DM_CLOSE = 0, DM_DIAG = 1, DM_FULL = 2 };

// The bra site of the pair (B: dm x 2 x dr) against U (dm x 2W):
//   DM_CLOSE  vout[r][c]               = sum_ij w_c[i][j] sum_m U[m][c + iW] B[m][j][r]
//             w_c = P^T for the Pauli letter codes[c * stride] (0 I, 1 X,
//             2 Y, 3 Z; codes == nullptr: I), so the pair contributes
//             Tr(rho_pair P) = sum_ij rho_ij P_ji
//   DM_DIAG   vout[r][c + iW]          = sum_m U[m][c + iW] B[m][i][r]
//   DM_FULL   vout[r][c + (i + 2j) W]  = sum_m U[m][c + iW] B[m][j][r]
template <typename T>
__global__ void k_dm_bra(const cx<T>* __restrict__ B, int dm, int dr, int64_t W, const cx<double>* __restrict__ U,
                         int mode, const uint8_t* __restrict__ codes, int stride, int64_t n_codes,
                         cx<double>* __restrict__ vout) {
  const int64_t wo = mode == DM_CLOSE ? W : (mode == DM_DIAG ? 2 * W : 4 * W);
  const int64_t total = (int64_t)dr * wo;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / wo);
    const int64_t col = t - (int64_t)r * wo;
    cx<double> acc = mk<double>(0, 0);
    auto bra = [&](int m, int j) {
      const cx<T> b = B[((int64_t)m * 2 + j) * dr + r];
      return mk<double>((double)b.re, (double)b.im);
    };
    if (mode == DM_CLOSE) {
      const int64_t c = col;
      const int code = (codes != nullptr && c < n_codes) ? codes[c * stride] : 0;
      for (int m = 0; m < dm; ++m) {
        const cx<double> u0 = U[(int64_t)m * 2 * W + c];
        const cx<double> u1 = U[(int64_t)m * 2 * W + W + c];
        const cx<double> b0 = bra(m, 0), b1 = bra(m, 1);
        switch (code) {
          case 0:  // I^T: (0,0) + (1,1)
            fma_c(acc, u0, b0);
            fma_c(acc, u1, b1);
            break;
          case 1:  // X^T: (0,1) + (1,0)
            fma_c(acc, u0, b1);
            fma_c(acc, u1, b0);
            break;
          case 2: {  // Y^T: i (0,1) - i (1,0)
            cx<double> s = mk<double>(0, 0);
            fma_c(s, u0, b1);
            cx<double> d = mk<double>(0, 0);
            fma_c(d, u1, b0);
            acc = acc + mk<double>(-(s.im - d.im), s.re - d.re);
            break;
          }
          default: {  // Z^T: (0,0) - (1,1)
            fma_c(acc, u0, b0);
            cx<double> s = mk<double>(0, 0);
            fma_c(s, u1, b1);
            acc = acc - s;
            break;
          }
        }
      }
    } else if (mode == DM_DIAG) {
      const int i = (int)(col / W);
      const int64_t c = col - (int64_t)i * W;
      for (int m = 0; m < dm; ++m) fma_c(acc, U[(int64_t)m * 2 * W + (int64_t)i * W + c], bra(m, i));
    } else {
      const int ij = (int)(col / W);
      const int64_t c = col - (int64_t)ij * W;
      const int i = ij & 1, j = ij >> 1;
      for (int m = 0; m < dm; ++m) fma_c(acc, U[(int64_t)m * 2 * W + (int64_t)i * W + c], bra(m, j));
    }
    vout[t] = acc;
  }
}

// One thread per output, grid-stride beyond 32 CTAs per SM.
static int grid_for(int64_t total, int sms) {
  int64_t g = (total + 255) / 256;
  if (g > (int64_t)sms * 32) g = (int64_t)sms * 32;
  if (g < 1) g = 1;
  return (int)g;
}

// Largest device buffers the contraction may take (three vectors of
// complex128 entries): requests beyond it are rejected.
constexpr size_t kDmWorkBytes = size_t(6) << 30;

// Walk the doubled chain.  sel[q]: DM_CLOSE (with codes, or the trace),
// DM_DIAG or DM_FULL for each qubit.  W0 columns enter (the rows of the
// left boundary vector are all ones: each column is one functional).
// Returns the final row vector (1 x W_final) in out_host.
static int dm_contract(mps_prog* p, const std::vector<int>& sel, int64_t W0, const uint8_t* d_codes, int stride,
                       int64_t n_codes, std::vector<cx<double>>& out_host) {
  mps_ctx* c = p->ctx;
  cudaStream_t st = c->lane0.stream;
  const int nq = p->nq;
  std::vector<int> bond(p->n + 1);
  cudaError_t e = cudaMemcpyAsync(bond.data(), p->d_bond, bond.size() * sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  // largest vector of the walk: the ket step's (bond x 2W) or the bra
  // step's (bond x W'), where W grows with the open indices so far
  int64_t W = W0;
  size_t elems = (size_t)W0;
  for (int q = 0; q < nq; ++q) {
    const int64_t wo = sel[q] == DM_DIAG ? 2 * W : (sel[q] == DM_FULL ? 4 * W : W);
    elems = std::max(elems, (size_t)bond[2 * q + 1] * 2 * (size_t)W);
    elems = std::max(elems, (size_t)bond[2 * q + 2] * (size_t)wo);
    W = wo;
  }
  if (3 * elems * sizeof(cx<double>) > kDmWorkBytes)
    return fail(MPS_ERR_UNSUPPORTED, "density-matrix contraction too large for the work buffers");
  cx<double>* buf = nullptr;
  if (cudaMalloc(&buf, 3 * elems * sizeof(cx<double>)) != cudaSuccess) {
    cudaGetLastError();
    return fail(MPS_ERR_OOM, "device allocation failed");
  }
  cx<double>* vin = buf;
  cx<double>* U = buf + elems;
  cx<double>* vout = buf + 2 * elems;
  // left boundary: one row (bond 1) of W0 ones
  std::vector<cx<double>> ones((size_t)W0, mk<double>(1, 0));
  e = cudaMemcpyAsync(vin, ones.data(), ones.size() * sizeof(cx<double>), cudaMemcpyHostToDevice, st);
  const size_t eb = p->prec == MPS_PREC_FP64 ? 16 : 8;
  W = W0;
  for (int q = 0; q < nq && e == cudaSuccess; ++q) {
    const int s0 = 2 * q, s1 = 2 * q + 1;
    const int dl = bond[s0], dm = bond[s0 + 1], dr = bond[s1 + 1];
    const char* A = (const char*)p->d_sites + p->off[s0] * eb;
    const char* B = (const char*)p->d_sites + p->off[s1] * eb;
    const int gk = grid_for((int64_t)dm * 2 * W, c->num_sms);
    if (p->prec == MPS_PREC_FP64)
      k_dm_ket<double><<<gk, 256, 0, st>>>((const cx<double>*)A, dl, dm, W, vin, U);
    else
      k_dm_ket<float><<<gk, 256, 0, st>>>((const cx<float>*)A, dl, dm, W, vin, U);
    const int mode = sel[q];
    const int64_t wo = mode == DM_CLOSE ? W : (mode == DM_DIAG ? 2 * W : 4 * W);
    const uint8_t* cq = (mode == DM_CLOSE && d_codes) ? d_codes + q : nullptr;
    const int gb = grid_for((int64_t)dr * wo, c->num_sms);
    if (p->prec == MPS_PREC_FP64)
      k_dm_bra<double><<<gb, 256, 0, st>>>((const cx<double>*)B, dm, dr, W, U, mode, cq, stride, n_codes, vout);
    else
      k_dm_bra<float><<<gb, 256, 0, st>>>((const cx<float>*)B, dm, dr, W, U, mode, cq, stride, n_codes, vout);
    e = cudaGetLastError();
    std::swap(vin, vout);
    W = wo;
  }
  if (e == cudaSuccess) {
    out_host.resize((size_t)W);
    e = cudaMemcpyAsync(out_host.data(), vin, (size_t)W * sizeof(cx<double>), cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(buf);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  return prog_check_err(p);
}

static int flush(mps_prog* p) {
  if (p->pending.empty()) return MPS_OK;
  return launch_programs(p->ctx, p->ctx->lane0, &p, 1, (p->flags & MPS_FLAG_PER_GATE) != 0);
}

static int check_selection(const mps_prog* p, int n_sel, const int* qubits, std::vector<int>& pos) {
  pos.assign(p->nq, -1);
  for (int a = 0; a < n_sel; ++a) {
    if (qubits[a] < 0 || qubits[a] >= p->nq) return fail(MPS_ERR_ARG, "qubit index out of range");
    if (pos[qubits[a]] >= 0) return fail(MPS_ERR_ARG, "qubit selected twice");
    pos[qubits[a]] = a;
  }
  return MPS_OK;
}

// Tr(rho P_t) for n_terms Pauli strings (codes: n_terms x nq) plus Tr(rho)
// as one more column; res gets n_terms + 1 complex values.
int density_expect(mps_prog* p, const uint8_t* codes, int n_terms, std::vector<cx<double>>& res) {
  mps_ctx* c = p->ctx;
  uint8_t* d_codes = nullptr;
  const size_t bytes = (size_t)n_terms * p->nq;
  if (bytes > 0) {
    if (cudaMalloc(&d_codes, bytes) != cudaSuccess) {
      cudaGetLastError();
      return fail(MPS_ERR_OOM, "device allocation failed");
    }
    cudaError_t e = cudaMemcpyAsync(d_codes, codes, bytes, cudaMemcpyHostToDevice, c->lane0.stream);
    if (e != cudaSuccess) {
      cudaFree(d_codes);
      return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
    }
  }
  std::vector<int> sel(p->nq, DM_CLOSE);
  const int rc = dm_contract(p, sel, (int64_t)n_terms + 1, d_codes, p->nq, n_terms, res);
  if (d_codes) cudaFree(d_codes);
  return rc;
}

// The superoperator of rho -> sum_k K_k rho K_k^H on the adjacent sites
// (2q, 2q+1): S[(2i + j)][(2i' + j')] = sum_k K[i][i'] conj(K[j][j']), rows and
// columns 2 * phys(ket site) + phys(bra site) with the ket site the lower one.
// kraus: n_kraus 2x2 matrices, row-major (re, im) pairs.
int kraus_superop(int qubit, int n_kraus, const double* kraus, GateRec& g) {
  g.nq = 2;
  g.q0 = 2 * qubit;
  g.q1 = 2 * qubit + 1;
  for (int i = 0; i < 16; ++i) g.m[i] = 0.0;
  for (int k = 0; k < n_kraus; ++k) {
    const double* K = kraus + 8 * (size_t)k;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        for (int i2 = 0; i2 < 2; ++i2)
          for (int j2 = 0; j2 < 2; ++j2) {
            const cd a(K[2 * (2 * i + i2)], K[2 * (2 * i + i2) + 1]);
            const cd b(K[2 * (2 * j + j2)], -K[2 * (2 * j + j2) + 1]);
            g.m[(2 * i + j) * 4 + (2 * i2 + j2)] += a * b;
          }
  }
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(g.m[i].real()) || !std::isfinite(g.m[i].imag())) return fail(MPS_ERR_ARG, "non-finite Kraus entry");
  return MPS_OK;
}

}  // namespace gbmps

using namespace gbmps;

extern "C" {

int mps_channel1(mps_prog* p, int qubit, int n_kraus, const double* kraus) {
  if (!p || !kraus || n_kraus < 1) return fail(MPS_ERR_ARG, "bad argument");
  if (!p->density) return fail(MPS_ERR_STATE, "channels need a program begun with MPS_FLAG_DENSITY");
  if (qubit < 0 || qubit >= p->nq) return fail(MPS_ERR_ARG, "qubit index out of range");
  GateRec g;
  const int rc = kraus_superop(qubit, n_kraus, kraus, g);
  if (rc) return rc;
  p->pending.push_back(g);
  return MPS_OK;
}

int mps_density_matrix(mps_prog* p, int n_sel, const int* qubits, double* out) {
  if (!p || !out || n_sel < 1 || !qubits) return fail(MPS_ERR_ARG, "bad argument");
  if (!p->density) return fail(MPS_ERR_STATE, "not a density program (MPS_FLAG_DENSITY)");
  if (n_sel > MPS_DM_QUBITS_MAX) return fail(MPS_ERR_UNSUPPORTED, "too many qubits for a density matrix");
  std::vector<int> pos;
  int rc = check_selection(p, n_sel, qubits, pos);
  if (rc) return rc;
  mps_ctx* c = p->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(MPS_ERR_CUDA, "cudaSetDevice failed");
  rc = flush(p);
  if (rc) return rc;
  std::vector<int> sel(p->nq, DM_CLOSE);
  std::vector<int> chain;  // selected qubits in chain order: base-4 digit t of the result
  for (int q = 0; q < p->nq; ++q)
    if (pos[q] >= 0) {
      sel[q] = DM_FULL;
      chain.push_back(q);
    }
  std::vector<cx<double>> res;
  rc = dm_contract(p, sel, 1, nullptr, 0, 0, res);
  if (rc) return rc;
  const int64_t dim = (int64_t)1 << n_sel;
  for (int64_t col = 0; col < (int64_t)res.size(); ++col) {
    int64_t x = 0, y = 0;
    for (size_t t = 0; t < chain.size(); ++t) {
      const int d = (int)((col >> (2 * t)) & 3);
      x |= (int64_t)(d & 1) << pos[chain[t]];
      y |= (int64_t)(d >> 1) << pos[chain[t]];
    }
    out[2 * (x * dim + y)] = res[col].re;
    out[2 * (x * dim + y) + 1] = res[col].im;
  }
  return MPS_OK;
}

int mps_density_diag(mps_prog* p, int n_sel, const int* qubits, double* out) {
  if (!p || !out || n_sel < 1 || !qubits) return fail(MPS_ERR_ARG, "bad argument");
  if (!p->density) return fail(MPS_ERR_STATE, "not a density program (MPS_FLAG_DENSITY)");
  if (n_sel > MPS_DIAG_QUBITS_MAX) return fail(MPS_ERR_UNSUPPORTED, "too many qubits for a diagonal");
  std::vector<int> pos;
  int rc = check_selection(p, n_sel, qubits, pos);
  if (rc) return rc;
  mps_ctx* c = p->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(MPS_ERR_CUDA, "cudaSetDevice failed");
  rc = flush(p);
  if (rc) return rc;
  std::vector<int> sel(p->nq, DM_CLOSE);
  std::vector<int> chain;
  for (int q = 0; q < p->nq; ++q)
    if (pos[q] >= 0) {
      sel[q] = DM_DIAG;
      chain.push_back(q);
    }
  std::vector<cx<double>> res;
  rc = dm_contract(p, sel, 1, nullptr, 0, 0, res);
  if (rc) return rc;
  for (int64_t col = 0; col < (int64_t)res.size(); ++col) {
    int64_t x = 0;
    for (size_t t = 0; t < chain.size(); ++t) x |= (int64_t)((col >> t) & 1) << pos[chain[t]];
    out[x] = res[col].re;
  }
  return MPS_OK;
}

}  // extern "C"

namespace gbmps {

// Shots of a density program: the diagonal of the reduced density matrix of
// the measured qubits on the device, then one Philox uniform per shot and a
// walk of the cumulative distribution (the draw of generateResultBitString,
// ExaTnPmpsVisitor.cpp:133-171, without its readout flips, which belong to
// the noise model of the caller).
int density_sample(mps_prog* p, int shots, uint64_t seed, uint8_t* bits) {
  std::vector<int> meas = p->measured;
  if (meas.empty())
    for (int q = 0; q < p->nq; ++q) meas.push_back(q);
  std::vector<int> uniq = meas;
  std::sort(uniq.begin(), uniq.end());
  uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
  if ((int)uniq.size() > MPS_DIAG_QUBITS_MAX) return fail(MPS_ERR_UNSUPPORTED, "too many measured qubits");
  std::vector<int> pos(p->nq, -1);
  for (size_t a = 0; a < uniq.size(); ++a) pos[uniq[a]] = (int)a;
  std::vector<int> sel(p->nq, DM_CLOSE);
  for (int q : uniq) sel[q] = DM_DIAG;
  std::vector<cx<double>> res;
  int rc = dm_contract(p, sel, 1, nullptr, 0, 0, res);
  if (rc) return rc;
  // res[col]: bit t of col is the t-th selected qubit in chain order = uniq[t]
  std::vector<double> cdf(res.size());
  double acc = 0.0;
  for (size_t i = 0; i < res.size(); ++i) {
    acc += std::max(0.0, res[i].re);
    cdf[i] = acc;
  }
  if (!(acc > 0.0)) return fail(MPS_ERR_NUMERIC, "density matrix with no positive diagonal");
  for (int s = 0; s < shots; ++s) {
    // one uniform per shot (counter = shot), on a stream tag of its own
    const double u = philox_uniform(seed, (uint32_t)s, 0u, 0x5D3A7u) * acc;
    size_t k = std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin();
    if (k >= cdf.size()) k = cdf.size() - 1;
    for (size_t a = 0; a < meas.size(); ++a) bits[(size_t)s * meas.size() + a] = (uint8_t)((k >> pos[meas[a]]) & 1);
  }
  return MPS_OK;
}

}  // namespace gbmps
