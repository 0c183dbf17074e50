// Wide two-site path: bond dimensions above the single-CTA limit (up to
// kWideChi).  Host-driven per gate: complex GEMMs (tcgen05 for complex64,
// CUDA cores for complex128), a cooperative (grid-wide) tridiagonal
// eigensolver and a cooperative Householder QR.  Declarations shared by
// k_gemm.cu, k_coop.cu and wide.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mps_common.cuh"

namespace gbmps {

constexpr int kWideChi = 1024;          // largest bond of the wide path
constexpr int kWideM = 2 * kWideChi;    // largest Gram / theta side

// Strided complex matrix: element (i, j) is p[i * rs + j * cs], conjugated
// when conj != 0.
template <typename T>
struct CMat {
  const cx<T>* p;
  int64_t rs, cs;
  int rows, cols;
  int conj;
};
template <typename T>
struct CMatOut {
  cx<T>* p;
  int64_t rs, cs;
  int rows, cols;
};

template <typename T>
inline CMat<T> cmat(const void* p, int rows, int cols, int64_t rs, int64_t cs, int conj = 0) {
  CMat<T> v;
  v.p = reinterpret_cast<const cx<T>*>(p);
  v.rs = rs;
  v.cs = cs;
  v.rows = rows;
  v.cols = cols;
  v.conj = conj;
  return v;
}
// The conjugate transpose of a view.
template <typename T>
inline CMat<T> adj(CMat<T> v) {
  CMat<T> r = v;
  r.rs = v.cs;
  r.cs = v.rs;
  r.rows = v.cols;
  r.cols = v.rows;
  r.conj = !v.conj;
  return r;
}
template <typename T>
inline CMatOut<T> cout_(void* p, int rows, int cols, int64_t rs, int64_t cs) {
  CMatOut<T> v;
  v.p = reinterpret_cast<cx<T>*>(p);
  v.rs = rs;
  v.cs = cs;
  v.rows = rows;
  v.cols = cols;
  return v;
}

// Kernels a complex GEMM can run on: CUDA-core tiles of rows x columns of
// complex outputs per CTA, and (complex64 only) the tensor-core kernel.
enum GemmKind {
  GEMM_SIMT_64x64 = 0,
  GEMM_SIMT_32x32 = 1,
  GEMM_SIMT_16x64 = 2,
  GEMM_SIMT_64x16 = 3,
  GEMM_TC = 4,
  GEMM_KINDS = 5
};

// Device workspace of the GEMMs: the split (hi/lo) real-embedded operands of
// the tensor-core path.  Sized for the largest wide product.
struct GemmWs {
  float* a_hi = nullptr;
  float* a_lo = nullptr;
  float* b_hi = nullptr;
  float* b_lo = nullptr;
  size_t a_elems = 0, b_elems = 0;
  int* d_err = nullptr;  // barrier/wait time-outs of the tensor-core kernel
  bool split_bf16 = false;  // tensor-core products with bf16 hi/lo operands (MPS_PREC_SPLIT_BF16)
  int tc_launches = 0;   // tensor-core GEMM launches issued (diagnostics)
  int simt_launches = 0;
  // autotuner: output buffer of the trial launches and their timing events
  void* tune_c = nullptr;
  size_t tune_c_bytes = 0;
  cudaEvent_t tune_ev[2] = {nullptr, nullptr};
  int tunings = 0;  // shape buckets tuned with this workspace
};
int gemm_ws_init(GemmWs& ws, size_t a_elems, size_t b_elems);
void gemm_ws_free(GemmWs& ws);

// C = alpha * A * B + beta * C with A (M x K), B (K x N), C (M x N) views.
// complex64 runs on tcgen05 (3xTF32: hi*hi + hi*lo + lo*hi, FP32
// accumulation in tensor memory) for products of at least ~2M complex MACs,
// else on CUDA cores; complex128 runs on CUDA cores.
cudaError_t cgemm(const CMat<float>& A, const CMat<float>& B, const CMatOut<float>& C, float alpha, float beta,
                  GemmWs& ws, cudaStream_t st);
cudaError_t cgemm(const CMat<double>& A, const CMat<double>& B, const CMatOut<double>& C, double alpha,
                  double beta, GemmWs& ws, cudaStream_t st);
// Force the CUDA-core kernel (cross-checks of the tensor-core path).
cudaError_t cgemm_simt(const CMat<float>& A, const CMat<float>& B, const CMatOut<float>& C, float alpha,
                       float beta, cudaStream_t st);
// Run one given kernel (GemmKind); GEMM_TC only for complex64 products the
// tensor-core kernel accepts (else cudaErrorInvalidValue).
cudaError_t cgemm_kind(int kind, const CMat<float>& A, const CMat<float>& B, const CMatOut<float>& C, float alpha,
                       float beta, GemmWs& ws, cudaStream_t st);
cudaError_t cgemm_kind(int kind, const CMat<double>& A, const CMat<double>& B, const CMatOut<double>& C,
                       double alpha, double beta, GemmWs& ws, cudaStream_t st);

// GEMM autotuner.  Products are grouped into buckets by device, precision,
// ceil(log2) of M, N and K, and which index of A, B and C is unit-stride.
// Mode 0 uses the static rule (tensor cores for complex64 products of at
// least ~2M complex MACs, else 64 x 64 CUDA-core tiles); mode 1 times every
// eligible kernel on the first product of a new bucket (trial launches write
// a scratch output, the inputs are only read) and keeps the fastest; mode 2
// uses tuned or loaded entries without tuning new buckets.  The table is
// shared by every context of the process; the initial mode is 1 unless the
// environment variable GB300MPS_AUTOTUNE names another.
constexpr int kTuneCols = 9;  // device, prec, lg M, lg N, lg K, layout, kernel, ns, ns of the static rule
void gemm_tune_set_mode(int mode);
int gemm_tune_mode();
int gemm_tune_table(int* out, int cap);
int gemm_tune_save(const char* path);
int gemm_tune_load(const char* path);
void gemm_tune_clear();

// ------------------------------------------------------------ cooperative
constexpr int32_t kCoopTimeout = 1 << 8;

// Eigen-decomposition of the m x m Hermitian Gram matrix G (row-major, ld m)
// in two cooperative launches.  phase 0: tridiagonalisation (the reflectors
// overwrite G), every eigenvalue, descending order -> lam[0..m).  phase 1:
// eigenvectors of ranks 0..kv-1 -> columns of W (row stride ld).  The work
// buffer carries the state from phase 0 to phase 1; status_err receives
// kCoopTimeout when a grid barrier gave up.
struct WideEigArgs {
  void* G;
  void* W;
  double* lam;
  int m;
  int phase;
  int kv;
  int ld;
  int grid0;        // grid of the launches (work-buffer layout); set by launch_wide_eig
  void* work;       // cooperative scratch (wide_eig_work_bytes)
  int* status_err;
};
size_t wide_eig_work_bytes(int prec, int m);
cudaError_t launch_wide_eig(int prec, const WideEigArgs& a, int grid, cudaStream_t st);

// Householder QR of the view M (mr x nc): Q (mr x k, k = min(mr, nc)) is
// written through the view Q (conjugated when qconj), R (k x nc) row-major to
// R.  The input is copied to the work buffer first, so Q may alias M.
size_t wide_qr_work_bytes(int prec, int mr, int nc);
template <typename T>
cudaError_t launch_wide_qr_t(const CMat<T>& M, const CMatOut<T>& Q, int qconj, void* R, void* work, int* err,
                             int grid, cudaStream_t st);
int coop_grid(int prec, int which);  // co-resident grid of the cooperative kernels (0 eig, 1 qr)

}  // namespace gbmps
