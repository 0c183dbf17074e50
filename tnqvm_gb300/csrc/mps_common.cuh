// Shared host/device definitions of the GB300 MPS engine.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbmps {

// Interleaved complex number; 8-byte (complex64) or 16-byte (complex128).
template <typename T>
struct __align__(2 * sizeof(T)) cx {
  T re, im;
};

template <typename T>
__host__ __device__ __forceinline__ cx<T> mk(T r, T i) {
  cx<T> z;
  z.re = r;
  z.im = i;
  return z;
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) {
  return mk<T>(a.re + b.re, a.im + b.im);
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) {
  return mk<T>(a.re - b.re, a.im - b.im);
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(cx<T> a, cx<T> b) {
  return mk<T>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> scl(cx<T> a, T s) {
  return mk<T>(a.re * s, a.im * s);
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> conj(cx<T> a) {
  return mk<T>(a.re, -a.im);
}
// acc += a * b
template <typename T>
__host__ __device__ __forceinline__ void fma_c(cx<T>& acc, cx<T> a, cx<T> b) {
  acc.re = fma(a.re, b.re, fma(-a.im, b.im, acc.re));
  acc.im = fma(a.re, b.im, fma(a.im, b.re, acc.im));
}
// acc += conj(a) * b
template <typename T>
__host__ __device__ __forceinline__ void fma_cj(cx<T>& acc, cx<T> a, cx<T> b) {
  acc.re = fma(a.re, b.re, fma(a.im, b.im, acc.re));
  acc.im = fma(a.re, b.im, fma(-a.im, b.re, acc.im));
}
template <typename T>
__host__ __device__ __forceinline__ T abs2(cx<T> a) {
  return a.re * a.re + a.im * a.im;
}

// Operation kinds of a compiled program.
enum OpKind : int32_t {
  OP_GATE1 = 0,   // 2x2 on the physical leg of one site
  OP_GATE2 = 1,   // 4x4 on sites (site, site+1): merge, gate, SVD, truncate, split
  OP_MOVE_R = 2,  // QR: orthogonality centre site -> site+1
  OP_MOVE_L = 3,  // LQ: orthogonality centre site -> site-1
};

// Where the singular values of a 2-site split go.
enum Orient : int32_t {
  ORIENT_TO_HI = 0,  // lo site left-isometric, S*V^H on hi (centre -> hi)
  ORIENT_TO_LO = 1,  // hi site right-isometric, U*S on lo (centre -> lo)
  ORIENT_SQRT = 2,   // sqrt(S) on both sides (exatn semantics)
};

struct DevOp {
  int32_t kind;
  int32_t site;
  int32_t orient;
  int32_t pad;
  double m[32];  // row-major interleaved complex; GATE2 rows/cols are 2*phys(site)+phys(site+1)
};

enum TruncMode : int32_t { TRUNC_EXATN = 0, TRUNC_ITENSOR = 1 };

// Per-program statistics written by the kernels.
enum StatSlot {
  ST_LOG_FID = 0,     // sum over 2-qubit gates of log(1 - discarded fraction)
  ST_MAX_DISC = 1,    // largest discarded fraction seen
  ST_N_GATE2 = 2,     // number of 2-qubit gate splits
  ST_N_OPS = 3,       // number of ops executed
  ST_FLOPS = 4,       // GEMM-class flops: theta merge + gate + Gram + split + centre-move products
  ST_EIG_FLOPS = 5,   // Householder reflections of the eigensolver and the centre-move QR
  ST_CYC_THETA = 6,   // SM clock cycles spent per phase (thread 0's clock64 deltas)
  ST_CYC_GRAM = 7,
  ST_CYC_EIG = 8,
  ST_CYC_SPLIT = 9,
  ST_CYC_MOVE = 10,
  ST_N_REFINE = 11,   // two-site splits whose small-eigenvalue block was re-solved
  ST_CYC_TRID = 12,   // within the eigensolver: Householder tridiagonalisation
  ST_CYC_BISECT = 13, //   bisection and ranking of the eigenvalues
  ST_CYC_VEC = 14,    //   twisted-factorisation vectors and their back-transform
  ST_CYC_ORTH = 15,   // orthonormalisation and the subspace step (within the split phase)
  ST_CYC_OBS = 16,    // attached observables evaluated by the program's CTA after its ops
  ST_COUNT = 17,
};

// Error bits written by the kernels into ProgDesc::err.
enum ErrBits : int32_t {
  ERR_NAN = 1,        // non-finite value met in a split
  ERR_DIMS = 2,       // bond dimension beyond what the kernel supports
  ERR_TIMEOUT = 4,    // a site-parallel op waited past its bound for an earlier op
};

struct ProgDesc {
  void* sites;              // complex<T> arena
  const int64_t* site_off;  // element offset of each site tensor
  int* bond;                // n+1 bond dimensions; bond[0] = bond[n] = 1
  const DevOp* ops;
  int32_t n_ops;
  int32_t n;
  int32_t chi_cap;
  int32_t mode;
  int32_t flags;
  int32_t prec;             // 0 complex128, 1 complex64 (MPS_PREC_FP64 / MPS_PREC_FP32)
  double cutoff;
  double* stats;            // ST_COUNT doubles
  int* err;
  // Optional observables evaluated by the same CTA right after the ops
  // (n_obs Pauli strings of n codes; results (re, im) per string to obs_out),
  // then done[1] = the error word and done[0] = 1 (host-mapped memory).
  const uint8_t* obs_codes;
  int32_t n_obs;
  int32_t pad2;
  double* obs_out;
  int* done;
  // Optional: the program's SM clock cycles on its CTA (ops + observables),
  // written when it finishes (captured batches order their next replay by it).
  double* cycles_out;
};

// Measurement task descriptors (k_measure.cu).
struct ExpTask {
  const void* sites;
  const int64_t* site_off;
  const int* bond;
  const uint8_t* codes;
  int32_t n;
  int32_t pad;
};
struct EnvTask {
  const void* sites;
  const int64_t* site_off;
  const int* bond;
  void* env;
  const int64_t* env_off;
  int32_t n;
  int32_t pad;
};
struct SampleTask {
  const void* sites;
  const int64_t* site_off;
  const int* bond;
  const void* env;
  const int64_t* env_off;
  uint8_t* bits;
  uint64_t seed;
  int32_t n;
  int32_t shots;
};

// Tuning constants of the single-CTA kernels.
constexpr int kChiLimit = 64;          // largest bond the fused gate kernel holds
constexpr int kMaxM = 2 * kChiLimit;   // largest Gram / theta side
constexpr int kOpThreads = 512;

}  // namespace gbmps
