// Measurement kernels of the GB300 MPS engine (sm_103a).
//
//  k_expect     transfer-matrix sweep for Pauli strings, one CTA per
//               (program, term): E <- A^H (E . P A) site by site
//               (ITensorMPSVisitor.cpp:173-250 for Z products; any Pauli here).
//  k_right_env  right environments R_i = sum_s A_i^s R_{i+1} A_i^s^H used by
//               the sampler (replaces the ket x bra contractions of
//               getMeasureSample, ExaTnMpsVisitor.cpp:2211-2364).
//  k_sample     one warp per shot, sequential conditional sampling left to
//               right with a Philox4x32-10 counter-based generator (Salmon et
//               al., SC'11); bit i is 0 when u <= p0 (ExaTnMpsVisitor.cpp:2342-2345).
//  k_amp_step   state-vector contraction, one site per launch, qubit k on
//               bit k of the index (ExaTnMpsVisitor.cpp:591-597,616-634).
//  k_amp_one    amplitude of one bit string (computeWaveFuncSlice :2588-2675
//               with every index closed).
#include "expect_sweep.cuh"
#include "mps_common.cuh"
#include "philox.cuh"

namespace gbmps {


// One CTA per (program, Pauli term): the sweep of expect_sweep.cuh.
template <typename T>
__global__ void __launch_bounds__(256) k_expect(const ExpTask* __restrict__ tasks, int n_tasks, char* scratch,
                                                size_t stride, double* out) {
  using L = ExpLayout<T>;
  extern __shared__ __align__(16) char smem[];
  cx<T>* E = reinterpret_cast<cx<T>*>(smem);  // ld kChiLimit
  cx<T>* As = L::staged ? E + L::e_elems : nullptr;  // staged A (FP32)
  cx<T>* X = L::staged ? E + L::e_elems + L::a_elems : reinterpret_cast<cx<T>*>(scratch + stride * blockIdx.x);
  const int task = blockIdx.x;
  if (task >= n_tasks) return;
  expect_sweep<T>(tasks[task], E, As, X, out + 2 * task);
}

template <typename T>
__global__ void __launch_bounds__(256) k_right_env(EnvTask tk, char* scratch) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const cx<T>* sites = reinterpret_cast<const cx<T>*>(tk.sites);
  cx<T>* env = reinterpret_cast<cx<T>*>(tk.env);
  cx<T>* Y = reinterpret_cast<cx<T>*>(scratch);
  if (tid == 0) env[tk.env_off[tk.n]] = mk<T>(1, 0);
  __syncthreads();
  for (int i = tk.n - 1; i >= 1; --i) {
    const int dl = tk.bond[i], dr = tk.bond[i + 1];
    const cx<T>* A = sites + tk.site_off[i];
    const cx<T>* Rn = env + tk.env_off[i + 1];
    cx<T>* Ri = env + tk.env_off[i];
    // Y[(l,s)][r'] = sum_r A[(l,s)][r] Rn[r][r']
    for (int t = tid; t < 2 * dl * dr; t += nt) {
      const int x = t / dr, rp = t - x * dr;
      cx<T> acc = mk<T>(0, 0);
      for (int r = 0; r < dr; ++r) fma_c(acc, A[x * dr + r], Rn[r * dr + rp]);
      Y[t] = acc;
    }
    __syncthreads();
    // Ri[l][l'] = sum_{s,r'} Y[(l,s)][r'] conj(A[(l',s)][r'])
    for (int t = tid; t < dl * dl; t += nt) {
      const int l = t / dl, lp = t - l * dl;
      cx<T> acc = mk<T>(0, 0);
      for (int s = 0; s < 2; ++s)
        for (int r = 0; r < dr; ++r) fma_cj(acc, A[(lp * 2 + s) * dr + r], Y[(l * 2 + s) * dr + r]);
      Ri[t] = acc;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ double uniform01(uint64_t seed, uint32_t shot, uint32_t site) {
  return philox_uniform(seed, shot, site, 0x4d505321u);
}


constexpr int kSampleWarps = 8;

template <typename T>
__global__ void __launch_bounds__(kSampleWarps * 32) k_sample(SampleTask tk) {
  __shared__ cx<T> sL[kSampleWarps][kChiLimit];
  __shared__ cx<T> sV[kSampleWarps][2][kChiLimit];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int shot = blockIdx.x * kSampleWarps + warp;
  if (shot >= tk.shots) return;
  const cx<T>* sites = reinterpret_cast<const cx<T>*>(tk.sites);
  const cx<T>* env = reinterpret_cast<const cx<T>*>(tk.env);
  cx<T>* L = sL[warp];
  if (lane == 0) L[0] = mk<T>(1, 0);
  __syncwarp();
  for (int i = 0; i < tk.n; ++i) {
    const int dl = tk.bond[i], dr = tk.bond[i + 1];
    const cx<T>* A = sites + tk.site_off[i];
    const cx<T>* Rn = env + tk.env_off[i + 1];
    for (int s = 0; s < 2; ++s)
      for (int r = lane; r < dr; r += 32) {
        cx<T> acc = mk<T>(0, 0);
        for (int l = 0; l < dl; ++l) fma_c(acc, L[l], A[(l * 2 + s) * dr + r]);
        sV[warp][s][r] = acc;
      }
    __syncwarp();
    double p[2];
    for (int s = 0; s < 2; ++s) {
      double part = 0.0;
      for (int r = lane; r < dr; r += 32) {
        cx<T> w = mk<T>(0, 0);
        for (int rp = 0; rp < dr; ++rp) fma_c(w, Rn[r * dr + rp], conj(sV[warp][s][rp]));
        const cx<T> v = sV[warp][s][r];
        part += (double)(v.re * w.re - v.im * w.im);
      }
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      p[s] = part > 0.0 ? part : 0.0;
    }
    const double tot = p[0] + p[1];
    const double p0 = tot > 0.0 ? p[0] / tot : 0.5;
    const double u = uniform01(tk.seed, (uint32_t)shot, (uint32_t)i);
    const int bit = (u <= p0) ? 0 : 1;
    const double nrm = p[bit] > 0.0 ? 1.0 / sqrt(p[bit]) : 0.0;
    for (int r = lane; r < dr; r += 32) L[r] = scl(sV[warp][bit][r], T(nrm));
    if (lane == 0) tk.bits[(size_t)shot * tk.n + i] = (uint8_t)bit;
    __syncwarp();
  }
}

template <typename T>
__global__ void k_amp_step(const cx<T>* __restrict__ A, int dl, int dr, int k, const cx<T>* __restrict__ vin,
                           cx<T>* __restrict__ vout) {
  // vout[r][c + s 2^k] = sum_l A[l][s][r] vin[l][c]   (vin: dl x 2^k, vout: dr x 2^(k+1))
  const int64_t w = (int64_t)1 << k;
  const int64_t total = (int64_t)dr * 2 * w;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / (2 * w));
    const int64_t col = t - (int64_t)r * 2 * w;
    const int s = (int)(col / w);
    const int64_t c = col - (int64_t)s * w;
    cx<T> acc = mk<T>(0, 0);
    for (int l = 0; l < dl; ++l) fma_c(acc, A[(l * 2 + s) * dr + r], vin[(int64_t)l * w + c]);
    vout[t] = acc;
  }
}

template <typename T>
__global__ void k_to_f64(const cx<T>* __restrict__ v, double* __restrict__ out, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    out[2 * t] = (double)v[t].re;
    out[2 * t + 1] = (double)v[t].im;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_amp_one(const void* sites_v, const int64_t* site_off, const int* bond,
                                                 const int* bits, int n, double* out) {
  __shared__ cx<T> v[2][kChiLimit];
  const cx<T>* sites = reinterpret_cast<const cx<T>*>(sites_v);
  const int tid = threadIdx.x;
  if (tid == 0) v[0][0] = mk<T>(1, 0);
  __syncthreads();
  int cur = 0;
  for (int i = 0; i < n; ++i) {
    const int dl = bond[i], dr = bond[i + 1], s = bits[i];
    const cx<T>* A = sites + site_off[i];
    for (int r = tid; r < dr; r += blockDim.x) {
      cx<T> acc = mk<T>(0, 0);
      for (int l = 0; l < dl; ++l) fma_c(acc, v[cur][l], A[(l * 2 + s) * dr + r]);
      v[1 - cur][r] = acc;
    }
    __syncthreads();
    cur = 1 - cur;
  }
  if (tid == 0) {
    out[0] = (double)v[cur][0].re;
    out[1] = (double)v[cur][0].im;
  }
}

// ------------------------------------------------------------- launchers
size_t expect_smem_bytes(int prec) { return prec == 0 ? ExpLayout<double>::smem : ExpLayout<float>::smem; }
size_t expect_scratch_bytes(int prec) { return prec == 0 ? ExpLayout<double>::scratch : ExpLayout<float>::scratch; }

template <typename T>
static cudaError_t launch_expect_t(const ExpTask* d_tasks, int n_tasks, char* scratch, double* d_out,
                                   cudaStream_t st) {
  const int prec = sizeof(T) == 8 ? 0 : 1;
  k_expect<T><<<n_tasks, 256, expect_smem_bytes(prec), st>>>(d_tasks, n_tasks, scratch, expect_scratch_bytes(prec),
                                                             d_out);
  return cudaGetLastError();
}

cudaError_t configure_expect() {
  cudaError_t e = cudaFuncSetAttribute(k_expect<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)expect_smem_bytes(1));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_expect<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)expect_smem_bytes(0));
}

cudaError_t launch_expect(int prec, const ExpTask* d_tasks, int n_tasks, char* scratch, double* d_out,
                          cudaStream_t st) {
  if (n_tasks <= 0) return cudaSuccess;
  return prec == 0 ? launch_expect_t<double>(d_tasks, n_tasks, scratch, d_out, st)
                   : launch_expect_t<float>(d_tasks, n_tasks, scratch, d_out, st);
}

cudaError_t launch_right_env(int prec, const EnvTask& tk, char* scratch, cudaStream_t st) {
  if (prec == 0)
    k_right_env<double><<<1, 256, 0, st>>>(tk, scratch);
  else
    k_right_env<float><<<1, 256, 0, st>>>(tk, scratch);
  return cudaGetLastError();
}

cudaError_t launch_sample(int prec, const SampleTask& tk, cudaStream_t st) {
  const int grid = (tk.shots + kSampleWarps - 1) / kSampleWarps;
  if (grid <= 0) return cudaSuccess;
  if (prec == 0)
    k_sample<double><<<grid, kSampleWarps * 32, 0, st>>>(tk);
  else
    k_sample<float><<<grid, kSampleWarps * 32, 0, st>>>(tk);
  return cudaGetLastError();
}

cudaError_t launch_amp_step(int prec, const void* A, int dl, int dr, int k, const void* vin, void* vout,
                            cudaStream_t st) {
  const int64_t total = (int64_t)dr * 2 * ((int64_t)1 << k);
  int grid = (int)((total + 255) / 256);
  if (grid > 65535) grid = 65535;
  if (prec == 0)
    k_amp_step<double><<<grid, 256, 0, st>>>((const cx<double>*)A, dl, dr, k, (const cx<double>*)vin,
                                             (cx<double>*)vout);
  else
    k_amp_step<float><<<grid, 256, 0, st>>>((const cx<float>*)A, dl, dr, k, (const cx<float>*)vin,
                                            (cx<float>*)vout);
  return cudaGetLastError();
}

cudaError_t launch_to_f64(int prec, const void* v, double* out, int64_t n, cudaStream_t st) {
  int grid = (int)((n + 255) / 256);
  if (grid > 65535) grid = 65535;
  if (grid < 1) grid = 1;
  if (prec == 0)
    k_to_f64<double><<<grid, 256, 0, st>>>((const cx<double>*)v, out, n);
  else
    k_to_f64<float><<<grid, 256, 0, st>>>((const cx<float>*)v, out, n);
  return cudaGetLastError();
}

cudaError_t launch_amp_one(int prec, const void* sites, const int64_t* site_off, const int* bond, const int* bits,
                           int n, double* out, cudaStream_t st) {
  if (prec == 0)
    k_amp_one<double><<<1, 256, 0, st>>>(sites, site_off, bond, bits, n, out);
  else
    k_amp_one<float><<<1, 256, 0, st>>>(sites, site_off, bond, bits, n, out);
  return cudaGetLastError();
}

}  // namespace gbmps

namespace gbmps {
// Reset programs to |0...0> on the device: bonds 1, each site [1, 0], stats
// 0; each program in its own precision.
template <typename T>
__device__ void reset_sites(const ProgDesc& P) {
  cx<T>* sites = reinterpret_cast<cx<T>*>(P.sites);
  for (int i = threadIdx.x; i < P.n; i += blockDim.x) {
    sites[P.site_off[i]] = mk<T>(1, 0);
    sites[P.site_off[i] + 1] = mk<T>(0, 0);
  }
}

__global__ void k_reset(const ProgDesc* __restrict__ progs, int n_progs) {
  const int pi = blockIdx.x;
  if (pi >= n_progs) return;
  const ProgDesc P = progs[pi];
  if (P.prec == 0)
    reset_sites<double>(P);
  else
    reset_sites<float>(P);
  for (int i = threadIdx.x; i <= P.n; i += blockDim.x) P.bond[i] = 1;
  if (threadIdx.x < ST_COUNT) P.stats[threadIdx.x] = 0.0;
  if (threadIdx.x == 0) *P.err = 0;
}

cudaError_t launch_reset(const ProgDesc* d_progs, int n_progs, cudaStream_t st) {
  if (n_progs <= 0) return cudaSuccess;
  k_reset<<<n_progs, 64, 0, st>>>(d_progs, n_progs);
  return cudaGetLastError();
}
}  // namespace gbmps

// ------------------------------------------------ CUDA-core FMA rate probe
// Peak fused multiply-add rate of the CUDA cores in one precision: every
// thread runs eight independent chains a <- a * b + c (b slightly below 1,
// so each chain settles at c / (1 - b) with no overflow), the grid fills
// every SM eight CTAs deep.  The denominator of the roofline of kernels that
// run on FP32/FP64 CUDA cores, measured on the GPU at hand.
namespace gbmps {
template <typename T>
__global__ void __launch_bounds__(256) k_fma_rate(T* out, int iters, T b, T c) {
  T a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = T(threadIdx.x + i);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = fma(a[i], b, c);
  }
  T s = T(0);
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  if (s == T(-1)) out[blockIdx.x] = s;  // never true; keeps the chains live
}
}  // namespace gbmps

#include <string>

#include "../../include/gb300mps.h"

namespace gbmps {
int fail(int code, const std::string& msg);
}

extern "C" int mps_diag_fma_rate(int device, int precision, double* flops_per_s) {
  using namespace gbmps;
  if (!flops_per_s) return fail(MPS_ERR_ARG, "NULL argument");
  if (precision != MPS_PREC_FP64 && precision != MPS_PREC_FP32) return fail(MPS_ERR_ARG, "bad precision");
  int prev = 0;
  cudaError_t e = cudaGetDevice(&prev);
  if (e == cudaSuccess) e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = 8 * (sms > 0 ? sms : 1), threads = 256;
  const int iters = precision == MPS_PREC_FP32 ? 1 << 16 : 1 << 11;
  void* out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float best = 0.0f;
  e = cudaMalloc(&out, sizeof(double) * blocks);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // first launch is a warm-up
    cudaEventRecord(e0, st);
    if (precision == MPS_PREC_FP32)
      k_fma_rate<float><<<blocks, threads, 0, st>>>(static_cast<float*>(out), iters, 0.999999f, 1e-6f);
    else
      k_fma_rate<double><<<blocks, threads, 0, st>>>(static_cast<double*>(out), iters, 0.999999, 1e-6);
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && rep > 0 && (best == 0.0f || ms < best)) best = ms;
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e1) cudaEventDestroy(e1);
  if (e0) cudaEventDestroy(e0);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  cudaSetDevice(prev);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  *flops_per_s = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3);
  return MPS_OK;
}
