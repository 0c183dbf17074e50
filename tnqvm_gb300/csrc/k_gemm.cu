// Complex GEMMs of the wide two-site path (sm_103a).
//
// complex64: tcgen05 tensor cores in kind::tf32 with FP32 accumulation in
// tensor memory.  A complex product is one real GEMM on a real embedding:
// A (M x K complex, interleaved) is the real M x 2K matrix as it lies in
// memory, and B enters K-major as the 2N x 2K real matrix whose rows 2n and
// 2n+1 hold (Re b, -Im b) and (Im b, Re b) of column n, so the real product
// is C (M x 2N real) = C (M x N complex, interleaved) with 8 real flops per
// complex MAC, as a complex GEMM.  Each operand is split into a TF32 head
// and a TF32 remainder (both rounded to nearest) and three products
// hi*hi + hi*lo + lo*hi recover ~FP32 accuracy (3xTF32).
//
// Operands reach shared memory by TMA (cp.async.bulk.tensor, 128-byte
// swizzle) through a 3-stage mbarrier pipeline; one thread issues the MMAs;
// four warps drain the accumulators from tensor memory.  Each MMA adds its
// products to the accumulator with a rounding step relative to the
// accumulator's magnitude, so one shared accumulator loses accuracy linearly
// in K.  The cross terms hi*lo + lo*hi therefore go to their own accumulator
// (errors relative to their ~2^-11 smaller size) and the main hi*hi term
// rotates over three accumulators by K step; the epilogue sums the four in
// FP32 registers (4 x 128 columns = all 512 columns of tensor memory).
// complex128 runs on a CUDA-core tiled kernel (FP64 has no fast tensor path
// on this part).
//
// Split-BF16 (a program precision mode): the same pipeline on tcgen05
// kind::f16 with bf16 operands, each split into a bf16 head and a bf16
// remainder (~16 significant bits together) and the three products hi*hi +
// hi*lo + lo*hi with FP32 accumulation: about twice the tensor rate of TF32
// at ~1e-5 relative error per product instead of ~1e-6.  A 128-byte operand
// row holds 32 fp32 or 64 bf16 values, so the tiles, swizzle and K steps (32
// bytes, K = 8 tf32 or 16 bf16 per MMA) are the same in bytes.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>

#include "wide.hpp"

namespace gbmps {

// ------------------------------------------------------------ CUDA cores
// Output tiles of BM x BN complex entries per 256-thread CTA (16 x 16
// threads, each holding (BM/16) x (BN/16) accumulators).  Every output sums
// its K terms in the same order whatever the tile, so the tile shapes give
// bit-identical results; the autotuner below picks among them by speed.
constexpr int kSK = 16;

template <typename T>
__device__ __forceinline__ cx<T> vload(const CMat<T>& v, int i, int j) {
  if (i >= v.rows || j >= v.cols) return mk<T>(T(0), T(0));
  cx<T> z = v.p[(int64_t)i * v.rs + (int64_t)j * v.cs];
  if (v.conj) z.im = -z.im;
  return z;
}

template <typename T, int BM, int BN>
__global__ void __launch_bounds__(256) k_cgemm_simt(CMat<T> A, CMat<T> B, CMatOut<T> C, T alpha, T beta) {
  constexpr int RM = BM / 16, RN = BN / 16;
  __shared__ cx<T> As[kSK][BM + 1];
  __shared__ cx<T> Bs[kSK][BN + 1];
  const int i0 = blockIdx.y * BM, j0 = blockIdx.x * BN;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int K = A.cols;
  cx<T> acc[RM][RN];
#pragma unroll
  for (int a = 0; a < RM; ++a)
#pragma unroll
    for (int b = 0; b < RN; ++b) acc[a][b] = mk<T>(T(0), T(0));
  // lanes walk the unit-stride index of each view (coalesced loads)
  const bool a_rows_fast = A.rs == 1 && A.cs != 1;
  const bool b_cols_fast = !(B.rs == 1 && B.cs != 1);
  for (int k0 = 0; k0 < K; k0 += kSK) {
    for (int t = threadIdx.x; t < BM * kSK; t += 256) {
      int ii, kk;
      if (a_rows_fast) {
        ii = t % BM;
        kk = t / BM;
      } else {
        kk = t % kSK;
        ii = t / kSK;
      }
      As[kk][ii] = vload(A, i0 + ii, k0 + kk);
    }
    for (int t = threadIdx.x; t < BN * kSK; t += 256) {
      int jj, k2;
      if (b_cols_fast) {
        jj = t % BN;
        k2 = t / BN;
      } else {
        k2 = t % kSK;
        jj = t / kSK;
      }
      Bs[k2][jj] = vload(B, k0 + k2, j0 + jj);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kSK; ++kk) {
      cx<T> a[RM], b[RN];
#pragma unroll
      for (int r = 0; r < RM; ++r) a[r] = As[kk][ty + 16 * r];
#pragma unroll
      for (int c = 0; c < RN; ++c) b[c] = Bs[kk][tx + 16 * c];
#pragma unroll
      for (int r = 0; r < RM; ++r)
#pragma unroll
        for (int c = 0; c < RN; ++c) fma_c(acc[r][c], a[r], b[c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < RM; ++r) {
    const int i = i0 + ty + 16 * r;
    if (i >= C.rows) continue;
#pragma unroll
    for (int c = 0; c < RN; ++c) {
      const int j = j0 + tx + 16 * c;
      if (j >= C.cols) continue;
      cx<T>* dst = C.p + (int64_t)i * C.rs + (int64_t)j * C.cs;
      cx<T> v = scl(acc[r][c], alpha);
      if (beta != T(0)) v = v + scl(*dst, beta);
      *dst = v;
    }
  }
}

template <typename T, int BM, int BN>
static cudaError_t simt_tile(const CMat<T>& A, const CMat<T>& B, const CMatOut<T>& C, T alpha, T beta,
                             cudaStream_t st) {
  dim3 grid((C.cols + BN - 1) / BN, (C.rows + BM - 1) / BM);
  k_cgemm_simt<T, BM, BN><<<grid, 256, 0, st>>>(A, B, C, alpha, beta);
  return cudaGetLastError();
}

template <typename T>
static cudaError_t simt_launch(const CMat<T>& A, const CMat<T>& B, const CMatOut<T>& C, T alpha, T beta,
                               cudaStream_t st, int kind = GEMM_SIMT_64x64) {
  if (C.rows <= 0 || C.cols <= 0) return cudaSuccess;
  switch (kind) {
    case GEMM_SIMT_32x32:
      return simt_tile<T, 32, 32>(A, B, C, alpha, beta, st);
    case GEMM_SIMT_16x64:
      return simt_tile<T, 16, 64>(A, B, C, alpha, beta, st);
    case GEMM_SIMT_64x16:
      return simt_tile<T, 64, 16>(A, B, C, alpha, beta, st);
    default:
      return simt_tile<T, 64, 64>(A, B, C, alpha, beta, st);
  }
}

// ------------------------------------------------------------ tcgen05 path
namespace tc {
constexpr int BM = 128;                  // rows per CTA (TMEM lanes)
constexpr int BN = 128;                  // real output columns per CTA (64 complex)
constexpr int BK = 32;                   // fp32 K elements per stage (128 B rows)
constexpr int STAGES = 3;
constexpr int TILE = BM * BK * 4;        // 16 KB per operand tile (BN == BM)
constexpr int STAGE = 4 * TILE;          // A_hi, A_lo, B_hi, B_lo
constexpr int SMEM = STAGES * STAGE + 1024 + 256;
constexpr int NBIG = 3;                  // accumulators of the hi*hi term
constexpr int TMEM_COLS = BN * (NBIG + 1);  // 512
constexpr int KP_ALIGN = 64;             // padded K (fp32) multiple of 64 (32 complex)
// instruction descriptor, kind::tf32: D f32 (bits 4-5 = 1), A/B tf32 (bits
// 7-9, 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);
// kind::f16 with bf16 A and B (bits 7-9, 10-12 = 1), D f32, both K-major
constexpr uint32_t IDESC_BF16 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                                ((uint32_t)(BM >> 4) << 24);
constexpr int BK_BF16 = 64;              // bf16 K elements per stage (the same 128 B rows)
constexpr long long kWaitNs = 2000000000LL;  // 2 s bound on every wait
}  // namespace tc

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ long long gtimer() {
  long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
               : "memory");
}
// Bounded wait for the phase of the given parity; false on time-out.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
  const uint32_t a = smem_u32(b);
  const long long t0 = gtimer();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (gtimer() - t0 > tc::kWaitNs) return false;
  }
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 B apart (SBO), version 1 (bits 46-47), layout SWIZZLE_128B (2 << 61).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
__device__ __forceinline__ void umma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(tc::IDESC), "r"(accum));
}
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(tc::IDESC_BF16), "r"(accum));
}
template <bool BF16>
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accum) {
  if (BF16)
    umma_bf16(tmem_d, adesc, bdesc, accum);
  else
    umma_tf32(tmem_d, adesc, bdesc, accum);
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// One 128 x 128 (real) output tile per CTA; 128 threads.  BF16: operands
// are bf16 (64 per 128-byte row) and the MMAs kind::f16.
template <bool BF16>
__global__ void __launch_bounds__(128, 1)
    k_cgemm_tc(const __grid_constant__ CUtensorMap tm_ahi, const __grid_constant__ CUtensorMap tm_alo,
               const __grid_constant__ CUtensorMap tm_bhi, const __grid_constant__ CUtensorMap tm_blo, int k_tiles,
               CMatOut<float> C, float alpha, float beta, int* err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + tc::STAGES * tc::STAGE);
  uint64_t* empty = full + tc::STAGES;
  uint64_t* done = empty + tc::STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  int* flag = reinterpret_cast<int*>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < tc::STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(tc::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const int m0 = blockIdx.y * tc::BM, n0 = blockIdx.x * tc::BN;

  if (warp == 0 && lane == 0) {
    // producer: TMA loads of the four operand tiles of each K step
    for (int kt = 0; kt < k_tiles; ++kt) {
      const int s = kt % tc::STAGES;
      const uint32_t ph = (uint32_t)(kt / tc::STAGES) & 1u;
      if (kt >= tc::STAGES && !mbar_wait(&empty[s], ph ^ 1u)) {
        atomicOr(flag, 1);
        break;
      }
      if (*((volatile int*)flag)) break;
      uint8_t* st = smem + s * tc::STAGE;
      mbar_expect_tx(&full[s], tc::STAGE);
      // x = the stage's first K element: 32 fp32 or 64 bf16 = 128 bytes per stage
      const int kx = kt * (BF16 ? tc::BK_BF16 : tc::BK);
      tma_load_2d(st + 0 * tc::TILE, &tm_ahi, kx, m0, &full[s]);
      tma_load_2d(st + 1 * tc::TILE, &tm_alo, kx, m0, &full[s]);
      tma_load_2d(st + 2 * tc::TILE, &tm_bhi, kx, n0, &full[s]);
      tma_load_2d(st + 3 * tc::TILE, &tm_blo, kx, n0, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: 4 K-steps of 32 bytes per stage (K = 8 tf32 or 16 bf16),
    // three products each
    for (int kt = 0; kt < k_tiles; ++kt) {
      const int s = kt % tc::STAGES;
      const uint32_t ph = (uint32_t)(kt / tc::STAGES) & 1u;
      if (!mbar_wait(&full[s], ph)) {
        atomicOr(flag, 1);
        break;
      }
      tc_fence_after();
      const uint32_t base = smem_u32(smem + s * tc::STAGE);
      const int b = kt % tc::NBIG;
      const uint32_t t_big = tmem + (uint32_t)(tc::BN * (1 + b)), t_small = tmem;
#pragma unroll
      for (int k = 0; k < tc::BK / 8; ++k) {
        const uint32_t ko = (uint32_t)k * 32u;
        const uint64_t ahi = sw128_desc(base + 0 * tc::TILE + ko), alo = sw128_desc(base + 1 * tc::TILE + ko);
        const uint64_t bhi = sw128_desc(base + 2 * tc::TILE + ko), blo = sw128_desc(base + 3 * tc::TILE + ko);
        umma<BF16>(t_big, ahi, bhi, (kt >= tc::NBIG || k > 0) ? 1u : 0u);
        umma<BF16>(t_small, ahi, blo, (kt > 0 || k > 0) ? 1u : 0u);
        umma<BF16>(t_small, alo, bhi, 1u);
      }
      umma_commit(&empty[s]);
    }
    umma_commit(done);
  }
  __syncwarp();
  // epilogue: warp w drains TMEM lanes 32w..32w+31 (rows of the tile)
  const bool ok = mbar_wait(done, 0);
  tc_fence_after();
  if (!ok) atomicOr(flag, 1);
  const int row = m0 + warp * 32 + lane;
  if (ok && k_tiles > 0) {
    const int nbig = k_tiles < tc::NBIG ? k_tiles : tc::NBIG;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int c = 0; c < tc::BN; c += 16) {
      float acc[16];
      uint32_t r[16];
      tmem_ld16(lane_base + (uint32_t)(tc::BN + c), r);
#pragma unroll
      for (int q = 0; q < 16; ++q) acc[q] = __uint_as_float(r[q]);
      for (int b = 1; b < nbig; ++b) {
        tmem_ld16(lane_base + (uint32_t)(tc::BN * (1 + b) + c), r);
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] += __uint_as_float(r[q]);
      }
      tmem_ld16(lane_base + (uint32_t)c, r);
#pragma unroll
      for (int q = 0; q < 16; ++q) acc[q] += __uint_as_float(r[q]);
      if (row < C.rows) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int j = (n0 + c) / 2 + q;
          if (j < C.cols) {
            cx<float>* dst = C.p + (int64_t)row * C.rs + (int64_t)j * C.cs;
            cx<float> v = mk<float>(alpha * acc[2 * q], alpha * acc[2 * q + 1]);
            if (beta != 0.0f) v = v + scl(*dst, beta);
            *dst = v;
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tc::TMEM_COLS));
  if (threadIdx.x == 0 && *flag && err) atomicOr(err, 1);
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// Pack a view into the split real-embedded operand of the tensor-core GEMM.
// Operand coordinates (r, k): A side r = view row, k = view column; B side
// r = view column, k = view row.  A side writes row r: (Re, Im) at 2k, 2k+1;
// B side writes rows 2r (Re, -Im) and 2r+1 (Im, Re).  32 x 32 complex tiles
// through shared memory so both the read and the write are coalesced.
template <bool BSIDE>
__global__ void __launch_bounds__(256) k_pack(CMat<float> V, float* hi, float* lo, int kp) {
  __shared__ cx<float> t[32][33];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  // lanes walk r when r is the view's unit-stride index
  const bool lanes_r = BSIDE ? (V.cs == 1) : (V.rs == 1 && V.cs != 1);
  for (int q = ty; q < 32; q += 8) {
    const int rr = lanes_r ? tx : q, kk = lanes_r ? q : tx;
    const int r = r0 + rr, k = k0 + kk;
    t[rr][kk] = BSIDE ? vload(V, k, r) : vload(V, r, k);
  }
  __syncthreads();
  for (int q = ty; q < 32; q += 8) {
    const int r = r0 + q, k = k0 + tx;
    const cx<float> z = t[q][tx];
    const float hr = tf32_rna(z.re), hm = tf32_rna(z.im);
    const float lr = tf32_rna(z.re - hr), lm = tf32_rna(z.im - hm);
    if (!BSIDE) {
      const int64_t o = (int64_t)r * kp + 2 * k;
      *reinterpret_cast<float2*>(hi + o) = make_float2(hr, hm);
      *reinterpret_cast<float2*>(lo + o) = make_float2(lr, lm);
    } else {
      const int64_t o0 = (int64_t)(2 * r) * kp + 2 * k, o1 = o0 + kp;
      *reinterpret_cast<float2*>(hi + o0) = make_float2(hr, -hm);
      *reinterpret_cast<float2*>(lo + o0) = make_float2(lr, -lm);
      *reinterpret_cast<float2*>(hi + o1) = make_float2(hm, hr);
      *reinterpret_cast<float2*>(lo + o1) = make_float2(lm, lr);
    }
  }
}

// The same packing into bf16 head and remainder: hi = bf16(x), lo =
// bf16(x - hi), each rounded to nearest.
template <bool BSIDE>
__global__ void __launch_bounds__(256) k_pack_bf16(CMat<float> V, __nv_bfloat16* hi, __nv_bfloat16* lo, int kp) {
  __shared__ cx<float> t[32][33];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const bool lanes_r = BSIDE ? (V.cs == 1) : (V.rs == 1 && V.cs != 1);
  for (int q = ty; q < 32; q += 8) {
    const int rr = lanes_r ? tx : q, kk = lanes_r ? q : tx;
    const int r = r0 + rr, k = k0 + kk;
    t[rr][kk] = BSIDE ? vload(V, k, r) : vload(V, r, k);
  }
  __syncthreads();
  for (int q = ty; q < 32; q += 8) {
    const int r = r0 + q, k = k0 + tx;
    const cx<float> z = t[q][tx];
    const __nv_bfloat16 hr = __float2bfloat16_rn(z.re), hm = __float2bfloat16_rn(z.im);
    const __nv_bfloat16 lr = __float2bfloat16_rn(z.re - __bfloat162float(hr));
    const __nv_bfloat16 lm = __float2bfloat16_rn(z.im - __bfloat162float(hm));
    const __nv_bfloat16 nhm = __float2bfloat16_rn(-__bfloat162float(hm));
    const __nv_bfloat16 nlm = __float2bfloat16_rn(-__bfloat162float(lm));
    if (!BSIDE) {
      const int64_t o = (int64_t)r * kp + 2 * k;
      *reinterpret_cast<__nv_bfloat162*>(hi + o) = __halves2bfloat162(hr, hm);
      *reinterpret_cast<__nv_bfloat162*>(lo + o) = __halves2bfloat162(lr, lm);
    } else {
      const int64_t o0 = (int64_t)(2 * r) * kp + 2 * k, o1 = o0 + kp;
      *reinterpret_cast<__nv_bfloat162*>(hi + o0) = __halves2bfloat162(hr, nhm);
      *reinterpret_cast<__nv_bfloat162*>(lo + o0) = __halves2bfloat162(lr, nlm);
      *reinterpret_cast<__nv_bfloat162*>(hi + o1) = __halves2bfloat162(hm, hr);
      *reinterpret_cast<__nv_bfloat162*>(lo + o1) = __halves2bfloat162(lm, lr);
    }
  }
}

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;
static cudaError_t g_attr_err = cudaSuccess;

static bool get_encode() {
  std::call_once(g_encode_once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    g_attr_err = cudaFuncSetAttribute(k_cgemm_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM);
    if (g_attr_err == cudaSuccess)
      g_attr_err = cudaFuncSetAttribute(k_cgemm_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM);
  });
  return g_encode != nullptr && g_attr_err == cudaSuccess;
}

// rows x kp fp32 row-major, box 32 (K) x 128 (rows), 128-byte swizzle
static bool make_map(CUtensorMap* m, float* base, int rows, int kp) {
  const cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kp * 4};
  const cuuint32_t box[2] = {(cuuint32_t)tc::BK, (cuuint32_t)tc::BM};
  const cuuint32_t es[2] = {1, 1};
  return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// rows x kp bf16 row-major, box 64 (K) x 128 (rows): the same 128-byte rows
static bool make_map_bf16(CUtensorMap* m, void* base, int rows, int kp) {
  const cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
  const cuuint32_t box[2] = {(cuuint32_t)tc::BK_BF16, (cuuint32_t)tc::BM};
  const cuuint32_t es[2] = {1, 1};
  return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int gemm_ws_init(GemmWs& ws, size_t a_elems, size_t b_elems) {
  if (ws.a_elems >= a_elems && ws.b_elems >= b_elems && ws.d_err) return 0;
  gemm_ws_free(ws);
  if (cudaMalloc(&ws.a_hi, a_elems * 4) != cudaSuccess || cudaMalloc(&ws.a_lo, a_elems * 4) != cudaSuccess ||
      cudaMalloc(&ws.b_hi, b_elems * 4) != cudaSuccess || cudaMalloc(&ws.b_lo, b_elems * 4) != cudaSuccess ||
      cudaMalloc(&ws.d_err, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    gemm_ws_free(ws);
    return 1;
  }
  cudaMemset(ws.d_err, 0, sizeof(int));
  ws.a_elems = a_elems;
  ws.b_elems = b_elems;
  return 0;
}

void gemm_ws_free(GemmWs& ws) {
  if (ws.a_hi) cudaFree(ws.a_hi);
  if (ws.a_lo) cudaFree(ws.a_lo);
  if (ws.b_hi) cudaFree(ws.b_hi);
  if (ws.b_lo) cudaFree(ws.b_lo);
  if (ws.d_err) cudaFree(ws.d_err);
  if (ws.tune_c) cudaFree(ws.tune_c);
  for (cudaEvent_t e : ws.tune_ev)
    if (e) cudaEventDestroy(e);
  ws = GemmWs();
}

// The tensor-core kernel takes products with N, K >= 16 whose padded
// operands fit the workspace.
static bool tc_eligible(int M, int N, int K, const GemmWs& ws) {
  if (N < 16 || K < 16 || !get_encode()) return false;
  const size_t mp = (size_t)(M + tc::BM - 1) / tc::BM * tc::BM;
  const size_t np = (size_t)(2 * N + tc::BN - 1) / tc::BN * tc::BN;
  const size_t kp = (size_t)(2 * K + tc::KP_ALIGN - 1) / tc::KP_ALIGN * tc::KP_ALIGN;
  return mp * kp <= ws.a_elems && np * kp <= ws.b_elems;
}

static cudaError_t tc_launch(const CMat<float>& A, const CMat<float>& B, const CMatOut<float>& C, float alpha,
                             float beta, GemmWs& ws, cudaStream_t st) {
  const int M = C.rows, N = C.cols, K = A.cols;
  const int mp = (M + tc::BM - 1) / tc::BM * tc::BM;
  const int np = (2 * N + tc::BN - 1) / tc::BN * tc::BN;
  const int kp = (2 * K + tc::KP_ALIGN - 1) / tc::KP_ALIGN * tc::KP_ALIGN;
  CUtensorMap ma, mal, mb, mbl;
  if (ws.split_bf16) {
    // bf16 operands in the same buffers (half the bytes)
    auto* ahi = reinterpret_cast<__nv_bfloat16*>(ws.a_hi);
    auto* alo = reinterpret_cast<__nv_bfloat16*>(ws.a_lo);
    auto* bhi = reinterpret_cast<__nv_bfloat16*>(ws.b_hi);
    auto* blo = reinterpret_cast<__nv_bfloat16*>(ws.b_lo);
    k_pack_bf16<false><<<dim3(kp / 64, mp / 32), 256, 0, st>>>(A, ahi, alo, kp);
    k_pack_bf16<true><<<dim3(kp / 64, np / 64), 256, 0, st>>>(B, bhi, blo, kp);
    if (!make_map_bf16(&ma, ahi, mp, kp) || !make_map_bf16(&mal, alo, mp, kp) || !make_map_bf16(&mb, bhi, np, kp) ||
        !make_map_bf16(&mbl, blo, np, kp))
      return cudaErrorInvalidValue;
    k_cgemm_tc<true><<<dim3(np / tc::BN, mp / tc::BM), 128, tc::SMEM, st>>>(ma, mal, mb, mbl, kp / tc::BK_BF16, C,
                                                                           alpha, beta, ws.d_err);
    return cudaGetLastError();
  }
  k_pack<false><<<dim3(kp / 64, mp / 32), 256, 0, st>>>(A, ws.a_hi, ws.a_lo, kp);
  k_pack<true><<<dim3(kp / 64, np / 64), 256, 0, st>>>(B, ws.b_hi, ws.b_lo, kp);
  if (!make_map(&ma, ws.a_hi, mp, kp) || !make_map(&mal, ws.a_lo, mp, kp) || !make_map(&mb, ws.b_hi, np, kp) ||
      !make_map(&mbl, ws.b_lo, np, kp))
    return cudaErrorInvalidValue;
  k_cgemm_tc<false><<<dim3(np / tc::BN, mp / tc::BM), 128, tc::SMEM, st>>>(ma, mal, mb, mbl, kp / tc::BK, C, alpha,
                                                                           beta, ws.d_err);
  return cudaGetLastError();
}

cudaError_t cgemm_simt(const CMat<float>& A, const CMat<float>& B, const CMatOut<float>& C, float alpha, float beta,
                       cudaStream_t st) {
  return simt_launch<float>(A, B, C, alpha, beta, st);
}

cudaError_t cgemm_kind(int kind, const CMat<float>& A, const CMat<float>& B, const CMatOut<float>& C, float alpha,
                       float beta, GemmWs& ws, cudaStream_t st) {
  if (C.rows <= 0 || C.cols <= 0) return cudaSuccess;
  if (kind == GEMM_TC) {
    if (!tc_eligible(C.rows, C.cols, A.cols, ws)) return cudaErrorInvalidValue;
    return tc_launch(A, B, C, alpha, beta, ws, st);
  }
  if (kind < 0 || kind >= GEMM_TC) return cudaErrorInvalidValue;
  return simt_launch<float>(A, B, C, alpha, beta, st, kind);
}

cudaError_t cgemm_kind(int kind, const CMat<double>& A, const CMat<double>& B, const CMatOut<double>& C,
                       double alpha, double beta, GemmWs&, cudaStream_t st) {
  if (kind < 0 || kind >= GEMM_TC) return cudaErrorInvalidValue;
  return simt_launch<double>(A, B, C, alpha, beta, st, kind);
}

// ------------------------------------------------------------ autotuner
namespace {

struct TuneEntry {
  int kind;                   // chosen kernel
  float ns[GEMM_KINDS];       // measured time per launch (0: not eligible)
  int static_kind;            // kernel of the static rule for this bucket
};

std::mutex g_tune_mu;
std::map<uint32_t, TuneEntry> g_tune;
int g_tune_mode = -1;  // -1: not read from the environment yet (default 1, tune)

constexpr size_t kTuneMaxBytes = size_t(64) << 20;  // largest trial output (64 MiB)
constexpr int kTuneReps = 3;                         // timed launches per kernel after one warm-up
constexpr float kTuneMargin = 0.95f;                 // a kernel must beat the static rule by 5 %

int lg2(int x) {
  int l = 0;
  while ((1 << l) < x && l < 15) ++l;
  return l;
}

// Which index of each view is unit-stride: bit 0 A's rows, bit 1 B's
// columns, bit 2 C's rows.
template <typename T>
int layout_bits(const CMat<T>& A, const CMat<T>& B, const CMatOut<T>& C) {
  return (A.rs == 1 && A.cs != 1 ? 1 : 0) | (!(B.rs == 1 && B.cs != 1) ? 2 : 0) | (C.rs == 1 && C.cs != 1 ? 4 : 0);
}

uint32_t tune_key(int dev, int prec, int M, int N, int K, int layout) {
  return ((uint32_t)(dev & 63) << 20) | ((uint32_t)(prec & 1) << 19) | ((uint32_t)lg2(M) << 15) |
         ((uint32_t)lg2(N) << 11) | ((uint32_t)lg2(K) << 7) | (uint32_t)(layout & 7);
}

int mode_now() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (g_tune_mode < 0) {
    const char* e = getenv("GB300MPS_AUTOTUNE");
    g_tune_mode = (e && *e) ? atoi(e) : 1;
    if (g_tune_mode < 0 || g_tune_mode > 2) g_tune_mode = 1;
  }
  return g_tune_mode;
}

template <typename T>
int static_kind(int M, int N, int K, const GemmWs& ws) {
  if (sizeof(T) == 8) return GEMM_SIMT_64x64;  // complex128: CUDA cores only
  // small products (under ~2M complex MACs, or too thin to fill a tile
  // pair) stay on the CUDA cores; the rest are padded to 128 x 128 tiles
  if ((double)M * N * K < 2097152.0 || !tc_eligible(M, N, K, ws)) return GEMM_SIMT_64x64;
  return GEMM_TC;
}

// Time every eligible kernel on this product, writing a scratch output of
// C's shape and layout (alpha 1, beta 0), and record the fastest.  Returns
// the kernel to use; on a trial failure returns -1 with the error in *err.
template <typename T>
int tune_bucket(uint32_t key, const CMat<T>& A, const CMat<T>& B, const CMatOut<T>& C, GemmWs& ws, int skind,
                cudaStream_t st, cudaError_t* err) {
  *err = cudaSuccess;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return skind;  // no trial launches or allocation inside a capture
  }
  const int M = C.rows, N = C.cols;
  const size_t bytes = (size_t)M * N * sizeof(cx<T>);
  if (bytes > kTuneMaxBytes) return skind;
  if (ws.tune_c_bytes < bytes) {
    if (ws.tune_c) cudaFree(ws.tune_c);
    ws.tune_c = nullptr;
    ws.tune_c_bytes = 0;
    if (cudaMalloc(&ws.tune_c, kTuneMaxBytes) != cudaSuccess) {
      cudaGetLastError();
      ws.tune_c = nullptr;
      return skind;
    }
    ws.tune_c_bytes = kTuneMaxBytes;
  }
  for (cudaEvent_t& e : ws.tune_ev)
    if (!e && cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      e = nullptr;
      return skind;
    }
  // the trial output keeps C's layout (row- or column-major)
  const CMatOut<T> Ct = (C.rs == 1 && C.cs != 1) ? cout_<T>(ws.tune_c, M, N, 1, M) : cout_<T>(ws.tune_c, M, N, N, 1);
  TuneEntry en;
  en.static_kind = skind;
  for (float& t : en.ns) t = 0.0f;
  for (int kind = 0; kind < GEMM_KINDS; ++kind) {
    if (kind == GEMM_TC && (sizeof(T) == 8 || !tc_eligible(M, N, A.cols, ws))) continue;
    cudaError_t e = cgemm_kind(kind, A, B, Ct, T(1), T(0), ws, st);
    if (e == cudaSuccess) e = cudaEventRecord(ws.tune_ev[0], st);
    for (int r = 0; r < kTuneReps && e == cudaSuccess; ++r) e = cgemm_kind(kind, A, B, Ct, T(1), T(0), ws, st);
    if (e == cudaSuccess) e = cudaEventRecord(ws.tune_ev[1], st);
    if (e == cudaSuccess) e = cudaEventSynchronize(ws.tune_ev[1]);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ws.tune_ev[0], ws.tune_ev[1]);
    if (e != cudaSuccess) {
      *err = e;
      return -1;
    }
    en.ns[kind] = ms * 1e6f / kTuneReps;
  }
  // the static rule unless another kernel beats it by the margin; then the fastest
  int best = skind;
  float best_ns = en.ns[skind];
  for (int kind = 0; kind < GEMM_KINDS; ++kind)
    if (en.ns[kind] > 0.0f && en.ns[kind] < en.ns[skind] * kTuneMargin && en.ns[kind] < best_ns) {
      best = kind;
      best_ns = en.ns[kind];
    }
  en.kind = best;
  ++ws.tunings;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = en;
  return best;
}

template <typename T>
cudaError_t cgemm_tuned(const CMat<T>& A, const CMat<T>& B, const CMatOut<T>& C, T alpha, T beta, GemmWs& ws,
                        cudaStream_t st) {
  const int M = C.rows, N = C.cols, K = A.cols;
  if (M <= 0 || N <= 0) return cudaSuccess;
  const int skind = static_kind<T>(M, N, K, ws);
  int kind = skind;
  const int mode = mode_now();
  if (mode != 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    // precision as in the C ABI: 0 complex128, 1 complex64
    const uint32_t key = tune_key(dev, sizeof(T) == 8 ? 0 : 1, M, N, K, layout_bits(A, B, C)) |
                         (sizeof(T) == 4 && ws.split_bf16 ? (1u << 26) : 0u);
    bool found = false;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tune.find(key);
      if (it != g_tune.end()) {
        kind = it->second.kind;
        found = true;
      }
    }
    if (!found && mode == 1) {
      cudaError_t e;
      kind = tune_bucket<T>(key, A, B, C, ws, skind, st, &e);
      if (kind < 0) return e;
    }
    // an entry tuned on a larger workspace may name a kernel this product cannot take here
    if (kind == GEMM_TC && (sizeof(T) == 8 || !tc_eligible(M, N, K, ws))) kind = skind;
  }
  if (kind == GEMM_TC)
    ++ws.tc_launches;
  else
    ++ws.simt_launches;
  return cgemm_kind(kind, A, B, C, alpha, beta, ws, st);
}

}  // namespace

cudaError_t cgemm(const CMat<double>& A, const CMat<double>& B, const CMatOut<double>& C, double alpha, double beta,
                  GemmWs& ws, cudaStream_t st) {
  return cgemm_tuned<double>(A, B, C, alpha, beta, ws, st);
}

cudaError_t cgemm(const CMat<float>& A, const CMat<float>& B, const CMatOut<float>& C, float alpha, float beta,
                  GemmWs& ws, cudaStream_t st) {
  return cgemm_tuned<float>(A, B, C, alpha, beta, ws, st);
}

void gemm_tune_set_mode(int mode) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_mode = (mode < 0 || mode > 2) ? 0 : mode;
}

int gemm_tune_mode() { return mode_now(); }

void gemm_tune_clear() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
}

static void entry_row(uint32_t key, const TuneEntry& en, int* row) {
  row[0] = (int)((key >> 20) & 63);
  row[1] = (key >> 26) & 1 ? 3 : (int)((key >> 19) & 1);  // 3: split-BF16 tensor-core products
  row[2] = (int)((key >> 15) & 15);
  row[3] = (int)((key >> 11) & 15);
  row[4] = (int)((key >> 7) & 15);
  row[5] = (int)(key & 7);
  row[6] = en.kind;
  row[7] = (int)en.ns[en.kind];
  row[8] = (int)en.ns[en.static_kind];
}

int gemm_tune_table(int* out, int cap) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  int n = 0;
  for (const auto& kv : g_tune) {
    if (out && n < cap) entry_row(kv.first, kv.second, out + (size_t)n * kTuneCols);
    ++n;
  }
  return n;
}

// Text cache: one line per bucket, "key kind static_kind ns_0 .. ns_4".
int gemm_tune_save(const char* path) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  FILE* f = fopen(path, "w");
  if (!f) return 1;
  fprintf(f, "# gb300mps gemm tuning v1: key kind static_kind ns[%d]\n", (int)GEMM_KINDS);
  for (const auto& kv : g_tune) {
    fprintf(f, "%u %d %d", kv.first, kv.second.kind, kv.second.static_kind);
    for (float t : kv.second.ns) fprintf(f, " %.9g", (double)t);  // exact float round trip
    fprintf(f, "\n");
  }
  return fclose(f) == 0 ? 0 : 1;
}

int gemm_tune_load(const char* path) {
  FILE* f = fopen(path, "r");
  if (!f) return 1;
  char line[512];
  std::map<uint32_t, TuneEntry> got;
  bool bad = false;
  while (fgets(line, sizeof line, f)) {
    if (line[0] == '#' || line[0] == '\n') continue;
    unsigned key = 0;
    TuneEntry en;
    int n = sscanf(line, "%u %d %d %f %f %f %f %f", &key, &en.kind, &en.static_kind, &en.ns[0], &en.ns[1], &en.ns[2],
                   &en.ns[3], &en.ns[4]);
    if (n != 3 + GEMM_KINDS || en.kind < 0 || en.kind >= GEMM_KINDS || en.static_kind < 0 ||
        en.static_kind >= GEMM_KINDS || (key >> 27) != 0) {
      bad = true;
      break;
    }
    got[(uint32_t)key] = en;
  }
  fclose(f);
  if (bad) return 2;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (const auto& kv : got) g_tune[kv.first] = kv.second;
  return 0;
}

}  // namespace gbmps
