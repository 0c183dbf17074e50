// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11), the generator of shot
// sampling.  Host and device share this one definition, so a host test can
// check it against the published known-answer vectors.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbmps {

// High 32 bits of the 64-bit product a * b.
__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

// Ten rounds of the Philox4x32 bijection of counter c under key k.
__host__ __device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

// Uniform double in [0, 1) from the first 53 bits of the Philox output of
// counter (shot, site, stream tag, 0) under the 64-bit seed.
__host__ __device__ __forceinline__ double philox_uniform(uint64_t seed, uint32_t shot, uint32_t site,
                                                          uint32_t tag) {
  const uint4 r = philox4x32_10(make_uint4(shot, site, tag, 0u), make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  const uint64_t v = ((uint64_t)r.x << 32) | r.y;
  return (double)(v >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace gbmps
