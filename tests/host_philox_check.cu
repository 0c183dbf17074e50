// Host-side check of the shot sampler's generator (tnqvm_gb300/csrc/philox.cuh,
// the definition the sampling kernels use), built with nvcc as host code and
// driven by tests/test_host_philox.py.  Each input line is a counter (4 words)
// and a key (2 words) in hex; each output line is the Philox4x32-10 output.
#include <cstdio>

#include "../tnqvm_gb300/csrc/philox.cuh"

int main() {
  unsigned c0, c1, c2, c3, k0, k1;
  while (std::scanf("%x %x %x %x %x %x", &c0, &c1, &c2, &c3, &k0, &k1) == 6) {
    const uint4 r = gbmps::philox4x32_10(make_uint4(c0, c1, c2, c3), make_uint2(k0, k1));
    std::printf("%08x %08x %08x %08x\n", r.x, r.y, r.z, r.w);
  }
  std::printf("u %.17g\n", gbmps::philox_uniform(0x0123456789abcdefull, 7u, 3u, 0x4d505321u));
  return 0;
}
