// Host-side check of the engine's truncation rule (tnqvm_gb300/csrc/keep.cuh,
// the same function the split kernels call), built with nvcc as host code
// and driven by tests/test_host_keep.py.  Each input line is
// "mode cutoff cap mm lam_0 .. lam_{mm-1}"; each output line is the kept
// dimension.
#include <cstdio>
#include <iostream>
#include <vector>

#include "../tnqvm_gb300/csrc/keep.cuh"

int main() {
  int mode, cap, mm;
  double cutoff;
  while (std::cin >> mode >> cutoff >> cap >> mm) {
    std::vector<double> lam(mm);
    for (int i = 0; i < mm; ++i) std::cin >> lam[i];
    std::printf("%d\n", gbmps::keep_rule(lam.data(), mm, mode, cutoff, cap));
  }
  return 0;
}
