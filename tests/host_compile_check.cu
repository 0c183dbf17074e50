// Host-side check of the engine's program compiler (gbmps::compile_program in
// libgb300mps.so: SWAP routing, 1-qubit fusion into 2-qubit gates, sweep
// scheduling and gauge-move planning), built with nvcc as host code and
// driven by tests/test_host_compile.py.  No device is touched: the program
// record is filled on the host and only compiled.
// Input: "n mode flags", then gate lines "name q0 q1 n_params p0 p1 p2".
// Output: one line per op, "kind site orient m_0 .. m_31".
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "../include/gb300mps.h"
#include "../tnqvm_gb300/csrc/engine_internal.hpp"

int main() {
  mps_prog p;
  if (!(std::cin >> p.n >> p.mode >> p.flags)) return 1;
  p.center = 0;
  std::string name;
  int q0, q1, np;
  double par[3];
  while (std::cin >> name >> q0 >> q1 >> np >> par[0] >> par[1] >> par[2]) {
    gbmps::GateRec g{};
    g.nq = gbmps::gate_matrix(name, par, np, g.m);
    if (g.nq <= 0) continue;
    g.q0 = q0;
    g.q1 = q1;
    p.pending.push_back(g);
  }
  std::vector<gbmps::DevOp> ops;
  gbmps::compile_program(&p, ops);
  for (const auto& o : ops) {
    std::printf("%d %d %d", o.kind, o.site, o.orient);
    for (int i = 0; i < 32; ++i) std::printf(" %.17g", o.m[i]);
    std::printf("\n");
  }
  return 0;
}
