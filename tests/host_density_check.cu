// Host-side check of a density program's recording and compilation
// (gbmps::record_gate, gbmps::kraus_superop and gbmps::compile_program in
// libgb300mps.so), built with nvcc as host code and driven by
// tests/test_host_density.py.  No device is touched: a density program
// record (n qubits on 2n sites) is filled on the host and only compiled.
// Input: "n mode flags", then lines "G name q0 q1 n_params p0 p1 p2" (a gate)
// or "K q n_kraus" followed by 8 doubles per Kraus matrix (a channel).
// Output: one line per op, "kind site orient m_0 .. m_31".
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "../include/gb300mps.h"
#include "../tnqvm_gb300/csrc/engine_internal.hpp"

int main() {
  mps_prog p;
  int nq = 0;
  if (!(std::cin >> nq >> p.mode >> p.flags)) return 1;
  p.nq = nq;
  p.n = 2 * nq;
  p.density = true;
  p.center = 0;
  std::string tag;
  while (std::cin >> tag) {
    if (tag == "G") {
      std::string name;
      int q0, q1, np;
      double par[3];
      std::cin >> name >> q0 >> q1 >> np >> par[0] >> par[1] >> par[2];
      gbmps::GateRec g{};
      g.nq = gbmps::gate_matrix(name, par, np, g.m);
      if (g.nq <= 0) continue;
      g.q0 = q0;
      g.q1 = q1;
      gbmps::record_gate(&p, g);
    } else if (tag == "K") {
      int q, nk;
      std::cin >> q >> nk;
      std::vector<double> k(8 * (size_t)nk);
      for (auto& x : k) std::cin >> x;
      gbmps::GateRec g{};
      if (gbmps::kraus_superop(q, nk, k.data(), g)) return 2;
      p.pending.push_back(g);
    }
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
