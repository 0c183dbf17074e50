// Host-side check of the site-parallel schedule (gbmps::site_schedule in
// libgb300mps.so) on a program compiled by gbmps::compile_program, built
// with nvcc as host code and driven by tests/test_host_schedule.py.  No
// device is touched.
// Input: "n mode flags", then gate lines "name q0 q1 n_params p0 p1 p2".
// Output: "P <count>" and the program-order ops, then "S <count>" and the
// scheduled ops with their two dependency counts; one op per line as
// "kind site orient dep0 dep1 m_0 .. m_31" (deps 0 0 in the program list).
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "../include/gb300mps.h"
#include "../tnqvm_gb300/csrc/engine_internal.hpp"

static void print(const gbmps::DevOp& o, int d0, int d1) {
  std::printf("%d %d %d %d %d", o.kind, o.site, o.orient, d0, d1);
  for (int i = 0; i < 32; ++i) std::printf(" %.17g", o.m[i]);
  std::printf("\n");
}

int main() {
  mps_prog p;
  if (!(std::cin >> p.n >> p.mode >> p.flags)) return 1;
  p.nq = p.n;
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
  std::vector<gbmps::DevOp> ops, sorted;
  std::vector<int> deps;
  gbmps::compile_program(&p, ops);
  gbmps::site_schedule(ops, p.n, sorted, deps);
  std::printf("P %zu\n", ops.size());
  for (const auto& o : ops) print(o, 0, 0);
  std::printf("S %zu\n", sorted.size());
  for (size_t k = 0; k < sorted.size(); ++k) print(sorted[k], deps[2 * k], deps[2 * k + 1]);
  return 0;
}
