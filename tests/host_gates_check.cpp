// Host-side check of the engine's gate table and SWAP router
// (tnqvm_gb300/csrc/gates.hpp), built and driven by tests/test_host_gates.py.
// Reads gate lines "name q0 q1 n_params p0 p1 p2" from stdin (q1 = -1 for one
// qubit).  Without arguments it prints each gate's matrix ("nq re im ..."); with
// "route" it routes the whole list and prints each routed record
// ("nq q0 q1 re im ...").
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "../tnqvm_gb300/csrc/gates.hpp"

static void print_matrix(const gbmps::GateRec& g) {
  const int cnt = g.nq == 1 ? 4 : (g.nq == 2 ? 16 : 0);
  for (int i = 0; i < cnt; ++i) std::printf(" %.17g %.17g", g.m[i].real(), g.m[i].imag());
  std::printf("\n");
}

int main(int argc, char** argv) {
  const bool route = argc > 1 && std::string(argv[1]) == "route";
  std::string name;
  int q0, q1, np;
  double p[3];
  std::vector<gbmps::GateRec> out;
  while (std::cin >> name >> q0 >> q1 >> np >> p[0] >> p[1] >> p[2]) {
    gbmps::GateRec g{};
    g.nq = gbmps::gate_matrix(name, p, np, g.m);
    g.q0 = q0;
    g.q1 = q1;
    if (route) {
      gbmps::route_append(g, out);
    } else {
      std::printf("%d", g.nq);
      print_matrix(g);
    }
  }
  for (const auto& g : out) {
    std::printf("%d %d %d", g.nq, g.q0, g.q1);
    print_matrix(g);
  }
  return 0;
}
