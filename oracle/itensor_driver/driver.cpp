// Standalone driver of the reference's itensor-mps arithmetic, linked against
// the vendored ITensor v3 (test infrastructure only, built into oracle/_ref/).
//
// It applies gates exactly as ITensorMPSVisitor does
// (tnqvm/visitors/itensor/mps/ITensorMPSVisitor.cpp):
//   1 qubit  (:288-299): position(site); A' = Op * A; noPrime
//   2 qubits (:312-331): position(site1); wf = A1 * A2 * Op; noPrime;
//                        [U,S,V] = svd(wf, inds(A1), {Cutoff, MaxDim}); A1 = U; A2 = S*V
// with site1 the site of the gate's first qubit, and evaluates <P> for Pauli
// strings as <psi|P|psi> (innerC).  Gate matrices arrive as numbers on stdin:
//   n maxdim cutoff
//   G1 q  <8 doubles: row-major 2x2, (re, im)>
//   G2 q0 q1 <32 doubles: row-major 4x4, q0 = most significant bit>
//   P <n chars of IXYZ, char i on qubit i>
//   END
// Output: one JSON object with the link dimensions and the <P> values.
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "itensor/all.h"

using namespace itensor;

static ITensor op1(Index const& s, const std::vector<Cplx>& m) {
  auto T = ITensor(prime(s), s);
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < 2; ++c) T.set(prime(s) = r + 1, s = c + 1, m[2 * r + c]);
  return T;
}

static ITensor pauli(Index const& s, char p) {
  const Cplx I(0, 1);
  std::vector<Cplx> m;
  if (p == 'X') m = {0, 1, 1, 0};
  if (p == 'Y') m = {0, -I, I, 0};
  if (p == 'Z') m = {1, 0, 0, -1};
  return op1(s, m);
}

int main() {
  int n = 0, maxdim = 0;
  double cutoff = 0.0;
  std::cin >> n >> maxdim >> cutoff;
  auto sites = SpinHalf(n, {"ConserveQNs=", false});
  auto psi = MPS(InitState(sites, "Up"));  // |0...0>, as ITensorMPSVisitor.cpp:107-110
  std::vector<std::string> paulis;
  std::string tok;
  while (std::cin >> tok && tok != "END") {
    if (tok == "G1") {
      int q;
      std::cin >> q;
      std::vector<Cplx> m(4);
      for (auto& z : m) {
        double re, im;
        std::cin >> re >> im;
        z = Cplx(re, im);
      }
      const int site = q + 1;
      psi.position(site);
      auto A = op1(sites(site), m) * psi(site);
      A.noPrime();
      psi.set(site, A);
    } else if (tok == "G2") {
      int q0, q1;
      std::cin >> q0 >> q1;
      std::vector<Cplx> m(16);
      for (auto& z : m) {
        double re, im;
        std::cin >> re >> im;
        z = Cplx(re, im);
      }
      const int s1 = q0 + 1, s2 = q1 + 1;
      auto a = sites(s1), b = sites(s2);
      auto Op = ITensor(prime(a), prime(b), a, b);
      for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c)
          Op.set(prime(a) = (r >> 1) + 1, prime(b) = (r & 1) + 1, a = (c >> 1) + 1, b = (c & 1) + 1, m[4 * r + c]);
      psi.position(s1);
      auto wf = psi(s1) * psi(s2);
      wf *= Op;
      wf.noPrime();
      auto [U, S, V] = svd(wf, inds(psi(s1)), {"Cutoff=", cutoff, "MaxDim=", maxdim});
      psi.set(s1, U);
      psi.set(s2, S * V);
    } else if (tok == "P") {
      std::string p;
      std::cin >> p;
      paulis.push_back(p);
    }
  }
  std::printf("{\"bonds\": [");
  for (int b = 1; b < n; ++b) std::printf("%s%ld", b > 1 ? ", " : "", (long)dim(linkIndex(psi, b)));
  std::printf("], \"paulis\": [");
  for (size_t t = 0; t < paulis.size(); ++t) {
    auto phi = psi;
    for (int q = 0; q < n; ++q) {
      if (paulis[t][q] == 'I') continue;
      auto A = pauli(sites(q + 1), paulis[t][q]) * phi(q + 1);
      A.noPrime();
      phi.set(q + 1, A);
    }
    const Cplx v = innerC(psi, phi);
    std::printf("%s[%.17g, %.17g]", t ? ", " : "", v.real(), v.imag());
  }
  std::printf("]}\n");
  return 0;
}
