// Host-side gate table and SWAP router of the GB300 MPS engine.
//
// Matrices follow tnqvm/base/Gates.hpp:131-334 (FP64, row-major; for two
// qubits the first qubit is the most significant bit of the row/column
// index, Gates.hpp:238-246).  The router restates the meet-in-the-middle
// strategy of tnqvm/visitors/exatn-mps/NearestNeighborTransform.hpp:43-135.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <string>
#include <vector>

namespace gbmps {

using cd = std::complex<double>;

struct GateRec {
  int nq;
  int q0, q1;
  cd m[16];  // 2x2 in m[0..3] or 4x4 row-major
};

// Returns the number of qubits of the gate (1 or 2), or 0 if the name is unknown
// or the parameter count is wrong.  "Measure" and "I" return -1 (no-op).
inline int gate_matrix(const std::string& name, const double* p, int np, cd* m) {
  const double s2 = std::sqrt(0.5);
  const cd I(0, 1);
  auto set2 = [&](cd a, cd b, cd c, cd d) {
    m[0] = a;
    m[1] = b;
    m[2] = c;
    m[3] = d;
    return 1;
  };
  auto diag4 = [&](cd a, cd b, cd c, cd d) {
    for (int i = 0; i < 16; ++i) m[i] = 0.0;
    m[0] = a;
    m[5] = b;
    m[10] = c;
    m[15] = d;
    return 2;
  };
  auto need = [&](int k) { return np == k; };
  if (name == "I" || name == "Identity" || name == "Measure") return -1;
  if (name == "H" && need(0)) return set2(s2, s2, s2, -s2);
  if (name == "X" && need(0)) return set2(0, 1, 1, 0);
  if (name == "Y" && need(0)) return set2(0, -I, I, 0);
  if (name == "Z" && need(0)) return set2(1, 0, 0, -1);
  if (name == "S" && need(0)) return set2(1, 0, 0, I);
  if (name == "Sdg" && need(0)) return set2(1, 0, 0, -I);
  if (name == "T" && need(0)) return set2(1, 0, 0, std::exp(I * (M_PI / 4)));
  if (name == "Tdg" && need(0)) return set2(1, 0, 0, std::exp(-I * (M_PI / 4)));
  if (name == "Rx" && need(1)) {
    const double c = std::cos(0.5 * p[0]), s = std::sin(0.5 * p[0]);
    return set2(c, -I * s, -I * s, c);
  }
  if (name == "Ry" && need(1)) {
    const double c = std::cos(0.5 * p[0]), s = std::sin(0.5 * p[0]);
    return set2(c, -s, s, c);
  }
  if (name == "Rz" && need(1)) return set2(std::exp(-0.5 * I * p[0]), 0, 0, std::exp(0.5 * I * p[0]));
  if ((name == "U" || name == "U3") && need(3)) {
    const double th = p[0], ph = p[1], la = p[2];
    return set2(std::cos(th / 2), -std::exp(I * la) * std::sin(th / 2), std::exp(I * ph) * std::sin(th / 2),
                std::exp(I * (ph + la)) * std::cos(th / 2));
  }
  if ((name == "CNOT" || name == "CX") && need(0)) {
    for (int i = 0; i < 16; ++i) m[i] = 0.0;
    m[0] = m[5] = m[11] = m[14] = 1.0;
    return 2;
  }
  if (name == "CZ" && need(0)) return diag4(1, 1, 1, -1);
  if (name == "CY" && need(0)) {
    for (int i = 0; i < 16; ++i) m[i] = 0.0;
    m[0] = m[5] = 1.0;
    m[11] = -I;
    m[14] = I;
    return 2;
  }
  if (name == "CH" && need(0)) {
    for (int i = 0; i < 16; ++i) m[i] = 0.0;
    m[0] = m[5] = 1.0;
    m[10] = m[11] = m[14] = s2;
    m[15] = -s2;
    return 2;
  }
  if (name == "CRZ" && need(1)) return diag4(1, 1, std::exp(-0.5 * I * p[0]), std::exp(0.5 * I * p[0]));
  if (name == "CPhase" && need(1)) return diag4(1, 1, 1, std::exp(I * p[0]));
  if (name == "RZZ" && need(1)) {
    const cd a = std::exp(-0.5 * I * p[0]), b = std::exp(0.5 * I * p[0]);
    return diag4(a, b, b, a);
  }
  if (name == "Swap" && need(0)) {
    for (int i = 0; i < 16; ++i) m[i] = 0.0;
    m[0] = m[6] = m[9] = m[15] = 1.0;
    return 2;
  }
  if (name == "iSwap" && need(0)) {
    for (int i = 0; i < 16; ++i) m[i] = 0.0;
    m[0] = m[15] = 1.0;
    m[6] = m[9] = I;
    return 2;
  }
  if (name == "fSim" && need(2)) {
    for (int i = 0; i < 16; ++i) m[i] = 0.0;
    m[0] = 1.0;
    m[5] = m[10] = std::cos(p[0]);
    m[6] = m[9] = -I * std::sin(p[0]);
    m[15] = std::exp(-I * p[1]);
    return 2;
  }
  return 0;
}

inline GateRec swap_rec(int a, int b) {
  GateRec g;
  g.nq = 2;
  g.q0 = a;
  g.q1 = b;
  gate_matrix("Swap", nullptr, 0, g.m);
  return g;
}

// SWAP routing (NearestNeighborTransform.hpp:77-127): swap the lower qubit up
// and the upper qubit down alternately until they are adjacent, apply the gate
// on the moved qubits in the original bit order, then undo the swaps.
inline void route_append(const GateRec& g, std::vector<GateRec>& out) {
  if (g.nq != 2 || std::abs(g.q0 - g.q1) <= 1) {
    out.push_back(g);
    return;
  }
  const int lo0 = std::min(g.q0, g.q1), hi0 = std::max(g.q0, g.q1);
  int lo = lo0, hi = hi0;
  for (;;) {
    out.push_back(swap_rec(lo, lo + 1));
    ++lo;
    if (std::abs(lo - hi) <= 1) break;
    out.push_back(swap_rec(hi, hi - 1));
    --hi;
    if (std::abs(lo - hi) <= 1) break;
  }
  GateRec moved = g;
  if (g.q0 < g.q1) {
    moved.q0 = lo;
    moved.q1 = hi;
  } else {
    moved.q0 = hi;
    moved.q1 = lo;
  }
  out.push_back(moved);
  for (int i = lo; i > lo0; --i) out.push_back(swap_rec(i, i - 1));
  for (int i = hi; i < hi0; ++i) out.push_back(swap_rec(i, i + 1));
}

// The exact SWAP of two neighbouring sites.
inline bool is_adjacent_swap(const GateRec& g) {
  if (g.nq != 2 || std::abs(g.q0 - g.q1) != 1) return false;
  static const double S[16] = {1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 0, 0, 0, 1};
  for (int i = 0; i < 16; ++i)
    if (g.m[i] != cd(S[i], 0.0)) return false;
  return true;
}

// Peephole on a routed instruction stream (no reference counterpart; the
// reference applies every SWAP of its meet-in-the-middle chains,
// NearestNeighborTransform.hpp:83-121).  Two SWAPs on the same pair of
// sites (a, a+1) with nothing in between that acts on a or a+1 except
// 1-qubit gates are the identity: both are dropped and those 1-qubit gates
// move to the other site of the pair (SWAP (A x B) SWAP = B x A).  Gates on
// other sites commute with both SWAPs.  Scanning from the end removes nested
// pairs (the return chain of one routed gate against the outgoing chain of
// the next) innermost first.  Returns the number of SWAPs removed.
inline size_t cancel_swap_pairs(std::vector<GateRec>& g) {
  const size_t n = g.size();
  std::vector<char> dead(n, 0);
  std::vector<size_t> ones;
  size_t removed = 0;
  for (size_t i = n; i-- > 0;) {
    if (dead[i] || !is_adjacent_swap(g[i])) continue;
    const int a = std::min(g[i].q0, g[i].q1), b = a + 1;
    ones.clear();
    for (size_t j = i + 1; j < n; ++j) {
      if (dead[j]) continue;
      const GateRec& h = g[j];
      const bool touch = h.q0 == a || h.q0 == b || (h.nq == 2 && (h.q1 == a || h.q1 == b));
      if (!touch) continue;
      if (h.nq == 1) {
        ones.push_back(j);
        continue;
      }
      if (is_adjacent_swap(h) && std::min(h.q0, h.q1) == a) {
        dead[i] = dead[j] = 1;
        removed += 2;
        for (size_t k : ones) g[k].q0 = g[k].q0 == a ? b : a;
      }
      break;
    }
  }
  if (removed) {
    size_t w = 0;
    for (size_t i = 0; i < n; ++i)
      if (!dead[i]) g[w++] = g[i];
    g.resize(w);
  }
  return removed;
}

// 4x4 re-expressed with its two qubits exchanged (row 2a+b -> 2b+a).
inline void swap_bits4(const cd* in, cd* out) {
  static const int p[4] = {0, 2, 1, 3};
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) out[r * 4 + c] = in[p[r] * 4 + p[c]];
}

}  // namespace gbmps
