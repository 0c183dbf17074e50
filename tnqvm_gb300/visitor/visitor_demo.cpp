// Drives GpuMpsVisitor the way TNQVM::execute does (TNQVM.cpp:106-139):
// setOptions, initialize, accept() every instruction, finalize, then prints
// the AcceleratorBuffer contents as JSON.  Input on stdin, one gate per line:
//   n_qubits shots
//   <name> <nbits> <b0> [b1] <nparams> [p0 p1 p2]
//   ... ; optional "opt <key> <value>" lines before the gates, and
//   "obs <name> <nbits> <b0> [b1] <nparams> [p...]" lines that form one
//   observed circuit (basis change + Measure) whose VQE-mode value
//   getExpectationValueZ returns (TNQVM.cpp:82-89) before finalize.
// "opt visitor pmps" drives the noisy visitor (GpuPmpsVisitor) instead, with
// a noise model from "noise <gate> <nbits> <b0> [b1] <nkraus> <8 doubles per
// Kraus matrix, row-major (re, im)>" and "readout <qubit> <P(0|1)> <P(1|0)>"
// lines, and prints the density matrix too.
#include <iostream>
#include <map>
#include <sstream>

#include "GpuMpsVisitor.hpp"
#include "GpuPmpsVisitor.hpp"

namespace {
// A noise model given as a table: channels per (gate name, qubits), readout
// errors per qubit.
class TableNoiseModel : public xacc::NoiseModel {
 public:
  std::map<std::pair<std::string, std::vector<std::size_t>>, std::vector<xacc::NoiseChannelKraus>> gates;
  std::map<std::size_t, std::pair<double, double>> readout;
  std::vector<xacc::NoiseChannelKraus> getNoiseChannels(xacc::Instruction& g) override {
    auto it = gates.find({g.name(), g.bits()});
    return it == gates.end() ? std::vector<xacc::NoiseChannelKraus>{} : it->second;
  }
  std::pair<double, double> readoutError(std::size_t q) override {
    auto it = readout.find(q);
    return it == readout.end() ? std::make_pair(0.0, 0.0) : it->second;
  }
};
}  // namespace

int main() {
  int n = 0, shots = 0;
  std::cin >> n >> shots;
  auto buffer = std::make_shared<xacc::AcceleratorBuffer>(n);
  auto program = std::make_shared<xacc::CompositeInstruction>("demo");
  auto observed = std::make_shared<xacc::CompositeInstruction>("observed");
  xacc::HeterogeneousMap opts;
  auto noise = std::make_shared<TableNoiseModel>();
  bool noisy = false, pmps = false;
  std::string tok;
  while (std::cin >> tok) {
    if (tok == "noise") {
      std::string g;
      int nb = 0, nk = 0;
      std::cin >> g >> nb;
      std::vector<std::size_t> bits(nb);
      for (auto& b : bits) std::cin >> b;
      std::cin >> nk;
      xacc::NoiseChannelKraus ch;
      ch.noise_qubits = bits;
      for (int k = 0; k < nk; ++k) {
        std::vector<std::vector<std::complex<double>>> m(2, std::vector<std::complex<double>>(2));
        for (int r = 0; r < 2; ++r)
          for (int c = 0; c < 2; ++c) {
            double re, im;
            std::cin >> re >> im;
            m[r][c] = {re, im};
          }
        ch.mats.push_back(m);
      }
      noise->gates[{g, bits}].push_back(ch);
      noisy = true;
      continue;
    }
    if (tok == "readout") {
      std::size_t q;
      double a, b;
      std::cin >> q >> a >> b;
      noise->readout[q] = {a, b};
      noisy = true;
      continue;
    }
    bool obs = false;
    if (tok == "obs") {
      obs = true;
      std::cin >> tok;
    }
    if (tok == "opt") {
      std::string key, val;
      std::cin >> key >> val;
      if (key == "visitor") {
        pmps = val == "pmps";
        continue;
      }
      if (key == "svd-cutoff") opts.insert("svd-cutoff", std::stod(val));
      else if (key == "max-bond-dim" || key == "seed") opts.insert(key, std::stoi(val));
      else opts.insert(key, val);
      continue;
    }
    int nb = 0, np = 0;
    std::cin >> nb;
    std::vector<std::size_t> bits(nb);
    for (auto& b : bits) std::cin >> b;
    std::cin >> np;
    std::vector<double> ps(np);
    for (auto& p : ps) std::cin >> p;
    (obs ? observed : program)->addInstruction(xacc::quantum::make_gate(tok, bits, ps));
  }
  if (noisy) opts.insert("noise-model", std::shared_ptr<xacc::NoiseModel>(noise));
  std::shared_ptr<tnqvm::TNQVMVisitor> visitor;
  if (pmps)
    visitor = std::make_shared<tnqvm::GpuPmpsVisitor>();
  else
    visitor = std::make_shared<tnqvm::GpuMpsVisitor>();
  visitor->setOptions(opts);
  visitor->initialize(buffer, shots);
  xacc::InstructionIterator it(program);
  while (it.hasNext()) {
    auto inst = it.next();
    if (inst->isEnabled()) inst->accept(*visitor);
  }
  const bool vqe = observed->nInstructions() > 0;
  const double vqe_val = vqe ? visitor->getExpectationValueZ(observed) : 0.0;
  visitor->finalize();
  std::cout.precision(17);
  std::cout << "{\"name\": \"" << visitor->name() << "\"";
  if (vqe) std::cout << ", \"vqe-exp-val\": " << vqe_val;
  for (auto& kv : buffer->getInformation()) {
    if (kv.second.type() == typeid(double))
      std::cout << ", \"" << kv.first << "\": " << std::any_cast<double>(kv.second);
    if (kv.second.type() == typeid(std::vector<std::pair<double, double>>)) {
      std::cout << ", \"" << kv.first << "\": [";
      const auto& v = std::any_cast<const std::vector<std::pair<double, double>>&>(kv.second);
      for (size_t i = 0; i < v.size(); ++i) std::cout << (i ? ", " : "") << "[" << v[i].first << ", " << v[i].second << "]";
      std::cout << "]";
    }
  }
  std::cout << ", \"counts\": {";
  bool first = true;
  for (auto& kv : buffer->getMeasurementCounts()) {
    std::cout << (first ? "" : ", ") << "\"" << kv.first << "\": " << kv.second;
    first = false;
  }
  std::cout << "}}" << std::endl;
  return 0;
}
