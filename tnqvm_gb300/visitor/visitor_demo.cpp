// Drives GpuMpsVisitor the way TNQVM::execute does (TNQVM.cpp:106-139):
// setOptions, initialize, accept() every instruction, finalize, then prints
// the AcceleratorBuffer contents as JSON.  Input on stdin, one gate per line:
//   n_qubits shots
//   <name> <nbits> <b0> [b1] <nparams> [p0 p1 p2]
//   ... ; optional "opt <key> <value>" lines before the gates, and
//   "obs <name> <nbits> <b0> [b1] <nparams> [p...]" lines that form one
//   observed circuit (basis change + Measure) whose VQE-mode value
//   getExpectationValueZ returns (TNQVM.cpp:82-89) before finalize.
#include <iostream>
#include <sstream>

#include "GpuMpsVisitor.hpp"

int main() {
  int n = 0, shots = 0;
  std::cin >> n >> shots;
  auto buffer = std::make_shared<xacc::AcceleratorBuffer>(n);
  auto program = std::make_shared<xacc::CompositeInstruction>("demo");
  auto observed = std::make_shared<xacc::CompositeInstruction>("observed");
  xacc::HeterogeneousMap opts;
  std::string tok;
  while (std::cin >> tok) {
    bool obs = false;
    if (tok == "obs") {
      obs = true;
      std::cin >> tok;
    }
    if (tok == "opt") {
      std::string key, val;
      std::cin >> key >> val;
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
  auto visitor = std::make_shared<tnqvm::GpuMpsVisitor>();
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
