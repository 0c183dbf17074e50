// GB300 noisy-circuit visitor plugin: ``tnqvm-visitor`` name "gb300-pmps".
//
// Drop-in for the purified-MPS visitor exatn-pmps
// (tnqvm/visitors/exatn-mpo/ExaTnPmpsVisitor.hpp): the same visit() set, the
// same "noise-model" option (an xacc::NoiseModel whose single-qubit Kraus
// channels follow each gate, :838-847,875-884), "shots" defaulting to 1024
// (:539), and the same results: "density_matrix" (the register's density
// matrix, or the measured qubits' reduced one for larger registers) and shot
// bit strings with readout errors (finalize :658-795).  The density matrix
// is held on the GPU as a vectorised MPS (MPS_FLAG_DENSITY); gates and
// channels are recorded and submitted once per circuit.
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "../../include/gb300mps.h"
#include "tnqvm_visitor.hpp"

namespace tnqvm {

class GpuPmpsVisitor : public TNQVMVisitor {
 public:
  GpuPmpsVisitor();
  ~GpuPmpsVisitor() override;

  void initialize(std::shared_ptr<AcceleratorBuffer> buffer, int nbShots) override;
  void finalize() override;
  // Tr(rho P) / Tr(rho) of the observed circuit's Pauli string (the
  // reference returns 0, :1233-1236)
  const double getExpectationValueZ(std::shared_ptr<CompositeInstruction> function) override;

  const std::string name() const override { return "gb300-pmps"; }
  const std::string description() const override {
    return "Noisy-circuit simulator (density matrix as a vectorised MPS) on one GB300 GPU";
  }
  std::shared_ptr<TNQVMVisitor> clone() override { return std::make_shared<GpuPmpsVisitor>(); }

#define GB300_VISIT_DECL(cls, nm) void visit(xacc::quantum::cls& g) override;
  GB300_SHIM_GATES(GB300_VISIT_DECL)
#undef GB300_VISIT_DECL

 private:
  void record(xacc::Instruction& g);
  void check(int rc, const char* what) const;
  mps_prog* prog_ = nullptr;
  int shots_ = 1024;
  std::vector<int> measured_;
  std::shared_ptr<xacc::NoiseModel> noise_;
};

}  // namespace tnqvm
