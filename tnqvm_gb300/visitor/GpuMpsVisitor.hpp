// GB300 MPS visitor plugin: ``tnqvm-visitor`` name "gb300-mps".
//
// Drop-in for the exatn-mps visitor (tnqvm/visitors/exatn-mps/ExaTnMpsVisitor.hpp:
// same visit() set, same options "svd-cutoff" / "max-bond-dim" / "bitstring",
// same AcceleratorBuffer keys).  Each visit() only records the gate; finalize()
// or getExpectationValueZ() submit the whole program through the gb300mps C ABI,
// so the host-device boundary is crossed once per program, not once per gate.
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "../../include/gb300mps.h"
#include "tnqvm_visitor.hpp"

namespace tnqvm {

class GpuMpsVisitor : public TNQVMVisitor {
 public:
  GpuMpsVisitor();
  ~GpuMpsVisitor() override;

  void initialize(std::shared_ptr<AcceleratorBuffer> buffer, int nbShots) override;
  void finalize() override;
  const double getExpectationValueZ(std::shared_ptr<CompositeInstruction> function) override;
  const std::vector<std::complex<double>> getState() override;
  bool supportVqeMode() const override { return true; }

  const std::string name() const override { return "gb300-mps"; }
  const std::string description() const override {
    return "Matrix-product-state simulator on one GB300 GPU (sm_103a kernels)";
  }
  std::shared_ptr<TNQVMVisitor> clone() override { return std::make_shared<GpuMpsVisitor>(); }

#define GB300_VISIT_DECL(cls, nm) void visit(xacc::quantum::cls& g) override;
  GB300_SHIM_GATES(GB300_VISIT_DECL)
#undef GB300_VISIT_DECL

 private:
  void record(xacc::Instruction& g);
  void check(int rc, const char* what) const;
  void sample(int shots);
  mps_prog* prog_ = nullptr;
  int shots_ = 1;
  std::vector<int> measured_;
};

// Process-wide engine context on device 0 (created on first use).
mps_ctx* gb300_context();

}  // namespace tnqvm
