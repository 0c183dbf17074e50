// The TNQVM visitor plugin interface, restated with the same method set as
// tnqvm/visitors/TNQVMVisitor.hpp:58-82 so that the GB300 visitor is a drop-in
// plugin: initialize(buffer, shots), one visit() per gate (AllGateVisitor),
// finalize(), getExpectationValueZ(observed circuit), getState(),
// setOptions(), supportVqeMode(), getExecutionInfo(), name()/clone().
// With a real XACC + TNQVM build (GB300MPS_WITH_XACC) TNQVM's own header is
// used instead and this file only supplies the shim types.
#pragma once
#ifdef GB300MPS_WITH_XACC
#include "TNQVMVisitor.hpp"
#else
#include "xacc_shim.hpp"

namespace tnqvm {
using xacc::AcceleratorBuffer;
using xacc::CompositeInstruction;
using xacc::HeterogeneousMap;

class TNQVMVisitor : public xacc::quantum::AllGateVisitor,
                     public xacc::OptionsProvider,
                     public xacc::Cloneable<TNQVMVisitor> {
 public:
  virtual void initialize(std::shared_ptr<AcceleratorBuffer> buffer, int nbShots = 1) = 0;
  virtual const double getExpectationValueZ(std::shared_ptr<CompositeInstruction> function) = 0;
  virtual const std::vector<std::complex<double>> getState() { return {}; }
  virtual void finalize() = 0;
  void setOptions(const HeterogeneousMap& in_options) { options = in_options; }
  virtual void setKernelName(const std::string&) {}
  virtual bool supportVqeMode() const { return false; }
  HeterogeneousMap getExecutionInfo() const { return executionInfo; }
  virtual const std::string name() const = 0;
  virtual const std::string description() const = 0;

 protected:
  std::shared_ptr<AcceleratorBuffer> buffer;
  HeterogeneousMap options;
  HeterogeneousMap executionInfo;
};
}  // namespace tnqvm
#endif
