// Minimal stand-in for the XACC types a TNQVM visitor touches, so that the
// GB300 visitor plugin compiles and runs without an XACC installation.
// Only the calls the visitor uses exist here: gate instructions with
// name()/bits()/getParameter(), composites and their iteration, the
// AllGateVisitor double dispatch, HeterogeneousMap options and the
// AcceleratorBuffer result sink (addExtraInfo / appendMeasurement).  Against a
// real XACC build the plugin includes XACC's own headers instead
// (GB300MPS_WITH_XACC).
#pragma once
#include <any>
#include <complex>
#include <cstddef>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace xacc {

class HeterogeneousMap {
 public:
  HeterogeneousMap() = default;
  template <typename T>
  void insert(const std::string& k, const T& v) {
    m_[k] = v;
  }
  template <typename T>
  bool keyExists(const std::string& k) const {
    auto it = m_.find(k);
    return it != m_.end() && it->second.type() == typeid(T);
  }
  template <typename T>
  T get(const std::string& k) const {
    return std::any_cast<T>(m_.at(k));
  }

 private:
  std::map<std::string, std::any> m_;
};

class AcceleratorBuffer {
 public:
  explicit AcceleratorBuffer(std::size_t n) : n_(n) {}
  std::size_t size() const { return n_; }
  template <typename T>
  void addExtraInfo(const std::string& k, const T& v) {
    extra_[k] = v;
  }
  const std::map<std::string, std::any>& getInformation() const { return extra_; }
  void appendMeasurement(const std::string& bits) { counts_[bits] += 1; }
  void appendMeasurement(const std::string& bits, int count) { counts_[bits] += count; }
  const std::map<std::string, int>& getMeasurementCounts() const { return counts_; }

 private:
  std::size_t n_;
  std::map<std::string, std::any> extra_;
  std::map<std::string, int> counts_;
};

class OptionsProvider {
 public:
  virtual ~OptionsProvider() = default;
};

template <typename T>
class Cloneable {
 public:
  virtual ~Cloneable() = default;
  virtual std::shared_ptr<T> clone() = 0;
};

namespace quantum {
class AllGateVisitor;
}

class Instruction {
 public:
  Instruction(std::string name, std::vector<std::size_t> bits, std::vector<double> params = {})
      : name_(std::move(name)), bits_(std::move(bits)), params_(std::move(params)) {}
  virtual ~Instruction() = default;
  const std::string& name() const { return name_; }
  const std::vector<std::size_t>& bits() const { return bits_; }
  void setBits(const std::vector<std::size_t>& b) { bits_ = b; }
  std::size_t nParameters() const { return params_.size(); }
  double getParameter(std::size_t i) const { return params_.at(i); }
  bool isEnabled() const { return true; }
  virtual bool isComposite() const { return false; }
  virtual void accept(quantum::AllGateVisitor& v) = 0;

 private:
  std::string name_;
  std::vector<std::size_t> bits_;
  std::vector<double> params_;
};

class CompositeInstruction {
 public:
  explicit CompositeInstruction(std::string name) : name_(std::move(name)) {}
  void addInstruction(std::shared_ptr<Instruction> i) { insts_.push_back(std::move(i)); }
  std::size_t nInstructions() const { return insts_.size(); }
  std::shared_ptr<Instruction> getInstruction(std::size_t i) const { return insts_.at(i); }
  const std::string& name() const { return name_; }

 private:
  std::string name_;
  std::vector<std::shared_ptr<Instruction>> insts_;
};

class InstructionIterator {
 public:
  explicit InstructionIterator(std::shared_ptr<CompositeInstruction> c) : c_(std::move(c)) {}
  bool hasNext() const { return i_ < c_->nInstructions(); }
  std::shared_ptr<Instruction> next() { return c_->getInstruction(i_++); }

 private:
  std::shared_ptr<CompositeInstruction> c_;
  std::size_t i_ = 0;
};

namespace quantum {
#define GB300_SHIM_GATES(F)                                                                                   \
  F(Identity, "I") F(Hadamard, "H") F(CNOT, "CNOT") F(Rx, "Rx") F(Ry, "Ry") F(Rz, "Rz") F(Swap, "Swap")     \
  F(U, "U") F(X, "X") F(Y, "Y") F(Z, "Z") F(Measure, "Measure") F(CZ, "CZ") F(CPhase, "CPhase")             \
  F(S, "S") F(Sdg, "Sdg") F(T, "T") F(Tdg, "Tdg") F(CY, "CY") F(CH, "CH") F(CRZ, "CRZ") F(iSwap, "iSwap")   \
  F(fSim, "fSim")

#define GB300_FWD(cls, nm) class cls;
GB300_SHIM_GATES(GB300_FWD)
#undef GB300_FWD

class AllGateVisitor {
 public:
  virtual ~AllGateVisitor() = default;
#define GB300_VISIT(cls, nm) \
  virtual void visit(cls&) {}
  GB300_SHIM_GATES(GB300_VISIT)
#undef GB300_VISIT
};

#define GB300_GATE(cls, nm)                                                            \
  class cls : public Instruction {                                                     \
   public:                                                                             \
    explicit cls(std::vector<std::size_t> b, std::vector<double> p = {})               \
        : Instruction(nm, std::move(b), std::move(p)) {}                               \
    void accept(AllGateVisitor& v) override { v.visit(*this); }                        \
  };
GB300_SHIM_GATES(GB300_GATE)
#undef GB300_GATE

// Builds a gate instruction from its XACC name.
std::shared_ptr<Instruction> make_gate(const std::string& name, std::vector<std::size_t> bits,
                                       std::vector<double> params = {});
}  // namespace quantum

// The two NoiseModel calls the noisy visitor makes (ExaTnPmpsVisitor.cpp
// :157-160,838-847): the Kraus channels that follow a gate, and a qubit's
// readout error as (P(meas 0 | prep 1), P(meas 1 | prep 0)).
enum class KrausMatBitOrder { MSB, LSB };
struct NoiseChannelKraus {
  std::vector<std::size_t> noise_qubits;
  std::vector<std::vector<std::vector<std::complex<double>>>> mats;
  KrausMatBitOrder bit_order = KrausMatBitOrder::MSB;
};
class NoiseModel {
 public:
  virtual ~NoiseModel() = default;
  virtual std::vector<NoiseChannelKraus> getNoiseChannels(Instruction& gate) = 0;
  virtual std::pair<double, double> readoutError(std::size_t qubit) = 0;
};
}  // namespace xacc
