// GB300 MPS visitor plugin (see GpuMpsVisitor.hpp).
#include "GpuMpsVisitor.hpp"

#include <chrono>
#include <cmath>
#include <map>
#include <mutex>
#include <stdexcept>

namespace xacc {
namespace quantum {
std::shared_ptr<Instruction> make_gate(const std::string& name, std::vector<std::size_t> bits,
                                       std::vector<double> params) {
#define GB300_MAKE(cls, nm) \
  if (name == nm) return std::make_shared<cls>(std::move(bits), std::move(params));
  GB300_SHIM_GATES(GB300_MAKE)
#undef GB300_MAKE
  if (name == "CX") return std::make_shared<CNOT>(std::move(bits), std::move(params));
  throw std::invalid_argument("unknown gate " + name);
}
}  // namespace quantum
}  // namespace xacc

namespace tnqvm {

// ExaTnMpsVisitor.cpp:55: below this many qubits the state vector is formed
constexpr int kMaxQubitsForStateVec = 20;

mps_ctx* gb300_context() {
  static std::mutex mu;
  static mps_ctx* ctx = nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!ctx) {
    mps_cfg cfg{0, 0};
    if (mps_ctx_create(&cfg, &ctx) != MPS_OK)
      throw std::runtime_error(std::string("gb300-mps: ") + mps_last_error());
  }
  return ctx;
}

GpuMpsVisitor::GpuMpsVisitor() = default;

GpuMpsVisitor::~GpuMpsVisitor() {
  if (prog_) mps_program_destroy(prog_);
}

void GpuMpsVisitor::check(int rc, const char* what) const {
  // xacc::error in the reference (TNQVM.hpp:106); an exception here
  if (rc != MPS_OK) throw std::runtime_error(std::string("gb300-mps ") + what + ": " + mps_last_error());
}

void GpuMpsVisitor::initialize(std::shared_ptr<AcceleratorBuffer> in_buffer, int nbShots) {
  // Options as read by ExaTnMpsVisitor::initialize (ExaTnMpsVisitor.cpp:257-271)
  double cutoff = -1.0;  // DBL_MIN for exatn semantics
  if (options.keyExists<double>("svd-cutoff")) cutoff = options.get<double>("svd-cutoff");
  int chi = 0;
  if (options.keyExists<int>("max-bond-dim")) chi = options.get<int>("max-bond-dim");
  int mode = MPS_TRUNC_EXATN;
  if (options.keyExists<std::string>("truncation-mode") &&
      options.get<std::string>("truncation-mode") == "itensor")
    mode = MPS_TRUNC_ITENSOR;
  int prec = MPS_PREC_FP64;
  if (options.keyExists<std::string>("precision")) {
    const std::string v = options.get<std::string>("precision");
    if (v == "fp32")
      prec = MPS_PREC_FP32;
    else if (v == "auto")
      prec = MPS_PREC_AUTO;
    else if (v == "split-bf16")
      prec = MPS_PREC_SPLIT_BF16;
  }
  int flags = 0;
  if (options.keyExists<bool>("renormalize") && options.get<bool>("renormalize")) flags |= MPS_FLAG_RENORM;
  if (options.keyExists<bool>("per-gate") && options.get<bool>("per-gate")) flags |= MPS_FLAG_PER_GATE;
  // independent two-site updates on different SMs (default on; same results)
  const bool parallel = !(options.keyExists<bool>("parallel") && !options.get<bool>("parallel"));
  if (parallel && !(flags & MPS_FLAG_PER_GATE)) flags |= MPS_FLAG_PARALLEL;
  // GEMM kernel choice of the wide path (bond caps above 64); no counterpart in
  // the reference: "gemm-tune-cache" loads a saved table and uses it without
  // trial launches, "gemm-autotune" sets the mode (0 static, 1 tune, 2 table)
  if (options.keyExists<std::string>("gemm-tune-cache")) {
    check(mps_autotune_load(options.get<std::string>("gemm-tune-cache").c_str()), "gemm-tune-cache");
    check(mps_autotune_set_mode(2), "gemm-tune-cache");
  }
  if (options.keyExists<int>("gemm-autotune"))
    check(mps_autotune_set_mode(options.get<int>("gemm-autotune")), "gemm-autotune");
  buffer = std::move(in_buffer);
  shots_ = nbShots;
  measured_.clear();
  if (prog_) mps_program_destroy(prog_);
  prog_ = nullptr;
  check(mps_program_begin(gb300_context(), (int)buffer->size(), chi, cutoff, mode, prec, flags, &prog_),
        "initialize");
}

void GpuMpsVisitor::record(xacc::Instruction& g) {
  int q[2] = {0, 0};
  const int nq = (int)g.bits().size();
  for (int i = 0; i < nq && i < 2; ++i) q[i] = (int)g.bits()[i];
  double p[3] = {0, 0, 0};
  const int np = (int)g.nParameters();
  for (int i = 0; i < np && i < 3; ++i) p[i] = g.getParameter(i);
  if (g.name() == "Measure") measured_.push_back(q[0]);  // ExaTnMpsVisitor.cpp:991-994
  check(mps_gate_named(prog_, g.name().c_str(), q, nq, p, np), "visit");
}

#define GB300_VISIT_DEF(cls, nm) \
  void GpuMpsVisitor::visit(xacc::quantum::cls& g) { record(g); }
GB300_SHIM_GATES(GB300_VISIT_DEF)
#undef GB300_VISIT_DEF

void GpuMpsVisitor::sample(int shots) {
  int nm = 0;
  check(mps_n_measured(prog_, &nm), "measure");
  std::vector<uint8_t> bits((size_t)shots * nm);
  uint64_t seed;
  if (options.keyExists<int>("seed"))
    seed = (uint64_t)options.get<int>("seed");
  else
    seed = (uint64_t)std::chrono::steady_clock::now().time_since_epoch().count();
  check(mps_sample(prog_, shots, seed, bits.data()), "sample");
  std::map<std::string, int> counts;
  for (int s = 0; s < shots; ++s) {
    std::string k(nm, '0');
    for (int i = 0; i < nm; ++i)
      if (bits[(size_t)s * nm + i]) k[i] = '1';
    counts[k] += 1;
  }
  for (auto& kv : counts) buffer->appendMeasurement(kv.first, kv.second);
}

// ExaTnMpsVisitor::finalize (ExaTnMpsVisitor.cpp:576-681) on the device MPS.
void GpuMpsVisitor::finalize() {
  check(mps_submit(prog_), "submit");
  check(mps_wait(prog_, -1), "run");
  const int n = (int)buffer->size();
  double st[4];
  check(mps_stats(prog_, st), "stats");
  executionInfo.insert("truncation-fidelity", st[0]);
  executionInfo.insert("max-discarded-weight", st[1]);
  if (options.keyExists<std::vector<int>>("bitstring")) {
    const std::vector<int> bs = options.get<std::vector<int>>("bitstring");
    if ((int)bs.size() != n) throw std::runtime_error("Bitstring size must match the number of qubits.");
    std::vector<int> open;
    for (int i = 0; i < n; ++i)
      if (bs[i] == -1) open.push_back(i);
    if (open.empty()) {
      double a[2];
      check(mps_amplitude(prog_, bs.data(), a), "amplitude");
      buffer->addExtraInfo("amplitude-real", a[0]);
      buffer->addExtraInfo("amplitude-imag", a[1]);
      return;
    }
    std::vector<double> re, im;
    double nrm = 0.0;
    for (long k = 0; k < (1L << open.size()); ++k) {
      std::vector<int> b = bs;
      for (size_t j = 0; j < open.size(); ++j) b[open[j]] = (int)((k >> j) & 1);
      double a[2];
      check(mps_amplitude(prog_, b.data(), a), "amplitude");
      re.push_back(a[0]);
      im.push_back(a[1]);
      nrm += a[0] * a[0] + a[1] * a[1];
    }
    if (nrm > 1e-12)
      for (size_t i = 0; i < re.size(); ++i) {
        re[i] /= std::sqrt(nrm);
        im[i] /= std::sqrt(nrm);
      }
    buffer->addExtraInfo("amplitude-real-vec", re);
    buffer->addExtraInfo("amplitude-imag-vec", im);
    return;
  }
  if (n < kMaxQubitsForStateVec) {
    double nrm = 0.0;
    check(mps_norm(prog_, &nrm), "norm");
    buffer->addExtraInfo("norm", nrm);
    if (!measured_.empty()) {
      if (shots_ < 1) {
        std::string z(n, 'I');
        for (int q : measured_) z[q] = z[q] == 'Z' ? 'I' : 'Z';
        double v[2];
        check(mps_expect_pauli(prog_, z.c_str(), 1, nullptr, v), "exp-val-z");
        buffer->addExtraInfo("exp-val-z", v[0]);
      } else {
        sample(shots_);
      }
    }
  } else if (!measured_.empty()) {
    sample(shots_ < 1 ? 1 : shots_);
  }
}

// VQE mode: the observed circuit is a basis change plus Measure on the
// resident ansatz state (TNQVM.cpp:82-89); the basis change folds into a
// local Pauli evaluated by the transfer-matrix sweep.  Measuring Z after a
// gate U measures U^H Z U: H -> X, and Rx(t)^H Z Rx(t) = cos(t) Z + sin(t) Y,
// so Rx(pi/2) -> +Y and Rx(-pi/2) -> -Y.
const double GpuMpsVisitor::getExpectationValueZ(std::shared_ptr<CompositeInstruction> function) {
  const int n = (int)buffer->size();
  std::string pauli(n, 'I');
  std::map<int, std::pair<char, int>> basis;  // letter and sign per qubit
  int sign = 1;
  bool any = false;
  xacc::InstructionIterator it(function);
  while (it.hasNext()) {
    auto inst = it.next();
    if (!inst->isEnabled()) continue;
    const int q = (int)inst->bits()[0];
    if (inst->name() == "Measure") {
      const auto b = basis.count(q) ? basis[q] : std::make_pair('Z', 1);
      pauli[q] = b.first;
      sign *= b.second;
      any = true;
    } else if (inst->name() == "H") {
      basis[q] = std::make_pair('X', 1);
    } else if (inst->name() == "Rx" && std::abs(std::abs(inst->getParameter(0)) - M_PI / 2) < 1e-12) {
      basis[q] = std::make_pair('Y', inst->getParameter(0) > 0.0 ? 1 : -1);
    } else {
      throw std::runtime_error("gb300-mps: unsupported basis-change gate " + inst->name());
    }
  }
  if (!any) return 0.0;
  double v[2];
  check(mps_expect_pauli(prog_, pauli.c_str(), 1, nullptr, v), "getExpectationValueZ");
  return sign * v[0];
}

const std::vector<std::complex<double>> GpuMpsVisitor::getState() {
  const int n = (int)buffer->size();
  std::vector<std::complex<double>> out((size_t)1 << n);
  check(mps_amplitudes(prog_, reinterpret_cast<double*>(out.data())), "getState");
  return out;
}

}  // namespace tnqvm
