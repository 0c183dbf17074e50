// GB300 noisy-circuit visitor plugin (see GpuPmpsVisitor.hpp).
#include "GpuPmpsVisitor.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <random>
#include <stdexcept>

namespace tnqvm {

mps_ctx* gb300_context();

GpuPmpsVisitor::GpuPmpsVisitor() = default;

GpuPmpsVisitor::~GpuPmpsVisitor() {
  if (prog_) mps_program_destroy(prog_);
}

void GpuPmpsVisitor::check(int rc, const char* what) const {
  if (rc != MPS_OK) throw std::runtime_error(std::string("gb300-pmps ") + what + ": " + mps_last_error());
}

// ExaTnPmpsVisitor::initialize (:482-542)
void GpuPmpsVisitor::initialize(std::shared_ptr<AcceleratorBuffer> in_buffer, int nbShots) {
  double cutoff = -1.0;
  if (options.keyExists<double>("svd-cutoff")) cutoff = options.get<double>("svd-cutoff");
  int chi = 0;
  if (options.keyExists<int>("max-bond-dim")) chi = options.get<int>("max-bond-dim");
  int mode = MPS_TRUNC_EXATN;
  if (options.keyExists<std::string>("truncation-mode") &&
      options.get<std::string>("truncation-mode") == "itensor")
    mode = MPS_TRUNC_ITENSOR;
  int prec = MPS_PREC_FP64;
  if (options.keyExists<std::string>("precision") && options.get<std::string>("precision") == "fp32")
    prec = MPS_PREC_FP32;
  noise_.reset();
#ifdef GB300MPS_WITH_XACC
  // as ExaTnPmpsVisitor::initialize (:518-536): a NoiseModel object, or the
  // IBM noise-model service initialised from a backend description or name
  if (options.pointerLikeExists<xacc::NoiseModel>("noise-model")) {
    noise_ = xacc::as_shared_ptr(options.getPointerLike<xacc::NoiseModel>("noise-model"));
  } else {
    if (options.stringExists("backend-json")) {
      noise_ = xacc::getService<xacc::NoiseModel>("IBM");
      noise_->initialize({{"backend-json", options.getString("backend-json")}});
    }
    if (options.stringExists("backend")) {
      noise_ = xacc::getService<xacc::NoiseModel>("IBM");
      noise_->initialize({{"backend", options.getString("backend")}});
    }
  }
#else
  if (options.keyExists<std::shared_ptr<xacc::NoiseModel>>("noise-model"))
    noise_ = options.get<std::shared_ptr<xacc::NoiseModel>>("noise-model");
#endif
  buffer = std::move(in_buffer);
  // a noisy simulation always runs shots (:539)
  shots_ = nbShots < 1 ? 1024 : nbShots;
  measured_.clear();
  if (prog_) mps_program_destroy(prog_);
  prog_ = nullptr;
  // the ket and bra halves of a gate, and gates on disjoint qubits, run on
  // different SMs at once (same results); "parallel" false turns it off
  int flags = MPS_FLAG_DENSITY;
  if (!(options.keyExists<bool>("parallel") && !options.get<bool>("parallel"))) flags |= MPS_FLAG_PARALLEL;
  check(mps_program_begin(gb300_context(), (int)buffer->size(), chi, cutoff, mode, prec, flags, &prog_),
        "initialize");
}

// applySingleQubitGate / applyTwoQubitGate (:820-885): the gate, then the
// noise model's channels for it; like convertNoiseChannel (:797-818) only
// single-qubit channels are applied.
void GpuPmpsVisitor::record(xacc::Instruction& g) {
  int q[2] = {0, 0};
  const int nq = (int)g.bits().size();
  for (int i = 0; i < nq && i < 2; ++i) q[i] = (int)g.bits()[i];
  double p[3] = {0, 0, 0};
  const int np = (int)g.nParameters();
  for (int i = 0; i < np && i < 3; ++i) p[i] = g.getParameter(i);
  if (g.name() == "Measure") measured_.push_back(q[0]);
  check(mps_gate_named(prog_, g.name().c_str(), q, nq, p, np), "visit");
  if (!noise_ || g.name() == "Measure") return;
  for (const auto& ch : noise_->getNoiseChannels(g)) {
    if (ch.noise_qubits.size() != 1 || ch.mats.empty() || ch.mats[0].size() != 2) continue;
    std::vector<double> k;
    for (const auto& m : ch.mats)
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
          k.push_back(m[r][c].real());
          k.push_back(m[r][c].imag());
        }
    check(mps_channel1(prog_, (int)ch.noise_qubits[0], (int)ch.mats.size(), k.data()), "channel");
  }
}

#define GB300_VISIT_DEF(cls, nm) \
  void GpuPmpsVisitor::visit(xacc::quantum::cls& g) { record(g); }
GB300_SHIM_GATES(GB300_VISIT_DEF)
#undef GB300_VISIT_DEF

// ExaTnPmpsVisitor::finalize (:658-795)
void GpuPmpsVisitor::finalize() {
  check(mps_submit(prog_), "submit");
  check(mps_wait(prog_, -1), "run");
  if (measured_.empty()) return;
  const int n = (int)buffer->size();
  std::vector<int> sel;
  if (n <= MPS_DM_QUBITS_MAX) {
    for (int q = 0; q < n; ++q) sel.push_back(q);
  } else {
    sel = measured_;
    std::sort(sel.begin(), sel.end());
    sel.erase(std::unique(sel.begin(), sel.end()), sel.end());
    if ((int)sel.size() > MPS_DM_QUBITS_MAX)
      throw std::runtime_error("gb300-pmps: Measure more than " + std::to_string(MPS_DM_QUBITS_MAX) +
                               " is not supported.");
  }
  const size_t dim = (size_t)1 << sel.size();
  std::vector<double> dm(2 * dim * dim);
  check(mps_density_matrix(prog_, (int)sel.size(), sel.data(), dm.data()), "density matrix");
  std::vector<std::pair<double, double>> pairs(dim * dim);
  for (size_t i = 0; i < dim * dim; ++i) pairs[i] = {dm[2 * i], dm[2 * i + 1]};
  buffer->addExtraInfo("density_matrix", pairs);
  // shots from the diagonal, then each measured bit flipped with the readout
  // error (generateResultBitString :133-171)
  uint64_t seed;
  if (options.keyExists<int>("seed"))
    seed = (uint64_t)options.get<int>("seed");
  else
    seed = (uint64_t)std::chrono::steady_clock::now().time_since_epoch().count();
  const int nm = (int)measured_.size();
  std::vector<uint8_t> bits((size_t)shots_ * nm);
  check(mps_sample(prog_, shots_, seed, bits.data()), "sample");
  std::mt19937_64 rng(seed ^ 0x5EEDull);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  std::map<std::string, int> counts;
  for (int s = 0; s < shots_; ++s) {
    std::string key(nm, '0');
    for (int a = 0; a < nm; ++a) {
      bool b = bits[(size_t)s * nm + a] != 0;
      if (noise_) {
        const auto ro = noise_->readoutError((std::size_t)measured_[a]);
        if (u(rng) < (b ? ro.first : ro.second)) b = !b;
      }
      if (b) key[a] = '1';
    }
    counts[key] += 1;
  }
  for (auto& kv : counts) buffer->appendMeasurement(kv.first, kv.second);
  measured_.clear();
}

const double GpuPmpsVisitor::getExpectationValueZ(std::shared_ptr<CompositeInstruction> function) {
  const int n = (int)buffer->size();
  std::string pauli(n, 'I');
  std::map<int, std::pair<char, int>> basis;
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
      throw std::runtime_error("gb300-pmps: unsupported basis-change gate " + inst->name());
    }
  }
  if (!any) return 0.0;
  double v[2];
  check(mps_expect_pauli(prog_, pauli.c_str(), 1, nullptr, v), "getExpectationValueZ");
  return sign * v[0];
}

}  // namespace tnqvm
