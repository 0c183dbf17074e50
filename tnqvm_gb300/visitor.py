"""Python mirror of TNQVM's visitor plugin interface for the GB300 MPS engine.

``GpuMpsVisitor`` has the method set of ``tnqvm::TNQVMVisitor``
(``tnqvm/visitors/TNQVMVisitor.hpp:58-82``): ``initialize(buffer, shots)``,
one ``visit`` per gate, ``finalize()``, ``getExpectationValueZ(circuit)``,
``getState()``, ``supportVqeMode()``, ``name()``.  Results go to an
``AcceleratorBuffer`` stand-in with XACC's ``addExtraInfo`` /
``appendMeasurement`` keys (``exp-val-z``, ``norm``, ``amplitude-real``,
``amplitude-imag``, ``amplitude-real-vec``, ``amplitude-imag-vec``).  The C++
plugin (``tnqvm_gb300/visitor/``) is the same logic against the XACC headers.

Options (``setOptions``), as in ``TNQVM::updateConfiguration``
(``tnqvm/TNQVM.hpp:61-125``) and the exatn-mps visitor
(``ExaTnMpsVisitor.cpp:257-271``): ``svd-cutoff`` (default DBL_MIN),
``max-bond-dim`` (default: the build's limit), ``shots``, ``seed``, plus
``truncation-mode`` (``exatn`` | ``itensor``), ``precision`` (``fp64`` |
``fp32``), ``renormalize``, ``per-gate`` (one launch per gate), ``parallel``
(default on: a circuit's two-site updates on disjoint sites run on different
SMs at once; results unchanged), and for bond
caps above 64 ``gemm-autotune`` (0 static, 1 tune, 2 table) and
``gemm-tune-cache`` (a saved tuning table, used without trial launches).
"""
from collections import Counter

import numpy as np

from . import mps as M

MAX_NUMBER_QUBITS_FOR_STATE_VEC = 20   # ExaTnMpsVisitor.cpp:55


class AcceleratorBuffer:
    """Result sink with the XACC AcceleratorBuffer calls the visitors use."""

    def __init__(self, n):
        self.n = n
        self.extra = {}
        self.counts = Counter()

    def size(self):
        return self.n

    def addExtraInfo(self, key, value):
        self.extra[key] = value

    def __getitem__(self, key):
        return self.extra[key]

    def __contains__(self, key):
        return key in self.extra

    def appendMeasurement(self, bits, count=1):
        self.counts[bits] += count

    def getMeasurementCounts(self):
        return dict(self.counts)

    def computeMeasurementProbability(self, bits):
        tot = sum(self.counts.values())
        return self.counts.get(bits, 0) / tot if tot else 0.0

    def getExpectationValueZ(self):
        if "exp-val-z" in self.extra:
            return self.extra["exp-val-z"]
        tot = sum(self.counts.values())
        if tot == 0:
            return 0.0
        e = 0.0
        for k, v in self.counts.items():
            e += (-1.0 if k.count("1") % 2 else 1.0) * v
        return e / tot


_CTX = None


def default_context():
    global _CTX
    if _CTX is None:
        _CTX = M.Context(0)
    return _CTX


class GpuMpsVisitor:
    """``tnqvm-visitor`` name ``gb300-mps``."""

    def __init__(self, ctx=None):
        self.ctx = ctx
        self.options = {}
        self.prog = None
        self.buffer = None
        self.shots = 1
        self.execution_info = {}

    # ---- plugin identity (Identifiable / Cloneable)
    def name(self):
        return "gb300-mps"

    def description(self):
        return "Matrix-product-state simulator on one GB300 GPU (sm_103a kernels)"

    def clone(self):
        v = GpuMpsVisitor(self.ctx)
        v.options = dict(self.options)
        return v

    def supportVqeMode(self):
        return True

    def setOptions(self, options):
        self.options = dict(options)

    def getExecutionInfo(self):
        return dict(self.execution_info)

    # ---- lifecycle
    def initialize(self, buffer, nbShots=1):
        if self.ctx is None:
            self.ctx = default_context()
        o = self.options
        mode = {"exatn": M.TRUNC_EXATN, "itensor": M.TRUNC_ITENSOR}[o.get("truncation-mode", "exatn")]
        prec = {"fp64": M.PREC_FP64, "fp32": M.PREC_FP32, "auto": M.PREC_AUTO,
                "split-bf16": M.PREC_SPLIT_BF16}[o.get("precision", "fp64")]
        flags = (M.FLAG_RENORM if o.get("renormalize", False) else 0) | \
                (M.FLAG_PER_GATE if o.get("per-gate", False) else 0)
        # independent two-site updates on different SMs (default on; same results)
        if o.get("parallel", True) and not (flags & M.FLAG_PER_GATE):
            flags |= M.FLAG_PARALLEL
        cutoff = float(o["svd-cutoff"]) if "svd-cutoff" in o else -1.0
        chi = int(o["max-bond-dim"]) if "max-bond-dim" in o else 0
        # GEMM kernel choice of the wide path (no counterpart in the reference)
        if "gemm-tune-cache" in o:
            M.autotune_load(o["gemm-tune-cache"])
            M.autotune_set_mode(2)
        if "gemm-autotune" in o:
            M.autotune_set_mode(int(o["gemm-autotune"]))
        if self.prog is not None:
            self.prog.close()
        self.buffer = buffer
        self.shots = nbShots
        self.prog = M.Program(self.ctx, buffer.size(), chi, cutoff, mode, prec, flags)
        self.measured = []

    def visit(self, name, qubits, params=()):
        if name == "Measure":
            self.measured.append(qubits[0])
            self.prog.measure(qubits[0])
            return
        self.prog.gate(name, list(qubits), list(params))

    def run(self, circuit):
        for name, qs, ps in circuit:
            self.visit(name, qs, ps)

    def finalize(self):
        """ExaTnMpsVisitor::finalize (ExaTnMpsVisitor.cpp:576-681)."""
        p, buf = self.prog, self.buffer
        n = buf.size()
        p.submit()
        p.wait()
        st = p.stats()
        self.execution_info.update({"truncation-fidelity": st["fidelity"],
                                    "max-discarded-weight": st["max_discarded"]})
        bitstring = self.options.get("bitstring")
        if bitstring is not None:
            self._bitstring(bitstring)
            return
        if n < MAX_NUMBER_QUBITS_FOR_STATE_VEC:
            buf.addExtraInfo("norm", p.norm())
            if self.measured:
                if self.shots < 1:
                    z = "".join("Z" if (self.measured.count(q) % 2) else "I" for q in range(n))
                    buf.addExtraInfo("exp-val-z", float(p.expect_pauli([z])[0].real))
                else:
                    self._sample(self.shots)
        elif self.measured:
            self._sample(max(self.shots, 1))

    def _sample(self, shots):
        seed = int(self.options.get("seed", np.random.SeedSequence().entropy % (1 << 63)))
        bits = self.prog.sample(shots, seed)
        keys = ["".join(map(str, row)) for row in bits]
        for k, v in Counter(keys).items():
            self.buffer.appendMeasurement(k, v)

    def _bitstring(self, bits):
        """``bitstring`` option (ExaTnMpsVisitor.cpp:776-822): -1 marks an open
        qubit; one amplitude, or the normalised slice over the open qubits."""
        n = self.buffer.size()
        if len(bits) != n:
            raise ValueError("Bitstring size must match the number of qubits.")
        open_q = [i for i, b in enumerate(bits) if b == -1]
        if not open_q:
            a = self.prog.amplitude([int(b) for b in bits])
            self.buffer.addExtraInfo("amplitude-real", a.real)
            self.buffer.addExtraInfo("amplitude-imag", a.imag)
            return
        vals = []
        for k in range(1 << len(open_q)):
            b = list(bits)
            for j, q in enumerate(open_q):
                b[q] = (k >> j) & 1
            vals.append(self.prog.amplitude(b))
        v = np.array(vals)
        nrm = float(np.sum(np.abs(v) ** 2))
        if nrm > 1e-12:
            v = v / np.sqrt(nrm)
        self.buffer.addExtraInfo("amplitude-real-vec", list(v.real))
        self.buffer.addExtraInfo("amplitude-imag-vec", list(v.imag))

    def getState(self):
        return self.prog.amplitudes()

    def getExpectationValueZ(self, observed_circuit):
        """VQE mode: ``observed_circuit`` is the basis change plus Measure gates
        of one Pauli term (``TNQVM.cpp:82-89``).  The basis change is folded
        into a local Pauli on the resident MPS instead of re-simulating
        (X basis: H, Y basis: Rx(pi/2), as XACC's observed composites emit).
        Measuring Z after U measures U^H Z U, and Rx(t)^H Z Rx(t) = cos(t) Z +
        sin(t) Y, so Rx(-pi/2) measures -Y."""
        n = self.buffer.size()
        letters = ["I"] * n
        pending = {}
        sign = 1.0
        for name, qs, ps in observed_circuit:
            if name == "Measure":
                q = qs[0]
                letter, s = pending.get(q, ("Z", 1.0))
                letters[q] = letter
                sign *= s
            elif name == "H":
                pending[qs[0]] = ("X", 1.0)
            elif name == "Rx" and abs(abs(ps[0]) - np.pi / 2) < 1e-12:
                pending[qs[0]] = ("Y", 1.0 if ps[0] > 0 else -1.0)
            else:
                raise ValueError("unsupported basis-change gate %s" % name)
        if all(c == "I" for c in letters):
            return 0.0
        v = self.prog.expect_pauli(["".join(letters)])[0]
        return sign * float(v.real)


MAX_QUBITS_FOR_DENSITY_MATRIX = M.DM_QUBITS_MAX   # the reference's bound is 15 (ExaTnPmpsVisitor.cpp:662)


class GpuPmpsVisitor:
    """``tnqvm-visitor`` name ``gb300-pmps``: noisy circuits, the drop-in for
    the purified-MPS visitor ``exatn-pmps``
    (``visitors/exatn-mpo/ExaTnPmpsVisitor.cpp``).  The density matrix is held
    as a vectorised MPS on the GPU (``DensityProgram``); each gate is followed
    by the single-qubit Kraus channels the noise model gives for it
    (``applySingleQubitGate`` / ``applyTwoQubitGate`` ``:820-885``).

    Options: ``noise-model`` (a ``JsonNoiseModel``, any object with its two
    methods, or the JSON text), ``backend-json`` (an IBM backend
    description: ``BackendNoiseModel``, thermal relaxation and depolarizing
    noise from its qubit and gate properties), ``shots`` (default 1024, ``:539``),
    ``seed``, ``max-bond-dim``, ``svd-cutoff``, ``precision``,
    ``truncation-mode``, ``parallel`` (default on: independent two-site
    updates of the doubled chain on different SMs, same results)."""

    def __init__(self, ctx=None):
        self.ctx = ctx
        self.options = {}
        self.prog = None
        self.buffer = None
        self.noise = None
        self.measured = []
        self.shots = 1024

    def name(self):
        return "gb300-pmps"

    def description(self):
        return "Noisy-circuit simulator (density matrix as a vectorised MPS) on one GB300 GPU"

    def clone(self):
        v = GpuPmpsVisitor(self.ctx)
        v.options = dict(self.options)
        return v

    def supportVqeMode(self):
        return False

    def setOptions(self, options):
        self.options = dict(options)

    def initialize(self, buffer, nbShots=1):
        """ExaTnPmpsVisitor::initialize (:482-542)."""
        from .noise import BackendNoiseModel, JsonNoiseModel
        if self.ctx is None:
            self.ctx = default_context()
        o = self.options
        nm = o.get("noise-model")
        if isinstance(nm, (str, bytes)):
            nm = JsonNoiseModel(nm)
        if nm is None and "backend-json" in o:
            nm = BackendNoiseModel(o["backend-json"])
        self.noise = nm
        mode = {"exatn": M.TRUNC_EXATN, "itensor": M.TRUNC_ITENSOR}[o.get("truncation-mode", "exatn")]
        prec = {"fp64": M.PREC_FP64, "fp32": M.PREC_FP32}[o.get("precision", "fp64")]
        cutoff = float(o["svd-cutoff"]) if "svd-cutoff" in o else -1.0
        chi = int(o["max-bond-dim"]) if "max-bond-dim" in o else 0
        if self.prog is not None:
            self.prog.close()
        self.buffer = buffer
        # a noisy simulation always runs shots (:539)
        self.shots = 1024 if nbShots < 1 else nbShots
        # the ket and bra halves of a gate, and gates on disjoint qubits, run on
        # different SMs at once (same results)
        flags = M.FLAG_PARALLEL if o.get("parallel", True) else 0
        self.prog = M.DensityProgram(self.ctx, buffer.size(), chi, cutoff, mode, prec, flags)
        self.measured = []

    def visit(self, name, qubits, params=()):
        if name == "Measure":
            self.measured.append(qubits[0])
            self.prog.measure(qubits[0])
            return
        self.prog.gate(name, list(qubits), list(params))
        if self.noise is None:
            return
        for cq, mats in self.noise.channels(name, list(qubits)):
            # single-qubit channels only (convertNoiseChannel :797-818)
            if len(cq) == 1 and np.asarray(mats[0]).shape == (2, 2):
                self.prog.channel(cq[0], mats)

    def run(self, circuit):
        for name, qs, ps in circuit:
            self.visit(name, qs, ps)

    def finalize(self):
        """ExaTnPmpsVisitor::finalize (:658-795): the density matrix of the
        register (or, for larger registers, of the measured qubits) as
        ``density_matrix`` (row-major (re, im) pairs, row = ket, bit a of an
        index = qubit a of the selection), then the shots drawn from its
        diagonal with each measured bit flipped by the readout error."""
        p, buf = self.prog, self.buffer
        n = buf.size()
        p.submit()
        p.wait()
        if not self.measured:
            return
        meas = list(self.measured)
        if n <= MAX_QUBITS_FOR_DENSITY_MATRIX:
            sel = list(range(n))
        elif len(set(meas)) <= MAX_QUBITS_FOR_DENSITY_MATRIX:
            sel = sorted(set(meas))
        else:
            raise ValueError("Measure more than %d is not supported." % MAX_QUBITS_FOR_DENSITY_MATRIX)
        dm = p.density_matrix(sel)
        # (re, im) rows, one per entry, row-major (a 13-qubit register has 4^13)
        buf.addExtraInfo("density_matrix", np.stack([dm.real.reshape(-1), dm.imag.reshape(-1)], axis=1))
        seed = int(self.options.get("seed", np.random.SeedSequence().entropy % (1 << 63)))
        bits = p.sample(self.shots, seed)
        if self.noise is not None:
            rng = np.random.default_rng(seed ^ 0x5EED)
            u = rng.random(bits.shape)
            for a, q in enumerate(meas):
                m0p1, m1p0 = self.noise.readout_error(q)
                flip = np.where(bits[:, a] == 1, m0p1, m1p0)
                bits[:, a] ^= (u[:, a] < flip).astype(np.uint8)
        keys = ["".join(map(str, row)) for row in bits]
        for k, v in Counter(keys).items():
            buf.appendMeasurement(k, v)
        self.measured = []

    def getExpectationValueZ(self, observed_circuit):
        """<Z...Z> on the measured qubits of ``observed_circuit`` after its
        basis change, as Tr(rho P) / Tr(rho) (the reference returns 0 here,
        :1233-1236)."""
        n = self.buffer.size()
        letters = ["I"] * n
        pending = {}
        sign = 1.0
        for name, qs, ps in observed_circuit:
            if name == "Measure":
                letter, s = pending.get(qs[0], ("Z", 1.0))
                letters[qs[0]] = letter
                sign *= s
            elif name == "H":
                pending[qs[0]] = ("X", 1.0)
            elif name == "Rx" and abs(abs(ps[0]) - np.pi / 2) < 1e-12:
                pending[qs[0]] = ("Y", 1.0 if ps[0] > 0 else -1.0)
            else:
                raise ValueError("unsupported basis-change gate %s" % name)
        if all(c == "I" for c in letters):
            return 0.0
        return sign * float(self.prog.expect_pauli(["".join(letters)])[0].real)
