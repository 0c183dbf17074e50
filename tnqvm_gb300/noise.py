"""Noise models for the noisy-circuit visitor (``gb300-pmps``).

The reference's purified-MPS visitor asks an XACC ``NoiseModel`` for the
Kraus channels that follow each gate (``getNoiseChannels``,
``visitors/exatn-mpo/ExaTnPmpsVisitor.cpp:838-847,875-884``) and for the
readout error of each measured qubit (``readoutError``, ``:157-160``).  XACC
is not part of this project, so ``JsonNoiseModel`` reads the JSON format of
XACC's ``json`` noise-model service, as the reference's tests write it
(``visitors/exatn-mpo/tests/JsonNoiseModelTester.cpp:7-25``):

* ``gate_noise``: entries ``{"gate_name", "register_location": ["q", ...],
  "noise_channels": [{"matrix": [K_0, K_1, ...]}]}``, each ``K`` a matrix of
  ``[re, im]`` pairs;
* ``readout_errors``: entries ``{"register_location": "q",
  "prob_meas0_prep1", "prob_meas1_prep0"}``;
* ``bit_order`` (``MSB`` / ``LSB``) only matters for multi-qubit channels,
  which the visitor skips as the reference does (``convertNoiseChannel``
  ``:797-818``).

Any object with the same two methods (``channels(name, qubits)`` and
``readout_error(qubit)``) can stand in for it.
"""
import json

import numpy as np

_ALIASES = {"CX": "CNOT", "CNOT": "CNOT", "U3": "U", "U": "U"}


def _canon(name):
    return _ALIASES.get(name, name)


class JsonNoiseModel:
    def __init__(self, text):
        doc = json.loads(text) if isinstance(text, (str, bytes)) else dict(text)
        self.bit_order = doc.get("bit_order", "MSB")
        self._gate = {}
        for e in doc.get("gate_noise", []):
            key = (_canon(e["gate_name"]), tuple(int(x) for x in e.get("register_location", [])))
            chans = self._gate.setdefault(key, [])
            for ch in e.get("noise_channels", []):
                mats = []
                for k in ch["matrix"]:
                    mats.append(np.array([[complex(v[0], v[1]) for v in row] for row in k], dtype=np.complex128))
                chans.append(mats)
        self._readout = {}
        for e in doc.get("readout_errors", []):
            self._readout[int(e["register_location"])] = (float(e["prob_meas0_prep1"]), float(e["prob_meas1_prep0"]))

    def channels(self, name, qubits):
        """Kraus channels after gate ``name`` on ``qubits``: a list of
        (qubits of the channel, [K_0, K_1, ...])."""
        chans = self._gate.get((_canon(name), tuple(int(q) for q in qubits)), [])
        return [(list(qubits), mats) for mats in chans]

    def readout_error(self, qubit):
        """(P(meas 0 | prep 1), P(meas 1 | prep 0)) of ``qubit``."""
        return self._readout.get(int(qubit), (0.0, 0.0))


# ---------------------------------------------------------------- device model
# The reference's noisy visitor can also build its noise model from an IBM
# backend description (``backend-json``, ExaTnPmpsVisitor.cpp:525-536) through
# XACC's IBM noise-model service, which is not part of the reference.  This
# model restates the common device-noise construction from such a description
# (per-qubit T1 and T2, per-gate error and duration, readout probabilities):
# each gate on a qubit is followed by thermal relaxation for the gate's
# duration, then by a depolarizing channel whose strength makes the combined
# average gate error equal to the reported one.  XACC gates are taken as
# the backend's basis gates: X and Y as one x, H as one sx, Rx, Ry and U as two
# sx, I as id, the Z rotations as the virtual rz (no error, no duration),
# CNOT as cx; CZ as cx with an sx before and after on the target; Swap as three
# cx.  A two-qubit gate adds thermal relaxation on both qubits for its
# duration; its two-qubit depolarizing part is a multi-qubit channel, which
# the visitor skips as the reference does (convertNoiseChannel :797-818).

def thermal_relaxation_kraus(t, t1, t2):
    """Kraus operators of relaxation for time t: rho00 += p rho11, rho11 *=
    1 - p with p = 1 - exp(-t/T1), coherences times exp(-t/T2) (T2 capped at
    2 T1): amplitude damping, then phase damping for the rest of the T2
    decay."""
    if t <= 0.0:
        return [np.eye(2, dtype=np.complex128)]
    t2 = min(t2, 2.0 * t1)
    p = 1.0 - np.exp(-t / t1)
    lam = np.exp(-t / t2) / np.sqrt(1.0 - p)  # <= 1 since T2 <= 2 T1
    amp = [np.array([[1, 0], [0, np.sqrt(1 - p)]], dtype=np.complex128),
           np.array([[0, np.sqrt(p)], [0, 0]], dtype=np.complex128)]
    pha = [np.sqrt((1 + lam) / 2) * np.eye(2, dtype=np.complex128),
           np.sqrt((1 - lam) / 2) * np.diag([1.0, -1.0]).astype(np.complex128)]
    return [b @ a for b in pha for a in amp]


def process_fidelity(kraus):
    """|Tr K|^2 summed over the Kraus operators, over d^2 (d = 2)."""
    return float(sum(abs(np.trace(k)) ** 2 for k in kraus)) / 4.0


def depolarizing_for(error, relax):
    """Depolarizing strength p (rho -> (1-p) rho + p I/2) that, after the
    relaxation channel, gives the average gate error ``error``: the process
    fidelity of Dep(p) after E is (1-p) F_E + p/4, and the average gate
    fidelity of a qubit channel is (2 F_pro + 1) / 3."""
    f_e = process_fidelity(relax)
    f_target = 1.0 - 1.5 * error
    if f_e <= 0.25:
        return 0.0
    return float(min(max((f_e - f_target) / (f_e - 0.25), 0.0), 1.0))


def depolarizing_kraus(p):
    s = np.sqrt(p / 4.0)
    return [np.sqrt(1.0 - 0.75 * p) * np.eye(2, dtype=np.complex128),
            s * np.array([[0, 1], [1, 0]], dtype=np.complex128),
            s * np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
            s * np.diag([1.0, -1.0]).astype(np.complex128)]


_BASIS = {"X": ["x"], "Y": ["x"], "H": ["sx"], "Rx": ["sx", "sx"], "Ry": ["sx", "sx"], "U": ["sx", "sx"],
          "U3": ["sx", "sx"], "I": ["id"], "Identity": ["id"]}
_VIRTUAL = {"Rz", "Z", "S", "Sdg", "T", "Tdg", "Measure"}


class BackendNoiseModel:
    """Noise of an IBM backend description (``qubits``: per-qubit property
    lists with T1 and T2 in us and the readout probabilities; ``gates``:
    per-gate ``gate_error`` and ``gate_length`` in ns)."""

    def __init__(self, text):
        doc = json.loads(text) if isinstance(text, (str, bytes)) else dict(text)
        self.t1, self.t2, self._readout = {}, {}, {}
        for q, props in enumerate(doc.get("qubits", [])):
            vals = {p["name"]: float(p["value"]) for p in props}
            self.t1[q] = vals.get("T1", float("inf")) * 1e3  # us -> ns
            self.t2[q] = vals.get("T2", float("inf")) * 1e3
            self._readout[q] = (vals.get("prob_meas0_prep1", 0.0), vals.get("prob_meas1_prep0", 0.0))
        self._gate = {}
        for g in doc.get("gates", []):
            vals = {p["name"]: float(p["value"]) for p in g.get("parameters", [])}
            self._gate[(g["gate"], tuple(int(q) for q in g["qubits"]))] = (vals.get("gate_error", 0.0),
                                                                          vals.get("gate_length", 0.0))

    def _one_qubit(self, gate, q):
        err, length = self._gate.get((gate, (q,)), (0.0, 0.0))
        relax = thermal_relaxation_kraus(length, self.t1.get(q, float("inf")), self.t2.get(q, float("inf")))
        p = depolarizing_for(err, relax)
        out = []
        if length > 0.0:
            out.append(([q], relax))
        if p > 0.0:
            out.append(([q], depolarizing_kraus(p)))
        return out

    def _cx(self, a, b):
        _, length = self._gate.get(("cx", (a, b)), self._gate.get(("cx", (b, a)), (0.0, 0.0)))
        out = []
        for q in (a, b):
            if length > 0.0:
                out.append(([q], thermal_relaxation_kraus(length, self.t1.get(q, float("inf")),
                                                          self.t2.get(q, float("inf")))))
        return out

    def channels(self, name, qubits):
        """Single-qubit channels after gate ``name`` on ``qubits``."""
        qs = [int(q) for q in qubits]
        name = _canon(name)
        if name in _VIRTUAL:
            return []
        if name in _BASIS:
            out = []
            for g in _BASIS[name]:
                out += self._one_qubit(g, qs[0])
            return out
        if name == "CNOT":
            return self._cx(qs[0], qs[1])
        if name == "CZ":
            return self._one_qubit("sx", qs[1]) + self._cx(qs[0], qs[1]) + self._one_qubit("sx", qs[1])
        if name == "Swap":
            return self._cx(qs[0], qs[1]) + self._cx(qs[1], qs[0]) + self._cx(qs[0], qs[1])
        return []

    def readout_error(self, qubit):
        return self._readout.get(int(qubit), (0.0, 0.0))
