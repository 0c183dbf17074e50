"""Dense density-matrix oracle for noisy circuits (test infrastructure only).

Restates what the reference's purified-MPS visitor
``tnqvm/visitors/exatn-mpo/ExaTnPmpsVisitor.cpp`` computes, as exact dense
linear algebra on ``rho`` (2^n x 2^n, complex128, n small):

* a gate: ``rho -> U rho U^H`` (``applySingleQubitGate`` ``:820-848``,
  ``applyTwoQubitGate`` ``:850-885``), with the gate matrices of
  ``oracle.gates``;
* after each gate, that gate's single-qubit Kraus channels from the noise
  model: ``rho -> sum_k K_k rho K_k^H`` (``applyKrausOp`` ``:887-907``,
  ``applyLocalKrausOp`` ``:909-1130``); channels on more than one qubit are
  ignored (``convertNoiseChannel`` ``:797-818``);
* ``finalize`` (``:658-795``): the density matrix of all qubits when
  ``n <= 15``, else the reduced density matrix of the measured qubits;
* shots (``generateResultBitString`` ``:133-171``): a CDF walk over the
  diagonal, then each measured bit flipped with the noise model's readout
  probability ``P(meas0|prep1)`` or ``P(meas1|prep0)``.

Index convention: qubit ``q`` is bit ``q`` of a row or column index of
``rho`` (the state-vector convention of ``oracle.dense``).  A bit string has
one character per measured qubit, in measure order.

The JSON noise-model reader follows the format of the reference's noise-model
test strings (``visitors/exatn-mpo/tests/JsonNoiseModelTester.cpp:7-25``):
``gate_noise`` entries with ``gate_name``, ``register_location`` and
``noise_channels[].matrix`` (a list of Kraus matrices of ``[re, im]``
pairs), optional ``readout_errors`` entries with ``register_location``,
``prob_meas0_prep1`` and ``prob_meas1_prep0``.
"""
import json

import numpy as np

from . import gates as G
from . import dense as D


def zero_rho(n):
    rho = np.zeros((1 << n, 1 << n), dtype=np.complex128)
    rho[0, 0] = 1.0
    return rho


def apply_1q(rho, n, q, m):
    """U rho U^H with U acting on qubit q."""
    r = np.stack([D.apply_1q(rho[:, j], n, q, m) for j in range(rho.shape[1])], axis=1)
    r = np.stack([D.apply_1q(r[i, :].conj(), n, q, m) for i in range(r.shape[0])], axis=0).conj()
    return r


def apply_2q(rho, n, a, b, m):
    r = np.stack([D.apply_2q(rho[:, j], n, a, b, m) for j in range(rho.shape[1])], axis=1)
    r = np.stack([D.apply_2q(r[i, :].conj(), n, a, b, m) for i in range(r.shape[0])], axis=0).conj()
    return r


def apply_channel(rho, n, q, kraus):
    """sum_k K_k rho K_k^H on qubit q (applyLocalKrausOp :909-1130)."""
    out = np.zeros_like(rho)
    for k in kraus:
        out += apply_1q(rho, n, q, np.asarray(k, dtype=np.complex128))
    return out


def run(n, circuit, noise=None):
    """``circuit``: ``[(name, qubits, params), ...]`` gates (Measure skipped)
    or ``("Kraus", [q], kraus_list)`` channels.  ``noise``: a NoiseModel whose
    channels follow each matching gate."""
    rho = zero_rho(n)
    for name, qs, ps in circuit:
        if name == "Measure":
            continue
        if name == "Kraus":
            rho = apply_channel(rho, n, qs[0], ps)
            continue
        m = G.matrix(name, ps)
        if len(qs) == 1:
            rho = apply_1q(rho, n, qs[0], m)
        else:
            rho = apply_2q(rho, n, qs[0], qs[1], m)
        if noise is not None:
            for cq, kraus in noise.channels(name, qs):
                rho = apply_channel(rho, n, cq, kraus)
    return rho


def reduced_dm(rho, n, keep):
    """Reduced density matrix over ``keep`` by explicit summation (bit i of
    the index = qubit keep[i])."""
    k = len(keep)
    dim = 1 << n
    out = np.zeros((1 << k, 1 << k), dtype=np.complex128)
    idx = np.arange(dim, dtype=np.int64)
    key = np.zeros(dim, dtype=np.int64)
    for i, q in enumerate(keep):
        key |= ((idx >> q) & 1) << i
    rest_mask = 0
    for q in range(n):
        if q not in keep:
            rest_mask |= 1 << q
    rest = idx & rest_mask
    for a in range(dim):
        same = rest == rest[a]
        out[key[a], key[same]] += rho[a, same]
    return out


def expect_pauli(rho, n, pauli):
    """Tr(rho P) / Tr(rho); character i of ``pauli`` acts on qubit i."""
    r = rho
    for q, c in enumerate(pauli):
        if c != "I":
            r = np.stack([D.apply_1q(r[:, j], n, q, G.PAULI[c]) for j in range(r.shape[1])], axis=1)
    return complex(np.trace(r) / np.trace(rho))


def probabilities(rho, n, bits):
    """Diagonal of the reduced density matrix of ``bits`` (index bit i =
    qubit bits[i]) normalised by the trace."""
    d = np.real(np.diag(rho))
    return D.probabilities(np.sqrt(np.maximum(d, 0.0)), bits) / np.sum(d)


def readout_probabilities(p, bits, readout):
    """Apply per-qubit readout flips to a distribution over ``bits``:
    ``readout[q] = (P(meas0|prep1), P(meas1|prep0))``."""
    out = np.asarray(p, dtype=np.float64).copy()
    for i, q in enumerate(bits):
        if q not in readout:
            continue
        m0p1, m1p0 = readout[q]
        new = np.zeros_like(out)
        idx = np.arange(out.size)
        b = (idx >> i) & 1
        flip = idx ^ (1 << i)
        stay = np.where(b == 1, 1.0 - m0p1, 1.0 - m1p0)
        go = np.where(b == 1, m0p1, m1p0)
        new += out * stay
        np.add.at(new, flip, out * go)
        out = new
    return out


class NoiseModel:
    """JSON noise model: Kraus channels per (gate name, qubits) and readout
    errors per qubit (the format of JsonNoiseModelTester.cpp:7-25)."""

    def __init__(self, text):
        doc = json.loads(text) if isinstance(text, str) else text
        self.gate_noise = []
        for e in doc.get("gate_noise", []):
            qs = [int(x) for x in e.get("register_location", [])]
            chans = []
            for ch in e.get("noise_channels", []):
                mats = [np.array([[complex(v[0], v[1]) for v in row] for row in k], dtype=np.complex128)
                        for k in ch["matrix"]]
                chans.append(mats)
            self.gate_noise.append((e["gate_name"], qs, chans))
        self.readout = {}
        for e in doc.get("readout_errors", []):
            self.readout[int(e["register_location"])] = (float(e["prob_meas0_prep1"]), float(e["prob_meas1_prep0"]))

    def channels(self, name, qubits):
        """Single-qubit Kraus channels that follow gate ``name`` on
        ``qubits`` (multi-qubit channels are skipped, as convertNoiseChannel
        :797-818 does)."""
        out = []
        names = {name}
        if name in ("CNOT", "CX"):
            names = {"CNOT", "CX"}
        for gname, qs, chans in self.gate_noise:
            if gname not in names or list(qs) != list(qubits):
                continue
            for mats in chans:
                if mats[0].shape == (2, 2):
                    out.append((qs[0] if len(qs) == 1 else None, mats))
        return [(q, m) for q, m in out if q is not None]
