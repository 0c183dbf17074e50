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
