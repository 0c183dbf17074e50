"""Extract the device properties of the IBM backend description that the
reference's noisy-visitor tests load (tnqvm/visitors/exatn-mpo/tests/
resources/ibmqx2.json) into ``ibmqx2_backend.json``: per qubit T1, T2 (us)
and the readout probabilities, per gate its error and length (ns), with the
values those tests expect (NoiseModelTester.cpp, ExaTnPmpsTester.cpp).  Run
where the reference tree exists, giving its root as the argument (or in
TNQVM_REFERENCE_ROOT; else a "reference" folder beside the repository):

    python tests/golden/make_backend_properties.py <reference root>
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = (sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TNQVM_REFERENCE_ROOT")
       or os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference"))
SRC = os.path.join(REF, "tnqvm", "visitors", "exatn-mpo", "tests", "resources", "ibmqx2.json")
KEEP_QUBIT = ("T1", "T2", "prob_meas0_prep1", "prob_meas1_prep0")
KEEP_GATE = ("gate_error", "gate_length")


def main():
    doc = json.load(open(SRC))
    qubits = [[p for p in q if p["name"] in KEEP_QUBIT] for q in doc["qubits"]]
    gates = [{"gate": g["gate"], "name": g["name"], "qubits": g["qubits"],
              "parameters": [p for p in g["parameters"] if p["name"] in KEEP_GATE]} for g in doc["gates"]]
    out = {
        "source": "tnqvm/visitors/exatn-mpo/tests/resources/ibmqx2.json (device properties only)",
        "backend": {"backend_name": doc["backend_name"], "qubits": qubits, "gates": gates},
        "expect": {
            "readout": "NoiseModelTester.cpp checkReadout: Measure(q0) alone, P('1') = 0.0154 +- 0.01",
            "gate_time": "NoiseModelTester.cpp checkGateTime: P('1') of X and of H Z H within 0.01",
            "gate_error": "NoiseModelTester.cpp checkGateError: 200 X then Measure, P('1') > 0.1",
            "simple": "ExaTnPmpsTester.cpp checkSimple: 100 X then Measure, P('1') > 0.01",
            "multiple": "ExaTnPmpsTester.cpp checkMultipleQubits: X on q0..q2, 0.8 < P('111') < 0.99",
            "bell": "ExaTnPmpsTester.cpp checkBell: X(q0), CX(q0, q1), 0.8 < P('11') < 0.99"},
    }
    with open(os.path.join(HERE, "ibmqx2_backend.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
