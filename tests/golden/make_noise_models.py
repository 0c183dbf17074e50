"""Extract the JSON noise models of the reference's noisy-visitor tests
(tnqvm/visitors/exatn-mpo/tests/JsonNoiseModelTester.cpp) into
``noise_models.json``, with the values those tests expect, so the oracle and
the engine can be pinned to them without the reference tree.  Run where the
reference tree exists, giving its root as the argument (or in
TNQVM_REFERENCE_ROOT; else a "reference" folder beside the repository):

    python tests/golden/make_noise_models.py <reference root>
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = (sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TNQVM_REFERENCE_ROOT")
       or os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference"))
SRC = os.path.join(REF, "tnqvm", "visitors", "exatn-mpo", "tests", "JsonNoiseModelTester.cpp")


def main():
    text = open(SRC).read()
    models = dict(re.findall(r'const std::string (\w+) =\s*R"\((.*?)\)";', text, re.S))
    for k in ("depol_json", "ad_json", "ro_error_noise_model"):
        json.loads(models[k])
    out = {
        "source": "tnqvm/visitors/exatn-mpo/tests/JsonNoiseModelTester.cpp",
        "depolarizing": {
            "model": models["depol_json"],
            "test": "checkSimple: X(q[0]); Measure(q[0]); density_matrix real parts, imaginary parts 0",
            "density_matrix_real": [0.00666667, 0.0, 0.0, 0.99333333], "tolerance": 1e-6},
        "amplitude_damping": {
            "model": models["ad_json"],
            "test": "checkSimple: X(q[0]); Measure(q[0]); P('0'), P('1') from shots",
            "probabilities": {"0": 0.25, "1": 0.75}, "tolerance": 0.1},
        "readout": {
            "model": models["ro_error_noise_model"],
            "test": "checkRoError: Measure(q[0]) gives P('1') = P(1|0); X(q[0]); Measure(q[0]) gives P('0') = P(0|1)",
            "prob_1_prep_0": 0.1, "prob_0_prep_1": 0.2, "tolerance": 0.05},
    }
    with open(os.path.join(HERE, "noise_models.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
