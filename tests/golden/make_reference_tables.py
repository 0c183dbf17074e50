"""Extract the hard-coded expectation tables of the reference's
ExatnExpValSumReduceTester (tnqvm/tests/ExatnExpValSumReduceTester.cpp) into
``reference_tables.json``, so the tests can pin the oracle and the engine to
them without the reference tree.  Run where the reference tree exists, giving
its root as the argument (or in TNQVM_REFERENCE_ROOT; else a "reference"
folder beside the repository is used):

    python tests/golden/make_reference_tables.py <reference root>
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = (sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TNQVM_REFERENCE_ROOT")
       or os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference"))
SRC = os.path.join(REF, "tnqvm", "tests", "ExatnExpValSumReduceTester.cpp")


def main():
    text = open(SRC).read()
    blocks = re.findall(r"expectedResults\{(.*?)\};", text, re.S)
    tables = [[float(x) for x in re.findall(r"[-+]?\d*\.?\d+(?:e[-+]?\d+)?", b)] for b in blocks]
    assert [len(t) for t in tables] == [20, 400], [len(t) for t in tables]
    out = {
        "source": "tnqvm/tests/ExatnExpValSumReduceTester.cpp",
        "deuteron_x0x1": {
            "test": "testDeuteron: X(0); Ry(1, t); CX(1, 0); H(0); H(1); <Z0 Z1>, t = linspace(-pi, pi, 20)",
            "tolerance": 1e-6, "values": tables[0]},
        "deuteron_h3_x0x1": {
            "test": "testDeuteronH3: X(0); exp_i_theta(t0, 0.5 X0 Y1 - 0.5 Y0 X1); "
                    "exp_i_theta(t1, 0.5 X0 Z1 Y2 - 0.5 X2 Z1 Y0); H(0); H(1); <Z0 Z1>, "
                    "t0 (outer) and t1 (inner) = linspace(-pi, pi, 20)",
            "tolerance": 1e-6, "values": tables[1]},
    }
    with open(os.path.join(HERE, "reference_tables.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
