"""Generate golden fixtures from the reference's own itensor-mps arithmetic.

Runs ``oracle/_ref/itensor_driver`` (the vendored ITensor v3 from the
reference tree, built by ``oracle/itensor_driver/Makefile``) on seeded
circuits with truncation active, and writes ``itensor_fixtures.json``:
per case the routed circuit, the bond cap and cutoff, the link dimensions
after the last gate and <P> for a few Pauli strings.  Run here, where the
reference tree exists:

    make -C oracle/itensor_driver && python tests/golden/make_itensor_fixtures.py
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import gates as G  # noqa: E402
from oracle import routing  # noqa: E402
from tnqvm_gb300 import circuits  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "itensor_driver")


def cases():
    rng = np.random.default_rng(77)
    out = []
    out.append(("brickwall8_cnot_chi4", 8, circuits.brickwall(8, 6, seed=1), 4, 1e-10))
    out.append(("brickwall10_cz_chi16_cut1e-6", 10, circuits.brickwall(10, 8, seed=2, entangler="CZ"), 16, 1e-6))
    out.append(("hea12_chi8", 12, circuits.hea(12, 5, seed=3), 8, 1e-12))
    qc, _ = circuits.qaoa_maxcut(8, 2, seed=4)
    out.append(("qaoa8_routed_exact", 8, qc, 16, 1e-14))
    mix = []
    names2 = [("CNOT", ()), ("CZ", ()), ("iSwap", ()), ("Swap", ()), ("CPhase", (0.7,)), ("fSim", (0.4, 0.3)),
              ("CRZ", (1.1,)), ("CY", ()), ("CH", ())]
    for _ in range(40):
        q = int(rng.integers(0, 6))
        mix.append(("U", (q,), tuple(rng.uniform(0, 2 * np.pi, 3))))
        a = int(rng.integers(0, 6))
        b = a + 1 if rng.random() < 0.5 else a - 1
        if 0 <= b < 6:
            nm, ps = names2[int(rng.integers(0, len(names2)))]
            mix.append((nm, (a, b), ps))
    out.append(("mixed6_exact", 6, mix, 64, 1e-14))
    out.append(("supremacy1d_12_exact", 12, circuits.supremacy_1d(12, 6, seed=5), 64, 1e-14))
    out.append(("brickwall12_cnot_chi6", 12, circuits.brickwall(12, 7, seed=9), 6, 1e-12))
    # truncations that land inside a degenerate singular-value subspace keep an
    # arbitrary basis of it, so truncating cases use generic random angles
    return out


def run_driver(n, routed, chi, cutoff, paulis):
    lines = ["%d %d %.17g" % (n, chi, cutoff)]
    for name, qs, ps in routed:
        if name == "Measure":
            continue
        m = G.matrix(name, ps)
        vals = " ".join("%.17g %.17g" % (z.real, z.imag) for z in m.reshape(-1))
        if len(qs) == 1:
            lines.append("G1 %d %s" % (qs[0], vals))
        else:
            lines.append("G2 %d %d %s" % (qs[0], qs[1], vals))
    for p in paulis:
        lines.append("P " + p)
    lines.append("END")
    r = subprocess.run([DRIVER], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    return json.loads(r.stdout)


def main():
    rng = np.random.default_rng(123)
    fixtures = []
    for name, n, circ, chi, cutoff in cases():
        routed = routing.route(circ)
        paulis = ["".join(rng.choice(list("IXYZ"), n)) for _ in range(5)] + ["Z" * n, "I" * n]
        res = run_driver(n, routed, chi, cutoff, paulis)
        fixtures.append({"name": name, "n": n, "chi": chi, "cutoff": cutoff,
                         "circuit": [[g, list(q), list(p)] for g, q, p in routed],
                         "paulis": paulis, "expect": res["paulis"], "bonds": res["bonds"]})
        print(name, res["bonds"])
    with open(os.path.join(HERE, "itensor_fixtures.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_itensor_fixtures.py",
                   "source": "vendored ITensor v3 from tnqvm/visitors/itensor/tpls, driven as "
                             "ITensorMPSVisitor.cpp:288-331", "cases": fixtures}, f, indent=1)


if __name__ == "__main__":
    main()
