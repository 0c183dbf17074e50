"""The C++ TNQVM visitor plugin (GpuMpsVisitor against the XACC interface
shim): it compiles and links here; on a GPU, circuits driven through it the
way TNQVM::execute does (TNQVM.cpp:106-139) give the oracle's results."""
import json
import subprocess

import numpy as np
import pytest

from oracle import dense
from tnqvm_gb300 import build as B
from tnqvm_gb300 import circuits


def test_plugin_compiles_and_links():
    path = B.build_visitor_demo()
    assert path.endswith("visitor_demo")


def _script(n, shots, circ, opts=(), obs=()):
    lines = ["%d %d" % (n, shots)]
    for k, v in opts:
        lines.append("opt %s %s" % (k, v))
    for prefix, gates in (("", circ), ("obs ", obs)):
        for name, qs, ps in gates:
            lines.append("%s%s %d %s %d %s" % (prefix, name, len(qs), " ".join(map(str, qs)), len(ps),
                                               " ".join("%.17g" % p for p in ps)))
    return "\n".join(lines) + "\n"


def _run(n, shots, circ, opts=(), obs=()):
    exe = B.build_visitor_demo()
    r = subprocess.run([exe], input=_script(n, shots, circ, opts, obs), capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


@pytest.mark.gpu
def test_plugin_exp_val_z_and_norm():
    n = 10
    circ = circuits.brickwall(n, 6, seed=4) + [("Measure", (q,), ()) for q in (0, 3, 7)]
    psi = dense.run(n, circ)
    out = _run(n, 0, circ, [("max-bond-dim", 32), ("svd-cutoff", 1e-14)])
    assert out["name"] == "gb300-mps"
    assert abs(out["norm"] - 1.0) < 1e-10
    assert abs(out["exp-val-z"] - dense.expect_z_parity(psi, [0, 3, 7])) < 1e-10


@pytest.mark.gpu
def test_plugin_sampling_and_itensor_mode():
    circ = [("X", (0,), ()), ("CNOT", (0, 3), ())] + [("Measure", (q,), ()) for q in range(4)]
    out = _run(4, 2000, circ, [("seed", 3), ("truncation-mode", "itensor")])
    assert out["counts"] == {"1001": 2000}
    # GHZ amplitude through the bitstring option (ITensorMPSVisitorTester.cpp:522-551)
    g = [("H", (0,), ()), ("Z", (0,), ()), ("CNOT", (0, 1), ()), ("CNOT", (1, 2), ())]
    psi = dense.run(3, g)
    out = _run(3, 0, g, [("precision", "fp32")])
    assert abs(out["norm"] - np.sum(np.abs(psi) ** 2)) < 1e-6


@pytest.mark.gpu
def test_plugin_wide_bond_cap():
    """max-bond-dim above 64 through the plugin: the splits run on the wide
    path; exp-val-z and the norm match the dense oracle."""
    n = 14
    circ = circuits.brickwall(n, 12, seed=6) + [("Measure", (q,), ()) for q in (1, 6, 12)]
    psi = dense.run(n, circ)
    out = _run(n, 0, circ, [("max-bond-dim", 128), ("svd-cutoff", 1e-14)])
    assert abs(out["norm"] - 1.0) < 1e-10
    assert abs(out["exp-val-z"] - dense.expect_z_parity(psi, [1, 6, 12])) < 1e-10


@pytest.mark.gpu
def test_plugin_vqe_basis_signs():
    """VQE mode through the plugin (TNQVM.cpp:82-89): measuring Z after H is
    <X>, after Rx(pi/2) <Y> and after Rx(-pi/2) -<Y> (Rx(t)^H Z Rx(t) = cos t Z
    + sin t Y)."""
    n = 3
    circ = circuits.hea(n, 2, seed=8)
    psi = dense.run(n, circ)
    for t, sign in ((np.pi / 2, 1.0), (-np.pi / 2, -1.0)):
        obs = [("H", (0,), ()), ("Rx", (2,), (t,)), ("Measure", (0,), ()), ("Measure", (2,), ())]
        out = _run(n, 0, circ, [("truncation-mode", "itensor")], obs)
        want = sign * dense.expect_pauli(psi, n, "XIY").real
        assert abs(out["vqe-exp-val"] - want) < 1e-10, (t, out["vqe-exp-val"], want)


def _noise_lines(model_json):
    """The demo driver's noise-model lines for a JSON noise model."""
    doc = json.loads(model_json)
    lines = []
    for e in doc.get("gate_noise", []):
        qs = [int(x) for x in e["register_location"]]
        for ch in e["noise_channels"]:
            flat = []
            for k in ch["matrix"]:
                for row in k:
                    for v in row:
                        flat += [v[0], v[1]]
            lines.append(("noise", "%s %d %s %d %s" % (e["gate_name"], len(qs), " ".join(map(str, qs)),
                                                      len(ch["matrix"]), " ".join("%.17g" % x for x in flat))))
    for e in doc.get("readout_errors", []):
        lines.append(("readout", "%s %.17g %.17g" % (e["register_location"], e["prob_meas0_prep1"],
                                                     e["prob_meas1_prep0"])))
    return lines


def _run_pmps(n, shots, circ, model_json=None, opts=()):
    exe = B.build_visitor_demo()
    script = _script(n, shots, circ, [("visitor", "pmps")] + list(opts))
    head, rest = script.split("\n", 1)
    extra = "".join("%s %s\n" % kv for kv in (_noise_lines(model_json) if model_json else []))
    r = subprocess.run([exe], input=head + "\n" + extra + rest, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


@pytest.mark.gpu
def test_plugin_pmps_noise_model_goldens():
    """The noisy visitor through the C++ plugin against the reference's
    JsonNoiseModelTester.cpp: depolarizing after X gives density_matrix
    diag(0.00666667, 0.99333333); readout errors P(1|0) = 0.1 +- 0.05."""
    import os
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "noise_models.json")))
    g = gold["depolarizing"]
    out = _run_pmps(1, 1024, [("X", (0,), ()), ("Measure", (0,), ())], g["model"], [("seed", 1)])
    assert out["name"] == "gb300-pmps"
    dm = out["density_matrix"]
    for (re, im), want in zip(dm, g["density_matrix_real"]):
        assert abs(re - want) < g["tolerance"] and abs(im) < 1e-6
    r = gold["readout"]
    out = _run_pmps(1, 8192, [("Measure", (0,), ())], r["model"], [("seed", 2)])
    p1 = out["counts"].get("1", 0) / 8192
    assert abs(p1 - r["prob_1_prep_0"]) < r["tolerance"]
