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
