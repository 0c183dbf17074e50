"""The engine's host gate table and SWAP router (tnqvm_gb300/csrc/gates.hpp,
compiled with g++ into a small driver, no GPU) against the oracle's gate
matrices (Gates.hpp:131-334) and routing (NearestNeighborTransform.hpp:43-135):
matrices to 1e-15, routed gate sequences identical."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import gates as G
from oracle import routing

HERE = os.path.dirname(os.path.abspath(__file__))

ONE = [("H", 0), ("X", 0), ("Y", 0), ("Z", 0), ("S", 0), ("Sdg", 0), ("T", 0), ("Tdg", 0), ("Rx", 1),
       ("Ry", 1), ("Rz", 1), ("U", 3)]
TWO = [("CNOT", 0), ("CX", 0), ("CZ", 0), ("CY", 0), ("CH", 0), ("CRZ", 1), ("CPhase", 1), ("RZZ", 1),
       ("Swap", 0), ("iSwap", 0), ("fSim", 2)]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("hostgates") / "host_gates_check")
    subprocess.run([gxx, "-std=c++17", "-O1", os.path.join(HERE, "host_gates_check.cpp"), "-o", exe], check=True)
    return exe


def _line(name, qs, ps):
    q0 = qs[0]
    q1 = qs[1] if len(qs) > 1 else -1
    p = list(ps) + [0.0] * (3 - len(ps))
    return "%s %d %d %d %.17g %.17g %.17g" % (name, q0, q1, len(ps), p[0], p[1], p[2])


def test_gate_table_matches_oracle(driver):
    rng = np.random.default_rng(11)
    gates = []
    for name, npar in ONE:
        for _ in range(3):
            gates.append((name, (0,), tuple(rng.uniform(-2 * np.pi, 2 * np.pi, npar))))
    for name, npar in TWO:
        for _ in range(3):
            gates.append((name, (0, 1), tuple(rng.uniform(-2 * np.pi, 2 * np.pi, npar))))
    r = subprocess.run([driver], input="\n".join(_line(*g) for g in gates) + "\n", capture_output=True, text=True,
                       check=True)
    lines = r.stdout.strip().splitlines()
    assert len(lines) == len(gates)
    for (name, qs, ps), line in zip(gates, lines):
        f = line.split()
        nq = int(f[0])
        assert nq == len(qs), name
        vals = np.array([float(x) for x in f[1:]])
        got = (vals[0::2] + 1j * vals[1::2]).reshape(2 ** nq, 2 ** nq)
        assert np.max(np.abs(got - G.matrix(name, ps))) < 1e-15, name


def test_unknown_gate_and_wrong_parameter_count(driver):
    lines = [_line("Foo", (0,), ()), _line("Rx", (0,), ()), _line("Measure", (0,), ()), _line("I", (0,), ())]
    r = subprocess.run([driver], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    assert [int(x.split()[0]) for x in r.stdout.strip().splitlines()] == [0, 0, -1, -1]


@pytest.mark.parametrize("seed", range(4))
def test_router_matches_oracle(driver, seed):
    rng = np.random.default_rng(100 + seed)
    n = 12
    circ = []
    for _ in range(60):
        if rng.random() < 0.3:
            circ.append(("U", (int(rng.integers(n)),), tuple(rng.uniform(0, 2 * np.pi, 3))))
        else:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            name, npar = TWO[int(rng.integers(len(TWO)))]
            circ.append((name, (a, b), tuple(rng.uniform(0, 2 * np.pi, npar))))
    want = routing.route(circ)
    r = subprocess.run([driver, "route"], input="\n".join(_line(*g) for g in circ) + "\n", capture_output=True,
                       text=True, check=True)
    got = r.stdout.strip().splitlines()
    assert len(got) == len(want)
    for (name, qs, ps), line in zip(want, got):
        f = line.split()
        nq, q0, q1 = int(f[0]), int(f[1]), int(f[2])
        assert nq == len(qs)
        assert (q0, q1) == (qs[0], qs[1] if len(qs) > 1 else -1)
        vals = np.array([float(x) for x in f[3:]])
        m = (vals[0::2] + 1j * vals[1::2]).reshape(2 ** nq, 2 ** nq)
        assert np.max(np.abs(m - G.matrix(name, ps))) < 1e-15, name
