"""The engine's host program compiler (compile_program: routing, 1-qubit
fusion, sweep scheduling, gauge moves), called on a host-built program
record and checked without a GPU: the compiled op list applied to a dense
state vector gives the circuit's state (1e-12), exatn semantics has no
centre moves and splits with sqrt(S) on both sides, and itensor semantics
keeps the orthogonality centre on every split pair (ITensorMPSVisitor.cpp:
312-331 gauges with position(site) before each gate)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import dense
from tnqvm_gb300 import circuits

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OP_GATE1, OP_GATE2, OP_MOVE_R, OP_MOVE_L = 0, 1, 2, 3
TO_HI, TO_LO, SQRT = 0, 1, 2


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    from tnqvm_gb300 import build as B
    lib = B.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path_factory.mktemp("hostcompile") / "host_compile_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", os.path.join(HERE, "host_compile_check.cu"), "-o", exe, "-L", libdir,
                    "-lgb300mps", "-Xlinker", "-rpath=" + libdir], check=True)
    return exe


def compile_ops(driver, n, mode, flags, circ):
    lines = ["%d %d %d" % (n, mode, flags)]
    for name, qs, ps in circ:
        p = list(ps) + [0.0] * (3 - len(ps))
        lines.append("%s %d %d %d %.17g %.17g %.17g" % (name, qs[0], qs[1] if len(qs) > 1 else -1, len(ps), *p))
    r = subprocess.run([driver], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    ops = []
    for line in r.stdout.strip().splitlines():
        f = line.split()
        m = np.array([float(x) for x in f[3:]])
        ops.append((int(f[0]), int(f[1]), int(f[2]), m[0::2] + 1j * m[1::2]))
    return ops


def apply_ops(n, ops):
    psi = dense.zero_state(n)
    for kind, site, orient, m in ops:
        if kind == OP_GATE1:
            psi = dense.apply_1q(psi, n, site, m[:4].reshape(2, 2))
        elif kind == OP_GATE2:
            psi = dense.apply_2q(psi, n, site, site + 1, m.reshape(4, 4))
    return psi


def check_structure(ops, mode):
    center = 0
    for kind, site, orient, _ in ops:
        if mode == 0:
            assert kind in (OP_GATE1, OP_GATE2)
            if kind == OP_GATE2:
                assert orient == SQRT
            continue
        if kind == OP_MOVE_R:
            assert site == center
            center += 1
        elif kind == OP_MOVE_L:
            assert site == center
            center -= 1
        elif kind == OP_GATE2:
            assert center in (site, site + 1) and orient in (TO_HI, TO_LO)
            center = site + 1 if orient == TO_HI else site


def mixed_circuit(n, count, seed):
    rng = np.random.default_rng(seed)
    names = [("CNOT", 0), ("CZ", 0), ("iSwap", 0), ("Swap", 0), ("CPhase", 1), ("fSim", 2), ("CRZ", 1), ("CY", 0),
             ("CH", 0), ("RZZ", 1)]
    circ = []
    for _ in range(count):
        if rng.random() < 0.45:
            circ.append(("U", (int(rng.integers(n)),), tuple(rng.uniform(0, 2 * np.pi, 3))))
        else:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            name, npar = names[int(rng.integers(len(names)))]
            circ.append((name, (a, b), tuple(rng.uniform(0, 2 * np.pi, npar))))
    return circ


@pytest.mark.parametrize("mode,flags", [(0, 0), (1, 0), (1, 4), (0, 8), (1, 8), (1, 12)])
@pytest.mark.parametrize("seed", range(3))
def test_compiled_ops_reproduce_the_circuit(driver, mode, flags, seed):
    n = 9
    circ = mixed_circuit(n, 70, seed)
    ops = compile_ops(driver, n, mode, flags, circ)
    check_structure(ops, mode)
    psi = dense.run(n, circ)
    assert np.max(np.abs(apply_ops(n, ops) - psi)) < 1e-12


def test_fusion_and_sweep_counts(driver):
    # a brick wall's 1-qubit layers fold into its 2-qubit gates, so only the
    # 2-qubit gates remain; in sweep order a layer costs at most one move per gate
    n, depth = 10, 6
    circ = circuits.brickwall(n, depth, seed=3)
    n2 = sum(1 for g in circ if len(g[1]) == 2)
    plain = compile_ops(driver, n, 1, 0, circ)
    swept = compile_ops(driver, n, 1, 4, circ)
    for ops in (plain, swept):
        assert sum(1 for o in ops if o[0] == OP_GATE2) == n2
        assert sum(1 for o in ops if o[0] == OP_GATE1) <= n
        check_structure(ops, 1)
        assert np.max(np.abs(apply_ops(n, ops) - dense.run(n, circ))) < 1e-12
    moves = lambda ops: sum(1 for o in ops if o[0] in (OP_MOVE_R, OP_MOVE_L))
    assert moves(swept) <= moves(plain)


def test_fused_routing_cuts_splits(driver):
    """MPS_FLAG_FUSE on the 64-qubit QAOA MaxCut circuit (3-regular graph, p =
    3, RZZ realised as CNOT . Rz . CNOT): cancelling routed SWAP pairs and
    multiplying consecutive gates on one pair leaves the same state (checked
    on a 12-qubit instance against the dense oracle) with far fewer two-site
    splits than NearestNeighborTransform's meet-in-the-middle stream."""
    small, _ = circuits.qaoa_maxcut(n=12, p=2, seed=5)
    for mode in (0, 1):
        ops = compile_ops(driver, 12, mode, 8, small)
        assert np.max(np.abs(apply_ops(12, ops) - dense.run(12, small))) < 1e-12
    big, _ = circuits.qaoa_maxcut(n=64, p=3, seed=7)
    plain = compile_ops(driver, 64, 1, 0, big)
    fused = compile_ops(driver, 64, 1, 8, big)
    n_plain = sum(1 for o in plain if o[0] == OP_GATE2)
    n_fused = sum(1 for o in fused if o[0] == OP_GATE2)
    assert n_fused < 0.6 * n_plain, (n_plain, n_fused)
