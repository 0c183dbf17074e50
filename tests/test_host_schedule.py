"""The site-parallel schedule (site_schedule in the engine: ops by
dependency level, with the count of earlier ops on each of their sites),
checked on the host without a GPU on programs compiled by the engine's own
compiler: every site sees its ops in program order, the dependency counts
are those of the scheduled order, the scheduled ops give the program's
state, and a brick-wall layer's gates share one level."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import dense
from tnqvm_gb300 import circuits

from .test_host_compile import OP_GATE1, OP_MOVE_L, apply_ops

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    from tnqvm_gb300 import build as B
    lib = B.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path_factory.mktemp("hostschedule") / "host_schedule_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", os.path.join(HERE, "host_schedule_check.cu"), "-o", exe, "-L", libdir,
                    "-lgb300mps", "-Xlinker", "-rpath=" + libdir], check=True)
    return exe


def schedule(driver, n, mode, flags, circ):
    lines = ["%d %d %d" % (n, mode, flags)]
    for name, qs, ps in circ:
        p = list(ps) + [0.0] * (3 - len(ps))
        lines.append("%s %d %d %d %.17g %.17g %.17g" % (name, qs[0], qs[1] if len(qs) > 1 else -1, len(ps), *p))
    r = subprocess.run([driver], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    prog, sched, cur = [], [], None
    for line in r.stdout.strip().splitlines():
        f = line.split()
        if f[0] in ("P", "S"):
            cur = prog if f[0] == "P" else sched
            continue
        m = np.array([float(x) for x in f[5:]])
        cur.append((int(f[0]), int(f[1]), int(f[2]), int(f[3]), int(f[4]), m[0::2] + 1j * m[1::2]))
    return prog, sched


def sites_of(op):
    kind, site = op[0], op[1]
    s0 = site - 1 if kind == OP_MOVE_L else site
    return [s0] if kind == OP_GATE1 else [s0, s0 + 1]


def levels(ops, n):
    last = [0] * n
    out = []
    for op in ops:
        ss = sites_of(op)
        lv = 1 + max(last[s] for s in ss)
        for s in ss:
            last[s] = lv
        out.append(lv)
    return out


def random_circuit(n, depth, seed):
    rng = np.random.default_rng(seed)
    c = []
    for _ in range(depth):
        for q in range(n):
            c.append(("U", [q], tuple(rng.uniform(0, 2 * np.pi, 3))))
        for _ in range(n // 2):
            a, b = rng.choice(n, 2, replace=False)
            c.append(("CNOT", [int(a), int(b)], ()))
    return c


@pytest.mark.parametrize("mode,flags", [(0, 0), (1, 0), (1, 4), (0, 8)])
@pytest.mark.parametrize("seed", [3, 4])
def test_schedule_keeps_site_order_and_state(driver, mode, flags, seed):
    n = 8
    circ = random_circuit(n, 5, seed)
    prog, sched = schedule(driver, n, mode, flags, circ)
    assert len(prog) == len(sched)
    # every site sees the same ops in the same order
    for s in range(n):
        a = [op[5] for op in prog if s in sites_of(op)]
        b = [op[5] for op in sched if s in sites_of(op)]
        assert len(a) == len(b) and all(np.array_equal(x, y) for x, y in zip(a, b)), s
    # dependency counts: earlier ops on each site in the scheduled order
    seen = [0] * n
    for op in sched:
        ss = sites_of(op)
        assert op[3] == seen[ss[0]] and op[4] == (seen[ss[1]] if len(ss) == 2 else -1)
        for x in ss:
            seen[x] += 1
    # levels never decrease along the schedule
    lv = levels(sched, n)
    assert lv == sorted(lv)
    # the scheduled ops give the program's state
    ops = lambda L: [(k, s, o, m) for k, s, o, _, _, m in L]
    assert np.max(np.abs(apply_ops(n, ops(sched)) - apply_ops(n, ops(prog)))) < 1e-12
    assert np.max(np.abs(apply_ops(n, ops(prog)) - dense.run(n, circ))) < 1e-12


def test_brick_wall_layers_share_a_level(driver):
    """exatn semantics: a brick wall of depth d on n qubits (each layer
    CNOTs on the even pairs, then on the odd pairs) is 2d levels of
    independent two-site updates (1-qubit gates fused into them)."""
    n, depth = 12, 6
    circ = circuits.brickwall(n, depth, seed=2)
    prog, sched = schedule(driver, n, 0, 0, circ)
    lv = levels(sched, n)
    assert max(lv) == 2 * depth and len(sched) == len(prog)
    assert all(op[0] != OP_GATE1 for op in sched)
