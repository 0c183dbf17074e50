"""Site-parallel runs (MPS_FLAG_PARALLEL): one circuit's two-site updates on
disjoint sites run on different SMs at once.  Every update must compute
exactly what it computes in program order, so the results are compared
bit for bit with the sequential run, and with the oracle at the usual
complex128 tolerance."""
import numpy as np
import pytest

from oracle import dense, routing
from oracle import mps as omps
from tnqvm_gb300 import circuits
from tnqvm_gb300 import mps as M

pytestmark = pytest.mark.gpu


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


def run(ctx, n, circ, chi, cutoff, mode, prec, flags):
    p = M.Program(ctx, n, chi, cutoff, mode, prec, flags)
    p.run(circ)
    p.submit()
    p.wait()
    return p


@pytest.mark.parametrize("prec", [M.PREC_FP64, M.PREC_FP32])
@pytest.mark.parametrize("mode", [M.TRUNC_EXATN, M.TRUNC_ITENSOR])
@pytest.mark.parametrize("chi", [8, 64])
def test_parallel_equals_sequential_bitwise(ctx, mode, prec, chi):
    n = 14
    circ = random_circuit(n, 10, seed=100 + chi + 7 * mode)
    cutoff = 1e-12
    with run(ctx, n, circ, chi, cutoff, mode, prec, 0) as a, \
            run(ctx, n, circ, chi, cutoff, mode, prec, M.FLAG_PARALLEL) as b:
        assert a.bond_dims() == b.bond_dims()
        assert np.array_equal(a.amplitudes(), b.amplitudes())
        zs = ["Z" * n, "X" + "I" * (n - 2) + "Y"]
        assert np.array_equal(a.expect_pauli(zs), b.expect_pauli(zs))
        assert a.stats()["gate2"] == b.stats()["gate2"]
        assert abs(a.truncation_fidelity() - b.truncation_fidelity()) < 1e-13


def test_parallel_truncated_vs_oracle(ctx):
    """exatn semantics at bond cap 8 against the oracle, routed long-range
    gates included."""
    n = 12
    circ = random_circuit(n, 8, seed=7)
    ref = omps.run(n, routing.route(circ), "exatn", 8, 1e-12)
    with run(ctx, n, circ, 8, 1e-12, M.TRUNC_EXATN, M.PREC_FP64, M.FLAG_PARALLEL) as p:
        assert p.bond_dims() == ref.bond_dims()
        for s in ("Z" * n, "XY" + "I" * (n - 4) + "ZX"):
            assert abs(p.expect_pauli([s])[0] - ref.expect_pauli(s)) < 1e-12


def test_parallel_hea_ladder_energy(ctx):
    """A hardware-efficient-ansatz circuit of the batched-VQE workload's shape
    (Ry/Rz layers, CNOT ladder, bond cap 64, 50 Pauli terms): same energy
    and amplitudes-free observables as the sequential run, exact to the bit."""
    inst = circuits.vqe_batch(64, seed=5)[0]
    # the costliest instance of a small sample
    insts = circuits.vqe_batch(32, seed=5)
    inst = max(insts, key=lambda it: it["n"] * it["layers"])
    n = inst["n"]
    with run(ctx, n, inst["circuit"], 64, 1e-12, M.TRUNC_EXATN, M.PREC_FP64, 0) as a, \
            run(ctx, n, inst["circuit"], 64, 1e-12, M.TRUNC_EXATN, M.PREC_FP64, M.FLAG_PARALLEL) as b:
        ea = a.expect_pauli(inst["paulis"], inst["coeffs"])[1]
        eb = b.expect_pauli(inst["paulis"], inst["coeffs"])[1]
        assert ea == eb
        assert a.bond_dims() == b.bond_dims()


def test_parallel_brickwall_exact(ctx):
    n = 12
    circ = circuits.brickwall(n, 20, seed=11)
    psi = dense.run(n, circ)
    with run(ctx, n, circ, 64, 1e-14, M.TRUNC_EXATN, M.PREC_FP64, M.FLAG_PARALLEL) as p:
        assert np.max(np.abs(p.amplitudes() - psi)) < 1e-10
