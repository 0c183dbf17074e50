"""Site-parallel runs (MPS_FLAG_PARALLEL): one circuit's two-site updates on
disjoint sites run on different SMs at once.  Every update reads only its
own sites and the bonds around them, so a run on many CTAs must equal, bit
for bit, the same kernel run one op at a time (width 1).  Against the
oracle the usual complex128 tolerances apply where the run is well
conditioned: itensor semantics, exact runs, and the workload's HEA circuits
in exatn semantics (two LAPACK drivers agree on their energies to 1e-15).
Heavily truncated random circuits in exatn semantics are not: there the
two drivers' amplitudes differ by ~25 % of the largest (no canonical form,
sqrt(S) on both sites), so only the bitwise comparison applies."""
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


def run(ctx, n, circ, chi, cutoff, mode, prec, flags, width=0):
    M.set_parallel_width(width)
    try:
        p = M.Program(ctx, n, chi, cutoff, mode, prec, flags)
        p.run(circ)
        p.submit()
        p.wait()
    finally:
        M.set_parallel_width(0)
    return p


@pytest.mark.parametrize("prec", [M.PREC_FP64, M.PREC_FP32])
@pytest.mark.parametrize("mode", [M.TRUNC_EXATN, M.TRUNC_ITENSOR])
@pytest.mark.parametrize("chi", [8, 64])
def test_parallel_equals_one_op_at_a_time_bitwise(ctx, mode, prec, chi):
    n = 14
    circ = random_circuit(n, 10, seed=100 + chi + 7 * mode)
    F = M.FLAG_PARALLEL
    with run(ctx, n, circ, chi, 1e-12, mode, prec, F, width=1) as a, \
            run(ctx, n, circ, chi, 1e-12, mode, prec, F) as b, \
            run(ctx, n, circ, chi, 1e-12, mode, prec, F) as c:
        assert a.bond_dims() == b.bond_dims() == c.bond_dims()
        assert np.array_equal(a.amplitudes(), b.amplitudes())
        assert np.array_equal(b.amplitudes(), c.amplitudes())
        zs = ["Z" * n, "X" + "I" * (n - 2) + "Y"]
        assert np.array_equal(a.expect_pauli(zs), b.expect_pauli(zs))
        assert a.stats()["gate2"] == b.stats()["gate2"]
        assert abs(a.truncation_fidelity() - b.truncation_fidelity()) < 1e-12


@pytest.mark.parametrize("prec,tol", [(M.PREC_FP64, 1e-12), (M.PREC_FP32, 2e-5)])
def test_parallel_itensor_truncated_vs_oracle_and_batch_kernel(ctx, prec, tol):
    """itensor semantics at bond cap 8 (routed long-range gates): against the
    oracle, and against the persistent batch kernel."""
    n = 12
    circ = random_circuit(n, 8, seed=7)
    ref = omps.run(n, routing.route(circ), "itensor", 8, 1e-12)
    with run(ctx, n, circ, 8, 1e-12, M.TRUNC_ITENSOR, prec, M.FLAG_PARALLEL) as p, \
            run(ctx, n, circ, 8, 1e-12, M.TRUNC_ITENSOR, prec, 0) as q:
        assert p.bond_dims() == ref.bond_dims() == q.bond_dims()
        for s in ("Z" * n, "XY" + "I" * (n - 4) + "ZX"):
            assert abs(p.expect_pauli([s])[0] - ref.expect_pauli(s)) < tol
            assert abs(p.expect_pauli([s])[0] - q.expect_pauli([s])[0]) < tol


def test_parallel_exact_brickwall_exatn(ctx):
    """An exact exatn run (12 qubits, depth 20, cap 64) against the dense
    oracle: brick-wall layers keep n/2 updates independent."""
    n = 12
    circ = circuits.brickwall(n, 20, seed=11)
    psi = dense.run(n, circ)
    with run(ctx, n, circ, 64, 1e-14, M.TRUNC_EXATN, M.PREC_FP64, M.FLAG_PARALLEL) as p:
        assert np.max(np.abs(p.amplitudes() - psi)) < 1e-10


def test_parallel_hea_energy_vs_oracle(ctx):
    """The costliest of 32 hardware-efficient-ansatz instances of the
    batched-VQE workload (Ry/Rz layers, CNOT ladder, cap 64, 50 Pauli terms)
    in exatn semantics: the site-parallel energy equals the one-op-at-a-time
    energy bit for bit and the exatn-mode oracle's to 1e-12."""
    insts = circuits.vqe_batch(32, seed=5)
    inst = max(insts, key=lambda it: it["n"] * it["layers"])
    n = inst["n"]
    ref = omps.run(n, routing.route(inst["circuit"]), "exatn", 64, 1e-12)
    e_ref = sum(c * ref.expect_pauli(s).real for s, c in zip(inst["paulis"], inst["coeffs"])) / ref.norm2()
    F = M.FLAG_PARALLEL
    with run(ctx, n, inst["circuit"], 64, 1e-12, M.TRUNC_EXATN, M.PREC_FP64, F, width=1) as a, \
            run(ctx, n, inst["circuit"], 64, 1e-12, M.TRUNC_EXATN, M.PREC_FP64, F) as b:
        ea = a.expect_pauli(inst["paulis"], inst["coeffs"])[1] / a.norm()
        eb = b.expect_pauli(inst["paulis"], inst["coeffs"])[1] / b.norm()
        assert ea == eb
        assert a.bond_dims() == b.bond_dims() == ref.bond_dims()
        assert abs(eb - e_ref) < 1e-12
