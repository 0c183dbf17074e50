"""GPU parity of noisy circuits (density programs, MPS_FLAG_DENSITY) against
the dense density-matrix oracle and the MPS oracle on the doubled chain, and
the noisy visitor against the reference's noise-model tests.  Tolerances:
1e-11 for complex128 runs, 2e-5 for complex64 runs; shot statistics at the
reference tests' own tolerances and by chi-square."""
import json
import os

import numpy as np
import pytest

from oracle import density as R
from tnqvm_gb300 import mps as M
from tnqvm_gb300.visitor import AcceleratorBuffer, GpuPmpsVisitor

from .test_oracle_density import _random_circuit, run_doubled_mps, vec_to_rho

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "noise_models.json")))
TOL64 = 1e-11
TOL32 = 2e-5


def record(p, circ, noise=None):
    for name, qs, ps in circ:
        if name == "Kraus":
            p.channel(qs[0], ps)
        elif name == "Measure":
            p.measure(qs[0])
        else:
            p.gate(name, list(qs), list(ps))
            if noise is not None:
                for cq, kraus in noise.channels(name, list(qs)):
                    p.channel(cq, kraus)


@pytest.mark.parametrize("prec,tol", [(M.PREC_FP64, TOL64), (M.PREC_FP32, TOL32)])
@pytest.mark.parametrize("mode", [M.TRUNC_EXATN, M.TRUNC_ITENSOR])
def test_density_exact_vs_dense_oracle(ctx, mode, prec, tol):
    """5 qubits, random U3 layers, long-range CNOTs and random CPTP channels,
    untruncated: the full density matrix, reduced ones, their diagonal, the
    trace and Pauli expectations against the dense oracle."""
    rng = np.random.default_rng(21 + mode)
    n = 5
    circ = _random_circuit(n, 5, rng)
    rho = R.run(n, circ)
    cutoff = -1.0 if mode == M.TRUNC_EXATN else 1e-16
    with M.DensityProgram(ctx, n, 64, cutoff, mode, prec) as p:
        record(p, circ)
        p.submit()
        p.wait()
        assert np.max(np.abs(p.density_matrix(range(n)) - rho)) < tol
        for sel in ([3, 1], [4, 0, 2], [2]):
            assert np.max(np.abs(p.density_matrix(sel) - R.reduced_dm(rho, n, sel))) < tol
            assert np.max(np.abs(p.density_diag(sel) - np.real(np.diag(R.reduced_dm(rho, n, sel))))) < tol
        assert abs(p.norm() - 1.0) < tol
        paulis = ["ZIXYI", "XXXXX", "IYZIZ", "IIIIZ"]
        got = p.expect_pauli(paulis)
        for s, g in zip(paulis, got):
            assert abs(g - R.expect_pauli(rho, n, s)) < tol


@pytest.mark.parametrize("mode,name", [(M.TRUNC_EXATN, "exatn"), (M.TRUNC_ITENSOR, "itensor")])
def test_density_truncated_vs_doubled_chain_oracle(ctx, mode, name):
    """6 qubits (12 sites) at bond cap 8: the engine's truncations of vec(rho)
    against the MPS oracle run on the same doubled chain, same semantics.

    Tolerance: 1e-10, or ten times the oracle's own spread between two
    LAPACK SVD drivers (gesdd, gesvd) where that is larger.  In exatn
    semantics the state is never brought to canonical form and both sites
    keep sqrt(S): the next truncation sees the individual singular vectors,
    not just the kept subspace, and on this noisy chain that makes the run
    ill-conditioned (the two drivers differ by ~3e-7, a 1e-15 relative
    perturbation of every theta moves the result by ~6e-7).  The itensor run
    (canonical form, the state depends on the kept subspace only) agrees with
    both drivers to 1e-15."""
    import scipy.linalg as SL
    rng = np.random.default_rng(33)
    n = 6
    circ = _random_circuit(n, 6, rng)
    cutoff = 1e-12
    ref = run_doubled_mps(n, circ, name, 8, cutoff)
    rho_ref = vec_to_rho(ref.amplitudes(), n)
    alt = run_doubled_mps(n, circ, name, 8, cutoff,
                          svd=lambda t, full_matrices=False: SL.svd(t, full_matrices=False, lapack_driver="gesvd"))
    spread = float(np.max(np.abs(vec_to_rho(alt.amplitudes(), n) - rho_ref)))
    tol = max(1e-10, 10.0 * spread)
    if mode == M.TRUNC_ITENSOR:
        assert spread < 1e-13
    with M.DensityProgram(ctx, n, 8, cutoff, mode, M.PREC_FP64) as p:
        record(p, circ)
        p.submit()
        p.wait()
        assert p.bond_dims() == ref.bond_dims()
        assert np.max(np.abs(p.density_matrix(range(n)) - rho_ref)) < tol
        # the trace sums 2^n diagonal entries, each within tol
        assert abs(p.norm() - np.trace(rho_ref).real) < (1 << n) * tol


def test_density_sampling_chi_square(ctx):
    """Shots of a density program against the exact measured distribution."""
    rng = np.random.default_rng(41)
    n = 4
    circ = _random_circuit(n, 4, rng)
    rho = R.run(n, circ)
    meas = [2, 0, 3]
    probs = R.probabilities(rho, n, meas)
    shots = 40000
    with M.DensityProgram(ctx, n, 64, -1.0, M.TRUNC_EXATN, M.PREC_FP64) as p:
        record(p, circ)
        for q in meas:
            p.measure(q)
        bits = p.sample(shots, seed=7)
        again = p.sample(shots, seed=7)
    assert np.array_equal(bits, again)
    keys = np.zeros(shots, dtype=np.int64)
    for i in range(len(meas)):
        keys |= bits[:, i].astype(np.int64) << i
    obs = np.bincount(keys, minlength=1 << len(meas))
    exp = probs * shots
    m = exp > 5
    chi2 = float(np.sum((obs[m] - exp[m]) ** 2 / exp[m]))
    from scipy.stats import chi2 as C2
    assert C2.sf(chi2, int(m.sum()) - 1) > 1e-3


def _visitor(ctx, n, circ, options, shots=8192):
    v = GpuPmpsVisitor(ctx)
    v.setOptions(options)
    buf = AcceleratorBuffer(n)
    v.initialize(buf, shots)
    v.run(circ)
    v.finalize()
    return buf


def test_pmps_visitor_depolarizing_golden(ctx):
    """JsonNoiseModelTester.cpp checkSimple: X under p = 0.01 depolarizing
    gives density_matrix diag(0.00666667, 0.99333333), imaginary parts 0."""
    g = GOLD["depolarizing"]
    buf = _visitor(ctx, 1, [("X", [0], ()), ("Measure", [0], ())], {"noise-model": g["model"], "seed": 3})
    dm = buf["density_matrix"]
    assert len(dm) == 4
    assert abs(dm[0][0] + dm[3][0] - 1.0) < 1e-6
    for (re, im), want in zip(dm, g["density_matrix_real"]):
        assert abs(re - want) < g["tolerance"]
        assert abs(im) < 1e-6


def test_pmps_visitor_amplitude_damping_and_readout_golden(ctx):
    """checkSimple (25% amplitude damping: P(0) = 0.25 +- 0.1) and
    checkRoError (P(1|0) = 0.1, P(0|1) = 0.2, +- 0.05)."""
    g = GOLD["amplitude_damping"]
    buf = _visitor(ctx, 1, [("X", [0], ()), ("Measure", [0], ())], {"noise-model": g["model"], "seed": 5})
    assert abs(buf["density_matrix"][0][0] - 0.25) < 1e-12
    assert abs(buf.computeMeasurementProbability("0") - g["probabilities"]["0"]) < g["tolerance"]
    assert abs(buf.computeMeasurementProbability("1") - g["probabilities"]["1"]) < g["tolerance"]
    r = GOLD["readout"]
    buf = _visitor(ctx, 1, [("Measure", [0], ())], {"noise-model": r["model"], "seed": 6})
    assert abs(buf.computeMeasurementProbability("1") - r["prob_1_prep_0"]) < r["tolerance"]
    buf = _visitor(ctx, 1, [("X", [0], ()), ("Measure", [0], ())], {"noise-model": r["model"], "seed": 7})
    assert abs(buf.computeMeasurementProbability("0") - r["prob_0_prep_1"]) < r["tolerance"]


def _depolarizing_model(gates_qubits, p=0.01):
    """JSON model: a depolarizing channel of strength p after each listed
    (gate, qubit)."""
    a, b = np.sqrt(1 - p), np.sqrt(p / 3)
    ks = [[[a, 0], [0, a]], [[0, b], [b, 0]], [[0, -1j * b], [1j * b, 0]], [[b, 0], [0, -b]]]
    mat = [[[[complex(x).real, complex(x).imag] for x in row] for row in k] for k in ks]
    return json.dumps({"gate_noise": [{"gate_name": g, "register_location": [str(q)],
                                       "noise_channels": [{"matrix": mat}]} for g, q in gates_qubits],
                       "bit_order": "MSB"})


def test_pmps_visitor_multiple_qubits_and_bell(ctx):
    """ExaTnPmpsTester.cpp checkMultipleQubits / checkBell with depolarizing
    noise in place of the IBM backend model: the ideal outcome is the most
    common but not certain (0.8 < P < 0.99)."""
    nm = _depolarizing_model([("X", 0), ("X", 1), ("X", 2)], p=0.05)
    circ = [("X", [0], ()), ("X", [1], ()), ("X", [2], ()), ("Measure", [0], ()), ("Measure", [1], ()),
            ("Measure", [2], ())]
    buf = _visitor(ctx, 3, circ, {"noise-model": nm, "seed": 11})
    p = buf.computeMeasurementProbability("111")
    assert 0.8 < p < 0.99
    exact = R.probabilities(R.run(3, circ, noise=R.NoiseModel(nm)), 3, [0, 1, 2])[7]
    assert abs(p - exact) < 0.02
    nm = _depolarizing_model([("X", 0)], p=0.1)
    circ = [("X", [0], ()), ("CNOT", [0, 1], ()), ("Measure", [0], ()), ("Measure", [1], ())]
    buf = _visitor(ctx, 2, circ, {"noise-model": nm, "seed": 12})
    assert 0.8 < buf.computeMeasurementProbability("11") < 0.99


def test_pmps_visitor_ghz_100_qubits(ctx):
    """ExaTnPmpsTester.cpp checkManyQubits: a 100-qubit GHZ chain without
    noise, 6 of 100 qubits measured: P(111111) = P(000000) = 0.5 +- 0.1 from
    1024 shots, and exactly 0.5 on the reduced diagonal."""
    n = 100
    circ = [("H", [0], ())] + [("CNOT", [i, i + 1], ()) for i in range(n - 1)]
    meas = [0, 6, 8, 36, 72, 98]
    circ += [("Measure", [q], ()) for q in meas]
    buf = _visitor(ctx, n, circ, {"seed": 13}, shots=1024)
    assert abs(buf.computeMeasurementProbability("111111") - 0.5) < 0.1
    assert abs(buf.computeMeasurementProbability("000000") - 0.5) < 0.1
    dm = np.array(buf["density_matrix"]).reshape(64, 64, 2)
    assert abs(dm[0, 0, 0] - 0.5) < 1e-12 and abs(dm[63, 63, 0] - 0.5) < 1e-12
    # tracing out the other 94 qubits removes the GHZ coherence
    assert abs(dm[0, 63, 0]) < 1e-12 and abs(dm[0, 63, 1]) < 1e-12


def test_density_errors(ctx):
    with M.Program(ctx, 3) as p:
        with pytest.raises(M.MpsError) as e:
            p.channel(0, [np.eye(2)])
        assert e.value.code == M.ERR_STATE
    with M.DensityProgram(ctx, 14) as p:
        p.gate("H", [0])
        with pytest.raises(M.MpsError) as e:
            p.amplitudes()
        assert e.value.code == M.ERR_UNSUPPORTED
        with pytest.raises(M.MpsError) as e:
            p.density_matrix(range(14))
        assert e.value.code == M.ERR_UNSUPPORTED
        with pytest.raises(M.MpsError) as e:
            p.set_observable(["Z" * 14], [1.0])
        assert e.value.code == M.ERR_UNSUPPORTED
        with pytest.raises(M.MpsError) as e:
            p.channel(14, [np.eye(2)])
        assert e.value.code == M.ERR_ARG
        with pytest.raises(M.MpsError) as e:
            M.Graph(ctx, [p])
        assert e.value.code == M.ERR_UNSUPPORTED
        assert abs(p.norm() - 1.0) < 1e-12


@pytest.mark.parametrize("mode", [M.TRUNC_EXATN, M.TRUNC_ITENSOR])
def test_density_site_parallel_equals_one_op_at_a_time(ctx, mode):
    """Density programs run site-parallel (the noisy visitor's default): the
    same density matrix, bit for bit, as the same kernel one op at a time."""
    rng = np.random.default_rng(55)
    n = 5
    circ = _random_circuit(n, 5, rng)
    outs = []
    for width in (1, 0):
        M.set_parallel_width(width)
        try:
            with M.DensityProgram(ctx, n, 16, 1e-12, mode, M.PREC_FP64, M.FLAG_PARALLEL) as p:
                record(p, circ)
                p.submit()
                p.wait()
                outs.append((p.density_matrix(range(n)), p.bond_dims()))
        finally:
            M.set_parallel_width(0)
    assert outs[0][1] == outs[1][1]
    assert np.array_equal(outs[0][0], outs[1][0])


def test_pmps_visitor_ibm_backend_reference_checks(ctx):
    """The reference's IBM-backend noise tests through the noisy visitor with
    the ibmqx2 description as ``backend-json`` (NoiseModelTester.cpp
    checkReadout, checkGateTime, checkGateError; ExaTnPmpsTester.cpp
    checkSimple, checkMultipleQubits, checkBell), 8192 shots each, at the
    tests' own tolerances."""
    backend = json.load(open(os.path.join(HERE, "golden", "ibmqx2_backend.json")))["backend"]
    text = json.dumps(backend)

    def p(n, circ, key, seed):
        buf = _visitor(ctx, n, circ, {"backend-json": text, "seed": seed}, shots=8192)
        return buf.computeMeasurementProbability(key)

    m0, m1, m2 = ("Measure", [0], ()), ("Measure", [1], ()), ("Measure", [2], ())
    x = ("X", [0], ())
    assert abs(p(1, [m0], "1", 1) - 0.0154) < 0.01
    hzh = [("H", [0], ()), ("Z", [0], ()), ("H", [0], ()), m0]
    assert abs(p(1, [x, m0], "1", 2) - p(1, hzh, "1", 3)) < 0.01
    assert p(1, [x] * 200 + [m0], "1", 4) > 0.1
    assert p(1, [x] * 100 + [m0], "1", 5) > 0.01
    assert 0.8 < p(3, [("X", [0], ()), ("X", [1], ()), ("X", [2], ()), m0, m1, m2], "111", 6) < 0.99
    assert 0.8 < p(2, [x, ("CNOT", [0, 1], ()), m0, m1], "11", 7) < 0.99
