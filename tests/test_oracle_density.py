"""Noisy-circuit oracle (``oracle/density.py``) pinned to the reference's
noise-model tests, and the vectorised-density mapping the engine uses,
checked on the CPU (no GPU needed)."""
import json
import os

import numpy as np
import pytest

from oracle import dense as D
from oracle import density as R
from oracle import gates as G
from oracle import mps as MO
from oracle import routing

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "noise_models.json")))


def test_depolarizing_golden():
    """JsonNoiseModelTester.cpp checkSimple: X then a depolarizing channel
    (p = 0.01) gives rho = diag(0.00666667, 0.99333333)."""
    g = GOLD["depolarizing"]
    nm = R.NoiseModel(g["model"])
    rho = R.run(1, [("X", [0], ())], noise=nm)
    assert np.allclose(rho.real.reshape(-1), g["density_matrix_real"], atol=g["tolerance"])
    assert np.allclose(rho.imag, 0.0, atol=1e-12)
    assert abs(np.trace(rho) - 1.0) < 1e-12


def test_amplitude_damping_golden():
    """checkSimple, second half: X then 25% amplitude damping: P(0) = 0.25."""
    g = GOLD["amplitude_damping"]
    nm = R.NoiseModel(g["model"])
    rho = R.run(1, [("X", [0], ())], noise=nm)
    p = R.probabilities(rho, 1, [0])
    assert abs(p[0] - 0.25) < 1e-12 and abs(p[1] - 0.75) < 1e-12
    assert abs(p[0] - g["probabilities"]["0"]) < g["tolerance"]


def test_readout_golden():
    """checkRoError: P(1|prep 0) = 0.1, P(0|prep 1) = 0.2 applied to the
    measured distribution."""
    g = GOLD["readout"]
    nm = R.NoiseModel(g["model"])
    p0 = R.readout_probabilities(R.probabilities(R.run(1, []), 1, [0]), [0], nm.readout)
    assert abs(p0[1] - g["prob_1_prep_0"]) < 1e-12
    p1 = R.readout_probabilities(R.probabilities(R.run(1, [("X", [0], ())]), 1, [0]), [0], nm.readout)
    assert abs(p1[0] - g["prob_0_prep_1"]) < 1e-12


def _random_circuit(n, depth, rng, with_channels=True):
    c = []
    for _ in range(depth):
        for q in range(n):
            c.append(("U", [q], tuple(rng.uniform(0, 2 * np.pi, 3))))
        a, b = rng.choice(n, 2, replace=False)
        c.append(("CNOT", [int(a), int(b)], ()))
        if with_channels:
            q = int(rng.integers(n))
            c.append(("Kraus", [q], random_channel(rng)))
    return c


def random_channel(rng, k=3):
    """A random CPTP map: K_k = A_k S^{-1/2} with S = sum A_k^H A_k."""
    a = rng.normal(size=(k, 2, 2)) + 1j * rng.normal(size=(k, 2, 2))
    s = sum(x.conj().T @ x for x in a)
    w, v = np.linalg.eigh(s)
    sm = v @ np.diag(w ** -0.5) @ v.conj().T
    return [x @ sm for x in a]


def test_noiseless_density_is_the_pure_state():
    rng = np.random.default_rng(3)
    n = 4
    circ = _random_circuit(n, 4, rng, with_channels=False)
    psi = D.run(n, circ)
    rho = R.run(n, circ)
    assert np.allclose(rho, np.outer(psi, psi.conj()), atol=1e-12)
    for pauli in ("ZIXY", "XXYZ", "IIIZ"):
        assert abs(R.expect_pauli(rho, n, pauli) - D.expect_pauli(psi, n, pauli)) < 1e-12


def test_channels_preserve_trace_and_positivity():
    rng = np.random.default_rng(4)
    n = 3
    rho = R.run(n, _random_circuit(n, 5, rng))
    assert abs(np.trace(rho) - 1.0) < 1e-12
    assert np.allclose(rho, rho.conj().T, atol=1e-13)
    assert np.linalg.eigvalsh(rho).min() > -1e-12


def test_reduced_density_matrix():
    rng = np.random.default_rng(5)
    n = 4
    rho = R.run(n, _random_circuit(n, 4, rng))
    red = R.reduced_dm(rho, n, [2, 0])
    # C-order axes of a row or column index: (q3, q2, q1, q0)
    t = rho.reshape([2] * 8)
    t2 = np.einsum("abcdaBcD->bdBD", t)  # keep q2 and q0; trace q3 and q1
    # bit 0 of the reduced index = qubit 2, bit 1 = qubit 0: index = q2 + 2 q0
    want = np.zeros((4, 4), dtype=np.complex128)
    for b in range(2):
        for d in range(2):
            for B in range(2):
                for Dd in range(2):
                    want[b + 2 * d, B + 2 * Dd] = t2[b, d, B, Dd]
    assert np.allclose(red, want, atol=1e-13)


# ----------------------------------------------------------------------------
# The engine holds vec(rho) as a state of 2n sites: ket of qubit q on site 2q,
# bra on 2q+1; U acts as U on the ket site(s) and conj(U) on the bra site(s),
# a channel as S = sum_k K_k (x) conj(K_k) on (2q, 2q+1).  These helpers
# restate that mapping for the tests (dense on 2n qubits, and the MPS oracle
# on the doubled chain for truncated runs).

def doubled_ops(circuit, noise=None):
    """Gate list on 2n sites (4x4/2x2 matrices) for a noisy circuit."""
    ops = []
    for name, qs, ps in circuit:
        if name == "Measure":
            continue
        if name == "Kraus":
            ops.append((None, [2 * qs[0], 2 * qs[0] + 1], superop(ps)))
            continue
        m = G.matrix(name, ps)
        if len(qs) == 1:
            ops.append((None, [2 * qs[0]], m))
            ops.append((None, [2 * qs[0] + 1], m.conj()))
        else:
            ops.append((None, [2 * qs[0], 2 * qs[1]], m))
            ops.append((None, [2 * qs[0] + 1, 2 * qs[1] + 1], m.conj()))
        if noise is not None:
            for cq, kraus in noise.channels(name, qs):
                ops.append((None, [2 * cq, 2 * cq + 1], superop(kraus)))
    return ops


def superop(kraus):
    s = np.zeros((4, 4), dtype=np.complex128)
    for k in kraus:
        s += np.kron(np.asarray(k), np.asarray(k).conj())
    return s


def vec_to_rho(v, n):
    """Dense doubled-chain state -> rho (qubit q on bit q of row and column)."""
    rho = np.zeros((1 << n, 1 << n), dtype=np.complex128)
    idx = np.arange(v.size)
    x = np.zeros_like(idx)
    y = np.zeros_like(idx)
    for q in range(n):
        x |= ((idx >> (2 * q)) & 1) << q
        y |= ((idx >> (2 * q + 1)) & 1) << q
    rho[x, y] = v
    return rho


def run_doubled_dense(n, circuit, noise=None):
    v = D.zero_state(2 * n)
    for _, qs, m in doubled_ops(circuit, noise):
        if len(qs) == 1:
            v = D.apply_1q(v, 2 * n, qs[0], m)
        else:
            v = D.apply_2q(v, 2 * n, qs[0], qs[1], m)
    return vec_to_rho(v, n)


def run_doubled_mps(n, circuit, mode, chi, cutoff, noise=None, svd=None):
    """The MPS oracle on the doubled chain, long-range pairs routed as the
    engine routes them (NearestNeighborTransform order)."""
    mps = MO.MPS(2 * n, mode, chi, cutoff, svd=svd)
    for _, qs, m in doubled_ops(circuit, noise):
        if len(qs) == 1:
            mps.gate1(qs[0], m)
            continue
        for name, rq, mat in routing.route([("Mat", tuple(qs), m)]):
            mps.gate2(rq[0], rq[1], G.matrix("Swap") if name == "Swap" else mat)
    return mps


def doubled_mps_expect(mps, n, pauli):
    """Tr(rho P) / Tr(rho) from the doubled-chain MPS by dense contraction
    of its amplitudes (small n)."""
    rho = vec_to_rho(mps.amplitudes(), n)
    return R.expect_pauli(rho, n, pauli)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_doubled_chain_reproduces_the_density_oracle(seed):
    rng = np.random.default_rng(10 + seed)
    n = 4
    circ = _random_circuit(n, 4, rng)
    want = R.run(n, circ)
    assert np.allclose(run_doubled_dense(n, circ), want, atol=1e-12)
    for mode in ("exatn", "itensor"):
        mps = run_doubled_mps(n, circ, mode, 256, 1e-300 if mode == "exatn" else 1e-16)
        assert np.allclose(vec_to_rho(mps.amplitudes(), n), want, atol=1e-10), mode


def test_product_json_model_reads_like_the_oracle():
    from tnqvm_gb300.noise import JsonNoiseModel
    for key in ("depolarizing", "amplitude_damping", "readout"):
        text = GOLD[key]["model"]
        a, b = JsonNoiseModel(text), R.NoiseModel(text)
        for name, qs in (("X", [0]), ("CNOT", [0, 1]), ("H", [0])):
            ca = [m for q, m in a.channels(name, qs) if len(q) == 1 and m[0].shape == (2, 2)]
            cb = [m for _, m in b.channels(name, qs)]
            assert len(ca) == len(cb)
            for x, y in zip(ca, cb):
                assert np.array_equal(np.array(x), np.array(y))
        assert a.readout_error(0) == b.readout.get(0, (0.0, 0.0))


def test_product_json_model_lookup_rules():
    """The product's JSON noise model: channels by gate name (CX and CNOT
    alike) and exact qubit list, none for other gates or qubits, readout
    (0, 0) for a qubit the model does not list."""
    from tnqvm_gb300.noise import JsonNoiseModel
    k = [[[1, 0], [0, 0]], [[0, 0], [0, 1]]]
    doc = {"gate_noise": [{"gate_name": "CX", "register_location": ["1", "2"], "noise_channels": [{"matrix": [
        [[[1, 0], [0, 0]], [[0, 0], [1, 0]]]]}]},
                          {"gate_name": "H", "register_location": ["0"], "noise_channels": [{"matrix": [k]}]}],
           "readout_errors": [{"register_location": "3", "prob_meas0_prep1": 0.25, "prob_meas1_prep0": 0.5}]}
    m = JsonNoiseModel(doc)
    assert len(m.channels("CNOT", [1, 2])) == 1 and len(m.channels("CX", [1, 2])) == 1
    assert m.channels("CNOT", [2, 1]) == [] and m.channels("H", [1]) == [] and m.channels("X", [0]) == []
    q, mats = m.channels("H", [0])[0]
    assert q == [0] and len(mats) == 1 and mats[0].shape == (2, 2)
    assert m.readout_error(3) == (0.25, 0.5) and m.readout_error(0) == (0.0, 0.0)


BACKEND = json.load(open(os.path.join(HERE, "golden", "ibmqx2_backend.json")))


def _oracle_noise(model):
    class Adapter:
        def channels(self, name, qs):
            return [(q[0], k) for q, k in model.channels(name, qs) if len(q) == 1]
    return Adapter()


def test_backend_model_channels():
    """The device model's channels are trace preserving; relaxation for time t
    decays the excited population by exp(-t/T1) and coherences by exp(-t/T2);
    relaxation plus depolarizing has the gate's reported average error."""
    from tnqvm_gb300 import noise as N
    m = N.BackendNoiseModel(BACKEND["backend"])
    for name, qs in (("X", [0]), ("H", [2]), ("Ry", [1]), ("CNOT", [0, 1]), ("CZ", [3, 4]), ("I", [4])):
        for q, kraus in m.channels(name, qs):
            assert np.allclose(sum(k.conj().T @ k for k in kraus), np.eye(2), atol=1e-12), (name, q)
    t, t1, t2 = 500.0, 40e3, 30e3
    k = N.thermal_relaxation_kraus(t, t1, t2)
    rho = np.array([[0.3, 0.2 + 0.1j], [0.2 - 0.1j, 0.7]])
    out = sum(x @ rho @ x.conj().T for x in k)
    assert abs(out[1, 1] - 0.7 * np.exp(-t / t1)) < 1e-14
    assert abs(out[0, 1] - rho[0, 1] * np.exp(-t / t2)) < 1e-14
    props = {(g["gate"], tuple(g["qubits"])): {p["name"]: p["value"] for p in g["parameters"]}
             for g in BACKEND["backend"]["gates"]}
    err = props[("x", (0,))]["gate_error"]
    chans = m.channels("X", [0])
    # compose relaxation then depolarizing: process fidelity -> average gate fidelity
    comp = [d @ r for d in chans[1][1] for r in chans[0][1]]
    f_avg = (2 * N.process_fidelity(comp) + 1) / 3
    assert abs((1 - f_avg) - err) < 1e-12
    assert m.channels("Rz", [0]) == [] and m.channels("Z", [1]) == []


def test_backend_model_reproduces_reference_checks():
    """The checks of the reference's IBM-backend tests on the dense oracle
    with the device model (NoiseModelTester.cpp, ExaTnPmpsTester.cpp):
    readout P(1|0) = 0.0154 +- 0.01, X against H Z H within 0.01, 100 X
    gives P(1) > 0.01, 200 X P(1) > 0.1, X on three qubits 0.8 < P(111) <
    0.99, a Bell pair 0.8 < P(11) < 0.99."""
    from tnqvm_gb300 import noise as N
    m = N.BackendNoiseModel(BACKEND["backend"])
    adapter = _oracle_noise(m)

    def probs(circ, n, meas):
        rho = R.run(n, circ, noise=adapter)
        return R.readout_probabilities(R.probabilities(rho, n, meas), meas, {q: m.readout_error(q) for q in meas})

    x = ("X", [0], ())
    assert abs(probs([], 1, [0])[1] - 0.0154) < 0.01
    assert abs(probs([x], 1, [0])[1] - probs([("H", [0], ()), ("Z", [0], ()), ("H", [0], ())], 1, [0])[1]) < 0.01
    assert probs([x] * 100, 1, [0])[1] > 0.01
    assert probs([x] * 200, 1, [0])[1] > 0.1
    assert 0.8 < probs([("X", [0], ()), ("X", [1], ()), ("X", [2], ())], 3, [0, 1, 2])[7] < 0.99
    assert 0.8 < probs([x, ("CNOT", [0, 1], ())], 2, [0, 1])[3] < 0.99
