"""Pin the CPU oracle against the golden values held by the reference's own
tests (analytic formulas, dense-helper results and hard-coded tables)."""
import numpy as np
import pytest
import scipy.linalg
import scipy.optimize

from oracle import dense, mps, routing
from oracle import gates as G

PI = np.pi


def linspace(a, b, n):
    # xacc::linspace
    return [a + (b - a) * i / (n - 1) for i in range(n)]


def both_modes(n, circ, **kw):
    out = []
    for mode in ("exatn", "itensor"):
        m = mps.run(n, routing.route(circ), mode=mode, cutoff=1e-14 if mode == "itensor" else None, **kw)
        out.append(m)
    return out


def z_expect(m, qubits):
    s = ["I"] * m.n
    for q in qubits:
        s[q] = "Z"
    return m.expect_pauli("".join(s)).real


def test_simple_simulation_vs_dense_helpers():
    # ITensorMPSVisitorTester.cpp:48-179: 2-qubit circuit, <Z0> vs dense helpers at 1e-12
    for theta in (-3.1415926, -1.44159, 1.25841, 1.85841, 3.1415926):
        circ = [("Rx", (0,), (3.1415926,)), ("Ry", (1,), (3.1415926 / 2,)), ("Rx", (0,), (7.8539752,)),
                ("CNOT", (1, 0), ()), ("Rz", (0,), (theta,)), ("CNOT", (1, 0), ()),
                ("Ry", (1,), (7.8539752,)), ("Rx", (0,), (3.1415926 / 2,))]
        psi = dense.run(2, circ)
        expected = -(abs(psi[1]) ** 2 + abs(psi[3]) ** 2) + (abs(psi[0]) ** 2 + abs(psi[2]) ** 2)
        for m in both_modes(2, circ):
            assert abs(z_expect(m, [0]) - expected) < 1e-12


@pytest.mark.parametrize("theta", linspace(-PI, PI, 20))
def test_parametric_rx(theta):
    # ITensorMPSVisitorTester.cpp:321-333: <Z> = 1 - 2 sin^2(theta/2) at 1e-6
    for m in both_modes(1, [("Rx", (0,), (theta,))]):
        assert abs(z_expect(m, [0]) - (1 - 2 * np.sin(theta / 2) ** 2)) < 1e-6


@pytest.mark.parametrize("theta", linspace(-PI, PI, 20))
def test_control_gate_cphase(theta):
    # ITensorMPSVisitorTester.cpp:351-363
    circ = [("X", (0,), ()), ("H", (1,), ()), ("CPhase", (0, 1), (theta,)), ("H", (1,), ())]
    for m in both_modes(2, circ):
        assert abs(z_expect(m, [1]) - (1 - 2 * np.sin(theta / 2) ** 2)) < 1e-6


@pytest.mark.parametrize("theta", linspace(-PI, PI, 20))
def test_u3_equals_rx(theta):
    # ITensorMPSVisitorTester.cpp:379-391
    for m in both_modes(1, [("U", (0,), (theta, -PI / 2, PI / 2))]):
        assert abs(z_expect(m, [0]) - (1 - 2 * np.sin(theta / 2) ** 2)) < 1e-6


DEUTERON_X0X1 = [0.0, -0.324699, -0.614213, -0.837166, -0.9694, -0.996584, -0.915773, -0.735724,
                 -0.475947, -0.164595, 0.164595, 0.475947, 0.735724, 0.915773, 0.996584, 0.9694,
                 0.837166, 0.614213, 0.324699, 0.0]  # visitors/exatn-mps/tests/MpsGateTester.cpp:375-396


@pytest.mark.parametrize("i", range(20))
def test_deuteron_table(i):
    t = linspace(-PI, PI, 20)[i]
    circ = [("X", (0,), ()), ("Ry", (1,), (t,)), ("CNOT", (1, 0), ()), ("H", (0,), ()), ("H", (1,), ())]
    for m in both_modes(2, circ):
        assert abs(z_expect(m, [0, 1]) - DEUTERON_X0X1[i]) < 1e-5


def test_ghz_amplitude_by_conjugate():
    # ITensorMPSVisitorTester.cpp:522-551: <111|H Z CX CX|000> = -1/sqrt(2)
    circ = [("H", (0,), ()), ("Z", (0,), ()), ("CNOT", (0, 1), ()), ("CNOT", (1, 2), ())]
    for m in both_modes(3, circ):
        a = m.amplitudes()[0b111]
        assert abs(a.real + 1 / np.sqrt(2)) < 1e-6 and abs(a.imag) < 1e-6


def _probs(n, circ, meas):
    return dense.probabilities(dense.run(n, routing.route(circ)), meas)


def _key(bits):
    return int("".join(reversed(bits)), 2)


def test_gate_tester_probabilities():
    # MpsGateTester.cpp:7-300 (probabilities at 0.05 / 0.01 from 10k shots)
    for q in range(4):
        p = _probs(4, [("H", (q,), ())], [0, 1, 2, 3])
        one = ["0"] * 4
        one[q] = "1"
        assert abs(p[0] - 0.5) < 1e-12 and abs(p[_key(one)] - 0.5) < 1e-12
    for a, b in ((0, 1), (1, 0), (1, 2), (2, 1), (2, 3), (3, 2)):
        p = _probs(4, [("H", (a,), ()), ("CNOT", (a, b), ())], [a, b])
        assert abs(p[0] - 0.5) < 1e-12 and abs(p[3] - 0.5) < 1e-12
    p = _probs(4, [("X", (0,), ()), ("CNOT", (0, 1), ()), ("CNOT", (1, 2), ()), ("CNOT", (2, 3), ())], [0, 1, 2, 3])
    assert abs(p[_key("1111")] - 1) < 1e-12
    p = _probs(4, [("X", (0,), ()), ("CNOT", (0, 3), ())], [0, 1, 2, 3])   # distance-3 CNOT
    assert abs(p[_key("1001")] - 1) < 1e-12
    p = _probs(3, [("X", (0,), ()), ("iSwap", (0, 1), ())], [0, 1, 2])
    assert abs(p[_key("010")] - 1) < 1e-12
    for a in linspace(-PI, PI, 10):
        p = _probs(2, [("X", (0,), ()), ("fSim", (0, 1), (a, 0.0))], [0, 1])
        assert abs(p[_key("01")] - np.sin(a) ** 2) < 1e-12
        assert abs(p[_key("10")] - (1 - np.sin(a) ** 2)) < 1e-12


GROVER = ("H0 H1 H2 X0 H2 H2 CNOT1,2 Tdg2 CNOT0,2 T2 CNOT1,2 Tdg2 CNOT0,2 T2 H2 T1 CNOT0,1 T0 Tdg1 "
          "CNOT0,1 X0 H2 H0 H1 H2 X0 X1 X2 H2 H2 CNOT1,2 Tdg2 CNOT0,2 T2 CNOT1,2 Tdg2 CNOT0,2 T2 H2 T1 "
          "CNOT0,1 T0 Tdg1 CNOT0,1 H2 X0 X1 X2 H0 H1 H2")   # MpsGateTester.cpp:409-462


def grover_circuit():
    c = []
    for tok in GROVER.split():
        name = tok.rstrip("0123456789,")
        qs = tuple(int(x) for x in tok[len(name):].split(","))
        c.append((name, qs, ()))
    return c


def test_grover():
    # MpsGateTester.cpp:463-499: P("110") > 0.5 with Measure order q2, q1, q0
    p = _probs(3, grover_circuit(), [2, 1, 0])
    assert p[_key("110")] > 0.5
    for m in both_modes(3, grover_circuit()):
        amps = m.amplitudes()
        assert np.allclose(amps, dense.run(3, grover_circuit()), atol=1e-12)


def _pauli_matrix(s):
    # Kronecker product with qubit 0 as the least significant bit
    m = np.array([[1.0 + 0j]])
    for c in reversed(s):
        m = np.kron(m, G.PAULI[c])
    return m


def test_deuteron_vqe_h2_minimum():
    # ITensorMPSVisitorTester.cpp:453-482 / tests/VQEModeTester.cpp:44: min = -1.74886 (1e-4)
    terms = [(5.907, "II"), (-2.1433, "XX"), (-2.1433, "YY"), (0.21829, "ZI"), (-6.125, "IZ")]
    best = 1e9
    for t in np.linspace(-PI, PI, 2001):
        circ = [("X", (0,), ()), ("Ry", (1,), (t,)), ("CNOT", (1, 0), ())]
        m = mps.run(2, circ)
        e = sum(c * m.expect_pauli(s).real for c, s in terms)
        best = min(best, e)
    assert abs(best + 1.74886) < 1e-4


def test_deuteron_vqe_h3_minimum():
    # ITensorMPSVisitorTester.cpp:484-520 / VQEModeTester.cpp:81: min = -2.04482 (1e-4)
    H = [(5.907, "III"), (-2.1433, "XXI"), (-2.1433, "YYI"), (0.21829, "ZII"), (-6.125, "IZI"),
         (9.625, "III"), (-9.625, "IIZ"), (-3.91, "IXX"), (-3.91, "IYY")]
    A1 = [(1.0, "XYI"), (-1.0, "YXI")]         # X0 Y1 - Y0 X1
    A2 = [(1.0, "XZY"), (-1.0, "YZX")]         # X0 Z1 Y2 - X2 Z1 Y0
    gen1 = sum(c * _pauli_matrix(s) for c, s in A1)
    gen2 = sum(c * _pauli_matrix(s) for c, s in A2)
    Hm = sum(c * _pauli_matrix(s) for c, s in H)

    def energy(x):
        psi = dense.run(3, [("X", (0,), ())])
        psi = scipy.linalg.expm(1j * x[0] * gen1) @ psi
        psi = scipy.linalg.expm(1j * x[1] * gen2) @ psi
        return float(np.real(np.vdot(psi, Hm @ psi)))

    res = scipy.optimize.minimize(energy, [0.1, 0.1], method="Nelder-Mead",
                                  options={"xatol": 1e-9, "fatol": 1e-12, "maxiter": 4000})
    assert abs(res.fun + 2.04482) < 1e-4


def test_routing_matches_reference_tests():
    # NearestNeighborTransformTester.cpp:24-63: all 2-qubit gates adjacent,
    # instruction count grows only by the inserted swaps.
    circ = [("X", (0,), ()), ("CNOT", (1, 3), ()), ("H", (7,), ()), ("CNOT", (6, 7), ()),
            ("CNOT", (7, 3), ()), ("X", (6,), ()), ("Swap", (4, 9), ()), ("S", (5,), ())]
    r = routing.route(circ)
    n_new_swaps = sum(1 for g in r if g[0] == "Swap") - 1
    assert len(r) == len(circ) + n_new_swaps
    assert all(abs(g[1][0] - g[1][1]) == 1 for g in r if len(g[1]) == 2)
    # max-distance 2 leaves CNOT(3,1) alone (:74-99)
    r2 = routing.route([("X", (0,), ()), ("CNOT", (1, 9), ()), ("H", (7,), ()), ("CNOT", (3, 1), ())], 2)
    assert r2[-1] == ("CNOT", (3, 1), ())
    # routing preserves the state
    rng = np.random.default_rng(3)
    c = [("U", (q,), tuple(rng.uniform(0, 6, 3))) for q in range(7)] + [("CNOT", (0, 6), ()), ("CZ", (5, 1), ())]
    assert np.allclose(dense.run(7, c), dense.run(7, routing.route(c)), atol=1e-13)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_mps_exact_equals_dense(seed):
    rng = np.random.default_rng(seed)
    n = 6
    circ = []
    for _ in range(5):
        for q in range(n):
            circ.append(("U", (q,), tuple(rng.uniform(0, 2 * PI, 3))))
        for q in range(0, n - 1, 2):
            circ.append(("CNOT", (q, q + 1), ()))
        for q in range(1, n - 1, 2):
            circ.append(("CZ", (q + 1, q), ()))
    circ.append(("fSim", (5, 1), (0.4, 0.9)))
    psi = dense.run(n, circ)
    for m in both_modes(n, circ):
        assert np.allclose(m.amplitudes(), psi, atol=1e-12)
        for p in ("XYZIZX", "ZZIIII", "IYXXYI"):
            assert abs(m.expect_pauli(p) - dense.expect_pauli(psi, n, p)) < 1e-12


def test_itensor_truncate_rule():
    # decomp.cc:307-463 with relative cutoff
    P = np.array([0.5, 0.3, 0.15, 0.04, 0.01])
    assert mps.itensor_truncate(P, 10, 0.011)[0] == 4       # drop 0.01 (<= 0.011 * 1.0)
    assert mps.itensor_truncate(P, 10, 0.05)[0] == 3        # drop 0.01 + 0.04 = 0.05
    assert mps.itensor_truncate(P, 2, 0.0)[0] == 2          # maxdim first
    assert mps.itensor_truncate(np.zeros(4), 10, 0.1)[0] == 1
    assert mps.exatn_keep(np.array([1.0, 0.5, 1e-20, 0.0]), 1e-14, 100) == 3   # i+1 quirk


def test_truncated_modes_consistent():
    # bounded bond: both oracles remain normalised up to the discarded weight
    circ = []
    rng = np.random.default_rng(5)
    n = 10
    for _ in range(8):
        for q in range(n):
            circ.append(("U", (q,), tuple(rng.uniform(0, 2 * PI, 3))))
        for q in range(n - 1):
            circ.append(("CNOT", (q, q + 1), ()))
    m = mps.run(n, circ, mode="itensor", chi_max=4, cutoff=1e-12)
    assert max(m.bond_dims()) <= 4
    assert abs(m.norm2() - m.fidelity) < 1e-10   # canonical truncation: norm^2 = prod(1 - eps)


def test_oracle_matches_itensor_reference_fixtures():
    """itensor-mode oracle vs the reference's vendored ITensor v3 run on the
    same routed circuits (tests/golden/itensor_fixtures.json, produced by
    tests/golden/make_itensor_fixtures.py): identical bond dimensions under
    cap and relative-cutoff truncation, <P> to 1e-12."""
    import json
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "itensor_fixtures.json")
    fx = json.load(open(path))
    assert len(fx["cases"]) >= 6
    for c in fx["cases"]:
        circ = [(g, tuple(q), tuple(p)) for g, q, p in c["circuit"]]
        m = mps.run(c["n"], circ, mode="itensor", chi_max=c["chi"], cutoff=c["cutoff"])
        assert m.bond_dims() == c["bonds"], c["name"]
        for p, v in zip(c["paulis"], c["expect"]):
            assert abs(m.expect_pauli(p) - complex(*v)) < 1e-12, (c["name"], p)


# ------------------------------------------------ ExatnExpValSumReduceTester
def reference_tables():
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_tables.json")
    with open(path) as f:
        return json.load(f)


def pauli_exp_gates(paulis, theta):
    """Gates of exp(-i theta P) for a Pauli string P (character q on qubit q):
    basis change to Z (H for X, Rx(pi/2) for Y), a CNOT ladder over the
    support, Rz(2 theta) on its last qubit, then the ladder and the basis
    change undone.  This is how XACC's exp_i_theta instruction expands."""
    sup = [q for q, c in enumerate(paulis) if c != "I"]
    pre, post = [], []
    for q in sup:
        if paulis[q] == "X":
            pre.append(("H", (q,), ()))
            post.append(("H", (q,), ()))
        elif paulis[q] == "Y":
            pre.append(("Rx", (q,), (PI / 2,)))
            post.append(("Rx", (q,), (-PI / 2,)))
    ladder = [("CNOT", (a, b), ()) for a, b in zip(sup, sup[1:])]
    return pre + ladder + [("Rz", (sup[-1],), (2.0 * theta,))] + ladder[::-1] + post


def deuteron_h3_circuit(t0, t1):
    # X(0); exp_i_theta(t0, 0.5 X0 Y1 - 0.5 Y0 X1); exp_i_theta(t1, 0.5 X0 Z1 Y2 - 0.5 X2 Z1 Y0),
    # each exp(-i t sum_k c_k P_k) with commuting terms; then H(0), H(1) for <X0 X1>
    circ = [("X", (0,), ())]
    circ += pauli_exp_gates("XYI", 0.5 * t0) + pauli_exp_gates("YXI", -0.5 * t0)
    circ += pauli_exp_gates("XZY", 0.5 * t1) + pauli_exp_gates("YZX", -0.5 * t1)
    return circ + [("H", (0,), ()), ("H", (1,), ())]


def test_deuteron_table_sum_reduce():
    # tests/ExatnExpValSumReduceTester.cpp:47-80 (the same circuit as MpsGateTester's table), 1e-6
    tab = reference_tables()["deuteron_x0x1"]["values"]
    for i, t in enumerate(linspace(-PI, PI, 20)):
        circ = [("X", (0,), ()), ("Ry", (1,), (t,)), ("CNOT", (1, 0), ()), ("H", (0,), ()), ("H", (1,), ())]
        for m in both_modes(2, circ):
            assert abs(z_expect(m, [0, 1]) - tab[i]) < 1e-6


def test_deuteron_h3_table_dense():
    # tests/ExatnExpValSumReduceTester.cpp:125-240: <X0 X1> on a 20 x 20 grid (1e-6), with
    # exp_i_theta as exp(-i t G) of the summed generator
    tab = reference_tables()["deuteron_h3_x0x1"]["values"]
    g1 = 0.5 * (_pauli_matrix("XYI") - _pauli_matrix("YXI"))
    g2 = 0.5 * (_pauli_matrix("XZY") - _pauli_matrix("YZX"))
    xx = _pauli_matrix("XXI")
    ang = linspace(-PI, PI, 20)
    for i0, t0 in enumerate(ang):
        for i1, t1 in enumerate(ang):
            psi = dense.run(3, [("X", (0,), ())])
            psi = scipy.linalg.expm(-1j * t1 * g2) @ (scipy.linalg.expm(-1j * t0 * g1) @ psi)
            assert abs(np.real(np.vdot(psi, xx @ psi)) - tab[20 * i0 + i1]) < 1e-6


def test_deuteron_h3_table_mps_gates():
    # the same table through the gate expansion of exp_i_theta on the MPS oracle, both truncation modes
    tab = reference_tables()["deuteron_h3_x0x1"]["values"]
    ang = linspace(-PI, PI, 20)
    for i0 in range(0, 20, 3):
        for i1 in range(0, 20, 2):
            for m in both_modes(3, deuteron_h3_circuit(ang[i0], ang[i1])):
                assert abs(z_expect(m, [0, 1]) - tab[20 * i0 + i1]) < 1e-6


UCC_TERMS = [(0.174073, "IIZZ"), (0.1202, "IZIZ"), (0.165607, "IZZI"), (0.165607, "ZIIZ"), (0.1202, "ZIZI"),
             (-0.0454063, "YYXX"), (-0.220041, "IIIZ"), (-0.106477, "IIII"), (0.17028, "ZIII"),
             (-0.220041, "IIZI"), (0.17028, "IZII"), (-0.0454063, "XXYY"), (0.0454063, "XYYX"),
             (0.168336, "ZZII"), (0.0454063, "YXXY")]  # tests/VQEModeTester.cpp:107-112


def ucc_circuit(t0):
    # tests/VQEModeTester.cpp:84-103
    c = [("X", (0,), ()), ("X", (1,), ()), ("Rx", (0,), (1.5707,)), ("H", (1,), ()), ("H", (2,), ()),
         ("H", (3,), ()), ("CNOT", (0, 1), ()), ("CNOT", (1, 2), ()), ("CNOT", (2, 3), ()), ("Rz", (3,), (t0,)),
         ("CNOT", (2, 3), ()), ("CNOT", (1, 2), ()), ("CNOT", (0, 1), ()), ("Rx", (0,), (-1.5707,)),
         ("H", (1,), ()), ("H", (2,), ()), ("H", (3,), ())]
    return c


def test_ucc_vqe_minimum():
    # tests/VQEModeTester.cpp:84-127: VQE minimum -1.13717 (1e-4), here by a bounded scalar search
    def energy(t):
        m = mps.run(4, ucc_circuit(float(t)), mode="itensor", cutoff=1e-14)
        return sum(c * m.expect_pauli(s).real for c, s in UCC_TERMS)

    grid = linspace(-PI, PI, 41)
    t_best = min(grid, key=energy)
    res = scipy.optimize.minimize_scalar(energy, bounds=(t_best - 0.2, t_best + 0.2), method="bounded",
                                         options={"xatol": 1e-10})
    assert abs(res.fun + 1.13717) < 1e-4


def test_deutsch_jozsa_16_routed():
    # visitors/exatn-mps/tests/BigCircuitTester.cpp:41-145: 16-bit Deutsch-Jozsa with a balanced
    # parity oracle (CNOTs from every input qubit to the ancilla q16, routed over up to 16 sites);
    # the inputs then read 1...1 with certainty
    n = 17
    evens = [("X", (q,), ()) for q in range(0, 16, 2)]
    circ = [("X", (16,), ())] + [("H", (q,), ()) for q in range(17)] + evens
    circ += [("CNOT", (q, 16), ()) for q in range(16)] + evens + [("H", (q,), ()) for q in range(16)]
    routed = routing.route(circ)
    assert all(len(q) == 1 or abs(q[0] - q[1]) == 1 for _, q, _ in routed)
    psi = dense.run(n, routed)
    for m in both_modes(n, circ, chi_max=64):
        for q in range(16):
            assert abs(z_expect(m, [q]) + 1.0) < 1e-10
    p = dense.probabilities(psi, list(range(16)))
    assert abs(p[(1 << 16) - 1] - 1.0) < 1e-10


def test_sampler_distribution():
    # visitors/exatn-mps/tests/NumericalTester.cpp: a 5-qubit random circuit, 100000 shots, every
    # sampled bit string's frequency within 0.01 of its probability; plus a chi-square test
    from scipy import stats
    from tnqvm_gb300 import circuits
    n = 5
    psi = dense.run(n, circuits.brickwall(n, 15, seed=31))
    meas = list(range(n))
    p = dense.probabilities(psi, meas)
    bits = dense.sample(psi, meas, 100000, np.random.default_rng(5))
    keys = (bits.astype(np.int64) << np.arange(n)).sum(axis=1)
    counts = np.bincount(keys, minlength=1 << n)
    assert np.max(np.abs(counts / 100000 - p)) < 0.01
    mask = p * 100000 >= 5
    chi2 = (((counts - 100000 * p) ** 2) / np.where(mask, 100000 * p, 1.0))[mask].sum()
    assert stats.chi2.sf(chi2, mask.sum() - 1) > 1e-4


@pytest.mark.parametrize("mode", ["exatn", "itensor"])
def test_renormalisation_is_a_global_scale(mode):
    # the renormalise flag rescales each truncated split to its pre-truncation weight: the state
    # changes only by a global factor (canonical itensor form then keeps norm 1)
    from tnqvm_gb300 import circuits
    n = 10
    circ = routing.route(circuits.brickwall(n, 8, seed=13))
    cut = 1e-3 if mode == "exatn" else 1e-12
    plain = mps.run(n, circ, mode=mode, chi_max=6, cutoff=cut)
    ren = mps.run(n, circ, mode=mode, chi_max=6, cutoff=cut, renorm=True)
    assert plain.bond_dims() == ren.bond_dims() and max(plain.bond_dims()) == 6
    assert plain.fidelity < 0.99
    if mode == "itensor":
        assert abs(ren.norm2() - 1.0) < 1e-12
        assert abs(plain.norm2() - plain.fidelity) < 1e-10
    for s in ["Z" * n, "XY" + "I" * (n - 2), "I" * 4 + "ZXZ" + "I" * 3]:
        a = plain.expect_pauli(s) / plain.norm2()
        b = ren.expect_pauli(s) / ren.norm2()
        assert abs(a - b) < 1e-12, s
