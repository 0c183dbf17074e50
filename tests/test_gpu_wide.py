"""GPU parity of the wide two-site path (bond caps above the single-CTA limit):
tensor-core complex GEMMs, the cooperative eigensolver and QR, centre moves,
GEMM-sweep expectations and sampling, called through the C ABI and checked
against the CPU oracle.  Tolerances: 1e-10 for complex128 runs against the
complex128 oracle (1e-12 for truncated runs, whose sums round to ~1e-16 of
the largest singular value of each split); 4e-6 relative (Frobenius)
for one complex64 3xTF32 GEMM with K up to 1000; 1e-4 on amplitudes and 2e-5
on expectation values for complex64 circuits."""
import numpy as np
import pytest

from oracle import dense, routing
from oracle import mps as omps
from tnqvm_gb300 import circuits
from tnqvm_gb300 import mps as M

pytestmark = pytest.mark.gpu

TOL64 = 1e-10


def run(ctx, n, circ, chi, cutoff, mode, prec, flags=0):
    p = M.Program(ctx, n, chi, cutoff, mode, prec, flags)
    p.run(circ)
    p.submit()
    p.wait()
    return p


def crand(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("M_,N_,K_", [(128, 64, 16), (256, 128, 128), (300, 257, 129), (512, 512, 1000),
                                      (1024, 96, 700)])
def test_tensor_core_gemm(ctx, M_, N_, K_):
    """3xTF32 tcgen05 product against complex128 numpy and the CUDA-core kernel."""
    rng = np.random.default_rng(M_ + N_ + K_)
    a = crand(rng, M_, K_)
    b = crand(rng, K_, N_)
    exact = a.astype(np.complex64).astype(np.complex128) @ b.astype(np.complex64).astype(np.complex128)
    ct, cs = ctx.diag_cgemm(a, b)
    scale = np.linalg.norm(exact)
    assert np.linalg.norm(cs - exact) / scale < 1e-6
    assert np.linalg.norm(ct - exact) / scale < 4e-6


@pytest.mark.parametrize("mode", [M.TRUNC_EXATN, M.TRUNC_ITENSOR])
def test_wide_exact_fp64(ctx, mode):
    """14 qubits, brick wall depth 14, cap 128 (= exact): every amplitude and
    <Z_i> against the dense oracle; bonds reach 128, so splits of a 256 x 256
    theta run on the cooperative eigensolver."""
    n = 14
    circ = circuits.brickwall(n, 14, seed=21)
    psi = dense.run(n, circ)
    with run(ctx, n, circ, 128, 1e-14, mode, M.PREC_FP64) as p:
        assert max(p.bond_dims()) == 128
        amp = p.amplitudes()
        assert np.max(np.abs(amp - psi)) < TOL64
        zs = p.expect_pauli(["I" * q + "Z" + "I" * (n - q - 1) for q in range(n)])
        for q in range(n):
            assert abs(zs[q].real - dense.expect_z_parity(psi, [q])) < TOL64
        assert abs(p.norm() - 1.0) < TOL64
        bits = [(q * 7) % 2 for q in range(n)]
        idx = sum(b << q for q, b in enumerate(bits))
        assert abs(p.amplitude(bits) - psi[idx]) < TOL64


@pytest.mark.parametrize("mode,omode", [(M.TRUNC_ITENSOR, "itensor"), (M.TRUNC_EXATN, "exatn")])
def test_wide_truncated_fp64_vs_oracle(ctx, mode, omode):
    """Cap 80 on 16 qubits (truncating, a non-power-of-two bond): bond
    dimensions, Pauli expectations and truncation fidelity against the
    complex128 oracle at the same cap and cutoff."""
    n = 16
    circ = circuits.brickwall(n, 12, seed=8)
    ref = omps.run(n, routing.route(circ), mode=omode, chi_max=80, cutoff=1e-12)
    rng = np.random.default_rng(3)
    paulis, _ = circuits.random_paulis(n, 6, rng)
    paulis = list(paulis) + ["I" * n]
    with run(ctx, n, circ, 80, 1e-12, mode, M.PREC_FP64) as p:
        assert p.bond_dims() == ref.bond_dims()
        vals = p.expect_pauli(paulis)
        tol = 1e-12
        for s, v in zip(paulis, vals):
            assert abs(v - ref.expect_pauli(s)) < tol, s
        assert abs(p.truncation_fidelity() - ref.fidelity) < tol


@pytest.mark.parametrize("mode", [M.TRUNC_EXATN, M.TRUNC_ITENSOR])
def test_wide_exact_fp32(ctx, mode):
    """complex64 wide path (tensor-core GEMMs) on the exact 14-qubit circuit."""
    n = 14
    circ = circuits.brickwall(n, 14, seed=21)
    psi = dense.run(n, circ)
    old = M.autotune_mode()
    M.autotune_set_mode(0)  # the static rule puts the large products on tensor cores
    try:
        t0, _ = ctx.gemm_counts()
        with run(ctx, n, circ, 128, 1e-14, mode, M.PREC_FP32) as p:
            amp = p.amplitudes()
            assert np.max(np.abs(amp - psi)) < 1e-4
            zs = p.expect_pauli(["I" * q + "Z" + "I" * (n - q - 1) for q in range(n)])
            for q in range(n):
                assert abs(zs[q].real - dense.expect_z_parity(psi, [q])) < 2e-5
        t1, _ = ctx.gemm_counts()
    finally:
        M.autotune_set_mode(old)
    assert t1 > t0  # the tensor-core kernel ran


@pytest.mark.parametrize("layout", [0, 7])
def test_split_bf16_gemm(ctx, layout):
    """The tensor-core kernel with split-BF16 operands (kind::f16, bf16 head
    and remainder, three products): within 6e-5 relative (Frobenius) of
    numpy on a ragged product in row- and column-major storage, and not
    equal to the 3xTF32 result (the other MMA kind ran)."""
    rng = np.random.default_rng(17 + layout)
    a = rng.standard_normal((257, 200)) + 1j * rng.standard_normal((257, 200))
    b = rng.standard_normal((200, 131)) + 1j * rng.standard_normal((200, 131))
    want = a @ b
    got = ctx.diag_cgemm_kind(a, b, M.GEMM_TC, M.PREC_FP32, layout | 8)
    tf32 = ctx.diag_cgemm_kind(a, b, M.GEMM_TC, M.PREC_FP32, layout)
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert rel < 6e-5, rel
    assert np.linalg.norm(tf32 - want) / np.linalg.norm(want) < 4e-6
    assert np.max(np.abs(got - tf32)) > 0.0


def test_split_bf16_program(ctx):
    """MPS_PREC_SPLIT_BF16 on the exact 14-qubit circuit at cap 128 (wide
    path, tensor-core products under the static rule): amplitudes within
    2e-3 and <Z_q> within 1e-3 of the dense oracle; the program reports the
    mode and the tensor-core kernel ran."""
    n = 14
    circ = circuits.brickwall(n, 14, seed=21)
    psi = dense.run(n, circ)
    old = M.autotune_mode()
    M.autotune_set_mode(0)
    try:
        t0, _ = ctx.gemm_counts()
        with run(ctx, n, circ, 128, 1e-14, M.TRUNC_ITENSOR, M.PREC_SPLIT_BF16) as p:
            assert p.precision == M.PREC_SPLIT_BF16
            amp = p.amplitudes()
            assert np.max(np.abs(amp - psi)) < 2e-3
            zs = p.expect_pauli(["I" * q + "Z" + "I" * (n - q - 1) for q in range(n)])
            for q in range(n):
                assert abs(zs[q].real - dense.expect_z_parity(psi, [q])) < 1e-3
        t1, _ = ctx.gemm_counts()
    finally:
        M.autotune_set_mode(old)
    assert t1 > t0


def test_wide_routed_itensor_fp64(ctx):
    """Non-adjacent gates (SWAP routing) and centre moves in both directions:
    a 3-regular QAOA circuit on 14 qubits, cap 100, against the oracle."""
    n = 14
    circ, _ = circuits.qaoa_maxcut(n, 1, seed=3)
    ref = omps.run(n, routing.route(circ), mode="itensor", chi_max=100, cutoff=1e-12)
    with run(ctx, n, circ, 100, 1e-12, M.TRUNC_ITENSOR, M.PREC_FP64) as p:
        assert p.bond_dims() == ref.bond_dims()
        for s in ["Z" * n, "ZZ" + "I" * (n - 2), "I" * (n - 2) + "XX", "Y" + "I" * (n - 2) + "Y"]:
            assert abs(p.expect_pauli([s])[0] - ref.expect_pauli(s)) < 1e-9, s


def test_wide_sampling_chi_square(ctx):
    """4096 shots of a 10-qubit state held at cap 96 against the exact
    probabilities (chi-square, p > 1e-4)."""
    from scipy import stats
    n = 10
    circ = circuits.brickwall(n, 6, seed=4)
    psi = dense.run(n, circ)
    probs = np.abs(psi) ** 2
    with run(ctx, n, circ, 96, 1e-14, M.TRUNC_EXATN, M.PREC_FP64) as p:
        bits = p.sample(4096, seed=17)
    idx = (bits.astype(np.int64) << np.arange(n)).sum(axis=1)
    counts = np.bincount(idx, minlength=1 << n)
    big = probs * 4096 >= 5
    obs = np.append(counts[big], counts[~big].sum())
    exp = np.append(probs[big], probs[~big].sum()) * 4096
    chi2 = ((obs - exp) ** 2 / np.maximum(exp, 1e-300)).sum()
    assert stats.chi2.sf(chi2, len(obs) - 1) > 1e-4


def test_wide_rejections(ctx):
    with pytest.raises(M.MpsError) as e:
        M.Program(ctx, 20, 2048, -1.0, M.TRUNC_EXATN, M.PREC_FP32)
    assert e.value.code == M.ERR_UNSUPPORTED
    with pytest.raises(M.MpsError) as e:
        M.Program(ctx, 20, 128, -1.0, M.TRUNC_EXATN, M.PREC_FP64, M.FLAG_PER_GATE)
    assert e.value.code == M.ERR_UNSUPPORTED


def test_wide_serve_same_alone_and_in_mix(ctx):
    """Requests with bond caps 16, 64, 128 and 256 in one Poisson-free burst:
    each wide request's energy and shots equal its result when served alone,
    and the narrow ones still complete beside it."""
    rng = np.random.default_rng(12)
    specs = []
    for i in range(12):
        n = int(rng.integers(10, 17))
        chi = [16, 64, 128, 256][i % 4]
        circ = circuits.brickwall(n, int(rng.integers(4, 9)), seed=100 + i)
        paulis, coeffs = circuits.random_paulis(n, 4, rng)
        specs.append((n, chi, circ, paulis, coeffs))

    def make(spec):
        n, chi, circ, paulis, coeffs = spec
        p = M.Program(ctx, n, chi, 1e-12, M.TRUNC_ITENSOR, M.PREC_FP32)
        p.run(circ)
        p.set_observable(paulis, coeffs)
        return p

    wide = [i for i, sp in enumerate(specs) if sp[1] > M.CHI_LIMIT]
    alone = {}
    ctx.serve_start(64)
    try:
        for i in wide:
            p = make(specs[i])
            t = ctx.serve_submit(p, 128, 9)
            e, bits, _ = ctx.serve_poll(t, p, 128)
            alone[i] = (e, bits.copy())
            p.close()
        progs = [make(sp) for sp in specs]
        tickets = [ctx.serve_submit(p, 128, 9) for p in progs]
        for i, (t, p) in enumerate(zip(tickets, progs)):
            e, bits, lat = ctx.serve_poll(t, p, 128)
            assert lat >= 0.0 and np.isfinite(e)
            if i in alone:
                assert abs(e - alone[i][0]) < 1e-9
                assert np.array_equal(bits, alone[i][1])
        for p in progs:
            p.close()
    finally:
        ctx.serve_stop()


@pytest.mark.parametrize("chi", [64, 128])
def test_sweep_schedule_exact(ctx, chi):
    """MPS_FLAG_SWEEP reorders gates on disjoint qubits: on an exact run the
    state equals the dense oracle's, with fewer centre moves than the
    recorded order."""
    n = 12
    circ = circuits.brickwall(n, 10, seed=31)
    psi = dense.run(n, circ)
    ops = {}
    for flags in (0, M.FLAG_SWEEP):
        with run(ctx, n, circ, chi, 1e-14, M.TRUNC_ITENSOR, M.PREC_FP64, flags) as p:
            amp = p.amplitudes()
            assert np.max(np.abs(amp - psi)) < TOL64
            ops[flags] = p.stats()["ops"]
    assert ops[M.FLAG_SWEEP] < ops[0]


def test_wide_itensor_fixtures_where_cap_is_loose(ctx):
    """The vendored-ITensor fixtures whose bond cap never binds (every bond
    below the cap) run as wide programs (cap 128): the same bond dimensions
    and <P> within 1e-10 as ITensor v3 (tests/golden/itensor_fixtures.json)."""
    import json
    import os
    fx = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "itensor_fixtures.json")))
    used = 0
    for c in fx["cases"]:
        if max(c["bonds"]) >= c["chi"]:
            continue
        used += 1
        circ = [(g, tuple(q), tuple(p)) for g, q, p in c["circuit"]]
        with run(ctx, c["n"], circ, 128, c["cutoff"], M.TRUNC_ITENSOR, M.PREC_FP64) as p:
            assert p.bond_dims() == c["bonds"], c["name"]
            vals = p.expect_pauli(c["paulis"])
            for s, v, want in zip(c["paulis"], vals, c["expect"]):
                assert abs(v - complex(*want)) < TOL64, (c["name"], s)
    assert used >= 3
