"""The wide path's GEMM kernels and their autotuner, through the C ABI.

Every kernel the autotuner can pick (four CUDA-core tile shapes and, for
complex64, the tcgen05 3xTF32 kernel) is checked against numpy on ragged
shapes and on every storage layout of A, B and C: 1e-12 relative (Frobenius)
for complex128, 1e-6 for the complex64 CUDA-core tiles, 4e-6 for the
tensor-core kernel; the CUDA-core tiles must agree bit for bit, since each
output sums its terms in the same order whatever the tile.  Then whole wide
circuits run with tuning on and off: complex128 results must be identical
(the tuner only picks among bit-identical tiles there), complex64 results
within 2e-5 of each other on expectation values; the tuned table survives a
save/clear/load round trip and mode 2 tunes nothing new."""
import numpy as np
import pytest

from tnqvm_gb300 import circuits
from tnqvm_gb300 import mps as M

pytestmark = pytest.mark.gpu

SIMT = [M.GEMM_SIMT_64x64, M.GEMM_SIMT_32x32, M.GEMM_SIMT_16x64, M.GEMM_SIMT_64x16]


@pytest.fixture
def tune_mode():
    old = M.autotune_mode()
    yield
    M.autotune_set_mode(old)


def crand(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("prec", [M.PREC_FP64, M.PREC_FP32])
@pytest.mark.parametrize("M_,N_,K_", [(1, 130, 97), (33, 17, 200), (130, 2, 64), (257, 129, 45)])
def test_every_kernel_every_layout(ctx, prec, M_, N_, K_):
    rng = np.random.default_rng(M_ * 7 + N_ * 3 + K_)
    a = crand(rng, M_, K_)
    b = crand(rng, K_, N_)
    if prec == M.PREC_FP32:
        a32 = a.astype(np.complex64).astype(np.complex128)
        b32 = b.astype(np.complex64).astype(np.complex128)
        exact = a32 @ b32
    else:
        exact = a @ b
    scale = np.linalg.norm(exact)
    tol = 1e-12 if prec == M.PREC_FP64 else 1e-6
    for flags in range(8):
        outs = [ctx.diag_cgemm_kind(a, b, k, prec, flags) for k in SIMT]
        for k, c in zip(SIMT, outs):
            assert np.linalg.norm(c - exact) / scale < tol, (k, flags)
            assert np.array_equal(c, outs[0]), (k, flags)
        if prec == M.PREC_FP32 and N_ >= 16 and K_ >= 16:
            c = ctx.diag_cgemm_kind(a, b, M.GEMM_TC, prec, flags)
            assert np.linalg.norm(c - exact) / scale < 4e-6, flags


def test_tc_rejected_where_it_cannot_run(ctx):
    rng = np.random.default_rng(5)
    with pytest.raises(M.MpsError) as e:
        ctx.diag_cgemm_kind(crand(rng, 8, 8), crand(rng, 8, 8), M.GEMM_TC, M.PREC_FP64)
    assert e.value.code == M.ERR_ARG
    with pytest.raises(M.MpsError):
        ctx.diag_cgemm_kind(crand(rng, 40, 40), crand(rng, 40, 8), M.GEMM_TC, M.PREC_FP32)  # N < 16


def _wide_run(ctx, prec, n=14, cap=100, seed=11):
    circ = circuits.brickwall(n, 12, seed=seed)
    p = M.Program(ctx, n, cap, 1e-12, M.TRUNC_ITENSOR, prec)
    p.run(circ)
    p.submit()
    p.wait()
    paulis = ["Z" * n, "I" * 3 + "XY" + "I" * (n - 5), "I" * (n - 2) + "ZZ"]
    vals = np.array(p.expect_pauli(paulis))
    bonds = p.bond_dims()
    fid = p.truncation_fidelity()
    p.close()
    return vals, bonds, fid


def test_tuned_fp64_circuit_is_identical(ctx, tune_mode):
    M.autotune_set_mode(0)
    ref = _wide_run(ctx, M.PREC_FP64)
    M.autotune_clear()
    M.autotune_set_mode(1)
    t0 = ctx.autotune_tunings()
    got = _wide_run(ctx, M.PREC_FP64)
    assert ctx.autotune_tunings() > t0
    rows = [r for r in M.autotune_table() if r["precision"] == M.PREC_FP64]
    assert rows and all(r["kernel"] != M.GEMM_TC for r in rows)
    assert got[1] == ref[1]
    assert np.array_equal(got[0], ref[0])
    assert got[2] == ref[2]


def test_tuned_fp32_circuit_and_cache(ctx, tune_mode, tmp_path):
    M.autotune_set_mode(0)
    ref = _wide_run(ctx, M.PREC_FP32, seed=12)
    M.autotune_clear()
    M.autotune_set_mode(1)
    got = _wide_run(ctx, M.PREC_FP32, seed=12)
    assert np.max(np.abs(got[0] - ref[0])) < 2e-5
    assert abs(got[2] - ref[2]) < 2e-5
    table = M.autotune_table()
    assert any(r["precision"] == M.PREC_FP32 for r in table)
    for r in table:
        assert 0 <= r["kernel"] < 5 and r["ns"] > 0 and r["static_ns"] > 0
        assert r["ns"] <= r["static_ns"]
    path = tmp_path / "tune.txt"
    M.autotune_save(str(path))
    M.autotune_clear()
    M.autotune_load(str(path))
    assert M.autotune_table() == table
    # mode 2: tuned entries only, nothing new is tuned
    M.autotune_set_mode(2)
    t0 = ctx.autotune_tunings()
    again = _wide_run(ctx, M.PREC_FP32, seed=12)
    assert ctx.autotune_tunings() == t0
    assert np.max(np.abs(again[0] - got[0])) < 2e-5
