"""The allocation-free two-site update (mps_gate2_apply_noalloc), called
through the C ABI, against the regular entry points.

It serves callers that cannot call cudaMalloc: a plugin inside a host
application whose device memory belongs to that application's own pool
allocator, or a process under a fixed device-memory cap.  Like such a
caller, the test owns the input/output tensors (allocated with torch) and
hands their device pointers over; the entry point must produce what the
allocating program path produces, on two calls in a row, within this
suite's tolerances (1e-10 for complex128, 2e-5 for complex64).  Kept in its
own file so that it runs last.
"""
import ctypes

import numpy as np
import pytest

from tnqvm_gb300 import mps as M

pytestmark = pytest.mark.gpu

TOL = {M.PREC_FP64: 1e-10, M.PREC_FP32: 2e-5}


def _unitary(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _call(prec, mode, chi, sites, hi_off, d_bonds, bonds, gate):
    import torch
    g = np.ascontiguousarray(gate, dtype=np.complex128).view(np.float64).reshape(-1)
    b = (ctypes.c_int * 3)(*bonds)
    rc = M._lib.mps_gate2_apply_noalloc(prec, mode, chi, -1.0, ctypes.c_void_p(sites.data_ptr()), hi_off,
                                        ctypes.c_void_p(d_bonds.data_ptr()), b,
                                        g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc


@pytest.mark.parametrize("prec", [M.PREC_FP64, M.PREC_FP32])
@pytest.mark.parametrize("mode", [M.TRUNC_EXATN, M.TRUNC_ITENSOR])
def test_noalloc_matches_program_path(ctx, prec, mode):
    import torch
    M.load_library()
    rng = np.random.default_rng(31 + 2 * prec + mode)
    g1, g2 = _unitary(rng, 4), _unitary(rng, 4)
    # allocating entry point: a 2-qubit program, two gates, amplitudes
    with M.Program(ctx, 2, 0, -1.0, mode, prec) as p:
        p.gate2(0, 1, g1)
        p.gate2(0, 1, g2)
        want = p.amplitudes()
    # allocation-free entry point on caller-owned buffers, two calls in a row
    dt = torch.complex128 if prec == M.PREC_FP64 else torch.complex64
    sites = torch.zeros(8, dtype=dt, device="cuda")
    sites[0] = 1.0          # lo site (1, 2, 1) = |0>
    sites[4] = 1.0          # hi site (1, 2, 1) = |0>
    d_bonds = torch.ones(3, dtype=torch.int32, device="cuda")
    bonds = [1, 1, 1]
    for g in (g1, g2):
        assert _call(prec, mode, 0, sites, 4, d_bonds, bonds, g) == M.OK, M._lib.mps_last_error()
        bonds = [int(x) for x in d_bonds.cpu()]
    k = bonds[1]
    s = sites.cpu().numpy().astype(np.complex128)
    lo = s[: 2 * k].reshape(1, 2, k)
    hi = s[4: 4 + 2 * k].reshape(k, 2, 1)
    theta = np.einsum("aij,jbc->ib", lo, hi)      # theta[p_lo, p_hi]
    got = np.array([theta[0, 0], theta[1, 0], theta[0, 1], theta[1, 1]])   # qubit 0 = lo = bit 0
    assert np.max(np.abs(got - want)) < TOL[prec]


@pytest.mark.parametrize("prec", [M.PREC_FP64, M.PREC_FP32])
def test_noalloc_wide_bonds_reconstruct_theta(prec):
    """dl = dm = dr = 8: with no truncation the split reproduces gate . (A B)."""
    import torch
    M.load_library()
    rng = np.random.default_rng(5 + prec)
    dl, dm, dr = 8, 8, 8
    a = rng.normal(size=(dl, 2, dm)) + 1j * rng.normal(size=(dl, 2, dm))
    b = rng.normal(size=(dm, 2, dr)) + 1j * rng.normal(size=(dm, 2, dr))
    cap_lo, cap_hi = dl * 2 * 16, 16 * 2 * dr
    dt = torch.complex128 if prec == M.PREC_FP64 else torch.complex64
    host = np.zeros(cap_lo + cap_hi, dtype=np.complex128)
    host[: a.size] = a.reshape(-1)
    host[cap_lo: cap_lo + b.size] = b.reshape(-1)
    sites = torch.tensor(host, dtype=dt, device="cuda")
    d_bonds = torch.tensor([dl, dm, dr], dtype=torch.int32, device="cuda")
    gates = [_unitary(rng, 4), _unitary(rng, 4)]
    theta = np.einsum("lim,mjr->lijr", a, b)
    for g in gates:
        bonds = [int(x) for x in d_bonds.cpu()]
        assert _call(prec, M.TRUNC_EXATN, 0, sites, cap_lo, d_bonds, bonds, g) == M.OK, M._lib.mps_last_error()
        theta = np.einsum("abij,lijr->labr", g.reshape(2, 2, 2, 2), theta)
    k = int(d_bonds.cpu()[1])
    s = sites.cpu().numpy().astype(np.complex128)
    lo = s[: dl * 2 * k].reshape(dl, 2, k)
    hi = s[cap_lo: cap_lo + k * 2 * dr].reshape(k, 2, dr)
    got = np.einsum("lim,mjr->lijr", lo, hi)
    scale = np.max(np.abs(theta))
    assert np.max(np.abs(got - theta)) / scale < 10 * TOL[prec]


def test_noalloc_rejects_bonds_beyond_limit():
    import torch
    M.load_library()
    sites = torch.zeros(4, dtype=torch.complex128, device="cuda")
    d_bonds = torch.ones(3, dtype=torch.int32, device="cuda")
    rc = _call(M.PREC_FP64, M.TRUNC_EXATN, 0, sites, 2, d_bonds, [65, 1, 1], np.eye(4))
    assert rc == M.ERR_UNSUPPORTED
    assert b"64" in M._lib.mps_last_error()
    # a hi site that would overlap the lo site's input or output is refused
    sites = torch.zeros(64, dtype=torch.complex128, device="cuda")
    for bonds, hi in (([2, 2, 2], 4), ([2, 4, 2], 12), ([1, 1, 1], -1)):
        rc = _call(M.PREC_FP64, M.TRUNC_EXATN, 0, sites, hi, d_bonds, bonds, np.eye(4))
        assert rc == M.ERR_ARG, (bonds, hi)
        assert b"hi_offset" in M._lib.mps_last_error()
