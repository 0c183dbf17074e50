"""The C-ABI library loads and exports every entry point ``include/*.h``
declares, and the Python binding covers them (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(mps_[a-z0-9_]+)\s*\(", src, re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    from tnqvm_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 30
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_binding_covers_header():
    from tnqvm_gb300 import mps as M
    bound = {s[0] for s in M.SIGNATURES}
    assert declared_symbols() <= bound


def test_host_only_calls(lib):
    from tnqvm_gb300 import mps as M
    M.load_library()
    assert b"sm_103a" in M._lib.mps_version()
    # footprint: 12 qubits, chi 64, complex128: sum chi_l*2*chi_r*16
    caps = [1, 2, 4, 8, 16, 32, 64, 32, 16, 8, 4, 2, 1]
    expect = sum(caps[i] * 2 * caps[i + 1] for i in range(12)) * 16
    assert M.footprint_bytes(12, 64, M.PREC_FP64) == expect
    assert M.footprint_bytes(12, 64, M.PREC_FP32) == expect // 2


def test_no_device_is_an_error_not_a_crash():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from tnqvm_gb300 import mps as M
    with pytest.raises(M.MpsError) as e:
        M.Context(0)
    assert e.value.code == M.ERR_CUDA
