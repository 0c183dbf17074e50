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


def test_autotune_host_calls(tmp_path):
    """The GEMM autotuner's mode, table and text cache work without a GPU:
    mode validation, a save/load round trip of a hand-written entry, and a
    malformed cache rejected without touching the table."""
    from tnqvm_gb300 import mps as M
    old = M.autotune_mode()
    try:
        with pytest.raises(M.MpsError) as e:
            M.autotune_set_mode(3)
        assert e.value.code == M.ERR_ARG
        M.autotune_set_mode(2)
        assert M.autotune_mode() == 2
        M.autotune_clear()
        assert M.autotune_table() == []
        # bucket: device 0, complex64 (1), M in (128, 256], N in (256, 512],
        # K in (512, 1024], A rows and B columns unit-stride (layout 3)
        key = (0 << 20) | (1 << 19) | (8 << 15) | (9 << 11) | (10 << 7) | 3
        src = tmp_path / "tune.txt"
        src.write_text("# comment\n%d 1 0 900.0 450.5 700.0 800.0 0.0\n" % key)
        M.autotune_load(str(src))
        rows = M.autotune_table()
        assert rows == [dict(device=0, precision=1, lg_m=8, lg_n=9, lg_k=10, layout=3, kernel=1, ns=450,
                             static_ns=900)]
        out = tmp_path / "saved.txt"
        M.autotune_save(str(out))
        M.autotune_clear()
        M.autotune_load(str(out))
        assert M.autotune_table() == rows
        bad = tmp_path / "bad.txt"
        bad.write_text("%d 9 0 1 2 3 4 5\n" % key)
        with pytest.raises(M.MpsError):
            M.autotune_load(str(bad))
        assert M.autotune_table() == rows
        with pytest.raises(M.MpsError):
            M.autotune_load(str(tmp_path / "missing.txt"))
    finally:
        M.autotune_clear()
        M.autotune_set_mode(old)


_NULL_SWEEP = r'''
import ctypes, sys
sys.path.insert(0, sys.argv[1])
from tnqvm_gb300 import mps as M
lib = M.load_library()
for name, res, argtypes in M.SIGNATURES:
    args = []
    for a in argtypes:
        if a in (ctypes.c_int, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_size_t):
            args.append(0)
        elif a is ctypes.c_double:
            args.append(0.0)
        else:
            args.append(None)
    rc = getattr(lib, name)(*args)
    print(name, rc if res is ctypes.c_int else "-", flush=True)
'''

# entry points for which NULL / zero arguments are a valid no-op (as free(NULL))
# or a valid setting
_NULL_OK = {"mps_ctx_destroy", "mps_program_destroy", "mps_graph_destroy", "mps_serve_stop",
            "mps_autotune_set_mode", "mps_autotune_clear", "mps_diag_set_parallel_width",
            "mps_gates_many", "mps_diag_set_coop_rows"}


def test_null_arguments_are_errors_not_crashes():
    """Every entry point called with NULL handles and zero sizes returns a
    status (MPS_ERR_ARG, or MPS_OK where that is a valid no-op) without
    touching memory; run in a child process so a crash cannot take pytest
    down."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, "-c", _NULL_SWEEP, ROOT], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-500:] + r.stderr[-500:]
    from tnqvm_gb300 import mps as M
    seen = {}
    for line in r.stdout.strip().splitlines():
        name, rc = line.split()
        seen[name] = rc
    assert set(seen) == {s[0] for s in M.SIGNATURES}
    for name, rc in seen.items():
        if rc == "-":
            continue
        if name in _NULL_OK:
            assert rc == "0", name
        else:
            assert rc == str(M.ERR_ARG), (name, rc)
