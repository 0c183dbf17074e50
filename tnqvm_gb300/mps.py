"""ctypes binding of the gb300mps C ABI (``include/gb300mps.h``).

This is the Python face of the engine: a ``Context`` owns the GPU stream and
memory, a ``Program`` is one MPS register with the gates recorded on it.  The
library must have been built (``tnqvm_gb300.build``); there is no CPU path and
loading fails loudly when the shared object is missing.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgb300mps.so")

OK, ERR_ARG, ERR_OOM, ERR_TIMEOUT, ERR_NUMERIC, ERR_CUDA, ERR_STATE, ERR_UNSUPPORTED = range(8)
TRUNC_EXATN, TRUNC_ITENSOR = 0, 1
PREC_FP64, PREC_FP32, PREC_AUTO, PREC_SPLIT_BF16 = 0, 1, 2, 3
AUTO_FP64_QUBITS = 12
FLAG_RENORM, FLAG_PER_GATE, FLAG_SWEEP, FLAG_FUSE, FLAG_DENSITY, FLAG_PARALLEL = 1, 2, 4, 8, 16, 32
DM_QUBITS_MAX, DIAG_QUBITS_MAX = 13, 24
CHI_LIMIT = 64
WIDE_CHI_LIMIT = 1024
# GEMM kernels of the wide path (MPS_GEMM_*) and the autotuner's row width
GEMM_SIMT_64x64, GEMM_SIMT_32x32, GEMM_SIMT_16x64, GEMM_SIMT_64x16, GEMM_TC = range(5)
GEMM_KERNEL_NAMES = ["simt64x64", "simt32x32", "simt16x64", "simt64x16", "tc"]
AUTOTUNE_COLS = 9
AUTOTUNE_FIELDS = ("device", "precision", "lg_m", "lg_n", "lg_k", "layout", "kernel", "ns", "static_ns")

_ERR_NAMES = {1: "MPS_ERR_ARG", 2: "MPS_ERR_OOM", 3: "MPS_ERR_TIMEOUT", 4: "MPS_ERR_NUMERIC",
              5: "MPS_ERR_CUDA", 6: "MPS_ERR_STATE", 7: "MPS_ERR_UNSUPPORTED"}

# (name, restype, argtypes) for every exported function
_c = ctypes
_P = _c.c_void_p
_DP = _c.POINTER(_c.c_double)
SIGNATURES = [
    ("mps_last_error", _c.c_char_p, []),
    ("mps_version", _c.c_char_p, []),
    ("mps_ctx_create", _c.c_int, [_P, _c.POINTER(_P)]),
    ("mps_ctx_destroy", _c.c_int, [_P]),
    ("mps_ctx_info", _c.c_int, [_P, _c.POINTER(_c.c_int), _c.POINTER(_c.c_size_t)]),
    ("mps_program_begin", _c.c_int, [_P, _c.c_int, _c.c_int, _c.c_double, _c.c_int, _c.c_int, _c.c_int,
                                      _c.POINTER(_P)]),
    ("mps_program_reset", _c.c_int, [_P]),
    ("mps_program_precision", _c.c_int, [_P, _c.POINTER(_c.c_int)]),
    ("mps_program_destroy", _c.c_int, [_P]),
    ("mps_gate1", _c.c_int, [_P, _c.c_int, _DP]),
    ("mps_gate2", _c.c_int, [_P, _c.c_int, _c.c_int, _DP]),
    ("mps_gate_named", _c.c_int, [_P, _c.c_char_p, _c.POINTER(_c.c_int), _c.c_int, _DP, _c.c_int]),
    ("mps_measure", _c.c_int, [_P, _c.c_int]),
    ("mps_submit", _c.c_int, [_P]),
    ("mps_wait", _c.c_int, [_P, _c.c_int]),
    ("mps_batch_submit", _c.c_int, [_P, _c.POINTER(_P), _c.c_int]),
    ("mps_norm", _c.c_int, [_P, _DP]),
    ("mps_amplitudes", _c.c_int, [_P, _DP]),
    ("mps_amplitude", _c.c_int, [_P, _c.POINTER(_c.c_int), _DP]),
    ("mps_expect_pauli", _c.c_int, [_P, _c.c_char_p, _c.c_int, _DP, _DP]),
    ("mps_set_observable", _c.c_int, [_P, _c.c_char_p, _c.c_int, _DP]),
    ("mps_batch_expect", _c.c_int, [_P, _c.POINTER(_P), _c.c_int, _DP]),
    ("mps_sample", _c.c_int, [_P, _c.c_int, _c.c_uint64, _c.POINTER(_c.c_uint8)]),
    ("mps_n_measured", _c.c_int, [_P, _c.POINTER(_c.c_int)]),
    ("mps_truncation_fidelity", _c.c_int, [_P, _DP]),
    ("mps_bond_dims", _c.c_int, [_P, _c.POINTER(_c.c_int)]),
    ("mps_stats", _c.c_int, [_P, _DP]),
    ("mps_serve_start", _c.c_int, [_P, _c.c_int]),
    ("mps_serve_submit", _c.c_int, [_P, _P, _c.c_int, _c.c_uint64, _c.POINTER(_c.c_uint64)]),
    ("mps_serve_poll", _c.c_int, [_P, _c.c_uint64, _c.c_int, _DP, _c.POINTER(_c.c_uint8), _DP]),
    ("mps_serve_stop", _c.c_int, [_P]),
    ("mps_footprint_bytes", _c.c_size_t, [_c.c_int, _c.c_int, _c.c_int]),
    ("mps_graph_create", _c.c_int, [_P, _c.POINTER(_P), _c.c_int, _c.POINTER(_P)]),
    ("mps_graph_launch", _c.c_int, [_P, _DP]),
    ("mps_graph_launch_async", _c.c_int, [_P]),
    ("mps_graph_sync", _c.c_int, [_P, _DP]),
    ("mps_graph_update", _c.c_int, [_P]),
    ("mps_graph_stream", _c.c_int, [_P, _c.POINTER(_P)]),
    ("mps_graph_destroy", _c.c_int, [_P]),
    ("mps_graph_timing", _c.c_int, [_P, _DP]),
    ("mps_graph_phase_cycles", _c.c_int, [_P, _DP]),
    ("mps_graph_stat_sums", _c.c_int, [_P, _DP, _c.c_int]),
    ("mps_gates", _c.c_int, [_P, _c.c_int, _c.POINTER(_c.c_int32), _c.POINTER(_c.c_int32), _DP]),
    ("mps_gates_many", _c.c_int, [_c.c_int, _c.POINTER(_P), _c.POINTER(_c.c_int64), _c.POINTER(_c.c_int32),
                                  _c.POINTER(_c.c_int32), _DP]),
    ("mps_gate2_apply_noalloc", _c.c_int, [_c.c_int, _c.c_int, _c.c_int, _c.c_double, _P, _c.c_int64,
                                            _P, _c.POINTER(_c.c_int), _DP, _P]),
    ("mps_diag_cgemm", _c.c_int, [_P, _c.c_int, _c.c_int, _c.c_int, _DP, _DP, _DP, _DP]),
    ("mps_diag_gemm_counts", _c.c_int, [_P, _c.POINTER(_c.c_int), _c.POINTER(_c.c_int)]),
    ("mps_diag_fma_rate", _c.c_int, [_c.c_int, _c.c_int, _DP]),
    ("mps_diag_cgemm_kind", _c.c_int, [_P, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _DP, _DP,
                                        _DP]),
    ("mps_autotune_set_mode", _c.c_int, [_c.c_int]),
    ("mps_autotune_get_mode", _c.c_int, [_c.POINTER(_c.c_int)]),
    ("mps_autotune_table", _c.c_int, [_c.POINTER(_c.c_int), _c.c_int, _c.POINTER(_c.c_int)]),
    ("mps_autotune_save", _c.c_int, [_c.c_char_p]),
    ("mps_autotune_load", _c.c_int, [_c.c_char_p]),
    ("mps_autotune_clear", _c.c_int, []),
    ("mps_autotune_tunings", _c.c_int, [_P, _c.POINTER(_c.c_int)]),
    ("mps_channel1", _c.c_int, [_P, _c.c_int, _c.c_int, _DP]),
    ("mps_diag_set_parallel_width", _c.c_int, [_c.c_int]),
    ("mps_diag_set_coop_rows", _c.c_int, [_c.c_int]),
    ("mps_density_matrix", _c.c_int, [_P, _c.c_int, _c.POINTER(_c.c_int), _DP]),
    ("mps_density_diag", _c.c_int, [_P, _c.c_int, _c.POINTER(_c.c_int), _DP]),
]

GATE_IDS = {name: i for i, name in enumerate(
    ["I", "H", "CNOT", "Rx", "Ry", "Rz", "Swap", "U", "X", "Y", "Z", "Measure", "CZ", "CPhase", "S", "Sdg",
     "T", "Tdg", "CY", "CH", "CRZ", "iSwap", "fSim", "RZZ"])}
GATE_IDS["CX"] = GATE_IDS["CNOT"]
GATE_IDS["U3"] = GATE_IDS["U"]


def encode_circuit(circuit):
    """Gate list -> (ids int32[g], qubits int32[g,2], params float64[g,3]) for ``Program.record``."""
    g = len(circuit)
    ids = np.zeros(g, dtype=np.int32)
    qs = np.zeros((g, 2), dtype=np.int32)
    ps = np.zeros((g, 3), dtype=np.float64)
    for i, (name, q, p) in enumerate(circuit):
        ids[i] = GATE_IDS[name]
        qs[i, : len(q)] = q
        ps[i, : len(p)] = p
    return ids, qs, ps

_lib = None


class MpsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (_ERR_NAMES.get(code, str(code)), msg))
        self.code = code


def load_library(path=LIB_PATH):
    """Load the engine.  Raises if the CUDA library was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libgb300mps.so not built (run tnqvm_gb300.build.build()); "
                          "there is no CPU fallback")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc):
    if rc != OK:
        raise MpsError(rc, _lib.mps_last_error().decode())


def _dptr(a):
    return a.ctypes.data_as(_DP)


class _Cfg(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_size_t)]


class Context:
    def __init__(self, device=0, hbm_budget_bytes=0):
        lib = load_library()
        cfg = _Cfg(device, hbm_budget_bytes)
        h = ctypes.c_void_p()
        _check(lib.mps_ctx_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self.serving = False

    def close(self):
        if self.h:
            _lib.mps_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def num_sms(self):
        n = ctypes.c_int()
        _check(_lib.mps_ctx_info(self.h, ctypes.byref(n), None))
        return n.value

    @property
    def bytes_resident(self):
        b = ctypes.c_size_t()
        _check(_lib.mps_ctx_info(self.h, None, ctypes.byref(b)))
        return b.value

    # ---- batches
    def batch_submit(self, programs):
        arr = (ctypes.c_void_p * len(programs))(*[p.h for p in programs])
        _check(_lib.mps_batch_submit(self.h, arr, len(programs)))

    def batch_expect(self, programs):
        arr = (ctypes.c_void_p * len(programs))(*[p.h for p in programs])
        out = np.zeros(len(programs))
        _check(_lib.mps_batch_expect(self.h, arr, len(programs), _dptr(out)))
        return out

    # ---- serving
    def serve_start(self, max_inflight=256):
        _check(_lib.mps_serve_start(self.h, max_inflight))
        self.serving = True

    def serve_submit(self, program, shots=0, seed=0):
        t = ctypes.c_uint64()
        _check(_lib.mps_serve_submit(self.h, program.h, shots, seed, ctypes.byref(t)))
        return t.value

    def serve_poll(self, ticket, program, shots=0, timeout_ms=-1):
        """Returns (energy, bits[shots, n_meas], latency_ms)."""
        e = ctypes.c_double()
        lat = ctypes.c_double()
        nm = program.n_measured
        bits = np.zeros((max(shots, 0), nm), dtype=np.uint8)
        bp = bits.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)) if shots > 0 else None
        _check(_lib.mps_serve_poll(self.h, ticket, timeout_ms, ctypes.byref(e), bp, ctypes.byref(lat)))
        return e.value, bits, lat.value

    def serve_stop(self):
        _check(_lib.mps_serve_stop(self.h))
        self.serving = False

    # ---- diagnostics of the wide path
    def diag_cgemm(self, a, b):
        """complex64 product a @ b on the tensor-core and on the CUDA-core
        kernel; returns (c_tc, c_simt) as complex128 arrays."""
        a = np.ascontiguousarray(a, dtype=np.complex128)
        b = np.ascontiguousarray(b, dtype=np.complex128)
        M, K = a.shape
        N = b.shape[1]
        ct = np.zeros((M, N), dtype=np.complex128)
        cs = np.zeros((M, N), dtype=np.complex128)
        _check(_lib.mps_diag_cgemm(self.h, M, N, K, _dptr(a.view(np.float64)), _dptr(b.view(np.float64)),
                                   _dptr(ct.view(np.float64)), _dptr(cs.view(np.float64))))
        return ct, cs

    def gemm_counts(self):
        """(tensor-core, CUDA-core) GEMM launches of the wide path so far."""
        t, s = ctypes.c_int(), ctypes.c_int()
        _check(_lib.mps_diag_gemm_counts(self.h, ctypes.byref(t), ctypes.byref(s)))
        return t.value, s.value

    def diag_cgemm_kind(self, a, b, kernel, precision=PREC_FP32, flags=0):
        """a @ b on one chosen GEMM kernel (GEMM_*) in complex64 or complex128;
        flags bits 0/1/2 store A/B/C column-major on the device."""
        a = np.ascontiguousarray(a, dtype=np.complex128)
        b = np.ascontiguousarray(b, dtype=np.complex128)
        M, K = a.shape
        N = b.shape[1]
        c = np.zeros((M, N), dtype=np.complex128)
        _check(_lib.mps_diag_cgemm_kind(self.h, precision, kernel, flags, M, N, K, _dptr(a.view(np.float64)),
                                        _dptr(b.view(np.float64)), _dptr(c.view(np.float64))))
        return c

    def autotune_tunings(self):
        """Shape buckets tuned by this context's wide workspaces so far."""
        n = ctypes.c_int()
        _check(_lib.mps_autotune_tunings(self.h, ctypes.byref(n)))
        return n.value


# ---- GEMM autotuner of the wide path (process-wide table)
def fma_rate(device=0, precision=PREC_FP32):
    """Measured peak CUDA-core FMA rate (flops/s, an FMA counts 2) of one
    precision on ``device``: the roofline denominator of CUDA-core kernels."""
    load_library()
    v = ctypes.c_double()
    _check(_lib.mps_diag_fma_rate(device, precision, ctypes.byref(v)))
    return v.value


def set_parallel_width(max_ctas):
    """Most CTAs a site-parallel run may use (0 = automatic); 1 runs the same
    kernel one op at a time."""
    load_library()
    _check(_lib.mps_diag_set_parallel_width(max_ctas))


def set_coop_rows(rows_per_cta):
    """Rows (or columns) per CTA of the wide path's cooperative launches
    (0 = the default, 8)."""
    load_library()
    _check(_lib.mps_diag_set_coop_rows(rows_per_cta))


def autotune_set_mode(mode):
    """0 static rule, 1 tune new shape buckets, 2 tuned/loaded entries only."""
    load_library()
    _check(_lib.mps_autotune_set_mode(mode))


def autotune_mode():
    load_library()
    m = ctypes.c_int()
    _check(_lib.mps_autotune_get_mode(ctypes.byref(m)))
    return m.value


def autotune_table():
    """List of dicts, one per tuned bucket (fields AUTOTUNE_FIELDS)."""
    load_library()
    n = ctypes.c_int()
    _check(_lib.mps_autotune_table(None, 0, ctypes.byref(n)))
    cap = n.value
    buf = (ctypes.c_int * max(1, cap * AUTOTUNE_COLS))()
    _check(_lib.mps_autotune_table(buf, cap, ctypes.byref(n)))
    rows = []
    for i in range(min(cap, n.value)):
        rows.append(dict(zip(AUTOTUNE_FIELDS, buf[i * AUTOTUNE_COLS:(i + 1) * AUTOTUNE_COLS])))
    return rows


def autotune_save(path):
    load_library()
    _check(_lib.mps_autotune_save(os.fsencode(path)))


def autotune_load(path):
    load_library()
    _check(_lib.mps_autotune_load(os.fsencode(path)))


def autotune_clear():
    load_library()
    _check(_lib.mps_autotune_clear())


class Graph:
    """Captured batch: reset + one persistent launch + observables + D2H,
    replayed by ``launch``; ``update`` loads newly recorded gates of the same
    structure (new parameters) into the captured op table."""

    def __init__(self, ctx, programs):
        self.programs = list(programs)
        arr = (ctypes.c_void_p * len(programs))(*[p.h for p in programs])
        h = ctypes.c_void_p()
        _check(_lib.mps_graph_create(ctx.h, arr, len(programs), ctypes.byref(h)))
        self.h = h
        self.out = np.zeros(len(programs))

    def launch(self):
        _check(_lib.mps_graph_launch(self.h, _dptr(self.out)))
        return self.out.copy()

    def launch_async(self):
        _check(_lib.mps_graph_launch_async(self.h))

    def sync(self):
        _check(_lib.mps_graph_sync(self.h, _dptr(self.out)))
        return self.out.copy()

    def update(self):
        _check(_lib.mps_graph_update(self.h))

    def timing(self):
        """(ms reset+ops, ms observables, GEMM-class flops, eigensolver flops,
        op-table bytes per update, result bytes per replay) of the last replay."""
        out = np.zeros(6)
        _check(_lib.mps_graph_timing(self.h, _dptr(out)))
        return tuple(out)

    def phase_cycles(self):
        """SM cycles of the last replay per phase: theta, Gram, eigensolver, split, centre moves."""
        out = np.zeros(5)
        _check(_lib.mps_graph_phase_cycles(self.h, _dptr(out)))
        return dict(zip(["theta", "gram", "eigensolver", "split", "moves"], out.tolist()))

    STAT_NAMES = ["log_fid", "max_disc", "gate2", "ops", "flops", "eig_flops", "cyc_theta", "cyc_gram",
                  "cyc_eig", "cyc_split", "cyc_move", "refined", "cyc_trid", "cyc_bisect", "cyc_vec", "cyc_orth",
                  "cyc_obs"]

    def stat_sums(self):
        """Per-program statistics of the last replay summed over the programs."""
        out = np.zeros(len(self.STAT_NAMES))
        _check(_lib.mps_graph_stat_sums(self.h, _dptr(out), len(self.STAT_NAMES)))
        return dict(zip(self.STAT_NAMES, out.tolist()))

    @property
    def stream(self):
        s = ctypes.c_void_p()
        _check(_lib.mps_graph_stream(self.h, ctypes.byref(s)))
        return s.value

    def close(self):
        if self.h:
            _lib.mps_graph_destroy(self.h)
            self.h = None


class BatchRecord:
    """Many programs' ``encode_circuit`` results concatenated once, then
    recorded on all of them by one C call (``mps_gates_many``; the library
    records the programs on host threads)."""

    def __init__(self, programs, encoded):
        self.programs = list(programs)
        self.arr = (ctypes.c_void_p * len(self.programs))(*[p.h for p in self.programs])
        counts = [len(e[0]) for e in encoded]
        self.first = np.zeros(len(counts) + 1, dtype=np.int64)
        self.first[1:] = np.cumsum(counts)
        self.ids = np.ascontiguousarray(np.concatenate([e[0] for e in encoded]), dtype=np.int32)
        self.qs = np.ascontiguousarray(np.concatenate([e[1] for e in encoded]), dtype=np.int32)
        self.ps = np.ascontiguousarray(np.concatenate([e[2] for e in encoded]), dtype=np.float64)

    def record(self):
        _check(_lib.mps_gates_many(len(self.programs), self.arr,
                                   self.first.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                   self.ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                   self.qs.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _dptr(self.ps)))


def footprint_bytes(n, chi_max, precision):
    load_library()
    return _lib.mps_footprint_bytes(n, chi_max, precision)


class Program:
    """One MPS register.  ``mode``: TRUNC_EXATN or TRUNC_ITENSOR;
    ``precision``: PREC_FP64 or PREC_FP32; ``chi_max <= 0`` means the build's
    limit; ``cutoff < 0`` selects the visitor default."""

    def __init__(self, ctx, n, chi_max=0, cutoff=-1.0, mode=TRUNC_EXATN, precision=PREC_FP64, flags=0):
        self.ctx = ctx
        self.n = n
        h = ctypes.c_void_p()
        _check(_lib.mps_program_begin(ctx.h, n, chi_max, cutoff, mode, precision, flags, ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            _lib.mps_program_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def reset(self):
        _check(_lib.mps_program_reset(self.h))

    @property
    def precision(self):
        """The precision this program runs in (PREC_AUTO resolved)."""
        v = ctypes.c_int()
        _check(_lib.mps_program_precision(self.h, ctypes.byref(v)))
        return v.value

    # ---- gates
    def gate(self, name, qubits, params=()):
        q = (ctypes.c_int * len(qubits))(*qubits)
        p = np.ascontiguousarray(params, dtype=np.float64)
        _check(_lib.mps_gate_named(self.h, name.encode(), q, len(qubits), _dptr(p) if p.size else None, p.size))

    def gate1(self, q, m):
        a = np.ascontiguousarray(np.asarray(m, dtype=np.complex128).reshape(2, 2)).view(np.float64).reshape(-1)
        _check(_lib.mps_gate1(self.h, q, _dptr(a)))

    def gate2(self, q0, q1, m):
        a = np.ascontiguousarray(np.asarray(m, dtype=np.complex128).reshape(4, 4)).view(np.float64).reshape(-1)
        _check(_lib.mps_gate2(self.h, q0, q1, _dptr(a)))

    def measure(self, q):
        _check(_lib.mps_measure(self.h, q))

    def run(self, circuit):
        """Record ``[(name, qubits, params), ...]`` (Measure included)."""
        for name, qs, ps in circuit:
            self.gate(name, list(qs), list(ps))
        return self

    def record(self, encoded):
        """Bulk-record an ``encode_circuit`` result with one C call."""
        ids, qs, ps = encoded
        _check(_lib.mps_gates(self.h, len(ids), ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                              qs.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _dptr(ps)))
        return self

    def submit(self):
        _check(_lib.mps_submit(self.h))

    def wait(self, timeout_ms=-1):
        _check(_lib.mps_wait(self.h, timeout_ms))

    # ---- results
    def norm(self):
        v = ctypes.c_double()
        _check(_lib.mps_norm(self.h, ctypes.byref(v)))
        return v.value

    def amplitudes(self):
        out = np.zeros(2 << self.n, dtype=np.float64)
        _check(_lib.mps_amplitudes(self.h, _dptr(out)))
        return out.view(np.complex128)

    def amplitude(self, bits):
        b = (ctypes.c_int * self.n)(*bits)
        out = np.zeros(2)
        _check(_lib.mps_amplitude(self.h, b, _dptr(out)))
        return complex(out[0], out[1])

    def expect_pauli(self, paulis, coeffs=None):
        """Returns complex <P_t> per term (unnormalised) and, with coeffs,
        also sum_t c_t Re<P_t>."""
        paulis = list(paulis)
        for s in paulis:
            if len(s) != self.n:
                raise ValueError("Pauli string length must equal the qubit count")
        buf = "".join(paulis).encode()
        out = np.zeros(2 * len(paulis) + 1)
        c = None
        if coeffs is not None:
            c = np.ascontiguousarray(coeffs, dtype=np.float64)
        _check(_lib.mps_expect_pauli(self.h, buf, len(paulis), _dptr(c) if c is not None else None, _dptr(out)))
        vals = out[: 2 * len(paulis)].view(np.complex128).copy()
        if coeffs is not None:
            return vals, float(out[2 * len(paulis)])
        return vals

    def set_observable(self, paulis, coeffs):
        paulis = list(paulis)
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        _check(_lib.mps_set_observable(self.h, "".join(paulis).encode(), len(paulis), _dptr(c)))

    @property
    def n_measured(self):
        v = ctypes.c_int()
        _check(_lib.mps_n_measured(self.h, ctypes.byref(v)))
        return v.value

    def sample(self, shots, seed=0):
        nm = self.n_measured
        out = np.zeros((shots, nm), dtype=np.uint8)
        _check(_lib.mps_sample(self.h, shots, seed, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return out

    def truncation_fidelity(self):
        v = ctypes.c_double()
        _check(_lib.mps_truncation_fidelity(self.h, ctypes.byref(v)))
        return v.value

    def bond_dims(self):
        out = (ctypes.c_int * max(self.n - 1, 1))()
        _check(_lib.mps_bond_dims(self.h, out))
        return list(out)[: self.n - 1]

    def stats(self):
        out = np.zeros(4)
        _check(_lib.mps_stats(self.h, _dptr(out)))
        return {"fidelity": out[0], "max_discarded": out[1], "gate2": int(out[2]), "ops": int(out[3])}

    # ---- noisy circuits (DensityProgram)
    def channel(self, q, kraus):
        """rho -> sum_k K_k rho K_k^H on qubit q (density programs)."""
        k = np.ascontiguousarray(np.asarray(kraus, dtype=np.complex128).reshape(-1, 2, 2))
        _check(_lib.mps_channel1(self.h, q, k.shape[0], _dptr(k.view(np.float64).reshape(-1))))

    def density_matrix(self, qubits):
        """rho reduced to ``qubits`` (bit a of an index = qubits[a]), not normalised."""
        qubits = list(qubits)
        k = len(qubits)
        out = np.zeros(2 << (2 * k), dtype=np.float64)
        q = (ctypes.c_int * k)(*qubits)
        _check(_lib.mps_density_matrix(self.h, k, q, _dptr(out)))
        return out.view(np.complex128).reshape(1 << k, 1 << k)

    def density_diag(self, qubits):
        qubits = list(qubits)
        k = len(qubits)
        out = np.zeros(1 << k, dtype=np.float64)
        q = (ctypes.c_int * k)(*qubits)
        _check(_lib.mps_density_diag(self.h, k, q, _dptr(out)))
        return out


class DensityProgram(Program):
    """Noisy circuit: the density matrix of ``n`` qubits as a vectorised MPS
    on 2n sites (MPS_FLAG_DENSITY).  Gates act as rho -> U rho U^H, ``channel``
    applies Kraus channels; ``bond_dims`` lists the 2n-1 bonds of the doubled
    chain."""

    def __init__(self, ctx, n, chi_max=0, cutoff=-1.0, mode=TRUNC_EXATN, precision=PREC_FP64, flags=0):
        super().__init__(ctx, n, chi_max, cutoff, mode, precision, flags | FLAG_DENSITY)

    def bond_dims(self):
        m = 2 * self.n
        out = (ctypes.c_int * (m - 1))()
        _check(_lib.mps_bond_dims(self.h, out))
        return list(out)
