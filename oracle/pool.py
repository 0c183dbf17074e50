"""Process-parallel runs of the complex128 MPS oracle (test infrastructure
only): one circuit per worker process, one worker per host core, each worker
with single-threaded BLAS (LAPACK on matrices of side <= 128 does not spread
over cores, so one circuit per core is how the host's cores are all used).

Workers are started with the ``spawn`` method, so a pool is safe to create
after the parent process has initialised CUDA.
"""
import multiprocessing as mp
import os
import time

_BLAS_ENV = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")


def _energy_task(task):
    """<H>/<psi|psi> of one circuit in the given truncation semantics, and the
    seconds it took."""
    from . import mps as omps
    from . import routing
    n, circuit, paulis, coeffs, chi, cutoff, mode = task
    t0 = time.perf_counter()
    m = omps.run(n, routing.route(circuit), mode=mode, chi_max=chi, cutoff=cutoff)
    e = sum(c * m.expect_pauli(s).real for s, c in zip(paulis, coeffs)) / m.norm2()
    return float(e), time.perf_counter() - t0


class OraclePool:
    """A pool of ``workers`` spawned processes (default: every host core)."""

    def __init__(self, workers=None):
        self.workers = max(1, workers or os.cpu_count() or 1)
        saved = {k: os.environ.get(k) for k in _BLAS_ENV}
        for k in _BLAS_ENV:
            os.environ[k] = "1"
        try:
            self.pool = mp.get_context("spawn").Pool(self.workers)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        # import the oracle in every worker before any timing
        self.pool.map(_warm, range(self.workers))

    def energies(self, insts, chi, cutoff, mode="itensor"):
        """Energies of ``insts`` (dicts with n, circuit, paulis, coeffs), in
        order, costliest first to balance the workers; returns (energies,
        wall seconds, summed worker seconds)."""
        order = sorted(range(len(insts)), key=lambda i: -insts[i]["n"] * len(insts[i]["circuit"]))
        tasks = [(insts[i]["n"], insts[i]["circuit"], list(insts[i]["paulis"]), list(insts[i]["coeffs"]), chi,
                  cutoff, mode) for i in order]
        t0 = time.perf_counter()
        res = self.pool.map(_energy_task, tasks, chunksize=1)
        wall = time.perf_counter() - t0
        out = [0.0] * len(insts)
        busy = 0.0
        for i, (e, dt) in zip(order, res):
            out[i] = e
            busy += dt
        return out, wall, busy

    def close(self):
        self.pool.close()
        self.pool.join()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _warm(_):
    from . import mps, routing  # noqa: F401
    return os.getpid()
