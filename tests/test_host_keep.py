"""The engine's truncation rule (keep.cuh, called by both split kernels),
built with nvcc as host code, against the oracle's restatements of ExaTN's
truncateSvdTensors (ExaTnMpsVisitor.cpp:2434-2445) and ITensor's truncate
(decomp.cc:307-463) on random spectra: the kept dimension must be equal."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import mps

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("hostkeep") / "host_keep_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", os.path.join(HERE, "host_keep_check.cu"), "-o", exe], check=True)
    return exe


def spectra(rng, count):
    out = []
    for _ in range(count):
        mm = int(rng.integers(1, 130))
        kind = rng.integers(5)
        if kind == 0:      # geometric decay over many decades
            lam = 10.0 ** (-rng.uniform(0, 30) * np.sort(rng.random(mm)))
        elif kind == 1:    # power law
            lam = (1.0 + np.arange(mm)) ** -rng.uniform(0.5, 8)
        elif kind == 2:    # exact zeros in the tail
            lam = np.sort(rng.random(mm))[::-1].copy()
            lam[int(rng.integers(0, mm)):] = 0.0
        elif kind == 3:    # degenerate plateaus
            lam = np.repeat(np.sort(rng.random(max(1, mm // 4)))[::-1], 4)[:mm].copy()
            lam = np.pad(lam, (0, mm - lam.size))
        else:              # rounding-level negative tail (FP32 Gram eigenvalues)
            lam = np.sort(rng.random(mm))[::-1] ** 6
            lam[int(rng.integers(0, mm)):] -= 1e-9
            lam = np.sort(lam)[::-1].copy()
        lam = lam * 10.0 ** rng.uniform(-6, 6)
        out.append(lam)
    return out


def run_driver(driver, cases):
    lines = ["%d %.17g %d %d %s" % (mode, cut, cap, lam.size, " ".join("%.17g" % v for v in lam))
             for mode, cut, cap, lam in cases]
    r = subprocess.run([driver], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    return [int(x) for x in r.stdout.split()]


def test_exatn_keep_rule_matches_oracle(driver):
    rng = np.random.default_rng(21)
    cases = []
    for lam in spectra(rng, 400):
        cut = 10.0 ** rng.uniform(-16, 0) * np.sqrt(lam[0]) if lam[0] > 0 else 1e-14
        cases.append((0, cut, int(rng.integers(1, 140)), lam))
    got = run_driver(driver, cases)
    for (mode, cut, cap, lam), k in zip(cases, got):
        s = np.sqrt(np.maximum(lam, 0.0))   # singular values; partial norms equal them
        assert k == mps.exatn_keep(s, cut, cap), (cut, cap, lam[:8])


def test_itensor_keep_rule_matches_oracle(driver):
    rng = np.random.default_rng(22)
    cases = []
    for lam in spectra(rng, 400):
        cut = [0.0, 1e-16, 1e-12, 1e-10, 1e-6, 1e-3, 0.1][int(rng.integers(7))]
        cases.append((1, cut, int(rng.integers(1, 140)), lam))
    got = run_driver(driver, cases)
    for (mode, cut, cap, lam), k in zip(cases, got):
        assert k == mps.itensor_truncate(lam, cap, cut)[0], (cut, cap, lam[:8])
