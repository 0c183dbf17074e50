"""The engine's recording of noisy circuits, checked without a GPU: a
density program's gates (U on the ket sites, conj(U) on the bra sites) and
Kraus channels (the two-site superoperator on a qubit's ket and bra sites),
compiled by the engine's own program compiler (routing of the distance-2
gates of the doubled chain, 1-qubit fusion, gauge moves), applied to a
dense state of the 2n sites: the result read as rho equals the dense
density-matrix oracle (ExaTnPmpsVisitor.cpp:820-1130 restated) to 1e-12."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import density as R

from .test_host_compile import OP_GATE1, OP_GATE2, apply_ops
from .test_oracle_density import _random_circuit, vec_to_rho

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    from tnqvm_gb300 import build as B
    lib = B.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path_factory.mktemp("hostdensity") / "host_density_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", os.path.join(HERE, "host_density_check.cu"), "-o", exe, "-L", libdir,
                    "-lgb300mps", "-Xlinker", "-rpath=" + libdir], check=True)
    return exe


def compile_noisy(driver, n, mode, flags, circ):
    lines = ["%d %d %d" % (n, mode, flags)]
    for name, qs, ps in circ:
        if name == "Kraus":
            flat = []
            for k in ps:
                for z in np.asarray(k, dtype=np.complex128).reshape(-1):
                    flat += [z.real, z.imag]
            lines.append("K %d %d %s" % (qs[0], len(ps), " ".join("%.17g" % x for x in flat)))
        else:
            p = list(ps) + [0.0] * (3 - len(ps))
            lines.append("G %s %d %d %d %.17g %.17g %.17g" % (name, qs[0], qs[1] if len(qs) > 1 else -1, len(ps),
                                                             *p))
    r = subprocess.run([driver], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    ops = []
    for line in r.stdout.strip().splitlines():
        f = line.split()
        m = np.array([float(x) for x in f[3:]])
        ops.append((int(f[0]), int(f[1]), int(f[2]), m[0::2] + 1j * m[1::2]))
    return ops


@pytest.mark.parametrize("mode,flags", [(0, 0), (1, 0), (1, 4), (0, 8)])
@pytest.mark.parametrize("seed", [1, 2])
def test_compiled_noisy_circuit_reproduces_the_density_oracle(driver, mode, flags, seed):
    rng = np.random.default_rng(70 + seed)
    n = 4
    circ = _random_circuit(n, 4, rng)
    want = R.run(n, circ)
    ops = compile_noisy(driver, n, mode, flags, circ)
    assert all(site + (1 if kind != OP_GATE1 else 0) < 2 * n for kind, site, _, _ in ops)
    got = vec_to_rho(apply_ops(2 * n, ops), n)
    assert np.max(np.abs(got - want)) < 1e-12


def test_channel_is_one_two_site_update(driver):
    """A channel on qubit q is one split on the sites (2q, 2q+1): amplitude
    damping after X on qubit 1 of 3."""
    g = 0.25
    kraus = [np.array([[1, 0], [0, np.sqrt(1 - g)]]), np.array([[0, np.sqrt(g)], [0, 0]])]
    circ = [("X", [1], ()), ("Kraus", [1], kraus)]
    ops = compile_noisy(driver, 3, 0, 0, circ)
    two = [op for op in ops if op[0] == OP_GATE2]
    assert len(two) == 1 and two[0][1] == 2
    rho = vec_to_rho(apply_ops(6, ops), 3)
    assert abs(rho[0, 0].real - g) < 1e-14 and abs(rho[2, 2].real - (1 - g)) < 1e-14
