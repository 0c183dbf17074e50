"""The shot sampler's Philox4x32-10 (philox.cuh, shared by the sampling
kernels), built with nvcc as host code, against the published known-answer
vectors of the generator (Salmon et al., SC'11, distributed with Random123),
and its uniform draw against a direct restatement."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

KAT = [  # counter, key -> output
    ("00000000 00000000 00000000 00000000", "00000000 00000000", "6627e8d5 e169c58d bc57ac4c 9b00dbd8"),
    ("ffffffff ffffffff ffffffff ffffffff", "ffffffff ffffffff", "408f276d 41c83b0e a20bc7c6 6d5451fd"),
    ("243f6a88 85a308d3 13198a2e 03707344", "a4093822 299f31d0", "d16cfe09 94fdcceb 5001e420 24126ea1"),
]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("hostphilox") / "host_philox_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", os.path.join(HERE, "host_philox_check.cu"), "-o", exe], check=True)
    return exe


def _philox_py(c, k):
    m = 0xFFFFFFFF
    c, k = list(c), list(k)
    for _ in range(10):
        p0, p1 = 0xD2511F53 * c[0], 0xCD9E8D57 * c[2]
        c = [(p1 >> 32) ^ c[1] ^ k[0], p1 & m, (p0 >> 32) ^ c[3] ^ k[1], p0 & m]
        k = [(k[0] + 0x9E3779B9) & m, (k[1] + 0xBB67AE85) & m]
    return c


def test_known_answer_vectors(driver):
    r = subprocess.run([driver], input="\n".join("%s %s" % (c, k) for c, k, _ in KAT) + "\n", capture_output=True,
                       text=True, check=True)
    lines = r.stdout.strip().splitlines()
    assert lines[:3] == [out for _, _, out in KAT]


def test_uniform_draw(driver):
    r = subprocess.run([driver], input="", capture_output=True, text=True, check=True)
    u = float(r.stdout.split()[-1])
    seed = 0x0123456789ABCDEF
    x = _philox_py([7, 3, 0x4D505321, 0], [seed & 0xFFFFFFFF, seed >> 32])
    assert u == ((x[0] << 32 | x[1]) >> 11) / 2.0 ** 53
    assert 0.0 <= u < 1.0
