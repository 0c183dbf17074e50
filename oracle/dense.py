"""Dense complex128 state-vector oracle (test infrastructure only).

Restates ``tnqvm/utils/GateMatrixAlgebra.hpp``: qubit ``q`` is bit ``q`` of the
amplitude index (``ApplySingleQubitGate`` ``:63-82``), expectation of a
product of Z on the measured bits is the parity sum of
``visitors/exatn-mps/ExaTnMpsVisitor.cpp:616-644``, and sampling follows the
sorted-uniform CDF walk of ``GenerateSamples`` ``:125-156``.
"""
import numpy as np

from . import gates as G


def zero_state(n):
    psi = np.zeros(1 << n, dtype=np.complex128)
    psi[0] = 1.0
    return psi


def _axis(n, q):
    # C-order reshape to (2,)*n puts bit q on axis n-1-q.
    return n - 1 - q


def apply_1q(psi, n, q, m):
    t = psi.reshape([2] * n)
    t = np.moveaxis(np.tensordot(m, t, axes=([1], [_axis(n, q)])), 0, _axis(n, q))
    return t.reshape(-1)


def apply_2q(psi, n, a, b, m):
    """Apply a 4x4 matrix whose row index is 2*bit(a)+bit(b) (a = bits()[0])."""
    t = psi.reshape([2] * n)
    m4 = m.reshape(2, 2, 2, 2)
    ax = (_axis(n, a), _axis(n, b))
    t = np.tensordot(m4, t, axes=([2, 3], list(ax)))
    t = np.moveaxis(t, [0, 1], list(ax))
    return t.reshape(-1)


def run(n, circuit):
    """Simulate a gate list ``[(name, qubits, params), ...]``; Measure is skipped."""
    psi = zero_state(n)
    for name, qs, ps in circuit:
        if name == "Measure":
            continue
        m = G.matrix(name, ps)
        if len(qs) == 1:
            psi = apply_1q(psi, n, qs[0], m)
        else:
            psi = apply_2q(psi, n, qs[0], qs[1], m)
    return psi


def expect_z_parity(psi, bits):
    """``exp-val-z`` of ExaTnMpsVisitor.cpp:616-644 (even parity -> +1)."""
    idx = np.arange(psi.size, dtype=np.uint64)
    par = np.zeros(psi.size, dtype=np.uint64)
    for b in bits:
        par ^= (idx >> np.uint64(b)) & np.uint64(1)
    sign = 1.0 - 2.0 * par.astype(np.float64)
    return float(np.sum(sign * np.abs(psi) ** 2))


def expect_pauli(psi, n, pauli):
    """<psi|P|psi> for a Pauli string; character i acts on qubit i."""
    phi = psi
    for q, c in enumerate(pauli):
        if c != "I":
            phi = apply_1q(phi, n, q, G.PAULI[c])
    return complex(np.vdot(psi, phi))


def probabilities(psi, bits):
    """Marginal distribution over the measured bits, keyed like the reference's
    bit strings: character i is the value of qubit ``bits[i]``."""
    p = np.abs(psi) ** 2
    idx = np.arange(psi.size, dtype=np.uint64)
    key = np.zeros(psi.size, dtype=np.uint64)
    for i, b in enumerate(bits):
        key |= ((idx >> np.uint64(b)) & np.uint64(1)) << np.uint64(i)
    out = np.bincount(key.astype(np.int64), weights=p, minlength=1 << len(bits))
    return out  # out[k]: bit i of k = char i of the bit string


def sample(psi, bits, shots, rng):
    """CDF walk over sorted uniforms (GateMatrixAlgebra.hpp:125-156)."""
    rs = np.sort(rng.random(shots))
    cdf = np.cumsum(np.abs(psi) ** 2)
    ks = np.searchsorted(cdf, rs, side="right")
    ks = np.minimum(ks, psi.size - 1).astype(np.uint64)
    out = np.zeros((shots, len(bits)), dtype=np.uint8)
    for i, b in enumerate(bits):
        out[:, i] = ((ks >> np.uint64(b)) & np.uint64(1)).astype(np.uint8)
    return out
