"""Gate matrices, restated from ``tnqvm/base/Gates.hpp:131-334`` (oracle).

Every matrix is complex128.  Two-qubit matrices use the reference convention
that ``bits()[0]`` is the most significant bit of the 4x4 row/column index
(``Gates.hpp:237-246`` CNOT; ``visitors/exatn-mps/ExatnUtils.cpp:116-130``).
"""
import numpy as np

_S2 = np.sqrt(0.5)


def _c(x):
    return np.array(x, dtype=np.complex128)


def matrix(name, params=()):
    """Return the gate matrix for an XACC gate name (``Gates.hpp:41-67``)."""
    p = [float(v) for v in params]
    e = np.exp
    if name == "I":
        return _c([[1, 0], [0, 1]])
    if name == "H":                                   # Gates.hpp:141-147
        return _c([[_S2, _S2], [_S2, -_S2]])
    if name == "X":
        return _c([[0, 1], [1, 0]])
    if name == "Y":
        return _c([[0, -1j], [1j, 0]])
    if name == "Z":
        return _c([[1, 0], [0, -1]])
    if name == "S":
        return _c([[1, 0], [0, 1j]])
    if name == "Sdg":
        return _c([[1, 0], [0, -1j]])
    if name == "T":                                   # Gates.hpp:207-213
        return _c([[1, 0], [0, e(1j * np.pi / 4)]])
    if name == "Tdg":
        return _c([[1, 0], [0, e(-1j * np.pi / 4)]])
    if name == "Rx":                                  # Gates.hpp:178-185
        t = p[0]
        return _c([[np.cos(t / 2), -1j * np.sin(t / 2)],
                   [-1j * np.sin(t / 2), np.cos(t / 2)]])
    if name == "Ry":                                  # Gates.hpp:188-194
        t = p[0]
        return _c([[np.cos(t / 2), -np.sin(t / 2)],
                   [np.sin(t / 2), np.cos(t / 2)]])
    if name == "Rz":                                  # Gates.hpp:198-204
        t = p[0]
        return _c([[e(-0.5j * t), 0], [0, e(0.5j * t)]])
    if name in ("U", "U3"):                           # Gates.hpp:224-235
        th, ph, lm = p
        return _c([[np.cos(th / 2), -e(1j * lm) * np.sin(th / 2)],
                   [e(1j * ph) * np.sin(th / 2), e(1j * (ph + lm)) * np.cos(th / 2)]])
    if name in ("CNOT", "CX"):                        # Gates.hpp:238-246
        return _c([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]])
    if name == "CZ":                                  # Gates.hpp:249-257
        return np.diag(_c([1, 1, 1, -1]))
    if name == "CY":
        return _c([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, -1j], [0, 0, 1j, 0]])
    if name == "CH":
        return _c([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, _S2, _S2], [0, 0, _S2, -_S2]])
    if name == "CRZ":
        t = p[0]
        return np.diag(_c([1, 1, e(-0.5j * t), e(0.5j * t)]))
    if name == "CPhase":
        t = p[0]
        return np.diag(_c([1, 1, 1, e(1j * t)]))
    if name == "Swap":                                # Gates.hpp:304-312
        return _c([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]])
    if name == "iSwap":
        return _c([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]])
    if name == "fSim":                                # Gates.hpp:326-334
        th, ph = p
        return _c([[1, 0, 0, 0],
                   [0, np.cos(th), -1j * np.sin(th), 0],
                   [0, -1j * np.sin(th), np.cos(th), 0],
                   [0, 0, 0, e(-1j * ph)]])
    if name == "RZZ":
        # exp(-i t/2 Z(x)Z): the diagonal that CNOT.Rz(t).CNOT produces.
        t = p[0]
        return np.diag(_c([e(-0.5j * t), e(0.5j * t), e(0.5j * t), e(-0.5j * t)]))
    raise KeyError(name)


PAULI = {
    "I": _c([[1, 0], [0, 1]]),
    "X": _c([[0, 1], [1, 0]]),
    "Y": _c([[0, -1j], [1j, 0]]),
    "Z": _c([[1, 0], [0, -1]]),
}
