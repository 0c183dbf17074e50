"""complex128 MPS oracle with the reference's two update semantics (test
infrastructure only).

Site tensors are stored as ``A[i]`` of shape ``(chi_left, 2, chi_right)``;
site 0 has ``chi_left == 1`` and the last site ``chi_right == 1``.  This is the
index order of the exatn-mps middle tensors ``Qi(left, phys, right)``
(``visitors/exatn-mps/ExaTnMpsVisitor.cpp:1684-1695``).

``mode="exatn"`` follows ``ExatnMpsVisitor``:

* 1-qubit gate: ``Q'(a,b,c) = sum_i Q(a,i,c) M[b][i]`` (``:1244-1247``).
* 2-qubit gate: merge the two neighbouring sites, contract the gate
  (``:1412-1524``), zero entries below 1e-100 (``stabilizeTensorBody``
  ``:141-161``), SVD into two factors with the singular values split as
  ``sqrt(S)`` on both sides (``decomposeTensorSVDLRSync`` ``:1623``), new bond
  ``min(vol(Qi\\bond), vol(Qj\\bond))`` (``:1594``), then
  ``truncateSvdTensors`` (``:2366-2536``): partial norms of both factors
  along the bond, keep ``i+1`` where ``i`` is the first index whose two
  partial norms are both below the cutoff, cap by ``max-bond-dim``; no
  renormalisation, no gauge moves.  The partial norm is taken as the sum of
  squared moduli over the other indices, as the reference's comment at
  ``:2418-2419`` states; with sqrt(S) on both sides it equals the singular
  value.

``mode="itensor"`` follows ``ITensorMPSVisitor``:

* orthogonality centre moved to the gate (``position``, ``.cpp:294,317``),
* two-site SVD with ITensor's relative truncation (``decomp.cc:307-463``,
  ``svd.cc:79-125``): ``P = s^2``, cut to ``maxdim`` first, then drop the tail
  while the dropped weight is ``<= cutoff * sum(P)``, keep at least one,
* ``U`` on the site of ``bits()[0]`` and ``S*V`` on the other (``.cpp:329-330``),
  no renormalisation.
"""
import sys

import numpy as np

from . import gates as G

DBL_MIN = sys.float_info.min
INT_MAX_M1 = 2 ** 31 - 2


def swap_bits_4x4(m):
    """Re-express a 4x4 matrix with the two qubits exchanged."""
    p = [0, 2, 1, 3]
    return m[np.ix_(p, p)]


def site_matrix(m, a, b):
    """4x4 matrix in site order (row = 2*phys(lo) + phys(hi))."""
    return m if a < b else swap_bits_4x4(m)


def itensor_truncate(P, maxdim, cutoff, mindim=1):
    """Number of kept values and truncation error; restates ITensor
    ``truncate`` (``decomp.cc:307-463``) with ``absoluteCutoff=false``,
    ``doRelCutoff=true`` and ``RespectDegenerate=false``."""
    P = np.array(P, dtype=np.float64)
    origm = P.size
    if P[0] == 0.0 or origm == 1:
        return 1, 0.0
    P0 = P[0]
    P = P / P0
    n = origm - 1
    for zn in range(n, -1, -1):
        if P[zn] >= 0:
            break
        P[zn] = 0.0
    truncerr = 0.0
    while n >= maxdim:
        truncerr += P[n]
        n -= 1
    scale = P.sum()
    if scale == 0.0:
        scale = 1.0
    while n >= mindim and truncerr + P[n] <= cutoff * scale:
        truncerr += P[n]
        n -= 1
    truncerr = truncerr / scale
    if n < 0:
        n = 0
    return n + 1, truncerr


def exatn_keep(s, cutoff, max_bond):
    """Bond kept by ``truncateSvdTensors`` (ExaTnMpsVisitor.cpp:2434-2445)."""
    bond = s.size
    k = bond
    for i in range(bond):
        if s[i] < cutoff:          # both partial norms equal s[i]
            k = i + 1
            break
    return min(k, max_bond)


class MPS:
    def __init__(self, n, mode="exatn", chi_max=None, cutoff=None, renorm=False, svd=None):
        """``svd``: the SVD routine (default numpy's LAPACK gesdd); another
        driver measures how sensitive a run is to the SVD's rounding."""
        assert mode in ("exatn", "itensor")
        self.svd = np.linalg.svd if svd is None else svd
        self.n = n
        self.mode = mode
        if mode == "exatn":
            self.chi_max = INT_MAX_M1 if chi_max is None else int(chi_max)
            self.cutoff = DBL_MIN if cutoff is None else float(cutoff)
        else:
            # ITensorMPSVisitor.cpp:115-116 defaults
            self.chi_max = 1024 if chi_max is None else int(chi_max)
            self.cutoff = 1e-6 if cutoff is None else float(cutoff)
        self.renorm = renorm
        self.A = []
        for _ in range(n):
            t = np.zeros((1, 2, 1), dtype=np.complex128)
            t[0, 0, 0] = 1.0
            self.A.append(t)
        self.center = 0
        self.discarded = []      # per 2-qubit gate: discarded weight fraction
        self.fidelity = 1.0

    # ----------------------------------------------------------- gauge
    def _move_right(self, c):
        a = self.A[c]
        dl, _, dr = a.shape
        q, r = np.linalg.qr(a.reshape(dl * 2, dr))
        k = q.shape[1]
        self.A[c] = q.reshape(dl, 2, k)
        self.A[c + 1] = np.tensordot(r, self.A[c + 1], axes=([1], [0]))

    def _move_left(self, c):
        a = self.A[c]
        dl, _, dr = a.shape
        q, r = np.linalg.qr(a.reshape(dl, 2 * dr).conj().T)
        k = q.shape[1]
        self.A[c] = q.conj().T.reshape(k, 2, dr)
        self.A[c - 1] = np.tensordot(self.A[c - 1], r.conj().T, axes=([2], [0]))

    def position(self, site):
        while self.center < site:
            self._move_right(self.center)
            self.center += 1
        while self.center > site:
            self._move_left(self.center)
            self.center -= 1

    # ----------------------------------------------------------- gates
    def gate1(self, q, m):
        self.A[q] = np.einsum("bi,aic->abc", m, self.A[q])

    def theta(self, lo, msite):
        a, b = self.A[lo], self.A[lo + 1]
        dl, dr = a.shape[0], b.shape[2]
        t = np.einsum("lim,mjr->lijr", a, b)
        th = np.einsum("abij,lijr->labr", msite.reshape(2, 2, 2, 2), t)
        return th.reshape(2 * dl, 2 * dr), dl, dr

    def gate2(self, qa, qb, m):
        assert abs(qa - qb) == 1, "nearest-neighbour only; route first"
        lo = min(qa, qb)
        msite = site_matrix(m, qa, qb)
        if self.mode == "itensor":
            # position(bits()[0]) (ITensorMPSVisitor.cpp:317)
            self.position(qa)
        th, dl, dr = self.theta(lo, msite)
        if self.mode == "exatn":
            th = np.where(np.abs(th) < 1e-100, 0.0, th)
        u, s, vh = self.svd(th, full_matrices=False)
        total = float(np.sum(s ** 2))
        if self.mode == "exatn":
            k = exatn_keep(s, self.cutoff, self.chi_max)
            sq = np.sqrt(s[:k])
            left = u[:, :k] * sq
            right = sq[:, None] * vh[:k]
        else:
            k, _ = itensor_truncate(s ** 2, self.chi_max, self.cutoff)
            if qa == lo:
                left = u[:, :k]
                right = s[:k, None] * vh[:k]
                self.center = lo + 1
            else:
                left = u[:, :k] * s[:k]
                right = vh[:k]
                self.center = lo
        kept = float(np.sum(s[:k] ** 2))
        frac = 0.0 if total == 0.0 else (total - kept) / total
        self.discarded.append(frac)
        self.fidelity *= (1.0 - frac)
        if self.renorm and kept > 0.0:
            scale = np.sqrt(total / kept)
            right = right * scale
        self.A[lo] = left.reshape(dl, 2, k)
        self.A[lo + 1] = right.reshape(k, 2, dr)

    def apply(self, name, qubits, params=()):
        m = G.matrix(name, params)
        if len(qubits) == 1:
            self.gate1(qubits[0], m)
        else:
            self.gate2(qubits[0], qubits[1], m)

    # ----------------------------------------------------------- measure
    def bond_dims(self):
        return [a.shape[2] for a in self.A[:-1]]

    def expect_ops(self, ops):
        """<psi| prod_i ops[i] |psi> by a left-to-right transfer-matrix sweep
        (ITensorMPSVisitor.cpp:173-250 generalised to any local operator)."""
        e = np.ones((1, 1), dtype=np.complex128)
        for i, a in enumerate(self.A):
            op = ops[i]
            if op is None:
                x = np.tensordot(e, a, axes=([1], [0]))            # (l, s, r')
            else:
                pa = np.einsum("st,ltr->lsr", op, a)
                x = np.tensordot(e, pa, axes=([1], [0]))
            e = np.tensordot(a.conj(), x, axes=([0, 1], [0, 1]))  # (r, r')
        return complex(e[0, 0])

    def expect_pauli(self, pauli):
        ops = [None if c == "I" else G.PAULI[c] for c in pauli]
        return self.expect_ops(ops)

    def norm2(self):
        return self.expect_ops([None] * self.n).real

    def amplitudes(self):
        """Full state vector with qubit k on bit k (n small)."""
        v = np.ones((1, 1), dtype=np.complex128)      # (bond, 2^k)
        for a in self.A:
            dl, _, dr = a.shape
            v0 = a[:, 0, :].T @ v
            v1 = a[:, 1, :].T @ v
            v = np.concatenate([v0, v1], axis=1)
        return v.reshape(-1)


def run(n, circuit, mode="exatn", chi_max=None, cutoff=None, renorm=False):
    """Simulate ``[(name, qubits, params), ...]``; non-adjacent 2-qubit gates
    must already be routed (``oracle.routing``)."""
    mps = MPS(n, mode, chi_max, cutoff, renorm)
    for name, qs, ps in circuit:
        if name == "Measure":
            continue
        mps.apply(name, qs, ps)
    return mps
