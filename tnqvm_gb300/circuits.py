"""Seeded synthetic circuit families for the MPS engine's workloads.

A circuit is a list of ``(name, qubits, params)`` with XACC gate names.
Families:

* ``brickwall``  - 1D random circuit: per layer U3(theta, phi, lambda) on every
  qubit with angles uniform in [0, 2pi), then an entangler on even pairs
  (2i, 2i+1) and on odd pairs (2i+1, 2i+2).  With CNOT, n=12, depth 20 this is
  the 12-qubit exact workload; with CZ, n=48, depth 30 the 48-qubit
  mixed-precision workload.
* ``hea``        - hardware-efficient ansatz: per layer Ry, Rz on every qubit
  (params uniform in [-pi, pi]) then a CNOT ladder (i, i+1), i = 0..n-2.
* ``vqe_batch``  - 1024 ``hea`` instances, qubits uniform in 8..32, layers
  uniform in 4..12, each with a random 50-term Pauli Hamiltonian (letters
  uniform over IXYZ, coefficients N(0,1)).
* ``qaoa_maxcut`` - H on all, then p rounds of RZZ(gamma) on the edges of a
  seeded random 3-regular graph and Rx(2 beta) on all.
* ``supremacy_1d`` - H on all, then per round a random local gate per qubit
  and CNOTs on even then odd pairs (the 1D circuits of the reference's
  memory-profiling study, ``examples/plos_one_experiments/experiments/profile_tnqvm.py:32-57``).
"""
import numpy as np


def brickwall(n, depth, seed, entangler="CNOT"):
    rng = np.random.default_rng(seed)
    c = []
    for _ in range(depth):
        for q in range(n):
            c.append(("U", (q,), tuple(rng.uniform(0.0, 2 * np.pi, 3))))
        for q in range(0, n - 1, 2):
            c.append((entangler, (q, q + 1), ()))
        for q in range(1, n - 1, 2):
            c.append((entangler, (q, q + 1), ()))
    return c


def hea(n, layers, seed):
    rng = np.random.default_rng(seed)
    c = []
    for _ in range(layers):
        for q in range(n):
            c.append(("Ry", (q,), (rng.uniform(-np.pi, np.pi),)))
            c.append(("Rz", (q,), (rng.uniform(-np.pi, np.pi),)))
        for q in range(n - 1):
            c.append(("CNOT", (q, q + 1), ()))
    return c


def random_paulis(n, terms, rng):
    letters = np.array(list("IXYZ"))
    strs = ["".join(letters[rng.integers(0, 4, n)]) for _ in range(terms)]
    coeffs = rng.normal(0.0, 1.0, terms)
    return strs, coeffs


def vqe_batch(instances=1024, seed=2024, qmin=8, qmax=32, lmin=4, lmax=12, terms=50):
    """List of dicts {n, layers, circuit, paulis, coeffs}."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(instances):
        n = int(rng.integers(qmin, qmax + 1))
        L = int(rng.integers(lmin, lmax + 1))
        circ = hea(n, L, int(rng.integers(0, 2 ** 31)))
        paulis, coeffs = random_paulis(n, terms, rng)
        out.append({"n": n, "layers": L, "circuit": circ, "paulis": paulis, "coeffs": coeffs})
    return out


def random_regular3(n, seed):
    """Seeded random 3-regular simple graph (pairing model with restarts)."""
    rng = np.random.default_rng(seed)
    assert (3 * n) % 2 == 0
    for _ in range(10000):
        stubs = np.repeat(np.arange(n), 3)
        rng.shuffle(stubs)
        pairs = stubs.reshape(-1, 2)
        ok = True
        seen = set()
        for a, b in pairs:
            if a == b:
                ok = False
                break
            e = (min(a, b), max(a, b))
            if e in seen:
                ok = False
                break
            seen.add(e)
        if ok:
            return sorted((int(a), int(b)) for a, b in seen)
    raise RuntimeError("no 3-regular graph found")


def qaoa_maxcut(n=64, p=3, seed=7, as_cnot=True):
    rng = np.random.default_rng(seed)
    edges = random_regular3(n, int(rng.integers(0, 2 ** 31)))
    gammas = rng.uniform(0.0, np.pi, p)
    betas = rng.uniform(0.0, np.pi, p)
    c = [("H", (q,), ()) for q in range(n)]
    for k in range(p):
        for a, b in edges:
            if as_cnot:
                c.append(("CNOT", (a, b), ()))
                c.append(("Rz", (b,), (float(gammas[k]),)))
                c.append(("CNOT", (a, b), ()))
            else:
                c.append(("RZZ", (a, b), (float(gammas[k]),)))
        for q in range(n):
            c.append(("Rx", (q,), (2.0 * float(betas[k]),)))
    return c, edges


def supremacy_1d(n, rounds, seed):
    rng = np.random.default_rng(seed)
    c = [("H", (q,), ()) for q in range(n)]
    local = ["X", "Y", "Z", "Rx", "Ry", "Rz", "H"]
    for _ in range(rounds):
        for q in range(n):
            g = local[int(rng.integers(0, len(local)))]
            c.append((g, (q,), (float(rng.uniform(0.0, np.pi)),) if g[0] == "R" else ()))
        for q in range(0, n - 1, 2):
            c.append(("CNOT", (q, q + 1), ()))
        for q in range(1, n - 1, 2):
            c.append(("CNOT", (q, q + 1), ()))
    return c
