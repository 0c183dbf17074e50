"""Meet-in-the-middle SWAP routing, restated from
``visitors/exatn-mps/NearestNeighborTransform.hpp:43-135`` (oracle).

For a 2-qubit gate with ``|q1 - q2| > max_distance`` the lower qubit is swapped
up and the upper qubit swapped down alternately until they are within the
distance (``:83-99``), the gate runs on the moved qubits keeping the original
bit order (``:102-104``), and the swaps are undone, lower side first
(``:107-115``).
"""


def route(circuit, max_distance=1):
    out = []
    for name, qs, ps in circuit:
        if len(qs) == 2 and abs(qs[0] - qs[1]) > max_distance:
            lo0, hi0 = min(qs), max(qs)
            lo, hi = lo0, hi0
            while True:
                out.append(("Swap", (lo, lo + 1), ()))
                lo += 1
                if abs(lo - hi) <= max_distance:
                    break
                out.append(("Swap", (hi, hi - 1), ()))
                hi -= 1
                if abs(lo - hi) <= max_distance:
                    break
            bits = (lo, hi) if qs[0] < qs[1] else (hi, lo)
            out.append((name, bits, ps))
            for i in range(lo, lo0, -1):
                out.append(("Swap", (i, i - 1), ()))
            for i in range(hi, hi0):
                out.append(("Swap", (i, i + 1), ()))
        else:
            out.append((name, tuple(qs), ps))
    return out
