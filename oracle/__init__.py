"""CPU oracle for the MPS circuit-simulation path (test infrastructure only).

This package restates, in numpy complex128, the arithmetic of the reference
TNQVM MPS visitors so that the GPU engine can be checked against it:

* ``gates``   - gate matrices of ``tnqvm/base/Gates.hpp:131-334``.
* ``dense``   - dense state-vector helpers of ``tnqvm/utils/GateMatrixAlgebra.hpp``
                (qubit 0 is the least significant bit, as in
                ``visitors/exatn-mps/ExaTnMpsVisitor.cpp:616-634``).
* ``mps``     - the two MPS update semantics:
                ``exatn`` (``visitors/exatn-mps/ExaTnMpsVisitor.cpp:1387-1730``
                and ``truncateSvdTensors`` ``:2366-2536``) and
                ``itensor`` (``visitors/itensor/mps/ITensorMPSVisitor.cpp:288-331``
                with ITensor's ``truncate``, ``tpls/itensor/decomp.cc:307-463``).
* ``routing`` - the meet-in-the-middle SWAP insertion of
                ``visitors/exatn-mps/NearestNeighborTransform.hpp:43-135``.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import this package, and only as
the checker or the timed CPU baseline.  The product path (``tnqvm_gb300``)
never imports it and has no CPU fallback.

Parity pins: the oracle is checked against the analytic and dense-helper
golden values of the reference's own tests (``tests/test_oracle_golden.py``)
and, where the vendored ITensor could be compiled here, against fixtures
produced by the ITensor driver in ``oracle/itensor_driver`` (committed under
``tests/golden/``).  The exatn-mode truncation rule (absolute per-index cutoff
on the partial norms of the split factors) is not pinned by any reference test
("parity unpinned" for bond dimensions under exatn-mode truncation); values
of observables are pinned through the dense oracle wherever the bond cap is
exact.
"""
