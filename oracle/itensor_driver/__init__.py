"""Build hook for the ITensor reference driver (test infrastructure only).

``build_if_available()`` runs the Makefile beside this file when the reference
tree and scipy's bundled OpenBLAS are present; the binary lands in
``oracle/_ref/itensor_driver``.  Elsewhere (e.g. a machine without the
reference tree) it does nothing; the committed fixtures in ``tests/golden``
carry its results.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree: TNQVM_REFERENCE_ROOT, else a "reference" folder beside the repository
REF = os.environ.get("TNQVM_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))),
                                                             "reference")
BINARY = os.path.join(os.path.dirname(HERE), "_ref", "itensor_driver")


def build_if_available():
    if not os.path.isdir(os.path.join(REF, "tnqvm", "visitors", "itensor", "tpls", "itensor")):
        return None
    if os.path.exists(BINARY):
        return BINARY
    jobs = str(max(1, min(8, os.cpu_count() or 1)))
    r = subprocess.run(["make", "-C", HERE, "-j", jobs, "REF=" + REF], capture_output=True, text=True)
    if r.returncode != 0:
        return None
    return BINARY
