"""GB300-native matrix-product-state circuit engine (TNQVM MPS visitor path).

Modules: ``mps`` (ctypes binding of the C ABI), ``visitor`` (TNQVM visitor
interface mirror), ``circuits`` (seeded workloads), ``build`` (nvcc build).
"""
from .mps import (Context, MpsError, Program, load_library, PREC_FP32, PREC_FP64,  # noqa: F401
                  TRUNC_EXATN, TRUNC_ITENSOR, FLAG_PER_GATE, FLAG_RENORM, CHI_LIMIT)
