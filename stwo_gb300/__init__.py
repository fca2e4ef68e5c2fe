"""stwo_gb300 — the reference's prover backend trait family on GB300 (sm_103a CUDA behind a C ABI).

`CudaBackend` mirrors ColumnOps / PolyOps / MerkleOps / FriOps / QuotientOps / AccumulationOps /
GrindOps over libstwo_gb300.so (include/stwo_cuda.h).
"""
from ._lib import LIB_PATH, StwoError, load  # noqa: F401

__all__ = ["LIB_PATH", "StwoError", "load"]
