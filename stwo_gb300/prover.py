"""Proving entry points over the C ABI (prove() of crates/prover/src/core/prover/mod.rs:27-79).

Trace columns live in HBM as torch int32 tensors; proofs come back as canonical bytes.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence, Tuple

import torch

from . import _lib
from ._lib import PcsConfig, call
from .backend import _ptrs, _stream

DEFAULT_CONFIG = (5, 1, 0, 3)  # PcsConfig::default(): pow_bits 5, FriConfig::new(0, 1, 3)

_OUT_CAP = 1 << 26
_out_buf = None


def _out():
    """A reusable host buffer for proof bytes (allocated once; proofs are far smaller)."""
    global _out_buf
    if _out_buf is None:
        _out_buf = (C.c_uint8 * _OUT_CAP)()
    return _out_buf


def pcs_config(cfg: Tuple[int, int, int, int] = DEFAULT_CONFIG) -> PcsConfig:
    """(pow_bits, log_blowup_factor, log_last_layer_degree_bound, n_queries)."""
    return PcsConfig(*cfg)


def wide_fib_trace(log_n_rows: int, n_cols: int, a: torch.Tensor, b: torch.Tensor):
    """generate_trace of the wide-Fibonacci example, on the device."""
    cols = [torch.empty(1 << log_n_rows, dtype=torch.int32, device="cuda") for _ in range(n_cols)]
    call("stwo_gen_wide_fib_trace", log_n_rows, n_cols, a.data_ptr(), b.data_ptr(), _ptrs(cols), _stream())
    return cols


def prove_wide_fib(log_n_rows: int, trace: Sequence[torch.Tensor], cfg=DEFAULT_CONFIG) -> bytes:
    """Proves the wide-Fibonacci AIR over `trace` (consumed: it holds coefficients afterwards)."""
    buf = _out()
    n = C.c_size_t()
    call("stwo_prove_wide_fib", log_n_rows, len(trace), _ptrs(trace), pcs_config(cfg), buf, _OUT_CAP, C.byref(n),
         _stream())
    return C.string_at(buf, n.value)


def prove_poseidon(log_n_rows: int, init=None, cfg=DEFAULT_CONFIG):
    """Proves the Poseidon2 AIR; `init` is None (reference inputs) or a device int32 tensor of
    initial states. Returns (proof bytes, claimed LogUp sum)."""
    from ._lib import QM31

    buf = _out()
    n = C.c_size_t()
    cs = QM31()
    call("stwo_prove_poseidon", log_n_rows, init.data_ptr() if init is not None else None, pcs_config(cfg), buf,
         _OUT_CAP, C.byref(n), C.byref(cs), _stream())
    return C.string_at(buf, n.value), tuple(cs.v)
