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
    """Proves the Poseidon2 AIR; `init` is None (reference inputs) or an int32 tensor of initial
    states, on the device or in pinned host memory (read by the trace kernel across the host
    link). Returns (proof bytes, claimed LogUp sum)."""
    from ._lib import QM31

    buf = _out()
    n = C.c_size_t()
    cs = QM31()
    call("stwo_prove_poseidon", log_n_rows, init.data_ptr() if init is not None else None, pcs_config(cfg), buf,
         _OUT_CAP, C.byref(n), C.byref(cs), _stream())
    return C.string_at(buf, n.value), tuple(cs.v)


def prove_blake_round(log_n_rows: int, inputs=None, cfg=DEFAULT_CONFIG):
    """Proves the Blake2s round AIR; `inputs` is None (the reference test's inputs) or a device
    int32 tensor of 32 words per row (16 state words, then 16 message words). Returns (proof
    bytes, claimed LogUp sum)."""
    from ._lib import QM31

    buf = _out()
    n = C.c_size_t()
    cs = QM31()
    call("stwo_prove_blake_round", log_n_rows, inputs.data_ptr() if inputs is not None else None, pcs_config(cfg),
         buf, _OUT_CAP, C.byref(n), C.byref(cs), _stream())
    return C.string_at(buf, n.value), tuple(cs.v)


# ------------------------------------------------------------------ batched and served proving
AIR_WIDE_FIB, AIR_POSEIDON, AIR_BLAKE_ROUND = 0, 1, 2


class Job:
    """One whole-proof job: wide-Fibonacci (a, b device tensors of 2^log_n_rows words), Poseidon2
    or the Blake2s round AIR (init: a device tensor of initial states / round inputs, or None for
    the reference inputs)."""

    def __init__(self, air: int, log_n_rows: int, cfg=DEFAULT_CONFIG, n_cols: int = 0, a=None, b=None, init=None,
                 capacity: int = 1 << 22):
        self.air, self.log_n_rows, self.cfg, self.n_cols = air, log_n_rows, cfg, n_cols
        self.a, self.b, self.init = a, b, init  # kept alive while the job runs
        self.buf = (C.c_uint8 * capacity)()
        self.c = _lib.ProofJob(air, log_n_rows, n_cols, a.data_ptr() if a is not None else None,
                               b.data_ptr() if b is not None else None,
                               init.data_ptr() if init is not None else None, pcs_config(cfg),
                               C.cast(self.buf, C.c_void_p), capacity)

    def hbm_bytes(self) -> int:
        return _lib.load().stwo_job_hbm_bytes(C.byref(self.c))


class Result:
    def __init__(self, job: Job, r):
        self.proof = C.string_at(job.buf, r.len)
        self.claimed_sum = tuple(r.claimed_sum.v)
        self.queue_ms, self.run_ms, self.latency_ms = r.queue_ms, r.run_ms, r.latency_ms


class Server:
    """A pool of workers, one CUDA stream each, running submitted jobs with HBM-budget
    admission (stwo_server_*)."""

    def __init__(self, n_workers: int = 8, hbm_budget: int = 0, device: int = None):
        dev = torch.cuda.current_device() if device is None else device
        h = C.c_void_p()
        call("stwo_server_create", n_workers, hbm_budget, dev, C.byref(h))
        self.h = h
        self.jobs = {}

    def submit(self, job: Job) -> int:
        t = C.c_uint64()
        call("stwo_server_submit", self.h, C.byref(job.c), C.byref(t))
        self.jobs[t.value] = job
        return t.value

    def wait(self, ticket: int) -> Result:
        r = _lib.ProofResult()
        call("stwo_server_wait", self.h, ticket, C.byref(r))
        job = self.jobs.pop(ticket)
        if r.status != 0:
            raise _lib.StwoError(r.status, "server job", r.error.decode(errors="replace"))
        return Result(job, r)

    def close(self):
        if self.h:
            _lib.load().stwo_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def prove_batch(jobs: Sequence[Job], n_workers: int = 8, hbm_budget: int = 0):
    """Runs all jobs on a temporary server (stwo_prove_batch); results in job order."""
    arr = (_lib.ProofJob * max(1, len(jobs)))(*[j.c for j in jobs])
    res = (_lib.ProofResult * max(1, len(jobs)))()
    call("stwo_prove_batch", arr, len(jobs), n_workers, hbm_budget, res)
    return [Result(j, res[i]) for i, j in enumerate(jobs)]
