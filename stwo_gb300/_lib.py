"""ctypes binding of include/stwo_cuda.h (libstwo_gb300.so, built in-tree for sm_103a).

Loading fails loudly: there is no CPU fallback for any backend operation.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libstwo_gb300.so")

STWO_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "TIMEOUT", 4: "CUDA_ERROR", 5: "UNSUPPORTED"}


class StwoError(RuntimeError):
    def __init__(self, status: int, fn: str, detail: str):
        super().__init__(f"{fn} failed: {STATUS_NAMES.get(status, status)}: {detail}")
        self.status = status


class Coset(C.Structure):
    _fields_ = [("initial_index", C.c_uint32), ("step_size", C.c_uint32), ("log_size", C.c_uint32)]


class QM31(C.Structure):
    _fields_ = [("v", C.c_uint32 * 4)]


class QM31Point(C.Structure):
    _fields_ = [("x", QM31), ("y", QM31)]


class PcsConfig(C.Structure):
    _fields_ = [("pow_bits", C.c_uint32), ("log_blowup_factor", C.c_uint32),
                ("log_last_layer_degree_bound", C.c_uint32), ("n_queries", C.c_uint32)]


class SampleBatch(C.Structure):
    _fields_ = [
        ("point", QM31Point),
        ("n_columns", C.c_uint32),
        ("h_column_indices", C.POINTER(C.c_uint32)),
        ("h_values", C.POINTER(QM31)),
    ]


P4 = C.c_void_p * 4
VP = C.c_void_p
U32 = C.c_uint32
PVP = C.POINTER(C.c_void_p)

# name -> (restype, argtypes); every symbol declared in include/stwo_cuda.h.
class ProofJob(C.Structure):
    _fields_ = [("air", C.c_uint32), ("log_n_rows", C.c_uint32), ("n_cols", C.c_uint32), ("d_a", C.c_void_p),
                ("d_b", C.c_void_p), ("d_init", C.c_void_p), ("cfg", PcsConfig), ("h_proof", C.c_void_p),
                ("capacity", C.c_size_t)]


class Component(C.Structure):
    _fields_ = [("air", C.c_uint32), ("log_n_rows", C.c_uint32), ("n_cols", C.c_uint32), ("claimed_sum", QM31),
                ("h_elements", C.POINTER(QM31)), ("n_elements", C.c_uint32)]


class ProofResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("len", C.c_size_t), ("claimed_sum", QM31), ("queue_ms", C.c_double),
                ("run_ms", C.c_double), ("latency_ms", C.c_double), ("error", C.c_char * 256)]


SIGNATURES = {
    "stwo_status_string": (C.c_char_p, [C.c_int32]),
    "stwo_last_error": (C.c_char_p, []),
    "stwo_device_init": (C.c_int32, [C.c_int]),
    "stwo_sync": (C.c_int32, [VP]),
    "stwo_kernel_launches": (C.c_uint64, []),
    "stwo_set_stage_timing": (C.c_int32, [C.c_int]),
    "stwo_butterfly_rate": (C.c_int32, [U32, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double), VP]),
    "stwo_blake2s_rate": (C.c_int32, [U32, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double), VP]),
    "stwo_autotune_mode": (C.c_int32, [C.c_int]),
    "stwo_autotune_entries": (U32, [C.POINTER(U32), C.POINTER(C.c_uint64), C.POINTER(U32), U32]),
    "stwo_autotune_set_entry": (C.c_int32, [U32, C.c_uint64, U32]),
    "stwo_autotune_clear": (C.c_int32, []),
    "stwo_stage_times": (C.c_uint32, [C.POINTER(C.c_char_p), C.POINTER(C.c_float), U32]),
    "stwo_buf_alloc": (C.c_int32, [PVP, C.c_size_t, VP]),
    "stwo_buf_free": (C.c_int32, [VP, VP]),
    "stwo_buf_upload": (C.c_int32, [VP, VP, C.c_size_t, VP]),
    "stwo_buf_download": (C.c_int32, [VP, VP, C.c_size_t, VP]),
    "stwo_buf_zero": (C.c_int32, [VP, C.c_size_t, VP]),
    "stwo_read_words": (C.c_int32, [VP, C.POINTER(C.c_uint64), C.c_size_t, C.POINTER(C.c_uint32), VP]),
    "stwo_read_words_cols": (C.c_int32, [VP, C.c_size_t, C.POINTER(C.c_uint64), C.c_size_t, C.POINTER(C.c_uint32),
                                         VP]),
    "stwo_twiddles_precompute": (C.c_int32, [Coset, PVP, VP]),
    "stwo_twiddles_free": (C.c_int32, [VP]),
    "stwo_twiddles_info": (C.c_int32, [VP, C.POINTER(Coset), PVP, PVP, C.POINTER(C.c_size_t)]),
    "stwo_interpolate_columns": (C.c_int32, [VP, Coset, PVP, U32, VP]),
    "stwo_evaluate_columns": (C.c_int32, [VP, Coset, PVP, U32, PVP, U32, VP]),
    "stwo_extend": (C.c_int32, [VP, U32, VP, U32, VP]),
    "stwo_eval_at_points": (C.c_int32, [PVP, C.POINTER(C.c_uint32), U32, C.POINTER(C.c_uint32),
                                        C.POINTER(QM31Point), U32, C.POINTER(QM31), VP]),
    "stwo_eval_at_points_noalloc": (C.c_int32, [PVP, C.POINTER(C.c_uint32), U32, C.POINTER(C.c_uint32),
                                                C.POINTER(QM31Point), U32, C.POINTER(QM31), VP]),
    "stwo_bit_reverse_column": (C.c_int32, [VP, U32, VP]),
    "stwo_merkle_commit_layer": (C.c_int32, [U32, VP, PVP, U32, VP, VP]),
    "stwo_fri_fold_line": (C.c_int32, [VP, Coset, PVP, QM31, PVP, VP]),
    "stwo_fri_fold_circle_into_line": (C.c_int32, [VP, Coset, PVP, PVP, QM31, VP]),
    "stwo_fri_decompose": (C.c_int32, [PVP, U32, PVP, C.POINTER(QM31), VP]),
    "stwo_accumulate_quotients": (C.c_int32, [U32, PVP, U32, QM31, C.POINTER(SampleBatch), U32, U32, PVP, VP]),
    "stwo_secure_accumulate": (C.c_int32, [PVP, PVP, C.c_size_t, VP]),
    "stwo_generate_secure_powers": (C.c_int32, [QM31, U32, C.POINTER(QM31), VP]),
    "stwo_gkr_gen_eq_evals": (C.c_int32, [C.POINTER(QM31), U32, QM31, PVP, VP]),
    "stwo_gkr_next_layer": (C.c_int32, [U32, U32, PVP, PVP, PVP, PVP, VP]),
    "stwo_gkr_sum_as_poly_in_first_variable": (C.c_int32, [U32, U32, PVP, PVP, PVP, C.POINTER(QM31), U32, QM31, QM31,
                                                           QM31, C.POINTER(QM31), C.POINTER(C.c_uint32), VP]),
    "stwo_mle_fix_first_variable_base": (C.c_int32, [U32, VP, QM31, PVP, VP]),
    "stwo_mle_fix_first_variable_secure": (C.c_int32, [U32, PVP, QM31, PVP, VP]),
    "stwo_gkr_prove_batch": (C.c_int32, [U32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), PVP, PVP, VP, VP,
                                         C.c_size_t, C.POINTER(C.c_size_t), VP, VP]),
    "stwo_grind_blake2s": (C.c_int32, [C.POINTER(C.c_uint32), U32, C.POINTER(C.c_uint64), VP]),
    "stwo_gen_wide_fib_trace": (C.c_int32, [U32, U32, VP, VP, PVP, VP]),
    "stwo_prove_wide_fib": (C.c_int32, [U32, U32, PVP, PcsConfig, VP, C.c_size_t, C.POINTER(C.c_size_t), VP]),
    "stwo_prove_poseidon": (C.c_int32, [U32, VP, PcsConfig, VP, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(QM31),
                                        VP]),
    "stwo_prove_blake_round": (C.c_int32, [U32, VP, PcsConfig, VP, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(QM31),
                                        VP]),
    "stwo_gen_blake_example_trace": (C.c_int32, [U32, VP, VP, VP]),
    "stwo_point_program_eval": (C.c_int32, [C.POINTER(C.c_uint32), C.c_size_t, C.POINTER(QM31), C.c_size_t, QM31, QM31,
                                            C.POINTER(QM31)]),
    "stwo_server_create": (C.c_int32, [U32, C.c_size_t, C.c_int, PVP]),
    "stwo_server_submit": (C.c_int32, [VP, C.POINTER(ProofJob), C.POINTER(C.c_uint64)]),
    "stwo_server_wait": (C.c_int32, [VP, C.c_uint64, C.POINTER(ProofResult)]),
    "stwo_server_destroy": (C.c_int32, [VP]),
    "stwo_job_hbm_bytes": (C.c_size_t, [C.POINTER(ProofJob)]),
    "stwo_prove_batch": (C.c_int32, [C.POINTER(ProofJob), U32, U32, C.c_size_t, C.POINTER(ProofResult)]),
    "stwo_merkle_commit_layer_poseidon252": (C.c_int32, [U32, VP, PVP, U32, VP, VP]),
    "stwo_grind_poseidon252": (C.c_int32, [C.POINTER(C.c_uint32), U32, C.POINTER(C.c_uint64), VP]),
    "stwo_component_info": (C.c_int32, [C.POINTER(Component), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "stwo_eval_constraints": (C.c_int32, [C.POINTER(Component), PVP, U32, C.POINTER(QM31), U32, PVP, VP]),
    "stwo_codegen_compile": (C.c_int32, [C.c_char_p, U32, U32, U32, C.c_int, PVP]),
    "stwo_codegen_cubin": (C.c_int32, [VP, VP, C.c_size_t, C.POINTER(C.c_size_t)]),
    "stwo_codegen_from_cubin": (C.c_int32, [VP, C.c_size_t, U32, U32, U32, C.c_int, PVP]),
    "stwo_codegen_destroy": (C.c_int32, [VP]),
    "stwo_logup_interaction_codegen": (C.c_int32, [VP, U32, PVP, U32, C.POINTER(QM31), U32, VP, C.POINTER(QM31), VP]),
    "stwo_eval_constraints_codegen": (C.c_int32, [VP, U32, U32, PVP, U32, C.POINTER(QM31), U32, C.POINTER(QM31), U32,
                                                  PVP, VP]),
}

_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Loads the backend library (raises if it is missing: no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
        )
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, fn: str) -> None:
    if status != STWO_OK:
        detail = load().stwo_last_error().decode(errors="replace")
        raise StwoError(status, fn, detail)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)
