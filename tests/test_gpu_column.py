"""The column model through the C ABI: Column::zeros / uninitialized / to_cpu / at
(crates/prover/src/core/backend/mod.rs:46-65) as stwo_buf_alloc / stwo_buf_zero /
stwo_buf_upload / stwo_buf_download / stwo_read_words (stwo_read_words_cols for several columns)
/ stwo_buf_free.

`at` backs the Merkle decommitment's queried values (crates/prover/src/core/vcs/prover.rs:80-149):
the words read at arbitrary indices must be those of the column, including the first and last.
"""
import ctypes as C

import numpy as np
import pytest

from tests import m31 as F

pytestmark = pytest.mark.gpu


def _alloc(lib, nbytes):
    p = C.c_void_p()
    assert lib.stwo_buf_alloc(C.byref(p), nbytes, None) == 0
    assert p.value
    return p


@pytest.mark.parametrize("log", [0, 5, 17, 22])
def test_alloc_upload_read_words_download_free(cuda, log):
    from stwo_gb300 import _lib

    lib = _lib.load()
    n = 1 << log
    rng = np.random.default_rng(1200 + log)
    words = F.rand_m31(rng, n)
    d = _alloc(lib, n * 4)
    assert lib.stwo_buf_upload(d, words.ctypes.data_as(C.c_void_p), n * 4, None) == 0
    idx = np.unique(np.concatenate([[0, n - 1], rng.integers(0, n, size=min(n, 500))])).astype(np.uint64)
    out = np.zeros(idx.size, np.uint32)
    st = lib.stwo_read_words(d, idx.ctypes.data_as(C.POINTER(C.c_uint64)), idx.size,
                             out.ctypes.data_as(C.POINTER(C.c_uint32)), None)
    assert st == 0
    assert np.array_equal(out, words[idx.astype(np.int64)])
    back = np.zeros(n, np.uint32)
    assert lib.stwo_buf_download(back.ctypes.data_as(C.c_void_p), d, n * 4, None) == 0
    assert np.array_equal(back, words)
    assert lib.stwo_buf_free(d, None) == 0
    assert lib.stwo_sync(None) == 0


@pytest.mark.parametrize("n_cols,log", [(1, 4), (7, 12), (300, 10)])
def test_read_words_cols_matches_per_column_reads(cuda, n_cols, log):
    """stwo_read_words_cols (one transfer for a layer's columns) returns, column by column, the
    words at the same indices, including the first and last."""
    from stwo_gb300 import _lib

    lib = _lib.load()
    n = 1 << log
    rng = np.random.default_rng(1300 + n_cols)
    cols = [F.rand_m31(rng, n) for _ in range(n_cols)]
    bufs = [_alloc(lib, n * 4) for _ in range(n_cols)]
    for b, w in zip(bufs, cols):
        assert lib.stwo_buf_upload(b, w.ctypes.data_as(C.c_void_p), n * 4, None) == 0
    idx = np.unique(np.concatenate([[0, n - 1], rng.integers(0, n, size=40)])).astype(np.uint64)
    out = np.zeros(n_cols * idx.size, np.uint32)
    tab = (C.c_void_p * n_cols)(*[b.value for b in bufs])
    assert lib.stwo_read_words_cols(tab, n_cols, idx.ctypes.data_as(C.POINTER(C.c_uint64)), idx.size,
                                    out.ctypes.data_as(C.POINTER(C.c_uint32)), None) == 0
    for c in range(n_cols):
        assert np.array_equal(out[c * idx.size:(c + 1) * idx.size], cols[c][idx.astype(np.int64)]), c
    for b in bufs:
        assert lib.stwo_buf_free(b, None) == 0


def test_zero_part_of_a_column_and_read_back(cuda):
    from stwo_gb300 import _lib

    lib = _lib.load()
    n = 4096
    words = np.arange(1, n + 1, dtype=np.uint32)
    d = _alloc(lib, n * 4)
    assert lib.stwo_buf_upload(d, words.ctypes.data_as(C.c_void_p), n * 4, None) == 0
    # Column::zeros of the upper half: the lower half keeps its words.
    assert lib.stwo_buf_zero(C.c_void_p(d.value + 2048 * 4), 2048 * 4, None) == 0
    idx = np.array([0, 1, 2047, 2048, 2049, 4095], np.uint64)
    out = np.zeros(idx.size, np.uint32)
    assert lib.stwo_read_words(d, idx.ctypes.data_as(C.POINTER(C.c_uint64)), idx.size,
                               out.ctypes.data_as(C.POINTER(C.c_uint32)), None) == 0
    assert out.tolist() == [1, 2, 2048, 0, 0, 0]
    assert lib.stwo_buf_free(d, None) == 0


def test_read_words_of_an_evaluation_matches_oracle(cuda, oracle):
    """`at` on a column the backend computed (an evaluation at blowup 2): the decommitment's use."""
    import torch

    from stwo_gb300 import _lib
    from stwo_gb300.backend import CudaBackend as B, TwiddleTree

    lib = _lib.load()
    rng = np.random.default_rng(1300)
    log, L = 12, 14
    coeffs = F.rand_m31(rng, 1 << log)
    t = TwiddleTree(_lib.Coset(*F.canonic_half(L)))
    (ev,) = B.evaluate_polynomials([torch.from_numpy(coeffs.view(np.int32)).cuda()], _lib.Coset(*F.canonic_half(L)), t)
    want = oracle.evaluate(F.canonic_half(L), F.canonic_half(L), coeffs)
    idx = rng.integers(0, 1 << L, size=64).astype(np.uint64)
    out = np.zeros(idx.size, np.uint32)
    assert lib.stwo_read_words(C.c_void_p(ev.data_ptr()), idx.ctypes.data_as(C.POINTER(C.c_uint64)), idx.size,
                               out.ctypes.data_as(C.POINTER(C.c_uint32)), None) == 0
    assert np.array_equal(out, want[idx.astype(np.int64)])


def test_null_arguments_are_rejected(cuda):
    from stwo_gb300 import _lib

    lib = _lib.load()
    assert lib.stwo_buf_alloc(None, 16, None) == 1
    idx = np.zeros(1, np.uint64)
    out = np.zeros(1, np.uint32)
    assert lib.stwo_read_words(None, idx.ctypes.data_as(C.POINTER(C.c_uint64)), 1,
                               out.ctypes.data_as(C.POINTER(C.c_uint32)), None) == 1
    assert lib.stwo_read_words(None, None, 0, None, None) == 0
