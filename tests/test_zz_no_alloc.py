"""stwo_eval_at_points_noalloc, the entry point for callers that cannot allocate device memory,
gives the same values as stwo_eval_at_points.

It is called through the C ABI twice in a row with different inputs: both calls share one static
device array, so the second call also checks that the accumulators left by the first are cleared.
Collected last so that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from tests import m31 as F

pytestmark = pytest.mark.gpu


def _dev(x):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, np.uint32)).view(np.int32)).cuda()


def _rq(rng):
    return tuple(int(v) for v in rng.integers(0, F.P, 4))


def _call(name, polys, queries):
    import torch

    from stwo_gb300 import _lib
    from stwo_gb300.backend import _point, _ptrs, _stream

    n = len(queries)
    logs = (C.c_uint32 * len(polys))(*[p.numel().bit_length() - 1 for p in polys])
    poly_of = (C.c_uint32 * n)(*[q[0] for q in queries])
    pts = (_lib.QM31Point * n)(*[_point(q[1]) for q in queries])
    out = (_lib.QM31 * n)()
    status = getattr(_lib.load(), name)(_ptrs(polys), logs, len(polys), poly_of, pts, n, out, _stream())
    torch.cuda.synchronize()
    return status, [tuple(out[i].v) for i in range(n)]


def _case(rng, n_polys, log, n_evals):
    polys = [_dev(F.rand_m31(rng, 1 << log)) for _ in range(n_polys)]
    queries = [(i % n_polys, (_rq(rng), _rq(rng))) for i in range(n_evals)]
    return polys, queries


def test_noalloc_matches_allocating_entry_point_twice(cuda):
    rng = np.random.default_rng(2024)
    for polys, queries in (_case(rng, 5, 14, 12), _case(rng, 3, 9, 40)):
        st_ref, want = _call("stwo_eval_at_points", polys, queries)
        st, got = _call("stwo_eval_at_points_noalloc", polys, queries)
        assert st_ref == 0 and st == 0
        assert got == want


def test_noalloc_matches_oracle_on_multi_block_polynomials(cuda, oracle):
    """Polynomials of 2^20 and 2^18 coefficients span several blocks of the table-less split, so
    each block's partial sum is scaled by the point's top-bit factors before the accumulation;
    several evaluations per polynomial share its coefficients. Two calls in a row, each checked
    against the oracle's eval_at_point."""
    rng = np.random.default_rng(2025)
    for log, n_polys, n_evals in ((20, 2, 6), (18, 3, 7)):
        host_polys = [F.rand_m31(rng, 1 << log) for _ in range(n_polys)]
        polys = [_dev(p) for p in host_polys]
        queries = [(i % n_polys, (_rq(rng), _rq(rng))) for i in range(n_evals)]
        st, got = _call("stwo_eval_at_points_noalloc", polys, queries)
        assert st == 0
        for (pi, pt), g in zip(queries, got):
            assert g == oracle.eval_at_point(host_polys[pi], pt)


def test_noalloc_rejects_sizes_beyond_its_maximum(cuda):
    from stwo_gb300 import _lib

    rng = np.random.default_rng(7)
    polys, queries = _case(rng, 1, 4, 2)
    max_evals = 2048  # STWO_NOALLOC_MAX_EVALS in include/stwo_cuda.h
    too_many = queries * (max_evals // 2 + 1)
    st, _ = _call("stwo_eval_at_points_noalloc", polys, too_many)
    assert st == 1
    assert b"maximum" in _lib.load().stwo_last_error()
