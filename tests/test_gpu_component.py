"""stwo_eval_constraints (ComponentProver::evaluate_constraint_quotients_on_domain,
crates/prover/src/constraint_framework/component.rs:278-416) against the oracle, bit for bit.

Each case fills the component's columns on its evaluation domain, the accumulator's slice of
coefficient powers and the accumulation column with seeded uniform words (the constraint sum is a
polynomial in the column words, so any words are a valid input), calls the entry point through
the C ABI and compares the accumulation column with the oracle's. The column starts non-zero, so
the test also checks that the call adds to it rather than overwriting it.
"""
import ctypes as C

import numpy as np
import pytest

from tests import m31 as F

pytestmark = pytest.mark.gpu


def _rq(rng):
    return tuple(int(v) for v in rng.integers(0, F.P, 4))


CASES = [(0, 4, 3), (0, 6, 10), (0, 9, 100), (1, 3, 0), (1, 6, 0), (2, 4, 0), (2, 7, 0)]


@pytest.mark.parametrize("air,log_n,n_cols", CASES)
def test_eval_constraints_matches_oracle(cuda, oracle, air, log_n, n_cols):
    import torch

    from stwo_gb300 import _lib
    from stwo_gb300.backend import _ptrs, _stream

    lib = _lib.load()
    rng = np.random.default_rng(3000 + 97 * air + log_n)
    n_el = {0: 0, 1: 2, 2: 12}[air]
    elements = [_rq(rng) for _ in range(n_el)]
    claimed = _rq(rng)
    els = (_lib.QM31 * max(1, n_el))(*[_lib.QM31(e) for e in elements])
    comp = _lib.Component(air, log_n, n_cols, _lib.QM31(claimed), els if n_el else None, n_el)
    n, el, nt = C.c_uint32(), C.c_uint32(), C.c_uint32()
    tc = (C.c_uint32 * 3)()
    assert lib.stwo_component_info(C.byref(comp), C.byref(n), C.byref(el), C.byref(nt), tc) == 0
    N = 1 << el.value
    host_cols, dev_cols = [], []
    for t in range(nt.value):
        if tc[t] == 0:
            continue
        block = F.rand_m31(rng, tc[t] * N).reshape(tc[t], N)
        d = torch.from_numpy(block.view(np.int32)).cuda()  # one contiguous block per tree
        host_cols += list(block)
        dev_cols += [d[c] for c in range(tc[t])]
    coeffs = [_rq(rng) for _ in range(n.value)]
    acc0 = [F.rand_m31(rng, N) for _ in range(4)]
    dacc = [torch.from_numpy(a.view(np.int32)).cuda() for a in acc0]
    pw = (_lib.QM31 * n.value)(*[_lib.QM31(c) for c in coeffs])
    st = lib.stwo_eval_constraints(C.byref(comp), _ptrs(dev_cols), len(dev_cols), pw, n.value, _ptrs(dacc), _stream())
    assert st == 0, lib.stwo_last_error()
    torch.cuda.synchronize()
    got = [a.cpu().numpy().view(np.uint32) for a in dacc]
    want = oracle.eval_constraints(air, log_n, n_cols, claimed, elements, host_cols, coeffs, acc0)
    for k in range(4):
        assert np.array_equal(got[k], want[k]), f"coordinate {k}"
