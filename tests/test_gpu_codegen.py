"""Generated constraint kernels on the GPU (stwo_eval_constraints_codegen), bit for bit.

Each example AIR is recorded with the expression framework, its kernel generated and compiled
with NVRTC, and run through the C ABI on seeded uniform column words (the constraint sum is a
polynomial in the words, so any words are a valid input), coefficient powers and a non-zero
starting accumulation column. The result must equal the oracle's restatement of the AIR
(oracle_eval_constraints) and, for the AIRs that also have a hand-written kernel, that kernel's
output (stwo_eval_constraints) at larger sizes.
"""
import ctypes as C

import numpy as np
import pytest

from stwo_gb300 import airs, codegen
from tests import m31 as F
from tests.test_codegen import make_case

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _run_generated(air, cols, powers, acc):
    import torch

    from stwo_gb300 import _lib
    from stwo_gb300.backend import _stream

    gc = codegen.GeneratedComponent(air)
    dcols = [_dev(c) for c in cols]
    dacc = [_dev(a.copy()) for a in acc]
    pw = (_lib.QM31 * len(powers))(*[_lib.QM31(p) for p in powers])
    gc.eval_constraints([c.data_ptr() for c in dcols], pw, [a.data_ptr() for a in dacc], _stream())
    torch.cuda.synchronize()
    return [a.cpu().numpy().view(np.uint32) for a in dacc]


@pytest.mark.parametrize("name", ["wide_fib", "poseidon", "plonk", "state_machine_x", "state_machine_y"])
@pytest.mark.parametrize("seed", [0, 1])
def test_generated_kernel_matches_oracle(cuda, oracle, name, seed):
    air_id, air, elements, cs, cols, powers, acc, n_fib = make_case(name, seed)
    got = _run_generated(air, cols, powers, acc)
    el = [elements[0], elements[1]] if air_id else []
    want = oracle.eval_constraints(air_id, air.log_size(), n_fib, cs, el, cols, powers, acc)
    for j in range(4):
        assert np.array_equal(got[j], want[j]), f"coordinate {j}"


@pytest.mark.parametrize("name,log_n", [("plonk", 12), ("state_machine_y", 11), ("poseidon", 6)])
def test_generated_kernel_matches_oracle_larger(cuda, oracle, name, log_n):
    air_id, air, elements, cs, cols, powers, acc, n_fib = make_case(name, 5, log_n)
    got = _run_generated(air, cols, powers, acc)
    el = [elements[0], elements[1]] if air_id else []
    want = oracle.eval_constraints(air_id, air.log_size(), n_fib, cs, el, cols, powers, acc)
    for j in range(4):
        assert np.array_equal(got[j], want[j]), f"coordinate {j}"


@pytest.mark.parametrize("air_id,log_n,n_cols", [(0, 12, 100), (1, 10, 0)])
def test_generated_kernel_matches_hand_written(cuda, air_id, log_n, n_cols):
    """Wide-Fibonacci (2^12 rows x 100 columns) and Poseidon2 (2^10 rows, 1,296 columns on 2^12
    points): the generated kernel and the hand-written one give the same words."""
    import torch

    from stwo_gb300 import _lib
    from stwo_gb300.backend import _ptrs, _stream

    rng = np.random.default_rng(77 + air_id)
    rq = lambda: tuple(int(v) for v in rng.integers(0, F.P, 4))  # noqa: E731
    elements = [rq(), rq()] if air_id == 1 else []
    cs = rq()
    air = airs.WideFibonacciEval(log_n, n_cols) if air_id == 0 else airs.PoseidonEval(log_n, tuple(elements), cs)
    gc = codegen.GeneratedComponent(air)
    N = 1 << air.max_constraint_log_degree_bound()
    blocks = []
    for m in gc.mask():
        if m:
            blocks.append(_dev(F.rand_m31(rng, len(m) * N).reshape(len(m), N)))
    dcols = [b[i] for b in blocks for i in range(b.shape[0])]
    powers = [rq() for _ in range(gc.n_constraints)]
    pw = (_lib.QM31 * len(powers))(*[_lib.QM31(p) for p in powers])
    acc0 = [F.rand_m31(rng, N) for _ in range(4)]
    acc_gen = [_dev(a.copy()) for a in acc0]
    acc_hand = [_dev(a.copy()) for a in acc0]
    gc.eval_constraints([c.data_ptr() for c in dcols], pw, [a.data_ptr() for a in acc_gen], _stream())
    els = (_lib.QM31 * 2)(*[_lib.QM31(e) for e in elements]) if elements else None
    comp = _lib.Component(air_id, log_n, n_cols, _lib.QM31(cs), els, len(elements))
    _lib.call("stwo_eval_constraints", C.byref(comp), _ptrs(dcols), len(dcols), pw, len(powers), _ptrs(acc_hand),
              _stream())
    torch.cuda.synchronize()
    for j in range(4):
        assert torch.equal(acc_gen[j], acc_hand[j]), f"coordinate {j}"


def test_generated_kernel_rejects_mismatched_sizes(cuda):
    from stwo_gb300 import _lib

    gc = codegen.GeneratedComponent(airs.StateTransitionEval(0, 4, ((1, 2, 3, 4), (5, 6, 7, 8))))
    pw = (_lib.QM31 * 1)()
    acc = (C.c_void_p * 4)(1, 1, 1, 1)
    cols = (C.c_void_p * 5)(*([1] * 5))
    st = _lib.load().stwo_eval_constraints_codegen(C.c_void_p(gc.handle), 4, 5, cols, 5, gc.param_values(), 4, pw,
                                                   1, acc, None)
    assert st == 1 and b"columns" in _lib.load().stwo_last_error()
