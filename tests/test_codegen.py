"""Constraint code generation on the CPU: the recorded example AIRs evaluate on the domain exactly
as the oracle's independent restatements of them (oracle_eval_constraints), and their generated
CUDA kernels compile with NVRTC for sm_103a (no device needed). The kernels themselves are run
against the oracle in tests/test_gpu_codegen.py."""
import ctypes as C
import re

import numpy as np
import pytest

from stwo_gb300 import airs, codegen, expr as X
from tests import codegen_host as H

P = X.P

# (oracle air id, factory(log_n, elements, claimed_sum), log_n, wide-Fibonacci columns)
CASES = {
    "wide_fib": (0, lambda l, e, cs: airs.WideFibonacciEval(l, 24), 5, 24),
    "poseidon": (1, lambda l, e, cs: airs.PoseidonEval(l, e, cs), 3, 0),
    "plonk": (3, lambda l, e, cs: airs.PlonkEval(l, e, cs), 5, 0),
    "state_machine_x": (4, lambda l, e, cs: airs.StateTransitionEval(0, l, e, cs), 5, 0),
    "state_machine_y": (5, lambda l, e, cs: airs.StateTransitionEval(1, l, e, cs), 4, 0),
}


def _rq(rng):
    return tuple(int(v) for v in rng.integers(0, P, 4))


def make_case(name, seed=0, log_n=None):
    """Random columns on the evaluation domain, relation elements, claimed sum, coefficient powers
    and starting accumulator for one example AIR."""
    air_id, make, default_log, n_fib = CASES[name]
    log_n = log_n or default_log
    rng = np.random.default_rng(seed)
    elements = (_rq(rng), _rq(rng))
    cs = _rq(rng)
    air = make(log_n, elements, cs)
    ev = air.evaluate(X.ExprEvaluator())
    n = 1 << air.max_constraint_log_degree_bound()
    cols = [rng.integers(0, P, n).astype(np.uint32) for m in ev.mask for _ in m]
    powers = [_rq(rng) for _ in range(ev.n_constraints())]
    acc = [rng.integers(0, P, n).astype(np.uint32) for _ in range(4)]
    return air_id, air, elements, cs, cols, powers, acc, n_fib


@pytest.mark.parametrize("name", sorted(CASES))
def test_recorded_air_matches_oracle_on_domain(name, oracle):
    air_id, air, elements, cs, cols, powers, acc, n_fib = make_case(name)
    got = H.accumulate(air, cols, air.params(), powers, acc)
    el = [elements[0], elements[1]] if air_id else []
    want = oracle.eval_constraints(air_id, air.log_size(), n_fib, cs, el, cols, powers, acc)
    for j in range(4):
        assert np.array_equal(got[j], want[j]), j


def make_blake_case(kind, seed=0):
    """A component of the full Blake example (scheduler, round or an XOR table) with random
    columns, relation elements, claimed sum, powers and accumulator; the oracle's air id, its
    n_cols argument and its flat element list."""
    rng = np.random.default_rng(seed)
    rels = [(_rq(rng), _rq(rng)) for _ in range(6)]
    cs = _rq(rng)
    if kind == "scheduler":
        air, air_id, n_cols, el = airs.BlakeSchedulerEval(4, {"blake": rels[0], "round": rels[1]}, cs), 6, 0, rels[:2]
    elif kind == "round":
        named = {"round": rels[0], **{w: rels[1 + i] for i, (w, _) in enumerate(airs.XOR_TABLES)}}
        air, air_id, n_cols, el = airs.BlakeRoundEval(4, named, cs), 2, 0, rels
    else:
        w = int(kind[3:])
        air, air_id, n_cols, el = airs.XorTableEval(w, dict(airs.XOR_TABLES)[w], rels[0], cs), 7, w, rels[:1]
    ev = air.evaluate(X.ExprEvaluator())
    n = 1 << air.max_constraint_log_degree_bound()
    cols = [rng.integers(0, P, n).astype(np.uint32) for m in ev.mask for _ in m]
    powers = [_rq(rng) for _ in range(ev.n_constraints())]
    acc = [rng.integers(0, P, n).astype(np.uint32) for _ in range(4)]
    return air, air_id, n_cols, [q for r in el for q in r], cs, cols, powers, acc


@pytest.mark.parametrize("kind", ["scheduler", "round", "xor4", "xor7", "xor9"])
def test_blake_components_match_oracle_on_domain(kind, oracle):
    """The full Blake example's components, recorded through the expression framework, evaluate on
    the domain as the oracle's restatements do (the 2^16-row XOR12 table runs in the GPU proof
    test)."""
    air, air_id, n_cols, el, cs, cols, powers, acc = make_blake_case(kind)
    got = H.accumulate(air, cols, air.params(), powers, acc)
    want = oracle.eval_constraints(air_id, air.log_size(), n_cols, cs, el, cols, powers, acc)
    for j in range(4):
        assert np.array_equal(got[j], want[j]), j


@pytest.mark.parametrize("name", ["wide_fib", "plonk", "state_machine_x", "poseidon"])
def test_generated_kernel_compiles(name):
    from stwo_gb300 import _lib

    _, air, *_ = make_case(name)
    gc = codegen.GeneratedComponent(air, load=False)
    size = C.c_size_t()
    _lib.call("stwo_codegen_cubin", gc.handle, None, 0, C.byref(size))
    assert size.value > 1000
    assert gc.n_constraints == air.evaluate(X.ExprEvaluator()).n_constraints()


@pytest.mark.parametrize("kind", ["scheduler", "round", "xor12", "xor4"])
def test_blake_generated_kernels_compile(kind):
    from stwo_gb300 import _lib

    air, *_ = make_blake_case(kind) if kind != "xor12" else (airs.XorTableEval(12, 4),)
    gc = codegen.GeneratedComponent(air, load=False)
    size = C.c_size_t()
    _lib.call("stwo_codegen_cubin", gc.handle, None, 0, C.byref(size))
    assert size.value > 1000


def test_poseidon_instances_share_one_loop_body():
    """The eight Poseidon2 instances of a row (each a run of constraint groups) are one unit
    class: one loop body over column tables, which loads each column of an instance once."""
    src, params = codegen.generate(airs.PoseidonEval(4).evaluate(X.ExprEvaluator()))
    assert re.findall(r"for \(int g = \w+; g < (\d+);", src) == ["8"]
    assert len(src.splitlines()) < 4000
    assert {n for n, _ in params} >= {"PoseidonElements_z", "claimed_sum", "column_size"}


def test_compile_error_is_reported():
    from stwo_gb300 import _lib

    out = C.c_void_p()
    st = _lib.load().stwo_codegen_compile(b"this is not CUDA", 1, 0, 1, 0, C.byref(out))
    assert st == 1
    assert b"does not compile" in _lib.load().stwo_last_error()


@pytest.mark.parametrize("kind", ["wide_fib", "poseidon", "plonk", "state_machine_x", "scheduler", "round", "xor12",
                                  "xor4"])
def test_point_evaluation_matches_interpreter(kind):
    """GeneratedComponent.eval_at_point (the library's stwo_point_program_eval running the
    component's compiled point program, on the host) equals the expression interpreter
    (with_intermediates + eval_expr) at random mask values."""
    import random

    if kind in CASES:
        air = make_case(kind)[1]
    elif kind == "xor12":
        air = airs.XorTableEval(12, 4, ((1, 2, 3, 4), (5, 6, 7, 8)), (9, 9, 9, 9))
    else:
        air = make_blake_case(kind)[0]
    gc = codegen.GeneratedComponent(air, load=False)
    ev = gc.ev
    rng = random.Random(11)
    mask = [[[tuple(rng.randrange(P) for _ in range(4)) for _ in offs] for offs in tree] for tree in ev.mask]
    rc, dinv = (3, 1, 4, 1), (5, 9, 2, 6)
    got = gc.eval_at_point(mask, rc, dinv)
    vals = {k: ((v % P, 0, 0, 0) if isinstance(v, int) else tuple(v)) for k, v in air.params().items()}
    for name in ev.preprocessed:
        vals.setdefault(name, mask[0][ev.preprocessed.index(name)][0])

    def col(c):
        return mask[c.interaction][c.local][ev.mask[c.interaction][c.local].index(c.offset)]

    vals = X.with_intermediates(ev, col, vals)
    want, memo = (0, 0, 0, 0), {}
    for c in ev.constraints:
        want = X.q_add(X.q_mul(want, rc), X.q_mul(dinv, X.eval_expr(c, col, vals, memo)))
    assert got == want


def test_point_program_rejects_malformed_programs():
    """stwo_point_program_eval checks every operand and length: a truncated program, an operand
    past the values, an unknown op or a combine reaching past the inputs is INVALID_ARG, not a read
    out of bounds."""
    from stwo_gb300 import _lib
    from stwo_gb300._lib import QM31

    lib = _lib.load()
    inputs = (QM31 * 2)(QM31((1, 2, 3, 4)), QM31((5, 6, 7, 8)))

    def run(words):
        arr = (C.c_uint32 * max(len(words), 1))(*words)
        acc = QM31((0, 0, 0, 0))
        return lib.stwo_point_program_eval(arr, len(words), inputs, 2, QM31((1, 0, 0, 0)), QM31((1, 0, 0, 0)),
                                           C.byref(acc)), tuple(acc.v)

    st, acc = run([1, 1, 0, 1, 1, 2])  # one add (v2 = v0 + v1), output v2
    assert st == 0 and acc == (6, 8, 10, 12)
    assert run([1, 1, 0])[0] == 1           # truncated add
    assert run([1, 1, 0, 5, 1, 2])[0] == 1  # operand past the values
    assert run([1, 9, 0, 1, 1, 2])[0] == 1  # unknown op
    assert run([1, 7, 3, 0, 1, 0, 1, 0, 1, 2])[0] == 1  # combine alphas past the values
    assert run([0, 1, 7])[0] == 1           # output past the values
