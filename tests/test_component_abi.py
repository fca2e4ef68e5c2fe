"""stwo_component_info and the argument checks of stwo_eval_constraints, without a GPU: the
constraint counts and evaluation-domain sizes of the three configured components are those of
the reference examples (wide-Fibonacci: n_cols - 2 constraints on log_n + 1; Poseidon2: 1,144 on
log_n + 2; Blake2s round: 129 on log_n + 1)."""
import ctypes as C

import pytest


def _component(air, log_n, n_cols=0, n_el=0):
    from stwo_gb300 import _lib

    els = (_lib.QM31 * max(1, n_el))()
    comp = _lib.Component(air, log_n, n_cols, _lib.QM31((0, 0, 0, 0)), els if n_el else None, n_el)
    return comp, els


def _info(comp):
    from stwo_gb300 import _lib

    n, el, nt = C.c_uint32(), C.c_uint32(), C.c_uint32()
    cols = (C.c_uint32 * 3)()
    st = _lib.load().stwo_component_info(C.byref(comp), C.byref(n), C.byref(el), C.byref(nt), cols)
    return st, n.value, el.value, nt.value, list(cols)


@pytest.mark.parametrize("air,log_n,n_cols,n_el,want", [
    (0, 12, 100, 0, (98, 13, 2, [0, 100, 0])),
    (0, 5, 3, 0, (1, 6, 2, [0, 3, 0])),
    (1, 16, 0, 2, (1144, 18, 3, [0, 1264, 32])),
    (2, 10, 0, 12, (129, 11, 3, [0, 384, 260])),
])
def test_component_info(air, log_n, n_cols, n_el, want):
    from stwo_gb300.build import build_backend

    build_backend()
    comp, _ = _component(air, log_n, n_cols, n_el)
    st, n, el, nt, cols = _info(comp)
    assert st == 0
    assert (n, el, nt, cols) == want


def test_component_argument_errors():
    from stwo_gb300 import _lib
    from stwo_gb300.build import build_backend

    build_backend()
    lib = _lib.load()
    # Unknown AIR id, missing relation elements, too few columns: INVALID_ARG before any device work.
    comp, _ = _component(7, 10)
    assert _info(comp)[0] == 1
    comp, _ = _component(1, 10, 0, 0)
    assert _info(comp)[0] == 1
    assert b"relation elements" in lib.stwo_last_error()
    comp, _ = _component(0, 8, 10)
    cols = (C.c_void_p * 5)()
    acc = (C.c_void_p * 4)(1, 1, 1, 1)
    pw = (_lib.QM31 * 8)()
    st = lib.stwo_eval_constraints(C.byref(comp), cols, 5, pw, 8, acc, None)
    assert st == 1 and b"reads 10 columns" in lib.stwo_last_error()
    cols = (C.c_void_p * 10)(*([1] * 10))
    st = lib.stwo_eval_constraints(C.byref(comp), cols, 10, pw, 7, acc, None)
    assert st == 1 and b"8 constraints" in lib.stwo_last_error()
