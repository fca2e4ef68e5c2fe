"""The expression framework (stwo_gb300.expr) against the reference's own expr tests.

Restated from crates/prover/src/constraint_framework/expr/:
  evaluator.rs:232-257  test_expr_evaluator (the format_constraints text, byte for byte)
  evaluator.rs:259-312  test_constraint_regression / _fails (equal values for equal AIRs)
  evaluator.rs:424-461  test_constraint_degree_bounds
  degree.rs:106-129     test_degree_bound
  simplify.rs:142-216   test_simplify_expr (simplification keeps the value)
"""
import random

import pytest

from stwo_gb300 import expr as X
from stwo_gb300.expr import BaseExpr, ExtExpr, ExprEvaluator, Relation

P = X.P
TEST_RELATION = Relation("TestRelation", 3)


def _test_struct(ev):
    x0, x1, x2 = ev.next_trace_mask(), ev.next_trace_mask(), ev.next_trace_mask()
    inter = ev.add_intermediate(x1 * x2)
    ev.add_constraint(x0 * inter * (x0 + x1).inverse())
    ev.add_to_relation(TEST_RELATION, ExtExpr.one(), [x0, x1, x2])
    ev.finalize_logup()
    return ev


def _equiv_struct(ev):
    x0, x1, x2 = ev.next_trace_mask(), ev.next_trace_mask(), ev.next_trace_mask()
    ev.add_constraint(x0 * (x1 * x2) * (x0 + x1).inverse())
    ev.add_to_relation(TEST_RELATION, ExtExpr.one(), [x0, x1, x2])
    ev.finalize_logup()
    return ev


def _diff_lookup_struct(ev):
    x0, x1, x2 = ev.next_trace_mask(), ev.next_trace_mask(), ev.next_trace_mask()
    inter = ev.add_intermediate(x1 * x2)
    ev.add_constraint(x0 * inter * (x0 + x1).inverse())
    ev.add_to_relation(TEST_RELATION, ExtExpr.one(), [x0, x1])
    ev.finalize_logup()
    return ev


def test_expr_evaluator_format():
    expected = (
        "let intermediate0 = (trace_1_column_1_offset_0) * (trace_1_column_2_offset_0);\n\n"
        "let intermediate1 = (TestRelation_alpha0) * (trace_1_column_0_offset_0) "
        "+ (TestRelation_alpha1) * (trace_1_column_1_offset_0) "
        "+ (TestRelation_alpha2) * (trace_1_column_2_offset_0) "
        "- (TestRelation_z);\n\n"
        "let constraint_0 = ((trace_1_column_0_offset_0) * (intermediate0)) * "
        "(1 / (trace_1_column_0_offset_0 + trace_1_column_1_offset_0));\n\n"
        "let constraint_1 = (QM31Impl::from_partial_evals([trace_2_column_3_offset_0, trace_2_column_4_offset_0, "
        "trace_2_column_5_offset_0, trace_2_column_6_offset_0]) "
        "- (QM31Impl::from_partial_evals([trace_2_column_3_offset_neg_1, trace_2_column_4_offset_neg_1, "
        "trace_2_column_5_offset_neg_1, trace_2_column_6_offset_neg_1])) "
        "+ (claimed_sum) * (1 / (column_size))) "
        "* (intermediate1) "
        "- (qm31(1, 0, 0, 0));")
    assert _test_struct(ExprEvaluator()).format_constraints() == expected


def _assignment(ev, seed):
    rng = random.Random(seed)
    cache = {}

    def col(c):
        k = (c.interaction, c.idx, c.offset)
        if k not in cache:
            cache[k] = (rng.randrange(P), 0, 0, 0)
        return cache[k]

    params = {"TestRelation_z": tuple(rng.randrange(P) for _ in range(4)), "claimed_sum":
              tuple(rng.randrange(P) for _ in range(4)), "column_size": (rng.randrange(1, P), 0, 0, 0)}
    for i in range(3):
        params[f"TestRelation_alpha{i}"] = tuple(rng.randrange(P) for _ in range(4))
    return col, X.with_intermediates(ev, col, params)


def _values(ev, seed):
    col, params = _assignment(ev, seed)
    return [X.eval_expr(c, col, params) for c in ev.constraints]


def test_constraint_regression():
    assert _values(_test_struct(ExprEvaluator()), 7) == _values(_equiv_struct(ExprEvaluator()), 7)


def test_constraint_regression_fails():
    assert _values(_test_struct(ExprEvaluator()), 7) != _values(_diff_lookup_struct(ExprEvaluator()), 7)


def test_constraint_degree_bounds():
    ev = ExprEvaluator()
    x0, x1, x2 = ev.next_trace_mask(), ev.next_trace_mask(), ev.next_trace_mask()
    ev.add_to_relation(TEST_RELATION, ExtExpr.one(), [x0])
    ev.add_to_relation(TEST_RELATION, ExtExpr.one(), [x0 * x1])
    ev.add_to_relation(TEST_RELATION, ExtExpr.one(), [x1 * x2])
    ev.finalize_logup_in_pairs()
    assert ev.constraint_degree_bounds() == [4, 3]


def test_degree_bound():
    col = BaseExpr.col
    inter = (BaseExpr.const(12) + col(1, 1, 0)) * BaseExpr.param("a") * col(1, 0, 0)
    qinter = ExtExpr.secure_col(inter, 12, BaseExpr.param("b"), 0)
    named = X.NamedExprs({"intermediate": inter, "low_degree_intermediate": BaseExpr.const(12345)},
                         {"qintermediate": qinter})
    e = BaseExpr.param("intermediate") * col(2, 1, 0)
    qe = BaseExpr.param("qintermediate") * ExtExpr.secure_col(col(2, 1, 0), e, 0, 1)
    assert inter.degree_bound(named) == 2
    assert qinter.degree_bound(named) == 2
    assert e.degree_bound(named) == 3
    assert qe.degree_bound(named) == 5
    low = e * BaseExpr.const(3141).inverse() * BaseExpr.param("low_degree_intermediate").inverse()
    assert low.degree_bound(named) == 3


def test_simplify_keeps_value():
    c0, c1 = BaseExpr.col(1, 0, 0), BaseExpr.col(1, 1, 0)
    a, b = BaseExpr.param("a"), ExtExpr.param("b")
    zero, one, minus_one = BaseExpr.const(0), BaseExpr.const(1), BaseExpr.const(P - 1)
    qzero, qone = ExtExpr.const((0, 0, 0, 0)), ExtExpr.const((1, 0, 0, 0))
    qminus_one = ExtExpr.const((P - 1, 0, 0, 0))
    base = ((((zero + c0) + (a + zero)) * ((-c1) + (-c0)) + (-(-(a + a + c0))) - zero) + (a - zero)
            + (-c1 - (a * a)) + (a * zero) - (zero * c1)
            + one * a * one * c1 * (-a) * c1 * (minus_one * c0))
    e = (qzero + ExtExpr.secure_col(base, base, zero, one) - qzero) * qone * b * qminus_one
    rng = random.Random(0)
    vals = {(1, 0, 0): rng.randrange(P), (1, 1, 0): rng.randrange(P)}
    params = {"a": (rng.randrange(P), 0, 0, 0), "b": tuple(rng.randrange(P) for _ in range(4))}
    col = lambda c: (vals[(c.interaction, c.idx, c.offset)], 0, 0, 0)
    s = e.simplify()
    assert X.eval_expr(e, col, params) == X.eval_expr(s, col, params)
    assert len(s.format_expr()) < len(e.format_expr())


def test_simplify_rules():
    c = BaseExpr.col(1, 0, 0)
    assert (BaseExpr.const(0) + c).simplify() is c
    assert (-(-c)).simplify() is c
    assert (c * BaseExpr.const(1)).simplify() is c
    assert (c.inverse().inverse()).simplify() is c
    assert BaseExpr.const(5).inverse().simplify() is BaseExpr.const(X.m31_inv(5))
    assert ExtExpr.from_secure((1, 2, 3, 4)).simplify() is ExtExpr.const((1, 2, 3, 4))
    with pytest.raises(ValueError):
        (c.inverse()).degree_bound(X.NamedExprs({}, {}))


def test_wide_relation_entry_is_one_combine_node():
    """A relation wider than COMBINE_LOOP_MIN is recorded as one combine node; its format, degree
    bound and value equal combine_formal's sum of alpha powers times values minus z."""
    rel = Relation("Wide", X.COMBINE_LOOP_MIN + 4)
    ev = ExprEvaluator()
    vals = [ev.next_trace_mask() * BaseExpr.const(k + 1) for k in range(rel.size)]
    ev.add_to_relation(rel, ExtExpr.one(), vals)
    ev.finalize_logup_in_pairs()
    node = next(e for e in ev.ext_intermediates.values() if e.kind == "combine")
    formal = X.combine_formal(rel, vals)
    assert node.format_expr() == formal.format_expr()
    named = X.NamedExprs(dict(ev.intermediates), dict(ev.ext_intermediates))
    assert node.degree_bound(named) == formal.degree_bound(named)
    rng = random.Random(5)
    cols = {}
    params = rel.param_values(tuple(rng.randrange(X.P) for _ in range(4)), tuple(rng.randrange(X.P) for _ in range(4)))

    def col(c):
        return cols.setdefault(c, (rng.randrange(X.P), 0, 0, 0))

    assert X.eval_expr(node, col, params) == X.eval_expr(formal, col, params)
    assert node.simplify().kind == "combine"
    narrow = ExprEvaluator()
    narrow.add_to_relation(Relation("Narrow", X.COMBINE_LOOP_MIN), ExtExpr.one(),
                           [narrow.next_trace_mask() for _ in range(X.COMBINE_LOOP_MIN)])
    assert all(e.kind != "combine" for e in narrow.ext_intermediates.values())


def test_long_flat_body_is_cut_into_blocks_and_marked():
    """A generated body of more than FLAT_SPLIT_MIN straight-line statements gets a block boundary
    every FLAT_BLOCK statements and the fast-compile mark; a shorter one, or one made of a loop,
    is left alone."""
    from stwo_gb300 import codegen as G

    body = [f"const uint32_t t{i} = {i}u;" for i in range(G.FLAT_SPLIT_MIN + 1)]
    out, flat = G._split_flat(body)
    assert flat
    cuts = [i for i, x in enumerate(out) if "asm volatile" in x]
    assert len(cuts) == (G.FLAT_SPLIT_MIN + 1) // G.FLAT_BLOCK
    assert [x for x in out if "asm volatile" not in x] == body
    short, flat = G._split_flat(body[:G.FLAT_SPLIT_MIN])
    assert not flat and short == body[:G.FLAT_SPLIT_MIN]
    loop = ["#pragma unroll 1", "for (int g = 0; g < 8; g++) {"] + ["  " + x for x in body] + ["}"]
    assert G._split_flat(loop) == (loop, False)
