"""Test helper: a vectorised host evaluation of a recorded component on its evaluation domain.

It applies the generator's own resolution of intermediates and preprocessed columns, then
evaluates the expression DAG row-wise with numpy (QM31 as four coordinate arrays) and
accumulates row_res * denom_inv exactly as FrameworkComponent::evaluate_constraint_quotients_on_
domain does (crates/prover/src/constraint_framework/component.rs:322-416). The tests compare it
with the oracle's independent restatement of each AIR, which pins the AIR definitions and the
expression semantics that the generated kernels are built from.
"""
import numpy as np

from stwo_gb300 import codegen, expr as X
from stwo_gb300.circle import canonic_half_coset, coset, subgroup_gen
from stwo_gb300.host_prover import _coset_vanishing, index_to_point

P = X.P


def _m(x):
    return np.asarray(x, np.int64) % P


def _cm(a, b):
    return (_m(a[0] * b[0] - a[1] * b[1]), _m(a[0] * b[1] + a[1] * b[0]))


def _qmul(x, y):
    xa, xb, ya, yb = (x[0], x[1]), (x[2], x[3]), (y[0], y[1]), (y[2], y[3])
    ac, bd = _cm(xa, ya), _cm(xb, yb)
    r = (_m(2 * bd[0] - bd[1]), _m(bd[0] + 2 * bd[1]))
    ad, bc = _cm(xa, yb), _cm(xb, ya)
    return (_m(ac[0] + r[0]), _m(ac[1] + r[1]), _m(ad[0] + bc[0]), _m(ad[1] + bc[1]))


def _lift(v):
    return v if isinstance(v, tuple) else (v, 0, 0, 0)


def offset_row(i, trace_log, eval_log, off):
    """offset_bit_reversed_circle_domain_index (crates/prover/src/core/utils.rs:74-90)."""
    def br(x):
        return int(format(x, f"0{eval_log}b")[::-1], 2)
    prev = br(i)
    half = 1 << (eval_log - 1)
    step = off * (1 << (eval_log - trace_log - 1))
    prev = (prev + step) % half if prev < half else (prev - step) % half + half
    return br(prev)


def denom_inv(trace_log, eval_log):
    """Bit-reversed 1 / coset_vanishing(trace coset, eval_domain.at(i)) for i < 2^(eval - trace)."""
    half = canonic_half_coset(eval_log)
    tc = coset(subgroup_gen(trace_log + 1), trace_log)
    out = []
    for i in range(1 << (eval_log - trace_log)):
        if i < (1 << half.log_size):
            x, y = index_to_point(half.initial_index + i * half.step_size)
        else:
            x, y = index_to_point(half.initial_index + (i - (1 << half.log_size)) * half.step_size)
            y = (-y) % P
        v = _coset_vanishing(tc, (x, 0, 0, 0), (y, 0, 0, 0))[0]
        out.append(pow(v, P - 2, P))
    k = eval_log - trace_log
    return [out[int(format(i, f"0{k}b")[::-1], 2) if k else 0] for i in range(len(out))]


def accumulate(air, cols, params, coeff_powers, acc):
    """acc (4 arrays) + row_res / Z over the evaluation domain of `air` (a FrameworkEval-like
    object); `cols` in table order (interaction 0, 1, 2), `coeff_powers` as the accumulator
    hands them."""
    ev = air.evaluate(X.ExprEvaluator())
    g = codegen._Gen(ev)
    roots = [g.resolve(c.simplify()) for c in ev.constraints]
    tl, el = air.log_size(), air.max_constraint_log_degree_bound()
    n = 1 << el
    rows = {0: np.arange(n)}
    vals = {k: _lift(tuple(v) if not isinstance(v, int) else v) for k, v in params.items()}
    memo = {}
    for node in g._topo(roots):
        k = node.kind
        if k == "col":
            c = node.val
            off = c.offset
            if off not in rows:
                rows[off] = np.array([offset_row(i, tl, el, off) for i in range(n)])
            v = (np.asarray(cols[g.col_base[c.interaction] + c.local], np.int64)[rows[off]], 0, 0, 0)
        elif k == "const":
            v = _lift(node.val)
        elif k == "param":
            v = vals[node.val]
        else:
            a = [memo[x.uid] for x in node.args]
            if k == "add":
                v = tuple(_m(p + q) for p, q in zip(a[0], a[1]))
            elif k == "sub":
                v = tuple(_m(p - q) for p, q in zip(a[0], a[1]))
            elif k == "mul":
                v = _qmul(a[0], a[1])
            elif k == "neg":
                v = tuple(_m(-p) for p in a[0])
            elif k == "inv":
                base = np.broadcast_to(np.asarray(a[0][0], np.int64), (n,))
                v = (np.array([pow(int(x), P - 2, P) for x in base], np.int64), 0, 0, 0)
            elif k == "secure_col":
                v = tuple(p[0] for p in a)
            elif k == "combine":
                name, _ = node.val
                v = (0, 0, 0, 0)
                for i, x in enumerate(a):
                    t = _qmul(vals[f"{name}_alpha{i}"], x)
                    v = tuple(_m(p + q) for p, q in zip(v, t))
                v = tuple(_m(p - q) for p, q in zip(v, vals[f"{name}_z"]))
            else:
                raise AssertionError(k)
        memo[node.uid] = v
    nc = len(roots)
    row_res = (0, 0, 0, 0)
    for i, r in enumerate(roots):
        pw = tuple(int(x) for x in coeff_powers[nc - 1 - i])
        t = _qmul(pw, memo[r.uid])
        row_res = tuple(_m(p + q) for p, q in zip(row_res, t))
    d = np.array(denom_inv(tl, el), np.int64)[np.arange(n) >> tl]
    out = []
    for j in range(4):
        prod = _m(np.broadcast_to(np.asarray(row_res[j], np.int64), (n,)) * d)
        out.append(((np.asarray(acc[j], np.int64) + prod) % P).astype(np.uint32))
    return out
