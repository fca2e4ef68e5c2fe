"""Symbolic constraint expressions and the expression-recording evaluator.

This is the constraint framework's `expr` module (crates/prover/src/constraint_framework/expr/
{mod,simplify,format,degree,evaluator}.rs) in Python: an AIR's `evaluate(eval)` runs once
against `ExprEvaluator`, which records every mask read, intermediate, LogUp fraction and
constraint as an expression DAG. `stwo_gb300.codegen` turns the recording into a CUDA kernel for
the evaluation domain; `eval_expr` evaluates it at an out-of-domain point on the host.

Semantics kept from the reference, because they are observable:
  * BaseExpr / ExtExpr node kinds, the mixed-type operator rules (mod.rs:150-351) and the
    SecureCol embedding of base values (mod.rs:94-123).
  * simplify (simplify.rs:7-140) and format_expr (format.rs:5-63), so that `format_constraints`
    reproduces the reference's text byte for byte.
  * degree_bound (degree.rs:38-104).
  * ExprEvaluator (evaluator.rs:54-227): column indices come from one counter shared by all
    interactions, intermediates are named `intermediate{k}`, preprocessed columns are parameters
    named by their id, relation entries become `<name>_alpha{i}` / `<name>_z` parameters
    (evaluator.rs:33-52), and the LogUp finalisation follows logup_proxy (mod.rs:165-240) with
    claimed_sum and column_size as parameters.
For code generation each column also keeps its index within its own interaction (the order in
which SimdDomainEvaluator reads them, simd_domain.rs:65-98).

Nodes are interned: structurally equal expressions are the same Python object, so equality is
identity and common subexpressions are shared for free.
"""
from __future__ import annotations

from typing import Dict, List, Optional, Sequence, Tuple

P = (1 << 31) - 1
Q = Tuple[int, int, int, int]


# ------------------------------------------------------------------ field constants (host)
def _cm_mul(a, b):
    return ((a[0] * b[0] - a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)


def q_add(a: Q, b: Q) -> Q:
    return tuple((x + y) % P for x, y in zip(a, b))


def q_sub(a: Q, b: Q) -> Q:
    return tuple((x - y) % P for x, y in zip(a, b))


def q_neg(a: Q) -> Q:
    return tuple((-x) % P for x in a)


def q_mul(a: Q, b: Q) -> Q:
    # (x + y u)(z + w u) = (xz + (2 + i) yw) + (xw + yz) u  (fields/qm31.rs:21-95)
    x, y, z, w = (a[0], a[1]), (a[2], a[3]), (b[0], b[1]), (b[2], b[3])
    xz, yw = _cm_mul(x, z), _cm_mul(y, w)
    r = _cm_mul((2, 1), yw)
    xw, yz = _cm_mul(x, w), _cm_mul(y, z)
    return ((xz[0] + r[0]) % P, (xz[1] + r[1]) % P, (xw[0] + yz[0]) % P, (xw[1] + yz[1]) % P)


def q_from_partial_evals(v: Sequence[Q]) -> Q:
    """QM31::from_partial_evals (fields/qm31.rs:52-58): v0 + v1 i + v2 u + v3 iu."""
    out = v[0]
    for k, e in ((1, (0, 1, 0, 0)), (2, (0, 0, 1, 0)), (3, (0, 0, 0, 1))):
        out = q_add(out, q_mul(v[k], e))
    return out


def m31_inv(a: int) -> int:
    return pow(a % P, P - 2, P)


def q_inv(a: Q) -> Q:
    """(a + bu)^-1 = (a - bu) / (a^2 - (2+i) b^2) (fields/qm31.rs:121-129); 0 maps to 0."""
    x, y = (a[0], a[1]), (a[2], a[3])
    yy = _cm_mul((2, 1), _cm_mul(y, y))
    xx = _cm_mul(x, x)
    den = ((xx[0] - yy[0]) % P, (xx[1] - yy[1]) % P)
    n = (den[0] * den[0] + den[1] * den[1]) % P
    ni = m31_inv(n)
    di = (den[0] * ni % P, (-den[1]) * ni % P)
    r0, r1 = _cm_mul(x, di), _cm_mul(((-y[0]) % P, (-y[1]) % P), di)
    return (r0[0], r0[1], r1[0], r1[1])


# ------------------------------------------------------------------ nodes
_INTERN: Dict[tuple, "Expr"] = {}
# Nodes are immutable and interned, so simplification is memoised by node: expressions with
# heavy sharing (a Poseidon2 partial round reuses the running sum in every lane) are DAGs whose
# trees are exponentially large.
_SIMPLIFIED: Dict[int, "Expr"] = {}


class Expr:
    """Common base of BaseExpr and ExtExpr. `kind` is one of col, const, param, add, sub, mul,
    neg, inv (base only), secure_col and combine (extension only); `args` are child nodes; `val`
    holds a constant (int for base, 4-tuple for extension), a parameter name, a ColumnExpr, or a
    combine node's (relation name, relation size)."""

    __slots__ = ("kind", "args", "val", "uid")
    is_ext = False

    def __new__(cls, kind, args=(), val=None):
        key = (cls.is_ext, kind, tuple(a.uid for a in args), val)
        node = _INTERN.get(key)
        if node is None:
            node = object.__new__(cls)
            node.kind, node.args, node.val = kind, tuple(args), val
            node.uid = len(_INTERN)
            _INTERN[key] = node
        return node

    def __repr__(self):
        return self.format_expr()

    def __hash__(self):
        return self.uid

    def __eq__(self, other):
        return self is other


class ColumnExpr(tuple):
    """(interaction, idx, offset) as in the reference (mod.rs:19-35), plus `local`, the column's
    index within its interaction (the order SimdDomainEvaluator reads columns in)."""

    def __new__(cls, interaction: int, idx: int, offset: int, local: int = -1):
        return tuple.__new__(cls, (interaction, idx, offset, local))

    interaction = property(lambda s: s[0])
    idx = property(lambda s: s[1])
    offset = property(lambda s: s[2])
    local = property(lambda s: s[3])


def _is_q(x) -> bool:
    return isinstance(x, tuple) and not isinstance(x, ColumnExpr) and len(x) == 4


def _as_base(x) -> "BaseExpr":
    if isinstance(x, BaseExpr):
        return x
    if isinstance(x, int):
        return BaseExpr.const(x)
    raise TypeError(f"not a base field expression: {x!r}")


def _as_ext(x) -> "ExtExpr":
    if isinstance(x, ExtExpr):
        return x
    if isinstance(x, BaseExpr):
        return ExtExpr.from_base(x)
    if isinstance(x, int):
        return ExtExpr.from_base(BaseExpr.const(x))
    if _is_q(x):
        return ExtExpr.from_secure(x)
    raise TypeError(f"not an extension field expression: {x!r}")


class BaseExpr(Expr):
    """A base field (M31) expression (mod.rs:37-58)."""

    is_ext = False

    @staticmethod
    def col(interaction: int, idx: int, offset: int, local: int = -1) -> "BaseExpr":
        return BaseExpr("col", (), ColumnExpr(interaction, idx, offset, local))

    @staticmethod
    def const(v: int) -> "BaseExpr":
        return BaseExpr("const", (), v % P)

    @staticmethod
    def param(name: str) -> "BaseExpr":
        return BaseExpr("param", (), name)

    @staticmethod
    def zero() -> "BaseExpr":
        return BaseExpr.const(0)

    @staticmethod
    def one() -> "BaseExpr":
        return BaseExpr.const(1)

    # Arithmetic (mod.rs:125-201, 242-351).
    def __add__(self, o):
        if isinstance(o, ExtExpr) or _is_q(o):
            return ExtExpr.from_base(self) + _as_ext(o)
        return BaseExpr("add", (self, _as_base(o)))

    def __radd__(self, o):
        return _as_base(o) + self

    def __sub__(self, o):
        if isinstance(o, ExtExpr) or _is_q(o):
            return ExtExpr.from_base(self) - _as_ext(o)
        return BaseExpr("sub", (self, _as_base(o)))

    def __rsub__(self, o):
        return _as_base(o) - self

    def __mul__(self, o):
        if isinstance(o, ExtExpr):
            return o * self  # impl Mul<ExtExpr> for BaseExpr: rhs * self
        if _is_q(o):
            return ExtExpr.from_base(self) * ExtExpr.from_secure(o)
        return BaseExpr("mul", (self, _as_base(o)))

    def __rmul__(self, o):
        return _as_base(o) * self

    def __neg__(self):
        return BaseExpr("neg", (self,))

    def inverse(self) -> "BaseExpr":
        return BaseExpr("inv", (self,))

    def square(self) -> "BaseExpr":
        return self * self

    # ---- simplify (simplify.rs:86-102)
    def simplify(self) -> "BaseExpr":
        done = _SIMPLIFIED.get(self.uid)
        if done is None:
            done = _SIMPLIFIED[self.uid] = self._simplify()
        return done

    def _simplify(self) -> "BaseExpr":
        s = _simplify_arith(self)
        if s.kind == "inv":
            a = s.args[0].simplify()
            if a.kind == "inv":
                return a.args[0]
            if a.kind == "const":
                return BaseExpr.const(m31_inv(a.val))
            return a.inverse()
        return s

    def simplify_and_format(self) -> str:
        return self.simplify().format_expr()

    # ---- format (format.rs:5-33)
    def format_expr(self) -> str:
        k = self.kind
        if k == "col":
            c = self.val
            off = str(c.offset) if c.offset >= 0 else f"neg_{-c.offset}"
            return f"trace_{c.interaction}_column_{c.idx}_offset_{off}"
        if k == "const":
            return f"m31({self.val}).into()"
        if k == "param":
            return self.val
        a = self.args
        if k == "add":
            return f"{a[0].format_expr()} + {a[1].format_expr()}"
        if k == "sub":
            return f"{a[0].format_expr()} - ({a[1].format_expr()})"
        if k == "mul":
            return f"({a[0].format_expr()}) * ({a[1].format_expr()})"
        if k == "neg":
            return f"-({a[0].format_expr()})"
        if k == "inv":
            return f"1 / ({a[0].format_expr()})"
        raise AssertionError(k)

    # ---- degree (degree.rs:38-84), memoised per NamedExprs
    def degree_bound(self, named: "NamedExprs") -> int:
        d = named.memo.get(self.uid)
        if d is None:
            d = named.memo[self.uid] = self._degree(named)
        return d

    def _degree(self, named: "NamedExprs") -> int:
        k = self.kind
        if k == "col":
            return 1
        if k == "const":
            return 0
        if k == "param":
            return named.degree_bound(self.val)
        if k in ("add", "sub"):
            return max(self.args[0].degree_bound(named), self.args[1].degree_bound(named))
        if k == "mul":
            return self.args[0].degree_bound(named) + self.args[1].degree_bound(named)
        if k == "neg":
            return self.args[0].degree_bound(named)
        if k == "inv":
            a = self.args[0]
            if a.kind == "const" or (a.kind == "param" and named.degree_bound(a.val) == 0):
                return 0
            raise ValueError("Cannot compute the degree of an inverse")
        raise AssertionError(k)


class ExtExpr(Expr):
    """A secure field (QM31) expression (mod.rs:60-78)."""

    is_ext = True

    @staticmethod
    def secure_col(a, b, c, d) -> "ExtExpr":
        return ExtExpr("secure_col", (_as_base(a), _as_base(b), _as_base(c), _as_base(d)))

    @staticmethod
    def const(v: Q) -> "ExtExpr":
        return ExtExpr("const", (), tuple(x % P for x in v))

    @staticmethod
    def param(name: str) -> "ExtExpr":
        return ExtExpr("param", (), name)

    @staticmethod
    def from_base(b: BaseExpr) -> "ExtExpr":
        z = BaseExpr.zero()
        return ExtExpr.secure_col(b, z, z, z)

    @staticmethod
    def from_secure(v: Q) -> "ExtExpr":
        # From<SecureField>: a SecureCol of the four coordinates as base constants (mod.rs:105-114).
        return ExtExpr.secure_col(*(BaseExpr.const(x) for x in v))

    @staticmethod
    def combine(relation: "Relation", values: Sequence["BaseExpr"]) -> "ExtExpr":
        """The relation entry value[0] * <name>_alpha0 + ... - <name>_z as one node, whose kernel
        code is a loop over the values rather than one product per value."""
        return ExtExpr("combine", tuple(_as_base(v) for v in values[:relation.size]), (relation.name, relation.size))

    def expanded(self) -> "ExtExpr":
        """A combine node written out as combine_formal's sum."""
        return combine_formal(Relation(*self.val), self.args)

    @staticmethod
    def zero() -> "ExtExpr":
        return ExtExpr.from_base(BaseExpr.zero())

    @staticmethod
    def one() -> "ExtExpr":
        return ExtExpr.from_base(BaseExpr.one())

    def __add__(self, o):
        return ExtExpr("add", (self, _as_ext(o)))

    def __radd__(self, o):
        return _as_ext(o) + self

    def __sub__(self, o):
        return ExtExpr("sub", (self, _as_ext(o)))

    def __rsub__(self, o):
        return _as_ext(o) - self

    def __mul__(self, o):
        return ExtExpr("mul", (self, _as_ext(o)))

    def __rmul__(self, o):
        return _as_ext(o) * self

    def __neg__(self):
        return ExtExpr("neg", (self,))

    def square(self) -> "ExtExpr":
        return self * self

    # ---- simplify (simplify.rs:104-140)
    def simplify(self) -> "ExtExpr":
        done = _SIMPLIFIED.get(self.uid)
        if done is None:
            done = _SIMPLIFIED[self.uid] = self._simplify()
        return done

    def _simplify(self) -> "ExtExpr":
        if self.kind == "combine":
            return ExtExpr("combine", tuple(a.simplify() for a in self.args), self.val)
        s = _simplify_arith(self)
        if s.kind == "secure_col":
            parts = [p.simplify() for p in s.args]
            if all(p.kind == "const" for p in parts):
                return ExtExpr.const(tuple(p.val for p in parts))
            return ExtExpr.secure_col(*parts)
        return s

    def simplify_and_format(self) -> str:
        return self.simplify().format_expr()

    # ---- format (format.rs:35-63)
    def format_expr(self) -> str:
        k = self.kind
        if k == "secure_col":
            a, b, c, d = self.args
            z = BaseExpr.zero()
            if b is z and c is z and d is z:
                return a.format_expr()
            return (f"QM31Impl::from_partial_evals([{a.format_expr()}, {b.format_expr()}, "
                    f"{c.format_expr()}, {d.format_expr()}])")
        if k == "const":
            v = self.val
            return f"qm31({v[0]}, {v[1]}, {v[2]}, {v[3]})"
        if k == "param":
            return self.val
        if k == "combine":
            return self.expanded().format_expr()
        a = self.args
        if k == "add":
            return f"{a[0].format_expr()} + {a[1].format_expr()}"
        if k == "sub":
            return f"{a[0].format_expr()} - ({a[1].format_expr()})"
        if k == "mul":
            return f"({a[0].format_expr()}) * ({a[1].format_expr()})"
        if k == "neg":
            return f"-({a[0].format_expr()})"
        raise AssertionError(k)

    # ---- degree (degree.rs:86-104), memoised per NamedExprs
    def degree_bound(self, named: "NamedExprs") -> int:
        d = named.memo.get(self.uid)
        if d is None:
            d = named.memo[self.uid] = self._degree(named)
        return d

    def _degree(self, named: "NamedExprs") -> int:
        k = self.kind
        if k == "combine":
            return self.expanded().degree_bound(named)
        if k == "secure_col":
            return max(p.degree_bound(named) for p in self.args)
        if k == "const":
            return 0
        if k == "param":
            return named.degree_bound(self.val)
        if k in ("add", "sub"):
            return max(self.args[0].degree_bound(named), self.args[1].degree_bound(named))
        if k == "mul":
            return self.args[0].degree_bound(named) + self.args[1].degree_bound(named)
        if k == "neg":
            return self.args[0].degree_bound(named)
        raise AssertionError(k)


def _is_zero(c: Expr) -> bool:
    return c.val == 0 if not c.is_ext else all(x == 0 for x in c.val)


def _is_one(c: Expr) -> bool:
    return c.val == 1 if not c.is_ext else c.val == (1, 0, 0, 0)


def _is_minus_one(c: Expr) -> bool:
    return c.val == P - 1 if not c.is_ext else c.val == (P - 1, 0, 0, 0)


def _cadd(a: Expr, b: Expr):
    return type(a).const(q_add(a.val, b.val) if a.is_ext else a.val + b.val)


def _csub(a: Expr, b: Expr):
    return type(a).const(q_sub(a.val, b.val) if a.is_ext else a.val - b.val)


def _cmul(a: Expr, b: Expr):
    return type(a).const(q_mul(a.val, b.val) if a.is_ext else a.val * b.val)


def _cneg(a: Expr):
    return type(a).const(q_neg(a.val) if a.is_ext else -a.val)


def _simplify_arith(e: Expr) -> Expr:
    """simplify_arithmetic! (simplify.rs:7-84), shared by both expression types."""
    T = type(e)
    k = e.kind
    if k == "add":
        a, b = (x.simplify() for x in e.args)
        if a.kind == "const" and b.kind == "const":
            return _cadd(a, b)
        if a.kind == "const" and _is_zero(a):
            return b
        if b.kind == "const" and _is_zero(b):
            return a
        if a.kind == "neg" and b.kind == "neg":
            return -(T("add", (a.args[0], b.args[0])))
        if a.kind == "neg":
            return T("sub", (b, a.args[0]))
        if b.kind == "neg":
            return T("sub", (a, b.args[0]))
        return T("add", (a, b))
    if k == "sub":
        a, b = (x.simplify() for x in e.args)
        if a.kind == "const" and b.kind == "const":
            return _csub(a, b)
        if a.kind == "const" and _is_zero(a):
            return -b
        if b.kind == "const" and _is_zero(b):
            return a
        if a.kind == "neg" and b.kind == "neg":
            return T("sub", (b.args[0], a.args[0]))
        if a.kind == "neg":
            return -(T("add", (a.args[0], b)))
        if b.kind == "neg":
            return T("add", (a, b.args[0]))
        return T("sub", (a, b))
    if k == "mul":
        a, b = (x.simplify() for x in e.args)
        if a.kind == "const" and b.kind == "const":
            return _cmul(a, b)
        if a.kind == "const" and _is_zero(a):
            return T.zero()
        if b.kind == "const" and _is_zero(b):
            return T.zero()
        if a.kind == "const" and _is_one(a):
            return b
        if b.kind == "const" and _is_one(b):
            return a
        if a.kind == "const" and _is_minus_one(a):
            return -b
        if b.kind == "const" and _is_minus_one(b):
            return -a
        if a.kind == "neg" and b.kind == "neg":
            return T("mul", (a.args[0], b.args[0]))
        if a.kind == "neg":
            return -(T("mul", (a.args[0], b)))
        if b.kind == "neg":
            return -(T("mul", (a, b.args[0])))
        return T("mul", (a, b))
    if k == "neg":
        a = e.args[0].simplify()
        if a.kind == "const":
            return _cneg(a)
        if a.kind == "neg":
            return a.args[0]
        if a.kind == "sub":
            return T("sub", (a.args[1], a.args[0]))
        return -a
    return e


class NamedExprs:
    """Named intermediates for degree bounds (degree.rs:14-36)."""

    def __init__(self, exprs: Dict[str, BaseExpr], ext_exprs: Dict[str, ExtExpr]):
        self.exprs, self.ext_exprs = exprs, ext_exprs
        self.memo: Dict[int, int] = {}
        self.name_memo: Dict[str, int] = {}

    def degree_bound(self, name: str) -> int:
        d = self.name_memo.get(name)
        if d is None:
            d = self.name_memo[name] = self._named_degree(name)
        return d

    def _named_degree(self, name: str) -> int:
        if name in self.exprs:
            return self.exprs[name].degree_bound(self)
        if name in self.ext_exprs:
            return self.ext_exprs[name].degree_bound(self)
        if name.startswith("preprocessed."):
            return 1
        return 0


# ------------------------------------------------------------------ relations and fractions
class Relation:
    """A LogUp relation (the `relation!` macro, constraint_framework/mod.rs:298-336): up to
    `size` values combined with alpha powers, minus z. In an ExprEvaluator only the name and size
    matter; `alpha_powers(z, alpha)` gives the parameter values that LookupElements::draw makes
    (constraint_framework/logup.rs:81-95)."""

    def __init__(self, name: str, size: int):
        self.name, self.size = name, size

    def param_values(self, z: Q, alpha: Q) -> Dict[str, Q]:
        out, cur = {f"{self.name}_z": tuple(z)}, (1, 0, 0, 0)
        for i in range(self.size):
            out[f"{self.name}_alpha{i}"] = cur
            cur = q_mul(cur, tuple(alpha))
        return out


class Fraction:
    """Fraction<N, D> with the reference's sum (core/lookups/utils.rs:210-251)."""

    def __init__(self, numerator, denominator):
        self.numerator, self.denominator = numerator, denominator

    def __add__(self, rhs: "Fraction") -> "Fraction":
        return Fraction(rhs.denominator * self.numerator + self.denominator * rhs.numerator,
                        self.denominator * rhs.denominator)


def _sum_fracs(fracs: List[Fraction]) -> Fraction:
    acc = fracs[0]
    for f in fracs[1:]:
        acc = acc + f
    return acc


def combine_formal(relation: Relation, values: Sequence[BaseExpr]) -> ExtExpr:
    """value[0] * <name>_alpha0 + ... - <name>_z (evaluator.rs:33-52)."""
    acc = ExtExpr.zero()
    for i, v in enumerate(values[:relation.size]):
        acc = acc + ExtExpr.param(f"{relation.name}_alpha{i}") * _as_base(v)
    return acc - ExtExpr.param(f"{relation.name}_z")


PREPROCESSED_TRACE_IDX, ORIGINAL_TRACE_IDX, INTERACTION_TRACE_IDX = 0, 1, 2
# Relations wider than this are recorded as combine nodes (a loop in the kernel); narrower ones as
# combine_formal's sum, which the kernel evaluates inline.
COMBINE_LOOP_MIN = 16


class ExprEvaluator:
    """EvalAtRow that records expressions (evaluator.rs:54-227)."""

    def __init__(self):
        self.cur_var_index = 0
        self.local_index = [0, 0, 0]
        self.constraints: List[ExtExpr] = []
        self.intermediates: Dict[str, BaseExpr] = {}
        self.ext_intermediates: Dict[str, ExtExpr] = {}
        self.ordered_intermediates: List[str] = []
        # Preprocessed column ids in the order they are requested; each is read as the next
        # column of interaction 0, as SimdDomainEvaluator reads them.
        self.preprocessed: List[str] = []
        # [interaction] -> offsets of each column, in read order (the component's mask).
        self.mask: List[List[List[int]]] = [[], [], []]
        # LogUp state (FormalLogupAtRow, evaluator.rs:13-31).
        self.logup_fracs: List[Fraction] = []
        self.logup_batches: List[Fraction] = []
        self.logup_finalized = True
        self.cumsum_shift = ExtExpr.param("claimed_sum") * BaseExpr.param("column_size").inverse()

    # ---- masks
    def next_interaction_mask(self, interaction: int, offsets: Sequence[int]) -> List[BaseExpr]:
        while len(self.local_index) <= interaction:
            self.local_index.append(0)
            self.mask.append([])
        local = self.local_index[interaction]
        self.local_index[interaction] += 1
        self.mask[interaction].append(list(offsets))
        res = [BaseExpr.col(interaction, self.cur_var_index, off, local) for off in offsets]
        self.cur_var_index += 1
        return res

    def next_trace_mask(self) -> BaseExpr:
        return self.next_interaction_mask(ORIGINAL_TRACE_IDX, [0])[0]

    def next_extension_interaction_mask(self, interaction: int, offsets: Sequence[int]) -> List[ExtExpr]:
        cols = [self.next_interaction_mask(interaction, offsets) for _ in range(4)]
        return [self.combine_ef([cols[k][j] for k in range(4)]) for j in range(len(offsets))]

    def get_preprocessed_column(self, column_id: str) -> BaseExpr:
        # The reference names the column (evaluator.rs:222-224); the domain kernel reads it as
        # the next column of interaction 0 (the default EvalAtRow::get_preprocessed_column).
        self.preprocessed.append(column_id)
        self.mask[PREPROCESSED_TRACE_IDX].append([0])
        self.local_index[PREPROCESSED_TRACE_IDX] += 1
        return BaseExpr.param(column_id)

    @staticmethod
    def combine_ef(values: Sequence[BaseExpr]) -> ExtExpr:
        return ExtExpr.secure_col(*values)

    # ---- constraints and intermediates
    def add_constraint(self, c) -> None:
        self.constraints.append(_as_ext(c))

    def _name(self) -> str:
        return f"intermediate{len(self.intermediates) + len(self.ext_intermediates)}"

    def add_intermediate(self, e) -> BaseExpr:
        name = self._name()
        self.intermediates[name] = _as_base(e)
        self.ordered_intermediates.append(name)
        return BaseExpr.param(name)

    def add_extension_intermediate(self, e) -> ExtExpr:
        name = self._name()
        self.ext_intermediates[name] = _as_ext(e)
        self.ordered_intermediates.append(name)
        return ExtExpr.param(name)

    # ---- LogUp (evaluator.rs:203-215 and logup_proxy, constraint_framework/mod.rs:165-240)
    def add_to_relation(self, relation: Relation, multiplicity, values: Sequence[BaseExpr]) -> None:
        combined = ExtExpr.combine(relation, values) if relation.size > COMBINE_LOOP_MIN else combine_formal(relation,
                                                                                                          values)
        inter = self.add_extension_intermediate(combined)
        self.write_logup_frac(Fraction(_as_ext(multiplicity), inter))

    def write_logup_frac(self, frac: Fraction) -> None:
        if not self.logup_fracs:
            self.logup_finalized = False
        self.logup_fracs.append(frac)

    def finalize_logup_batched(self, batching: Sequence[int]) -> None:
        assert not self.logup_finalized, "LogupAtRow was already finalized"
        assert len(batching) == len(self.logup_fracs), "Batching must be of the same length as the entries"
        last = max(batching)
        by_batch: Dict[int, List[Fraction]] = {}
        for b, f in zip(batching, self.logup_fracs):
            by_batch.setdefault(b, []).append(f)
        assert set(by_batch) == set(range(last + 1)), "Batching must contain all consecutive batches"
        prev_col = ExtExpr.zero()
        # The batch fractions, in column order: what the interaction trace's columns accumulate
        # (LogupColGenerator::write_frac, logup.rs:222-238).
        self.logup_batches = [_sum_fracs(by_batch[b]) for b in range(last + 1)]
        for b in range(last):
            frac = _sum_fracs(by_batch[b])
            cur, = self.next_extension_interaction_mask(INTERACTION_TRACE_IDX, [0])
            diff = cur - prev_col
            prev_col = cur
            self.add_constraint(diff * frac.denominator - frac.numerator)
        frac = _sum_fracs(by_batch[last])
        prev_row, cur = self.next_extension_interaction_mask(INTERACTION_TRACE_IDX, [-1, 0])
        diff = cur - prev_row - prev_col
        fixed = diff + self.cumsum_shift
        self.add_constraint(fixed * frac.denominator - frac.numerator)
        self.logup_finalized = True

    def finalize_logup(self) -> None:
        self.finalize_logup_batched(list(range(len(self.logup_fracs))))

    def finalize_logup_in_pairs(self) -> None:
        self.finalize_logup_batched([n // 2 for n in range(len(self.logup_fracs))])

    # ---- outputs
    def intermediate(self, name: str) -> Expr:
        e = self.intermediates.get(name)
        return e if e is not None else self.ext_intermediates[name]

    def format_constraints(self) -> str:
        """ExprEvaluator::format_constraints (evaluator.rs:88-132)."""
        inter = [f"let {n} = {self.intermediate(n).simplify_and_format()};" for n in self.ordered_intermediates]
        cons = [f"let constraint_{i} = {c.simplify_and_format()};" for i, c in enumerate(self.constraints)]
        parts = ["\n\n".join(inter), "\n\n".join(cons)]
        return "\n\n".join(p for p in parts if p)

    def constraint_degree_bounds(self) -> List[int]:
        named = NamedExprs(dict(self.intermediates), dict(self.ext_intermediates))
        return [c.degree_bound(named) for c in self.constraints]

    def n_constraints(self) -> int:
        return len(self.constraints)


# ------------------------------------------------------------------ evaluation on the host
def eval_expr(e: Expr, cols, params: Dict[str, object], memo: Optional[dict] = None) -> Q:
    """Evaluates e with `cols(ColumnExpr) -> value` and `params[name] -> value`, both QM31
    tuples or ints. Values are QM31 throughout (base values embedded as (v, 0, 0, 0)), as the
    PointEvaluator sees them at an out-of-domain point (constraint_framework/point.rs)."""
    if memo is None:
        memo = {}
    stack = [e]
    while stack:
        n = stack[-1]
        if n.uid in memo:
            stack.pop()
            continue
        pending = [a for a in n.args if a.uid not in memo]
        if pending:
            stack.extend(pending)
            continue
        stack.pop()
        k = n.kind
        if k == "col":
            v = cols(n.val)
        elif k == "const":
            v = n.val
        elif k == "param":
            v = params[n.val]
        else:
            a = [memo[x.uid] for x in n.args]
            a = [(x % P, 0, 0, 0) if isinstance(x, int) else x for x in a]
            if k == "add":
                v = q_add(a[0], a[1])
            elif k == "sub":
                v = q_sub(a[0], a[1])
            elif k == "mul":
                v = q_mul(a[0], a[1])
            elif k == "neg":
                v = q_neg(a[0])
            elif k == "inv":
                v = q_inv(a[0])
            elif k == "secure_col":
                v = q_from_partial_evals(a)
            elif k == "combine":
                name, _ = n.val
                v = (0, 0, 0, 0)
                for i, x in enumerate(a):
                    al = params[f"{name}_alpha{i}"]
                    v = q_add(v, q_mul((al % P, 0, 0, 0) if isinstance(al, int) else tuple(al), x))
                z = params[f"{name}_z"]
                v = q_sub(v, (z % P, 0, 0, 0) if isinstance(z, int) else tuple(z))
            else:
                raise AssertionError(k)
        if isinstance(v, int):
            v = (v % P, 0, 0, 0)
        memo[n.uid] = v
    return memo[e.uid]


def with_intermediates(ev: ExprEvaluator, cols, params: Dict[str, object]) -> Dict[str, object]:
    """`params` plus every intermediate's value, evaluated in definition order."""
    out = dict(params)
    for name in ev.ordered_intermediates:
        out[name] = eval_expr(ev.intermediate(name), cols, out)
    return out
