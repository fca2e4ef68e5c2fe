"""FrameworkEval definitions of the reference's example AIRs, written against the expression
framework (stwo_gb300.expr), so that their constraint kernels are generated rather than
hand-written.

Each class has the FrameworkEval surface (crates/prover/src/constraint_framework/component.rs:
33-47): `log_size()`, `max_constraint_log_degree_bound()` and `evaluate(eval)`, plus `params()`,
the values of the formal parameters its constraints name (relation elements, claimed sum, column
size), and `shape_key()`, which names what the recorded expressions depend on (not the log size,
the elements or the claimed sum), so that components of one shape share one generated kernel. `evaluate` restates the example's own `evaluate` step for step:
  WideFibonacciEval   crates/prover/src/examples/wide_fibonacci/mod.rs:25-44
  PoseidonEval        crates/prover/src/examples/poseidon/mod.rs:53-197 (constants all 1234)
  PlonkEval           crates/prover/src/examples/plonk/mod.rs:40-95
  StateTransitionEval crates/prover/src/examples/state_machine/components.rs:33-66
  BlakeSchedulerEval  crates/prover/src/examples/blake/scheduler/constraints.rs:10-67
  BlakeRoundEval      crates/prover/src/examples/blake/round/constraints.rs:22-206
  XorTableEval        crates/prover/src/examples/blake/xor_table/constraints.rs:1-61
"""
from __future__ import annotations

from typing import Dict, List, Optional

from .expr import BaseExpr, ExtExpr, Q, Relation

P = (1 << 31) - 1


def _lookup_params(rel: Relation, elements: Optional[tuple]) -> Dict[str, Q]:
    """<name>_z and <name>_alpha{i} from drawn (z, alpha) (LookupElements::draw, logup.rs:81-95)."""
    if elements is None:
        return {}
    return rel.param_values(*elements)


def _logup_params(claimed_sum: Q, log_size: int) -> Dict[str, object]:
    return {"claimed_sum": tuple(claimed_sum), "column_size": (1 << log_size) % P}


class WideFibonacciEval:
    def __init__(self, log_n_rows: int, n_cols: int):
        self.log_n_rows, self.n_cols = log_n_rows, n_cols

    def shape_key(self) -> tuple:
        return ("wide_fib", self.n_cols)

    def log_size(self) -> int:
        return self.log_n_rows

    def max_constraint_log_degree_bound(self) -> int:
        return self.log_n_rows + 1

    def evaluate(self, ev):
        a, b = ev.next_trace_mask(), ev.next_trace_mask()
        for _ in range(2, self.n_cols):
            c = ev.next_trace_mask()
            ev.add_constraint(c - (a.square() + b.square()))
            a, b = b, c
        return ev

    def params(self) -> Dict[str, object]:
        return {}


# ---------------------------------------------------------------- Poseidon2 (width 16, M31)
N_INSTANCES_PER_ROW = 8
N_STATE = 16
N_PARTIAL_ROUNDS = 14
N_HALF_FULL_ROUNDS = 4
ROUND_CONST = 1234  # EXTERNAL_ROUND_CONSTS / INTERNAL_ROUND_CONSTS of the example
POSEIDON_RELATION = Relation("PoseidonElements", N_STATE)


def apply_m4(x: List) -> List:
    """The M4 MDS matrix (poseidon/mod.rs:71-87)."""
    t0 = x[0] + x[1]
    t02 = t0 + t0
    t1 = x[2] + x[3]
    t12 = t1 + t1
    t2 = x[1] + x[1] + t1
    t3 = x[3] + x[3] + t0
    t4 = t12 + t12 + t3
    t5 = t02 + t02 + t2
    t6 = t3 + t5
    t7 = t2 + t4
    return [t6, t5, t7, t4]


def apply_external_round_matrix(state: List) -> None:
    """circ(2M4, M4, M4, M4) (poseidon/mod.rs:89-113)."""
    for i in range(4):
        state[4 * i:4 * i + 4] = apply_m4(state[4 * i:4 * i + 4])
    for j in range(4):
        s = state[j] + state[j + 4] + state[j + 8] + state[j + 12]
        for i in range(4):
            state[4 * i + j] = state[4 * i + j] + s


def apply_internal_round_matrix(state: List) -> None:
    """mu_i = 2^{i+1} + 1 (poseidon/mod.rs:115-132)."""
    total = state[0]
    for s in state[1:]:
        total = total + s
    for i in range(N_STATE):
        state[i] = state[i] * BaseExpr.const(1 << (i + 1)) + total


def pow5(x):
    x2 = x * x
    x4 = x2 * x2
    return x4 * x


class PoseidonEval:
    def __init__(self, log_n_rows: int, elements: Optional[tuple] = None, claimed_sum: Q = (0, 0, 0, 0)):
        self.log_n_rows, self.elements, self.claimed_sum = log_n_rows, elements, claimed_sum

    def shape_key(self) -> tuple:
        return ("poseidon",)

    def log_size(self) -> int:
        return self.log_n_rows

    def max_constraint_log_degree_bound(self) -> int:
        return self.log_n_rows + 2  # LOG_EXPAND

    def evaluate(self, ev):
        """eval_poseidon_constraints (poseidon/mod.rs:140-197)."""
        for _ in range(N_INSTANCES_PER_ROW):
            state = [ev.next_trace_mask() for _ in range(N_STATE)]
            initial = list(state)
            state = self._full_rounds(ev, state)
            for _ in range(N_PARTIAL_ROUNDS):
                state[0] = state[0] + BaseExpr.const(ROUND_CONST)
                apply_internal_round_matrix(state)
                state[0] = pow5(state[0])
                m = ev.next_trace_mask()
                ev.add_constraint(state[0] - m)
                state[0] = m
            state = self._full_rounds(ev, state)
            ev.add_to_relation(POSEIDON_RELATION, ExtExpr.one(), initial)
            ev.add_to_relation(POSEIDON_RELATION, -ExtExpr.one(), state)
        ev.finalize_logup_in_pairs()
        return ev

    @staticmethod
    def _full_rounds(ev, state):
        """N_HALF_FULL_ROUNDS full rounds: constants, external matrix, pow5, one new mask each."""
        for _ in range(N_HALF_FULL_ROUNDS):
            state = [s + BaseExpr.const(ROUND_CONST) for s in state]
            apply_external_round_matrix(state)
            state = [pow5(s) for s in state]
            for i in range(N_STATE):
                m = ev.next_trace_mask()
                ev.add_constraint(state[i] - m)
                state[i] = m
        return state

    def params(self) -> Dict[str, object]:
        return {**_lookup_params(POSEIDON_RELATION, self.elements),
                **_logup_params(self.claimed_sum, self.log_n_rows)}


# ---------------------------------------------------------------- Plonk
PLONK_RELATION = Relation("PlonkLookupElements", 2)


class PlonkEval:
    def __init__(self, log_n_rows: int, elements: Optional[tuple] = None, claimed_sum: Q = (0, 0, 0, 0)):
        self.log_n_rows, self.elements, self.claimed_sum = log_n_rows, elements, claimed_sum

    def shape_key(self) -> tuple:
        return ("plonk",)

    def log_size(self) -> int:
        return self.log_n_rows

    def max_constraint_log_degree_bound(self) -> int:
        return self.log_n_rows + 1

    def evaluate(self, ev):
        a_wire = ev.get_preprocessed_column("preprocessed_plonk_wire_a")
        b_wire = ev.get_preprocessed_column("preprocessed_plonk_wire_b")
        c_wire = ev.get_preprocessed_column("preprocessed_plonk_wire_c")
        op = ev.get_preprocessed_column("preprocessed_plonk_op")
        mult, a_val, b_val, c_val = (ev.next_trace_mask() for _ in range(4))
        ev.add_constraint(c_val - op * (a_val + b_val) + (BaseExpr.one() - op) * a_val * b_val)
        ev.add_to_relation(PLONK_RELATION, ExtExpr.one(), [a_wire, a_val])
        ev.add_to_relation(PLONK_RELATION, ExtExpr.one(), [b_wire, b_val])
        ev.add_to_relation(PLONK_RELATION, ExtExpr.from_base(-mult), [c_wire, c_val])
        ev.finalize_logup_in_pairs()
        return ev

    def params(self) -> Dict[str, object]:
        return {**_lookup_params(PLONK_RELATION, self.elements),
                **_logup_params(self.claimed_sum, self.log_n_rows)}


# ---------------------------------------------------------------- State machine
STATE_SIZE = 2
STATE_MACHINE_RELATION = Relation("StateMachineElements", STATE_SIZE)


class StateTransitionEval:
    def __init__(self, coordinate: int, log_n_rows: int, elements: Optional[tuple] = None,
                 claimed_sum: Q = (0, 0, 0, 0)):
        self.coordinate, self.log_n_rows = coordinate, log_n_rows
        self.elements, self.claimed_sum = elements, claimed_sum

    def shape_key(self) -> tuple:
        return ("state_transition", self.coordinate)

    def log_size(self) -> int:
        return self.log_n_rows

    def max_constraint_log_degree_bound(self) -> int:
        return self.log_n_rows + 1  # LOG_CONSTRAINT_DEGREE

    def evaluate(self, ev):
        inp = [ev.next_trace_mask() for _ in range(STATE_SIZE)]
        out = list(inp)
        out[self.coordinate] = out[self.coordinate] + BaseExpr.one()
        ev.add_to_relation(STATE_MACHINE_RELATION, ExtExpr.one(), inp)
        ev.add_to_relation(STATE_MACHINE_RELATION, -ExtExpr.one(), out)
        ev.finalize_logup_in_pairs()
        return ev

    def params(self) -> Dict[str, object]:
        return {**_lookup_params(STATE_MACHINE_RELATION, self.elements),
                **_logup_params(self.claimed_sum, self.log_n_rows)}


# ---------------------------------------------------------------- Blake (scheduler, round, XOR tables)
BLAKE_STATE = 16
BLAKE_ROUNDS = 10
BLAKE_ROUND_FELTS = 96  # (STATE_SIZE + STATE_SIZE + MESSAGE_SIZE) * N_FELTS_IN_U32
BLAKE_RELATION = Relation("BlakeElements", BLAKE_ROUND_FELTS)
ROUND_RELATION = Relation("RoundElements", BLAKE_ROUND_FELTS)
XOR_TABLES = ((12, 4), (9, 2), (8, 2), (7, 2), (4, 0))  # (elem_bits, expand_bits)
XOR_RELATIONS = {w: Relation(f"XorElements{w}", 3) for w, _ in XOR_TABLES}
# The BLAKE2s message schedule (RFC 7693, section 2.7).
BLAKE2S_SIGMA = (
    (0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15),
    (14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3),
    (11, 8, 12, 0, 5, 2, 15, 13, 10, 14, 3, 6, 7, 1, 9, 4),
    (7, 9, 3, 1, 13, 12, 11, 14, 2, 6, 5, 10, 4, 0, 15, 8),
    (9, 0, 5, 7, 2, 4, 10, 15, 14, 1, 11, 12, 6, 8, 3, 13),
    (2, 12, 6, 10, 0, 11, 8, 3, 4, 13, 7, 5, 15, 14, 1, 9),
    (12, 5, 1, 15, 14, 13, 4, 10, 0, 7, 6, 3, 9, 2, 8, 11),
    (13, 11, 7, 14, 12, 1, 3, 9, 5, 0, 15, 4, 8, 6, 2, 10),
    (6, 15, 14, 9, 11, 3, 0, 8, 12, 2, 13, 7, 1, 4, 10, 5),
    (10, 2, 8, 4, 7, 6, 1, 5, 15, 11, 9, 14, 3, 12, 13, 0),
)


def xor_table_id(elem_bits: int, expand_bits: int, index: int) -> str:
    """XorTable::id (blake/preprocessed_columns.rs:31-38)."""
    return f"preprocessed_xor_table_{elem_bits}_{expand_bits}_{index}"


def is_first_id(log_size: int) -> str:
    """IsFirst::id (constraint_framework/preprocessed_columns.rs:52-56)."""
    return f"preprocessed_is_first_{log_size}"


def _next_u32(ev):
    """A u32 as its (low, high) 16-bit limbs, two trace masks (Fu32)."""
    return (ev.next_trace_mask(), ev.next_trace_mask())


def _felts(words) -> List:
    return [x for w in words for x in w]


class BlakeSchedulerEval:
    """The scheduler: per row one BLAKE2s hash of 10 rounds, read as the messages and the 11
    states; each round is looked up in the Round relation, the whole hash in the Blake relation
    with multiplicity 0. `elements` maps "blake" and "round" to drawn (z, alpha)."""

    def __init__(self, log_n_rows: int, elements: Optional[dict] = None, claimed_sum: Q = (0, 0, 0, 0)):
        self.log_n_rows, self.elements, self.claimed_sum = log_n_rows, elements, claimed_sum

    def shape_key(self) -> tuple:
        return ("blake_scheduler",)

    def log_size(self) -> int:
        return self.log_n_rows

    def max_constraint_log_degree_bound(self) -> int:
        return self.log_n_rows + 1

    def evaluate(self, ev):
        messages = [_next_u32(ev) for _ in range(BLAKE_STATE)]
        states = [[_next_u32(ev) for _ in range(BLAKE_STATE)] for _ in range(BLAKE_ROUNDS + 1)]
        for r in range(BLAKE_ROUNDS):
            round_messages = [messages[k] for k in BLAKE2S_SIGMA[r]]
            ev.add_to_relation(ROUND_RELATION, ExtExpr.one(),
                               _felts(states[r]) + _felts(states[r + 1]) + _felts(round_messages))
        ev.add_to_relation(BLAKE_RELATION, ExtExpr.zero(),
                           _felts(states[0]) + _felts(states[BLAKE_ROUNDS]) + _felts(messages))
        ev.finalize_logup_in_pairs()
        return ev

    def params(self) -> Dict[str, object]:
        el = self.elements or {}
        return {**_lookup_params(BLAKE_RELATION, el.get("blake")), **_lookup_params(ROUND_RELATION, el.get("round")),
                **_logup_params(self.claimed_sum, self.log_n_rows)}


INV16 = 1 << 15  # 2^-16 mod P


class BlakeRoundEval:
    """One BLAKE2s round per row: 8 G functions over u32 limbs with carry constraints, XORs looked
    up in the XOR relations by width, and the round's (input, output, messages) removed from the
    Round relation. `elements` maps "round" and the XOR widths 12, 9, 8, 7, 4 to drawn (z, alpha)."""

    def __init__(self, log_n_rows: int, elements: Optional[dict] = None, claimed_sum: Q = (0, 0, 0, 0)):
        self.log_n_rows, self.elements, self.claimed_sum = log_n_rows, elements, claimed_sum

    def shape_key(self) -> tuple:
        return ("blake_round",)

    def log_size(self) -> int:
        return self.log_n_rows

    def max_constraint_log_degree_bound(self) -> int:
        return self.log_n_rows + 1

    def evaluate(self, ev):
        v = [_next_u32(ev) for _ in range(BLAKE_STATE)]
        input_v = list(v)
        m = [_next_u32(ev) for _ in range(BLAKE_STATE)]
        for k, idx in enumerate(((0, 4, 8, 12), (1, 5, 9, 13), (2, 6, 10, 14), (3, 7, 11, 15),
                                 (0, 5, 10, 15), (1, 6, 11, 12), (2, 7, 8, 13), (3, 4, 9, 14))):
            a, b, c, d = (v[i] for i in idx)
            a, b, c, d = self._g(ev, a, b, c, d, m[2 * k], m[2 * k + 1])
            for i, x in zip(idx, (a, b, c, d)):
                v[i] = x
        ev.add_to_relation(ROUND_RELATION, -ExtExpr.one(), _felts(input_v) + _felts(v) + _felts(m))
        ev.finalize_logup_in_pairs()
        return ev

    def _g(self, ev, a, b, c, d, m0, m1):
        a = self._add3(ev, a, b, m0)
        d = self._xor_rotr16(ev, a, d)
        c = self._add2(ev, c, d)
        b = self._xor_rotr(ev, b, c, 12)
        a = self._add3(ev, a, b, m1)
        d = self._xor_rotr(ev, a, d, 8)
        c = self._add2(ev, c, d)
        b = self._xor_rotr(ev, b, c, 7)
        return a, b, c, d

    @staticmethod
    def _add2(ev, a, b):
        sl, sh = ev.next_trace_mask(), ev.next_trace_mask()
        carry_l = (a[0] + b[0] - sl) * BaseExpr.const(INV16)
        ev.add_constraint(carry_l * carry_l - carry_l)
        carry_h = (a[1] + b[1] + carry_l - sh) * BaseExpr.const(INV16)
        ev.add_constraint(carry_h * carry_h - carry_h)
        return (sl, sh)

    @staticmethod
    def _add3(ev, a, b, c):
        sl, sh = ev.next_trace_mask(), ev.next_trace_mask()
        one, two = BaseExpr.one(), BaseExpr.const(2)
        carry_l = (a[0] + b[0] + c[0] - sl) * BaseExpr.const(INV16)
        ev.add_constraint(carry_l * (carry_l - one) * (carry_l - two))
        carry_h = (a[1] + b[1] + c[1] + carry_l - sh) * BaseExpr.const(INV16)
        ev.add_constraint(carry_h * (carry_h - one) * (carry_h - two))
        return (sl, sh)

    @staticmethod
    def _split(ev, a, r):
        h = ev.next_trace_mask()
        return a - h * BaseExpr.const(1 << r), h

    def _xor2(self, ev, w, a, b):
        c = [ev.next_trace_mask(), ev.next_trace_mask()]
        for k in range(2):
            ev.add_to_relation(XOR_RELATIONS[w], ExtExpr.one(), [a[k], b[k], c[k]])
        return c

    def _xor_rotr(self, ev, a, b, r):
        all_, alh = self._split(ev, a[0], r)
        ahl, ahh = self._split(ev, a[1], r)
        bll, blh = self._split(ev, b[0], r)
        bhl, bhh = self._split(ev, b[1], r)
        xorll, xorhl = self._xor2(ev, r, [all_, ahl], [bll, bhl])
        xorlh, xorhh = self._xor2(ev, 16 - r, [alh, ahh], [blh, bhh])
        s = BaseExpr.const(1 << (16 - r))
        return (xorhl * s + xorlh, xorll * s + xorhh)

    def _xor_rotr16(self, ev, a, b):
        all_, alh = self._split(ev, a[0], 8)
        ahl, ahh = self._split(ev, a[1], 8)
        bll, blh = self._split(ev, b[0], 8)
        bhl, bhh = self._split(ev, b[1], 8)
        xorll, xorhl = self._xor2(ev, 8, [all_, ahl], [bll, bhl])
        xorlh, xorhh = self._xor2(ev, 8, [alh, ahh], [blh, bhh])
        s = BaseExpr.const(1 << 8)
        return (xorhh * s + xorhl, xorlh * s + xorll)

    def params(self) -> Dict[str, object]:
        el = self.elements or {}
        out = {**_lookup_params(ROUND_RELATION, el.get("round")), **_logup_params(self.claimed_sum, self.log_n_rows)}
        for w, _ in XOR_TABLES:
            out.update(_lookup_params(XOR_RELATIONS[w], el.get(w)))
        return out


class XorTableEval:
    """The XOR table of `elem_bits`-bit words with `expand_bits` expanded: the preprocessed
    (al, bl, al ^ bl) over the low limbs, and one multiplicity column per (ah, bh), whose entry
    (al + ah 2^limb, bl + bh 2^limb, cl + (ah ^ bh) 2^limb) has multiplicity -mult."""

    def __init__(self, elem_bits: int, expand_bits: int, elements: Optional[tuple] = None,
                 claimed_sum: Q = (0, 0, 0, 0)):
        self.elem_bits, self.expand_bits = elem_bits, expand_bits
        self.elements, self.claimed_sum = elements, claimed_sum

    def limb_bits(self) -> int:
        return self.elem_bits - self.expand_bits

    def shape_key(self) -> tuple:
        return ("xor_table", self.elem_bits, self.expand_bits)

    def log_size(self) -> int:
        return 2 * self.limb_bits()

    def max_constraint_log_degree_bound(self) -> int:
        return self.log_size() + 1

    def evaluate(self, ev):
        e, x, lb = self.elem_bits, self.expand_bits, self.limb_bits()
        al, bl, cl = (ev.get_preprocessed_column(xor_table_id(e, x, k)) for k in range(3))
        for i in range(1 << (2 * x)):
            ih, jh = i >> x, i % (1 << x)
            mult = ev.next_trace_mask()
            vals = [al + BaseExpr.const(ih << lb), bl + BaseExpr.const(jh << lb),
                    cl + BaseExpr.const((ih ^ jh) << lb)]
            ev.add_to_relation(XOR_RELATIONS[e], -ExtExpr.from_base(mult), vals)
        ev.finalize_logup_in_pairs()
        return ev

    def params(self) -> Dict[str, object]:
        return {**_lookup_params(XOR_RELATIONS[self.elem_bits], self.elements),
                **_logup_params(self.claimed_sum, self.log_size())}
