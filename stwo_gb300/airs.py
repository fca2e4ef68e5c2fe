"""FrameworkEval definitions of the reference's example AIRs, written against the expression
framework (stwo_gb300.expr), so that their constraint kernels are generated rather than
hand-written.

Each class has the FrameworkEval surface (crates/prover/src/constraint_framework/component.rs:
33-47): `log_size()`, `max_constraint_log_degree_bound()` and `evaluate(eval)`, plus `params()`,
the values of the formal parameters its constraints name (relation elements, claimed sum, column
size). `evaluate` restates the example's own `evaluate` step for step:
  WideFibonacciEval   crates/prover/src/examples/wide_fibonacci/mod.rs:25-44
  PoseidonEval        crates/prover/src/examples/poseidon/mod.rs:53-197 (constants all 1234)
  PlonkEval           crates/prover/src/examples/plonk/mod.rs:40-95
  StateTransitionEval crates/prover/src/examples/state_machine/components.rs:33-66
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
