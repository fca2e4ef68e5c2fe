"""prove() for components written against the constraint framework, over the per-operation C ABI.

Each component is a FrameworkEval-like object (`stwo_gb300.airs`) whose constraint kernel and
LogUp interaction kernel are generated (`stwo_gb300.codegen`); any number of them, of different
sizes, share the trees as the reference lays them out. Restated from (file:line of the reference):
  prove                          crates/prover/src/core/prover/mod.rs:27-79
  Components (mask points, OODS) crates/prover/src/core/air/components.rs:15-137
  DomainEvaluationAccumulator    crates/prover/src/core/air/accumulation.rs:49-149
  TraceLocationAllocator         crates/prover/src/constraint_framework/component.rs:45-175
  FrameworkComponent             crates/prover/src/constraint_framework/component.rs:236-416
and the two examples without a hand-written device prover:
  prove_fibonacci_plonk          crates/prover/src/examples/plonk/mod.rs:153-266
  prove_state_machine            crates/prover/src/examples/state_machine/mod.rs:26-135, gen.rs:20-89
  prove_blake                    crates/prover/src/examples/blake/air.rs:308-460
Every O(trace) step after trace generation runs on the device: the generated constraint kernels,
the generated LogUp interaction kernels, and the backend operations of host_prover (FFT, Merkle,
quotients, FRI, grind). The Plonk circuit and the state-machine traces are built on the host, as
the reference's examples build them before prove(); the full Blake example's trace is generated
on the device (stwo_gen_blake_example_trace).
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import QM31, QM31Point, call
from .circle import canonic_half_coset, coset, subgroup_gen
from .codegen import GeneratedComponent

STWO_AIR_BLAKE_ROUND = 2  # include/stwo_cuda.h
from .host_prover import (Blake2sChannel, Buf, CommitmentSchemeProver, SecureCol, _block_views, _coset_vanishing,
                          _finish_proof, _log2, _ptr4, _ptrs, index_to_point, q_add, q_inv, q_m31, q_mul, q_sub)

P = (1 << 31) - 1
Q = Tuple[int, int, int, int]


class TraceLocationAllocator:
    """Columns of each tree handed out in component order; preprocessed columns by id
    (component.rs:45-175, dynamic allocation)."""

    def __init__(self):
        self.next = [0, 0, 0]
        self.preprocessed: List[str] = []

    def place(self, gc: GeneratedComponent) -> "PlacedComponent":
        spans = []
        for t, cols in enumerate(gc.mask()):
            if t == 0:
                spans.append((0, 0))
                continue
            while len(self.next) <= t:
                self.next.append(0)
            spans.append((self.next[t], self.next[t] + len(cols)))
            self.next[t] += len(cols)
        pre = []
        for cid in gc.ev.preprocessed:
            if cid not in self.preprocessed:
                self.preprocessed.append(cid)
            pre.append(self.preprocessed.index(cid))
        return PlacedComponent(gc, spans, pre)


class PlacedComponent:
    def __init__(self, gc: GeneratedComponent, spans, preprocessed: List[int]):
        self.gc, self.spans, self.preprocessed = gc, spans, preprocessed

    def polys(self, pcs: CommitmentSchemeProver, t: int) -> List[Buf]:
        if t == 0:
            return [pcs.trees[0].polys[i] for i in self.preprocessed]
        a, b = self.spans[t]
        return pcs.trees[t].polys[a:b]


def _pt_add(p, m) -> Tuple[Q, Q]:
    """A QM31 circle point plus an M31 one."""
    (x, y), (mx, my) = p, m
    return (q_sub(q_mul(x, q_m31(mx)), q_mul(y, q_m31(my))), q_add(q_mul(x, q_m31(my)), q_mul(y, q_m31(mx))))


def _mask_point(p, log_size: int, offset: int):
    """point + CanonicCoset(log_size).step() * offset (component.rs:236-247)."""
    step = subgroup_gen(log_size)
    idx = (step * abs(offset)) & P
    if offset < 0:
        idx = ((1 << 31) - idx) & P
    return _pt_add(p, index_to_point(idx))


def prove(components: Sequence[PlacedComponent], pcs: CommitmentSchemeProver, ch: Blake2sChannel,
          cfg: Tuple[int, int, int, int]) -> bytes:
    """prove (prover/mod.rs:27-79) for placed components; `pcs` holds the preprocessed, trace and
    interaction trees. Returns the canonical proof bytes."""
    rc = ch.draw_felt()
    # Composition polynomial (components.rs:122-137, accumulation.rs:49-149).
    total = sum(c.gc.n_constraints for c in components)
    comp_log = max(c.gc.max_constraint_log_degree_bound() for c in components)
    powers = (QM31 * max(total, 1))()
    call("stwo_generate_secure_powers", QM31(rc), total, powers, None)
    remaining = [tuple(powers[i].v) for i in range(total)]
    sub: Dict[int, SecureCol] = {}
    for c in components:
        n = c.gc.n_constraints
        mine, remaining = remaining[len(remaining) - n:], remaining[:len(remaining) - n]
        eval_log, log = c.gc.max_constraint_log_degree_bound(), c.gc.log_size()
        acc = sub.setdefault(eval_log, SecureCol(1 << eval_log, zero=True))
        cols: List[Buf] = []
        for t in range(len(c.gc.mask())):
            polys = c.polys(pcs, t)
            if not polys:
                continue
            ext = _block_views([1 << eval_log] * len(polys))  # the component's "Extension" (component.rs:305-322)
            call("stwo_evaluate_columns", pcs.tw, canonic_half_coset(eval_log), _ptrs(polys), log, _ptrs(ext),
                 len(ext), None)
            cols += ext
        arr = (QM31 * max(n, 1))(*[QM31(p) for p in mine])
        c.gc.eval_constraints([b.ptr for b in cols], arr, [b.ptr for b in acc.cols])
    cur: Optional[SecureCol] = None
    for log in sorted(sub):  # DomainEvaluationAccumulator::finalize
        vals = sub[log]
        if cur is not None:
            ev = SecureCol(1 << log, zero=False)
            call("stwo_evaluate_columns", pcs.tw, canonic_half_coset(log), _ptr4(cur.cols), _log2(cur.n),
                 _ptr4(ev.cols), 4, None)
            call("stwo_secure_accumulate", _ptr4(vals.cols), _ptr4(ev.cols), vals.n, None)
        call("stwo_interpolate_columns", pcs.tw, canonic_half_coset(log), _ptr4(vals.cols), 4, None)
        cur = vals
    pcs.commit_polys(cur.cols, ch)

    # Out-of-domain sampling (prover/mod.rs:51-68) with Components::mask_points.
    px, py = ch.random_point()
    oods = (px, py)
    points: List[List[list]] = [[[] for _ in tr.polys] for tr in pcs.trees]
    shifted: Dict[Tuple[int, int], tuple] = {}

    def mask_pt(log_size: int, offset: int):
        """oods shifted by `offset` steps of the log_size coset; the same for every column that
        asks for it."""
        key = (log_size, offset)
        if key not in shifted:
            shifted[key] = _mask_point(oods, log_size, offset)
        return shifted[key]

    for c in components:
        for i in c.preprocessed:
            points[0][i] = [oods]
        for t, offs_per_col in enumerate(c.gc.mask()):
            if t == 0:
                continue
            a, _ = c.spans[t]
            for k, offs in enumerate(offs_per_col):
                points[t][a + k] = [mask_pt(c.gc.log_size(), o) for o in offs]
    points[-1] = [[oods]] * 4
    polys = [p for tr in pcs.trees for p in tr.polys]
    poly_of, pts = [], []
    k = 0
    for ti, tr in enumerate(pcs.trees):
        for ci in range(len(tr.polys)):
            for pt in points[ti][ci]:
                poly_of.append(k)
                pts.append(pt)
            k += 1
    out = (QM31 * max(len(pts), 1))()
    logs = (C.c_uint32 * max(len(polys), 1))(*[_log2(p.n) for p in polys])
    call("stwo_eval_at_points", _ptrs(polys), logs, len(polys), (C.c_uint32 * max(len(pts), 1))(*poly_of),
         (QM31Point * max(len(pts), 1))(*[QM31Point(QM31(x), QM31(y)) for x, y in pts]), len(pts), out, None)
    vals = [tuple(out[i].v) for i in range(len(pts))]
    sampled, vi = [], 0
    for ti, tr in enumerate(pcs.trees):
        tv = []
        for ci in range(len(tr.polys)):
            tv.append(vals[vi:vi + len(points[ti][ci])])
            vi += len(points[ti][ci])
        sampled.append(tv)
    ch.mix_felts([v for tv in sampled for cv in tv for v in cv])
    # Components::eval_composition_polynomial_at_point: one accumulator across the components.
    acc = (0, 0, 0, 0)
    for c in components:
        mask = [[sampled[0][i] for i in c.preprocessed]]
        for t in range(1, len(c.gc.mask())):
            a, b = c.spans[t]
            mask.append(sampled[t][a:b])
        dinv = q_inv(_coset_vanishing(coset(subgroup_gen(c.gc.log_size() + 1), c.gc.log_size()), px, py))
        acc = c.gc.eval_at_point(mask, rc, dinv, acc=acc)
    comp = [cv[0] for cv in sampled[-1]]
    comp_at = q_add(q_add(comp[0], q_mul(comp[1], (0, 1, 0, 0))), q_add(q_mul(comp[2], (0, 0, 1, 0)),
                                                                        q_mul(comp[3], (0, 0, 0, 1))))
    if comp_at != acc:
        raise RuntimeError("ConstraintsNotSatisfied")
    return _finish_proof(pcs, ch, points, sampled, cfg)


# ------------------------------------------------------------------ examples
def _upload(cols: Sequence[np.ndarray]) -> List[Buf]:
    out = []
    for c in cols:
        a = np.ascontiguousarray(c, np.uint32)
        b = Buf(len(a))
        call("stwo_buf_upload", b.ptr, a.ctypes.data, a.nbytes, None)
        out.append(b)
    return out


def _commit_evals(pcs: CommitmentSchemeProver, evals: Sequence[Buf], ch: Blake2sChannel) -> None:
    """TreeBuilder::extend_evals + commit for columns of any sizes (interpolated in place)."""
    by_log: Dict[int, List[Buf]] = {}
    for e in evals:
        by_log.setdefault(_log2(e.n), []).append(e)
    for log in sorted(by_log):
        grp = by_log[log]
        call("stwo_interpolate_columns", pcs.tw, canonic_half_coset(log), _ptrs(grp), len(grp), None)
    pcs.commit_polys(list(evals), ch)


def _mix_config(ch: Blake2sChannel, cfg) -> None:
    """PcsConfig::mix_into (pcs/mod.rs:42-49, fri.rs:80-89)."""
    pow_bits, log_blowup, log_last, n_queries = cfg
    for v in (pow_bits, log_blowup, n_queries, log_last):
        ch.mix_u64(v)


def plonk_circuit(log_n: int) -> Dict[str, np.ndarray]:
    """The Fibonacci circuit of prove_fibonacci_plonk (plonk/mod.rs:159-176)."""
    n = 1 << log_n
    fib = [1, 1]
    for _ in range(n):
        fib.append((fib[-1] + fib[-2]) % P)
    i = np.arange(n, dtype=np.uint32)
    c = {"mult": np.full(n, 2, np.uint32), "a_wire": i, "b_wire": i + 1, "c_wire": i + 2,
         "op": np.ones(n, np.uint32), "a_val": np.array(fib[:n], np.uint32),
         "b_val": np.array(fib[1:n + 1], np.uint32), "c_val": np.array(fib[2:n + 2], np.uint32)}
    c["mult"][n - 1], c["mult"][n - 2] = 0, 1
    return c


def prove_plonk(log_n: int, cfg=(5, 1, 0, 3)) -> Tuple[bytes, Q]:
    """prove_fibonacci_plonk (plonk/mod.rs:153-266) on the device: the canonical proof bytes and
    the component's claimed sum."""
    from .airs import PlonkEval

    circuit = plonk_circuit(log_n)
    pcs = CommitmentSchemeProver(cfg, log_n + cfg[1] + 1)
    ch = Blake2sChannel()
    pre = [circuit[k] for k in ("a_wire", "b_wire", "c_wire", "op")]
    trace = [circuit[k] for k in ("mult", "a_val", "b_val", "c_val")]
    _commit_evals(pcs, _upload(pre), ch)
    _commit_evals(pcs, _upload(trace), ch)
    z, alpha = ch.draw_felts(2)
    gc = GeneratedComponent(PlonkEval(log_n, (z, alpha)))
    block = Buf(gc.n_interaction_columns() << log_n)
    cols = _upload(pre + trace)  # the interaction kernel reads the trace-domain evaluations
    cs = gc.interaction([b.ptr for b in cols], block.ptr)
    inter = _split(block, gc.n_interaction_columns(), 1 << log_n)
    _commit_evals(pcs, inter, ch)
    gc = GeneratedComponent(PlonkEval(log_n, (z, alpha), cs))
    alloc = TraceLocationAllocator()
    return prove([alloc.place(gc)], pcs, ch, cfg), cs


def _split(block: Buf, k: int, n: int) -> List[Buf]:
    """The k columns of n words of a contiguous block, as views that keep the block alive."""
    return [Buf.view(block, j * n, n) for j in range(k)]


def state_machine_trace(log_size: int, initial: Sequence[int], inc_index: int) -> List[np.ndarray]:
    """gen_trace (state_machine/gen.rs:20-48): row i holds the state plus i in coordinate
    inc_index, at the bit-reversed circle-domain position of coset index i."""
    n = 1 << log_size
    i = np.arange(n)
    circ = np.where(i % 2 == 0, i // 2, ((2 << log_size) - i) // 2)
    pos = np.array([int(format(x, f"0{log_size}b")[::-1], 2) for x in circ])
    cols = [np.zeros(n, np.uint32) for _ in range(2)]
    for j in range(2):
        vals = (int(initial[j]) + (i if j == inc_index else 0)) % P
        cols[j][pos] = vals
    return cols


def prove_state_machine(log_n: int, initial: Sequence[int], cfg=(5, 1, 0, 3)) -> Tuple[bytes, Tuple[Q, Q]]:
    """prove_state_machine (state_machine/mod.rs:26-135) on the device: two components, of 2^log_n
    and 2^(log_n - 1) rows. Returns the stark proof's canonical bytes and the claimed sums."""
    from .airs import StateTransitionEval

    logs = (log_n, log_n - 1)
    mid = ((initial[0] + (1 << logs[0])) % P, initial[1])
    traces = [state_machine_trace(logs[0], initial, 0), state_machine_trace(logs[1], mid, 1)]
    pcs = CommitmentSchemeProver(cfg, log_n + cfg[1] + 1)
    ch = Blake2sChannel()
    _mix_config(ch, cfg)
    pcs.commit_polys([], ch)
    ch.mix_u64(logs[0])
    ch.mix_u64(logs[1])
    _commit_evals(pcs, _upload(traces[0] + traces[1]), ch)
    z, alpha = ch.draw_felts(2)
    inter, sums = [], []
    for k in range(2):
        gc = GeneratedComponent(StateTransitionEval(k, logs[k], (z, alpha)))
        block = Buf(gc.n_interaction_columns() << logs[k])
        cols = _upload(traces[k])
        sums.append(gc.interaction([b.ptr for b in cols], block.ptr))
        inter += _split(block, gc.n_interaction_columns(), 1 << logs[k])
    ch.mix_felts(sums)
    _commit_evals(pcs, inter, ch)
    alloc = TraceLocationAllocator()
    comps = [alloc.place(GeneratedComponent(StateTransitionEval(k, logs[k], (z, alpha), sums[k]))) for k in range(2)]
    return prove(comps, pcs, ch, cfg), (sums[0], sums[1])


class HandWrittenComponent(GeneratedComponent):
    """A framework component whose evaluation on the domain runs one of the library's hand-written
    kernels (stwo_eval_constraints, as the Rust crate's CudaAir components do); its recorded
    expressions still give its mask, its LogUp interaction kernel and its evaluation at a point.
    `air_id` is STWO_AIR_*, `elements` the QM31 values that entry point takes for it."""

    def __init__(self, air, air_id: int, elements: Sequence[Q]):
        super().__init__(air)
        self.air_id, self.elements = air_id, [tuple(e) for e in elements]

    def eval_constraints(self, cols: Sequence[int], coeff_powers, accum4: Sequence[int], stream=None,
                         params: Dict[str, object] = None) -> None:
        el = (QM31 * len(self.elements))(*[QM31(e) for e in self.elements])
        comp = _lib.Component(self.air_id, self.log_size(), 0, QM31(tuple(self.air.claimed_sum)), el,
                              len(self.elements))
        call("stwo_eval_constraints", C.byref(comp), (C.c_void_p * max(len(cols), 1))(*cols), len(cols), coeff_powers,
             self.n_constraints, (C.c_void_p * 4)(*accum4), stream)


# ------------------------------------------------------------------ the full Blake example
def blake_preprocessed(log_n: int) -> List[np.ndarray]:
    """The preprocessed columns of prove_blake (air.rs:343-361): IsFirst(L), IsFirst(L+3),
    IsFirst(L+1), then per XOR table (al, bl, al ^ bl) in natural order and IsFirst of its size
    (blake/preprocessed_columns.rs:58-82)."""
    from .airs import XOR_TABLES

    def is_first(log):
        c = np.zeros(1 << log, np.uint32)
        c[0] = 1
        return c

    pre = [is_first(log_n), is_first(log_n + 3), is_first(log_n + 1)]
    for w, e in XOR_TABLES:
        lb = w - e
        i = np.arange(1 << (2 * lb), dtype=np.uint32)
        al, bl = i >> np.uint32(lb), i & np.uint32((1 << lb) - 1)
        pre += [al, bl, al ^ bl, is_first(2 * lb)]
    return pre


def blake_device_trace(log_n: int) -> List[Buf]:
    """prove_blake's trace columns generated in HBM (stwo_gen_blake_example_trace), in commit
    order, as views of one block: the scheduler, the two round components, the XOR tables'
    multiplicity columns."""
    from .airs import XOR_TABLES

    n = 1 << log_n
    sizes = [n] * 384 + [8 * n] * 384 + [2 * n] * 384
    for w, e in XOR_TABLES:
        sizes += [1 << (2 * (w - e))] * (1 << (2 * e))
    block = Buf(sum(sizes))
    scratch = Buf(320 * n)
    call("stwo_gen_blake_example_trace", log_n, block.ptr, scratch.ptr, None)
    out, at = [], 0
    for sz in sizes:
        out.append(Buf.view(block, at, sz))
        at += sz
    return out


def prove_blake(log_n: int, cfg=(5, 1, 0, 3)) -> Tuple[bytes, List[Q]]:
    """prove_blake (blake/air.rs:308-460) on the device for 2^log_n BLAKE2s instances: the
    scheduler, two round components (2^(L+3) and 2^(L+1) rows) and the XOR tables 12, 9, 8, 7, 4
    in one proof. Returns the stark proof's canonical bytes and the eight claimed sums (scheduler,
    round 0, round 1, XOR 12, 9, 8, 7, 4), which add to zero. The trace is generated in HBM
    (blake_device_trace) and everything after it runs in generated and library kernels; the
    preprocessed XOR tables are host constants."""
    from .airs import (BlakeRoundEval, BlakeSchedulerEval, XOR_TABLES, XorTableEval, is_first_id,
                       xor_table_id)

    pre = blake_preprocessed(log_n)
    trace = blake_device_trace(log_n)
    n_sched, n_round = 384, 384
    log_max_rows = max(log_n + 3, 16)
    pcs = CommitmentSchemeProver(cfg, log_max_rows + 1 + cfg[1])
    ch = Blake2sChannel()
    _commit_evals(pcs, _upload(pre), ch)
    ch.mix_u64(log_n)
    _commit_evals(pcs, trace, ch)
    trace = blake_device_trace(log_n)  # the committed columns were interpolated in place
    # AllElements::draw (air.rs:119-133): Blake, Round, then the XOR relations 12, 9, 8, 7, 4.
    el = {"blake": tuple(ch.draw_felts(2)), "round": tuple(ch.draw_felts(2))}
    for w, _ in XOR_TABLES:
        el[w] = tuple(ch.draw_felts(2))

    # Each component with its trace columns (its preprocessed ones first where it reads any).
    spans, at = [], 0
    for n_cols in (n_sched, n_round, n_round) + tuple(1 << (2 * e) for _, e in XOR_TABLES):
        spans.append((at, at + n_cols))
        at += n_cols
    assert at == len(trace)

    def evals(cs=None):
        cs = cs or [(0, 0, 0, 0)] * 8
        out = [BlakeSchedulerEval(log_n, el, cs[0]), BlakeRoundEval(log_n + 3, el, cs[1]),
               BlakeRoundEval(log_n + 1, el, cs[2])]
        out += [XorTableEval(w, e, el[w], cs[3 + t]) for t, (w, e) in enumerate(XOR_TABLES)]
        return out

    inter, sums = [], []
    for k, air in enumerate(evals()):
        gc = GeneratedComponent(air)
        a, b = spans[k]
        pre_cols = _upload([pre[3 + 4 * (k - 3) + j] for j in range(3)]) if k >= 3 else []
        cols = pre_cols + trace[a:b]
        block = Buf(gc.n_interaction_columns() << air.log_size())
        sums.append(gc.interaction([c.ptr for c in cols], block.ptr))
        inter += _split(block, gc.n_interaction_columns(), 1 << air.log_size())
    # BlakeStatement1::mix_into (air.rs:146-162): scheduler, XOR 12..4, then the rounds.
    ch.mix_felts([sums[0]] + sums[3:] + sums[1:3])
    _commit_evals(pcs, inter, ch)
    alloc = TraceLocationAllocator()
    alloc.preprocessed = [is_first_id(log_n), is_first_id(log_n + 3), is_first_id(log_n + 1)]
    for w, e in XOR_TABLES:
        alloc.preprocessed += [xor_table_id(w, e, j) for j in range(3)] + [is_first_id(2 * (w - e))]
    # The round components run the hand-written round kernel (STWO_AIR_BLAKE_ROUND: Round, then
    # the XOR relations 12, 9, 8, 7, 4), the others their generated kernels.
    round_el = [q for key in ("round",) + tuple(w for w, _ in XOR_TABLES) for q in el[key]]
    comps = [alloc.place(HandWrittenComponent(air, STWO_AIR_BLAKE_ROUND, round_el) if isinstance(air, BlakeRoundEval)
                         else GeneratedComponent(air)) for air in evals(sums)]
    return prove(comps, pcs, ch, cfg), sums
