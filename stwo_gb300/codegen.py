"""CUDA code generation for constraint evaluation on the domain.

An AIR written against the constraint framework (a FrameworkEval: `evaluate(eval)` over the
EvalAtRow surface) is recorded once with `expr.ExprEvaluator`, then emitted as one CUDA kernel
that evaluates every constraint at every row of the evaluation domain and adds
row_res * denom_inv to the accumulation column — what the reference does per row with
SimdDomainEvaluator inside FrameworkComponent::evaluate_constraint_quotients_on_domain
(crates/prover/src/constraint_framework/component.rs:278-416, simd_domain.rs:24-114). The
library compiles the source with NVRTC (stwo_codegen_compile) and launches it through
stwo_eval_constraints_codegen.

Kernel shape (one thread per row, a grid-stride loop):
  * The column table and the random-coefficient powers are staged in shared memory.
  * Every distinct subexpression is one SSA value (nodes are interned, so sharing is exact);
    values that depend on no column (parameters, their inverses and products) are computed once
    per thread before the row loop.
  * Extension values that are embedded base values stay 32-bit words: `ext * base` is four M31
    products, not a QM31 product.
  * Base-field constraints accumulate p_i * c_i into four 64-bit lanes, folded every third
    product; extension constraints take a QM31 product.
  * Mask offsets other than 0 read the row given by offset_bit_reversed_circle_domain_index
    (core/utils.rs:74-90), computed once per offset.
Any order of these exact field operations gives the same words, so the column equals the
reference's row by row.

`GeneratedComponent.eval_at_point` evaluates the same expressions at an out-of-domain point on
the host (PointEvaluator, constraint_framework/point.rs:15-70).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
from typing import Dict, List, Sequence, Tuple

from . import expr as X
from .expr import BaseExpr, Expr, ExprEvaluator

SMEM_BUDGET = 40 * 1024  # shared memory for the column table and the powers, bytes


# A row-loop body of more straight-line statements than this (no repeated group became a loop) is
# compiled for compile time: NVRTC's default pipeline is superlinear in the size of one basic block
# (a 2,700-statement Blake2s round body took minutes), so such a body is cut into blocks of
# FLAT_BLOCK statements by branches the compiler cannot remove, and the source asks for
# --Ofast-compile=mid (FAST_COMPILE_MARK, read by the library's NVRTC call).
FLAT_SPLIT_MIN = 1000
FLAT_BLOCK = 40
FAST_COMPILE_MARK = "// stwo-codegen: fast-compile"
# The library's NVRTC options (codegen.cu), part of the cubin cache key.
NVRTC_FLAGS = b"--gpu-architecture=sm_103a -std=c++17 -lineinfo; marked: --Ofast-compile=mid"


def _split_flat(body: List[str]) -> Tuple[List[str], bool]:
    """`body` with a block boundary after every FLAT_BLOCK top-level statements when it has more
    than FLAT_SPLIT_MIN of them; and whether it was split."""
    top = [i for i, x in enumerate(body) if not x.startswith((" ", "#", "for ", "}"))]
    if len(top) <= FLAT_SPLIT_MIN:
        return body, False
    cut = set(top[FLAT_BLOCK - 1::FLAT_BLOCK])
    out = []
    for i, x in enumerate(body):
        out.append(x)
        if i in cut:
            out.append('if (a.trace_log == 0xFFFFFFFFu) asm volatile("");')
    return out, True


class _Gen:
    def __init__(self, ev: ExprEvaluator):
        self.ev = ev
        self.col_base = [0]
        for m in ev.mask[:-1]:
            self.col_base.append(self.col_base[-1] + len(m))
        self.n_cols = sum(len(m) for m in ev.mask)
        self.params: List[Tuple[str, bool]] = []  # external parameters: (name, is_ext)
        self.param_index: Dict[str, int] = {}
        self.pre: List[str] = []
        self.tables: List[str] = []
        self.offsets: Dict[int, str] = {0: "row"}
        self.uniform_memo: Dict[int, Tuple[str, str, bool]] = {}
        self.pre_params: Dict[str, bool] = {}
        self.n_scopes = 0
        self.resolved: Dict[int, Expr] = {}

    # ---- intermediates and preprocessed columns substituted: a DAG over columns, constants and
    # external parameters only.
    def resolve(self, root: Expr) -> Expr:
        ev = self.ev
        stack = [root]
        while stack:
            n = stack[-1]
            if n.uid in self.resolved:
                stack.pop()
                continue
            if n.kind == "param":
                name = n.val
                if name in ev.intermediates or name in ev.ext_intermediates:
                    target = ev.intermediate(name).simplify()
                elif name in ev.preprocessed:
                    target = BaseExpr.col(0, -1, 0, ev.preprocessed.index(name))
                else:
                    target = n
                if target is n:
                    self.resolved[n.uid] = n
                    stack.pop()
                elif target.uid in self.resolved:
                    self.resolved[n.uid] = self.resolved[target.uid]
                    stack.pop()
                else:
                    stack.append(target)
                continue
            pending = [a for a in n.args if a.uid not in self.resolved]
            if pending:
                stack.extend(pending)
                continue
            stack.pop()
            args = tuple(self.resolved[a.uid] for a in n.args)
            self.resolved[n.uid] = n if all(x is y for x, y in zip(args, n.args)) else type(n)(n.kind, args, n.val)
        return self.resolved[root.uid]

    @staticmethod
    def _topo(roots: Sequence[Expr]) -> List[Expr]:
        """Every node reachable from roots, children before parents, roots in order."""
        seen, out = set(), []
        for r in roots:
            stack = [(r, False)]
            while stack:
                n, done = stack.pop()
                if done:
                    out.append(n)
                    continue
                if n.uid in seen:
                    continue
                seen.add(n.uid)
                stack.append((n, True))
                for a in reversed(n.args):
                    if a.uid not in seen:
                        stack.append((a, False))
        return out

    # ---- grouping: constraints that share a computed (non-uniform) node belong to one group;
    # groups with the same shape up to column renaming form a class, emitted once as a loop.
    def _groups(self, roots: List[Expr]) -> List[List[int]]:
        nodes = self._topo(roots)
        self.uniform = {}
        for n in nodes:
            if n.kind == "col":
                self.uniform[n.uid] = False
            elif n.kind in ("const", "param"):
                self.uniform[n.uid] = True
            else:
                self.uniform[n.uid] = all(self.uniform[a.uid] for a in n.args)
        parent: Dict[int, int] = {}

        def find(x):
            while parent.get(x, x) != x:
                parent[x] = parent.get(parent[x], parent[x])
                x = parent[x]
            return x

        for n in nodes:
            if n.args and not self.uniform[n.uid]:
                for a in n.args:
                    if a.args and not self.uniform[a.uid]:
                        ra, rb = find(a.uid), find(n.uid)
                        if ra != rb:
                            parent[ra] = rb
        by: Dict[int, List[int]] = {}
        for i, r in enumerate(roots):
            by.setdefault(find(r.uid), []).append(i)
        return sorted(by.values(), key=lambda g: g[0])

    def _signature(self, roots: List[Expr], idx: List[int]):
        """Canonical shape of a group: nodes in emission order with columns numbered by first
        use; returns (signature, column table indices in slot order)."""
        canon: Dict[int, int] = {}
        slots: Dict[int, int] = {}
        toks = []
        for n in self._topo([roots[i] for i in idx]):
            if self.uniform[n.uid] and n.args:
                tok = ("u", n.uid)
            elif n.kind == "col":
                c = n.val
                t = self.col_base[c.interaction] + c.local
                tok = ("c", slots.setdefault(t, len(slots)), c.offset)
            elif n.kind in ("const", "param"):
                tok = (n.kind, n.is_ext, n.val)
            elif n.kind == "combine":
                tok = (n.kind, n.is_ext, n.val) + tuple(canon[a.uid] for a in n.args)
            else:
                tok = (n.kind, n.is_ext) + tuple(canon[a.uid] for a in n.args)
            canon[n.uid] = len(toks)
            toks.append(tok)
        sig = (tuple(toks), tuple(canon[roots[i].uid] for i in idx))
        return sig, list(slots)

    def _units(self, roots: List[Expr]) -> List[List[int]]:
        """The emission units: the groups, except that a periodic run of repeated groups (an AIR
        that evaluates N identical instances per row, each a sequence of groups) becomes one unit
        per period, so that one loop body covers a whole instance and loads each of its columns
        once."""
        units = self._groups(roots)
        sigs = [self._signature(roots, u)[0] for u in units]
        count: Dict[tuple, int] = {}
        for sg in sigs:
            count[sg] = count.get(sg, 0) + 1
        rep = [i for i, sg in enumerate(sigs) if count[sg] > 1]
        seq = [sigs[i] for i in rep]
        for p in range(2, len(seq) // 2 + 1):
            if len(seq) % p or any(seq[k] != seq[k % p] for k in range(len(seq))):
                continue
            supers = [sorted(i for j in range(p) for i in units[rep[k * p + j]]) for k in range(len(seq) // p)]
            first = self._signature(roots, supers[0])[0]
            if all(self._signature(roots, sp)[0] == first for sp in supers[1:]):
                taken = set(rep)
                units = [u for i, u in enumerate(units) if i not in taken] + supers
                units.sort(key=lambda u: u[0])
            break
        return units

    # ---- emission
    def _param(self, name: str, is_ext: bool, out, memo) -> Tuple[str, str, bool]:
        """An external parameter, read where it is used: in the code before the row loop when a
        column-independent value needs it (out is None), else in the scope of the unit that uses
        it, so that the relation elements of a LogUp unit are not live across the whole row."""
        k = self.param_index.get(name)
        if k is None:
            k = self.param_index[name] = len(self.params)
            self.params.append((name, is_ext))
        if out is None:
            code, dest, key, seen = f"p{k}", self.pre, name, self.pre_params
        else:
            if "scope" not in memo:
                self.n_scopes += 1
                memo["scope"] = self.n_scopes
            code, dest, key, seen = f"q{k}_{memo['scope']}", out, ("param", name), memo
        if key not in seen:
            seen[key] = True
            if is_ext:
                dest.append(f"const qm31 {code} = gen_param_q(a.params, {k});")
            else:
                dest.append(f"const uint32_t {code} = __ldg(a.params + {4 * k});")
        return (code, "q" if is_ext else "b", out is None)

    def _param_block(self, name: str, size: int) -> int:
        """The parameter index of <name>_alpha0, with <name>_alpha0 .. <name>_alpha{size-1}
        registered as consecutive parameters (gen_combine reads them by index)."""
        first = f"{name}_alpha0"
        if first not in self.param_index:
            for i in range(size):
                nm = f"{name}_alpha{i}"
                assert nm not in self.param_index, nm
                self.param_index[nm] = len(self.params)
                self.params.append((nm, True))
        k0 = self.param_index[first]
        assert all(self.param_index.get(f"{name}_alpha{i}") == k0 + i for i in range(size)), name
        return k0

    def _offset(self, off: int) -> str:
        rv = self.offsets.get(off)
        if rv is None:
            rv = self.offsets[off] = f"r_{'m' if off < 0 else 'p'}{abs(off)}"
        return rv

    def _value(self, root: Expr, memo: Dict, out: List[str], col_ref) -> Tuple[str, str, bool]:
        for n in self._topo([root]):
            if n.kind in ("param", "const") or n.uid in memo or n.uid in self.uniform_memo:
                continue
            uni = self.uniform[n.uid] if n.uid in self.uniform else False
            (self.uniform_memo if uni else memo)[n.uid] = self._emit(n, memo, out, col_ref)
        return self._ref(root, memo, out, False)

    def _ref(self, n: Expr, memo: Dict, out: List[str], parent_uniform: bool) -> Tuple[str, str, bool]:
        """The code of a node for a parent: constants inline, parameters where the parent is."""
        if n.kind == "const":
            if not n.is_ext:
                return (f"{n.val}u", "b", True)
            v = n.val
            if v[1] == v[2] == v[3] == 0:
                return (f"{v[0]}u", "b", True)
            return (f"qm31_from_u32({v[0]}u, {v[1]}u, {v[2]}u, {v[3]}u)", "q", True)
        if n.kind == "param":
            return self._param(n.val, n.is_ext, None if parent_uniform else out, None if parent_uniform else memo)
        return self.uniform_memo.get(n.uid) or memo[n.uid]

    def _stmt(self, uniform: bool, ty: str, code: str, uid: int, out: List[str]) -> Tuple[str, str, bool]:
        name = f"t{uid}"
        decl = "uint32_t" if ty == "b" else "qm31"
        (self.pre if uniform else out).append(f"const {decl} {name} = {code};")
        return (name, ty, uniform)

    def _emit(self, n: Expr, memo: Dict, out: List[str], col_ref) -> Tuple[str, str, bool]:
        k = n.kind
        if k == "col":
            c = n.val
            name = f"c{n.uid}"
            out.append(f"const uint32_t {name} = __ldg({col_ref(self.col_base[c.interaction] + c.local)} + "
                       f"{self._offset(c.offset)});")
            return (name, "b", False)
        uni = self.uniform.get(n.uid, False)
        args = [self._ref(a, memo, out, uni) for a in n.args]
        if k == "combine":
            name, size = n.val
            k0 = self._param_block(name, size)
            zname = f"{name}_z"
            if zname not in self.param_index:
                self.param_index[zname] = len(self.params)
                self.params.append((zname, True))
            arr = f"v{n.uid}"
            (self.pre if uni else out).append(f"const uint32_t {arr}[{len(args)}] = {{{', '.join(a[0] for a in args)}}};")
            return self._stmt(uni, "q", f"gen_combine(a.params, {k0}, {arr}, {len(args)}, {self.param_index[zname]})",
                              n.uid, out)
        if k == "secure_col":
            zero = BaseExpr.zero()
            if all(a is zero for a in n.args[1:]):
                return args[0]
            return self._stmt(uni, "q", "qm31_from_u32({}, {}, {}, {})".format(*(a[0] for a in args)), n.uid, out)
        if k == "neg":
            (x, t, _), = args
            return self._stmt(uni, t, f"m31_neg({x})" if t == "b" else f"gen_q_neg({x})", n.uid, out)
        if k == "inv":
            (x, t, _), = args
            return self._stmt(uni, "b", f"m31_inv({x})", n.uid, out)
        (x, tx, _), (y, ty, _) = args
        if k == "add":
            if tx == ty == "b":
                return self._stmt(uni, "b", f"m31_add({x}, {y})", n.uid, out)
            if tx == "q" and ty == "q":
                return self._stmt(uni, "q", f"qm31_add({x}, {y})", n.uid, out)
            q, b = (x, y) if tx == "q" else (y, x)
            return self._stmt(uni, "q", f"gen_q_add_m31({q}, {b})", n.uid, out)
        if k == "sub":
            if tx == ty == "b":
                return self._stmt(uni, "b", f"m31_sub({x}, {y})", n.uid, out)
            if tx == "q" and ty == "q":
                return self._stmt(uni, "q", f"qm31_sub({x}, {y})", n.uid, out)
            if tx == "q":
                return self._stmt(uni, "q", f"gen_q_sub_m31({x}, {y})", n.uid, out)
            return self._stmt(uni, "q", f"gen_m31_sub_q({x}, {y})", n.uid, out)
        if k == "mul":
            if tx == ty == "b":
                # A power-of-two constant factor 2^j is a 31-bit rotation (2^31 = 1 mod P).
                for (a_, b_) in ((n.args[0], y), (n.args[1], x)):
                    if a_.kind == "const" and not a_.is_ext and a_.val and a_.val & (a_.val - 1) == 0:
                        return self._stmt(uni, "b", f"gen_mul_pow2({b_}, {a_.val.bit_length() - 1})", n.uid, out)
                    if (a_.kind == "const" and a_.is_ext and a_.val[1:] == (0, 0, 0) and a_.val[0]
                            and a_.val[0] & (a_.val[0] - 1) == 0):
                        return self._stmt(uni, "b", f"gen_mul_pow2({b_}, {a_.val[0].bit_length() - 1})", n.uid, out)
                return self._stmt(uni, "b", f"m31_mul({x}, {y})", n.uid, out)
            if tx == "q" and ty == "q":
                return self._stmt(uni, "q", f"qm31_mul({x}, {y})", n.uid, out)
            q, b = (x, y) if tx == "q" else (y, x)
            return self._stmt(uni, "q", f"qm31_mul_m31({q}, {b})", n.uid, out)
        raise AssertionError(k)

    def _accumulate(self, roots, idx, memo, out, col_ref, pw_ref) -> None:
        n_base = 0
        for j, i in enumerate(idx):
            code, ty, _ = self._value(roots[i], memo, out, col_ref)
            if ty == "b":
                out.append(f"gen_acc_base(acc, {pw_ref(j, i)}, {code});")
                n_base += 1
                if n_base % 3 == 0:
                    out.append("gen_fold(acc);")
            else:
                out.append(f"qacc = qm31_add(qacc, qm31_mul(gen_q_of_u4({pw_ref(j, i)}), {code}));")
        if n_base % 3:
            out.append("gen_fold(acc);")

    # ---- the kernel
    def source(self) -> str:
        ev = self.ev
        roots = [self.resolve(c.simplify()) for c in ev.constraints]
        n_cons = len(roots)
        smem_pw = n_cons * 16 + self.n_cols * 8 <= SMEM_BUDGET
        pw_at = (lambda e: f"s_pw[{e}]") if smem_pw else (lambda e: f"gen_ldg_u4(a.powers, {e})")
        classes: Dict[tuple, List[Tuple[List[int], List[int]]]] = {}
        order = []
        for g in self._units(roots):
            sig, slots = self._signature(roots, g)
            if sig not in classes:
                classes[sig] = []
                order.append(sig)
            classes[sig].append((g, slots))
        body: List[str] = []
        outer: Dict[int, Tuple[str, str, bool]] = {}  # values in the row loop's own scope
        for ci, sig in enumerate(order):
            members = classes[sig]
            if len(members) == 1:
                g, slots = members[0]
                self._accumulate(roots, g, outer, body, lambda t: f"s_cols[{t}]", lambda j, i: pw_at(i))
                continue
            # One loop over the members: column slots and constraint indices from tables.
            m, ns, nc = len(members), len(members[0][1]), len(members[0][0])
            cmap = ", ".join(str(t) for g, slots in members for t in slots)
            pmap = ", ".join(str(i) for g, slots in members for i in g)
            ctype = "uint16_t" if self.n_cols < 65536 else "uint32_t"
            ptype = "uint16_t" if n_cons < 65536 else "uint32_t"
            self.tables.append(f"__constant__ {ctype} g_cmap{ci}[{m * ns}] = {{{cmap}}};")
            self.tables.append(f"__constant__ {ptype} g_pmap{ci}[{m * nc}] = {{{pmap}}};")
            g0, slots0 = members[0]
            slot_of = {t: s for s, t in enumerate(slots0)}
            inner = []
            self._accumulate(roots, g0, {}, inner, lambda t: f"s_cols[g_cmap{ci}[g * {ns} + {slot_of[t]}]]",
                             lambda j, i: pw_at(f"g_pmap{ci}[g * {nc} + {j}]"))
            body.append("#pragma unroll 1")
            body.append(f"for (int g = 0; g < {m}; g++) {{")
            body += ["  " + x for x in inner]
            body.append("}")
        body, flat = _split_flat(body)
        nc = max(self.n_cols, 1)
        threads = rows_per_iter = 128
        lines = [
            "// Generated from a constraint-framework component by stwo_gb300/codegen.py.",
        ] + ([FAST_COMPILE_MARK] if flat else []) + [
            '#include "codegen_rt.cuh"',
            "using namespace stwo;",
            "typedef unsigned short uint16_t;",
            "__device__ __forceinline__ uint4 gen_ldg_u4(const uint32_t* p, int i) {",
            "  return __ldg(reinterpret_cast<const uint4*>(p) + i);",
            "}",
            "// Launch shape read by the library: threads per block, rows per block and iteration.",
            f'extern "C" __constant__ uint32_t stwo_generated_layout[2] = {{{threads}, {rows_per_iter}}};',
        ] + self.tables + [
            f'extern "C" __global__ void __launch_bounds__({threads}) stwo_generated_constraints(const GenArgs a) {{',
            f"  __shared__ const uint32_t* s_cols[{nc}];",
            f"  for (int i = threadIdx.x; i < {self.n_cols}; i += blockDim.x) s_cols[i] = a.cols[i];",
        ]
        if smem_pw:
            lines += [f"  __shared__ uint4 s_pw[{max(n_cons, 1)}];",
                      f"  for (int i = threadIdx.x; i < {n_cons}; i += blockDim.x) s_pw[i] = gen_ldg_u4(a.powers, i);"]
        lines += ["  __syncthreads();"]
        lines += ["  " + x for x in self.pre]
        offs = [f"const uint32_t {rv} = gen_offset_row(row, a.trace_log, a.eval_log, {off});"
                for off, rv in self.offsets.items() if off != 0]
        finish_row = [
            "rr = qm31_mul_m31(rr, __ldg(a.dinv + (row >> a.trace_log)));",
            "a.acc0[row] = m31_add(a.acc0[row], rr.a.a);",
            "a.acc1[row] = m31_add(a.acc1[row], rr.a.b);",
            "a.acc2[row] = m31_add(a.acc2[row], rr.b.a);",
            "a.acc3[row] = m31_add(a.acc3[row], rr.b.b);",
        ]
        reduce_acc = [
            "qm31 rr = qm31_add(qm31_from_u32(m31_reduce64(acc[0]), m31_reduce64(acc[1]), m31_reduce64(acc[2]),",
            "                                 m31_reduce64(acc[3])), qacc);",
        ]
        lines += ["  const uint32_t n_rows = 1u << a.eval_log;"]
        lines += [
            "  for (uint32_t row = blockIdx.x * blockDim.x + threadIdx.x; row < n_rows; row += gridDim.x * blockDim.x) {",
            "    uint64_t acc[4] = {0ull, 0ull, 0ull, 0ull};",
            "    qm31 qacc = qm31_zero();",
        ]
        lines += ["    " + x for x in offs]
        lines += ["    " + x for x in body]
        lines += ["    " + x for x in reduce_acc]
        lines += ["    " + x for x in finish_row]
        lines += ["  }", "}"]
        return "\n".join(lines) + "\n"


class _FracGen(_Gen):
    """The interaction trace of a component's LogUp relations (LogupTraceGenerator,
    crates/prover/src/constraint_framework/logup.rs:123-260): per row of the trace domain, the
    value num_b / den_b of each batch fraction that finalize_logup_batched formed, accumulated
    across the batches, written as four coordinate columns per batch. The library then finalises
    the last column (claimed sum, shift, prefix sum in coset order)."""

    def source(self) -> str:
        ev = self.ev
        assert ev.logup_batches, "the component has no LogUp relation"
        self.n_cols = len(ev.mask[0]) + len(ev.mask[1])
        roots = []
        for f in ev.logup_batches:
            roots += [self.resolve(X._as_ext(f.numerator).simplify()), self.resolve(X._as_ext(f.denominator).simplify())]
        nodes = self._topo(roots)
        self.uniform = {}
        for n in nodes:
            if n.kind == "col":
                assert n.val.interaction in (0, 1) and n.val.offset == 0, \
                    "relation entries read trace columns of the current row only"
                self.uniform[n.uid] = False
            elif n.kind in ("const", "param"):
                self.uniform[n.uid] = True
            else:
                self.uniform[n.uid] = all(self.uniform[a.uid] for a in n.args)
        body: List[str] = []
        memo: Dict = {}
        col = lambda t: f"s_cols[{t}]"  # noqa: E731
        body.append("qm31 prev = qm31_zero();")
        for b in range(len(ev.logup_batches)):
            num, den = (self._value(r, memo, body, col) for r in roots[2 * b:2 * b + 2])
            lift = lambda v: v[0] if v[1] == "q" else f"qm31_from_u32({v[0]}, 0u, 0u, 0u)"  # noqa: E731
            body.append(f"prev = qm31_add(prev, qm31_mul({lift(num)}, qm31_inv({lift(den)})));")
            for j, c in enumerate(("prev.a.a", "prev.a.b", "prev.b.a", "prev.b.b")):
                body.append(f"a.acc0[(size_t){4 * b + j} * n_rows + row] = {c};")
        body, flat = _split_flat(body)
        nc = max(self.n_cols, 1)
        lines = [
            "// Generated from a constraint-framework component by stwo_gb300/codegen.py.",
        ] + ([FAST_COMPILE_MARK] if flat else []) + [
            '#include "codegen_rt.cuh"',
            "using namespace stwo;",
            'extern "C" __constant__ uint32_t stwo_generated_layout[2] = {128, 128};',
            'extern "C" __global__ void __launch_bounds__(128) stwo_generated_fractions(const GenArgs a) {',
            f"  __shared__ const uint32_t* s_cols[{nc}];",
            f"  for (int i = threadIdx.x; i < {self.n_cols}; i += blockDim.x) s_cols[i] = a.cols[i];",
            "  __syncthreads();",
        ]
        lines += ["  " + x for x in self.pre]
        lines += [
            "  const uint32_t n_rows = 1u << a.eval_log;",
            "  for (uint32_t row = blockIdx.x * blockDim.x + threadIdx.x; row < n_rows; row += gridDim.x * blockDim.x) {",
        ]
        lines += ["    " + x for x in body]
        lines += ["  }", "}"]
        return "\n".join(lines) + "\n"


def generate_fractions(ev: ExprEvaluator) -> Tuple[str, List[Tuple[str, bool]]]:
    """CUDA source of the interaction-trace kernel of a recorded component and its parameters."""
    g = _FracGen(ev)
    src = g.source()
    return src, g.params


def generate(ev: ExprEvaluator) -> Tuple[str, List[Tuple[str, bool]]]:
    """CUDA source of the constraint kernel of a recorded component, and its external parameters
    (name, is_extension) in the order the kernel reads them."""
    g = _Gen(ev)
    src = g.source()
    return src, g.params


_CACHE: Dict[str, int] = {}  # source digest -> compiled component handle (process lifetime)
# Compiled kernels persist across processes here (the package's build directory), keyed by the
# digest of the source and the component's sizes.
CUBIN_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "codegen_cache")


def _compiled(source: str, sizes: Tuple[int, int, int], load: bool = True) -> int:
    """A compiled component handle for `source`: from this process's cache, the cubin cache on
    disk, or NVRTC."""
    from . import _lib

    key = hashlib.sha256(source.encode() + repr(sizes).encode() + _runtime_headers() + NVRTC_FLAGS).hexdigest()
    h = _CACHE.get(key)
    if h is None:
        out = C.c_void_p()
        path = os.path.join(CUBIN_CACHE, key + ".cubin")
        if os.path.exists(path):
            blob = open(path, "rb").read()
            _lib.call("stwo_codegen_from_cubin", blob, len(blob), *sizes, 1 if load else 0, C.byref(out))
        else:
            _lib.call("stwo_codegen_compile", source.encode(), *sizes, 1 if load else 0, C.byref(out))
            _store_cubin(out.value, path)
        h = _CACHE[key] = out.value
    return h


def _runtime_headers() -> bytes:
    """The text the library compiles generated kernels against (part of the cache key)."""
    csrc = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc")
    return b"".join(open(os.path.join(csrc, n), "rb").read() for n in ("field.cuh", "codegen_rt.cuh"))


def _store_cubin(handle: int, path: str) -> None:
    from . import _lib

    size = C.c_size_t()
    _lib.call("stwo_codegen_cubin", handle, None, 0, C.byref(size))
    buf = C.create_string_buffer(size.value)
    _lib.call("stwo_codegen_cubin", handle, buf, size.value, C.byref(size))
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + f".{os.getpid()}.tmp"
    with open(tmp, "wb") as f:
        f.write(buf.raw)
    os.replace(tmp, path)


def _point_program(ev: ExprEvaluator):
    """The component's constraints at a point as a program for stwo_point_program_eval: the
    intermediates in definition order, then the constraints, each node one op. Returns the program
    (uint32 words) and its inputs, in order: ("mask", interaction, local column, offset index),
    ("param", name) or ("const", QM31). A relation entry's alpha powers are consecutive inputs."""
    inputs: List[tuple] = []
    index: Dict[tuple, int] = {}
    ops: List[List[tuple]] = []  # each op: its words, operands as ("i", input) or ("o", op)
    ref: Dict[int, tuple] = {}
    inter: Dict[str, tuple] = {}

    def inp(key) -> tuple:
        if key not in index:
            index[key] = len(inputs)
            inputs.append(key)
        return ("i", index[key])

    def leaf(n: Expr) -> tuple:
        if n.kind == "col":
            c = n.val
            return inp(("mask", c.interaction, c.local, ev.mask[c.interaction][c.local].index(c.offset)))
        if n.kind == "const":
            v = n.val
            return inp(("const", (v % X.P, 0, 0, 0) if isinstance(v, int) else tuple(v)))
        name = n.val
        if name in inter:
            return inter[name]
        if name in ev.preprocessed:
            return inp(("mask", 0, ev.preprocessed.index(name), 0))
        return inp(("param", name))

    def emit(root: Expr) -> tuple:
        stack = [root]
        while stack:
            n = stack[-1]
            if n.uid in ref:
                stack.pop()
                continue
            if n.kind in ("col", "const", "param"):
                ref[n.uid] = leaf(n)
                stack.pop()
                continue
            pending = [a for a in n.args if a.uid not in ref]
            if pending:
                stack.extend(pending)
                continue
            stack.pop()
            args = [ref[x.uid] for x in n.args]
            k = n.kind
            if k == "combine":
                rel, size = n.val
                first = ("param", f"{rel}_alpha0")
                if first not in index:
                    for i in range(size):
                        inp(("param", f"{rel}_alpha{i}"))
                k0 = index[first]
                assert all(index.get(("param", f"{rel}_alpha{i}")) == k0 + i for i in range(size)), rel
                words = [7, len(args), ("a", k0), inp(("param", f"{rel}_z"))] + args
            else:
                words = [{"add": 1, "sub": 2, "mul": 3, "neg": 4, "inv": 5, "secure_col": 6}[k]] + args
            ops.append(words)
            ref[n.uid] = ("o", len(ops) - 1)
        return ref[root.uid]

    for name in ev.ordered_intermediates:
        inter[name] = emit(ev.intermediate(name))
    outs = [emit(c) for c in ev.constraints]
    n_in = len(inputs)

    def word(w):
        if isinstance(w, int):
            return w
        kind, k = w
        return k if kind in ("i", "a") else n_in + k

    prog = [len(ops)] + [word(w) for op in ops for w in op] + [len(outs)] + [word(o) for o in outs]
    return (C.c_uint32 * len(prog))(*prog), len(prog), inputs


# Recorded components by the AIR's shape_key(): the expressions, the kernel source and handle, and
# the interaction kernel, shared by every component of that shape (the recording does not depend on
# the log size, the relation elements or the claimed sum, which reach the kernels as parameters).
_RECORDED: Dict[tuple, dict] = {}


class GeneratedComponent:
    """A FrameworkEval-like object (`log_size`, `max_constraint_log_degree_bound`, `evaluate`,
    `params`) with its generated constraint kernel."""

    def __init__(self, air, load: bool = True):
        self.air = air
        key = air.shape_key() if hasattr(air, "shape_key") else None
        rec = _RECORDED.get((key, load)) if key is not None else None
        if rec is None:
            ev = air.evaluate(ExprEvaluator())
            source, names = generate(ev)
            n_cols = sum(len(m) for m in ev.mask)
            rec = {"ev": ev, "source": source, "names": names, "n_cols": n_cols, "n_constraints": len(ev.constraints),
                   "load": load, "handle": None, "frac": None}
            if key is not None:
                _RECORDED[(key, load)] = rec
        self._rec = rec
        self.ev, self.source, self.param_names = rec["ev"], rec["source"], rec["names"]
        self.n_cols, self.n_constraints = rec["n_cols"], rec["n_constraints"]

    @property
    def handle(self) -> int:
        """The compiled constraint kernel, compiled (or loaded from the cubin cache) on first use."""
        rec = self._rec
        if rec["handle"] is None:
            rec["handle"] = _compiled(rec["source"], (rec["n_cols"], len(rec["names"]), rec["n_constraints"]),
                                      rec["load"])
        return rec["handle"]

    def log_size(self) -> int:
        return self.air.log_size()

    def max_constraint_log_degree_bound(self) -> int:
        return self.air.max_constraint_log_degree_bound()

    def mask(self) -> List[List[List[int]]]:
        return self.ev.mask

    def param_values(self, params: Dict[str, object] = None, names=None):
        from ._lib import QM31

        names = self.param_names if names is None else names
        vals = dict(self.air.params())
        if params:
            vals.update(params)
        arr = (QM31 * max(len(names), 1))()
        for i, (name, _) in enumerate(names):
            v = vals[name]
            arr[i] = QM31(tuple(v) if not isinstance(v, int) else (v % X.P, 0, 0, 0))
        return arr

    def eval_constraints(self, cols: Sequence[int], coeff_powers, accum4: Sequence[int], stream=None,
                         params: Dict[str, object] = None) -> None:
        """stwo_eval_constraints_codegen: `cols` are device addresses of the columns on the
        evaluation domain (interaction 0, 1, 2 in mask order), `coeff_powers` the accumulator's
        QM31 slice, `accum4` the four coordinate columns."""
        from . import _lib

        n = len(cols)
        tab = (C.c_void_p * max(n, 1))(*cols)
        acc = (C.c_void_p * 4)(*accum4)
        _lib.call("stwo_eval_constraints_codegen", self.handle, self.log_size(),
                  self.max_constraint_log_degree_bound(), tab, n, self.param_values(params),
                  len(self.param_names), coeff_powers, self.n_constraints, acc, stream)

    def n_interaction_columns(self) -> int:
        return 4 * len(self.ev.logup_batches)

    def interaction(self, cols: Sequence[int], out: int, stream=None, params: Dict[str, object] = None) -> X.Q:
        """The LogUp interaction trace (stwo_logup_interaction_codegen): `cols` are device
        addresses of the preprocessed then trace columns on the trace domain, `out` a device block
        of n_interaction_columns() columns of 2^log_size words. Returns the claimed sum; the
        relation elements come from the AIR's params (its claimed sum is not read)."""
        from . import _lib
        from ._lib import QM31

        if self._rec["frac"] is None:
            src, names = generate_fractions(self.ev)
            n_in = len(self.ev.mask[0]) + len(self.ev.mask[1])
            self._rec["frac"] = (_compiled(src, (n_in, len(names), len(self.ev.logup_batches))), names, n_in)
        h, names, n_in = self._rec["frac"]
        vals = dict(params or {})
        vals.setdefault("claimed_sum", (0, 0, 0, 0))
        tab = (C.c_void_p * max(len(cols), 1))(*cols)
        cs = QM31()
        _lib.call("stwo_logup_interaction_codegen", h, self.log_size(), tab, len(cols),
                  self.param_values(vals, names), len(names), out, C.byref(cs), stream)
        return tuple(cs.v)

    def eval_at_point(self, mask_values: Sequence[Sequence[Sequence[X.Q]]], rc: X.Q, denom_inv: X.Q,
                      params: Dict[str, object] = None, acc: X.Q = (0, 0, 0, 0)) -> X.Q:
        """PointEvaluator (constraint_framework/point.rs:15-70): acc = acc * rc + denom_inv * c
        for every constraint in order, by the library on the host (stwo_point_program_eval, from
        the component's recorded expressions). `mask_values[interaction][local column][offset
        index]` are the sampled values; preprocessed columns are interaction 0 in request order."""
        vals = dict(self.air.params())
        if params:
            vals.update(params)
        vals = {k: ((v % X.P, 0, 0, 0) if isinstance(v, int) else tuple(v)) for k, v in vals.items()}
        from . import _lib
        from ._lib import QM31

        prog = self._rec.get("point")
        if prog is None:
            prog = self._rec["point"] = _point_program(self.ev)
        words, n_words, inputs = prog
        arr = (QM31 * max(len(inputs), 1))()
        for i, key in enumerate(inputs):
            if key[0] == "mask":
                arr[i] = QM31(tuple(mask_values[key[1]][key[2]][key[3]]))
            elif key[0] == "param":
                arr[i] = QM31(vals[key[1]])
            else:
                arr[i] = QM31(key[1])
        out = QM31(tuple(acc))
        _lib.call("stwo_point_program_eval", words, n_words, arr, len(inputs), QM31(tuple(rc)), QM31(tuple(denom_inv)),
                  C.byref(out))
        return tuple(out.v)
