"""prove() of the reference driven through the per-operation C ABI, as a Rust
`prove::<CudaBackend, Blake2sMerkleChannel>` over the backend traits would drive it.

Every O(trace) step is one backend entry point (interpolate, evaluate, commit_on_layer,
eval_at_points, accumulate_quotients, fold_circle_into_line, fold_line, grind,
generate_secure_powers, and the per-component stwo_eval_constraints); device memory comes only from
the column model (stwo_buf_alloc / upload / download / zero / read_words). What stays here is what
the reference keeps on its host: the Blake2s channel, the Merkle decommitment walk, the query
positions, the last FRI layer's interpolation and the out-of-domain constraint check.

Restated from (file:line of the reference):
  prove                  crates/prover/src/core/prover/mod.rs:27-79
  CommitmentSchemeProver crates/prover/src/core/pcs/prover.rs:25-243
  compute_fri_quotients  crates/prover/src/core/pcs/quotients.rs:49-101
  FriProver              crates/prover/src/core/fri.rs:168-336, :943-976
  MerkleProver           crates/prover/src/core/vcs/prover.rs:13-154
  Blake2sChannel         crates/prover/src/core/channel/blake2s.rs:15-110
  Queries                crates/prover/src/core/queries.rs:21-52
  DomainEvaluationAccumulator crates/prover/src/core/air/accumulation.rs:49-149
The proof bytes use the canonical form of the fused provers (little-endian u32 words, u64
lengths, fields in StarkProof order), so the three routes can be compared byte for byte.

This module drives the wide-Fibonacci AIR (crates/prover/src/examples/wide_fibonacci/mod.rs), whose
trace the device generates (stwo_gen_wide_fib_trace).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import struct
from typing import Dict, List, Sequence, Tuple

from . import _lib
from ._lib import Coset, QM31, QM31Point, SampleBatch, call
from .circle import canonic_half_coset, double, half_odds

P = (1 << 31) - 1
Q = Tuple[int, int, int, int]


# ------------------------------------------------------------------ host field arithmetic
def _cm_mul(a, b):
    return ((a[0] * b[0] - a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)


def q_add(a: Q, b: Q) -> Q:
    return tuple((x + y) % P for x, y in zip(a, b))


def q_sub(a: Q, b: Q) -> Q:
    return tuple((x - y) % P for x, y in zip(a, b))


def q_mul(a: Q, b: Q) -> Q:
    # (x + y u)(z + w u) = (xz + (2 + i) yw) + (xw + yz) u, u^2 = 2 + i (fields/qm31.rs:21-95)
    x, y, z, w = (a[0], a[1]), (a[2], a[3]), (b[0], b[1]), (b[2], b[3])
    xz, yw = _cm_mul(x, z), _cm_mul(y, w)
    r_yw = _cm_mul((2, 1), yw)
    xw, yz = _cm_mul(x, w), _cm_mul(y, z)
    return ((xz[0] + r_yw[0]) % P, (xz[1] + r_yw[1]) % P, (xw[0] + yz[0]) % P, (xw[1] + yz[1]) % P)


def q_inv(a: Q) -> Q:
    x, y = (a[0], a[1]), (a[2], a[3])
    yy = _cm_mul((2, 1), _cm_mul(y, y))
    den = ((_cm_mul(x, x)[0] - yy[0]) % P, (_cm_mul(x, x)[1] - yy[1]) % P)
    n = (den[0] * den[0] + den[1] * den[1]) % P
    ni = pow(n, P - 2, P)
    di = (den[0] * ni % P, (-den[1]) * ni % P)
    r0, r1 = _cm_mul(x, di), _cm_mul(((-y[0]) % P, (-y[1]) % P), di)
    return (r0[0], r0[1], r1[0], r1[1])


def q_m31(a: int) -> Q:
    return (a % P, 0, 0, 0)


# Circle points over M31: M31_CIRCLE_GEN (crates/prover/src/core/circle.rs:203-206), order 2^31.
_GEN = (2, 1268011823)


def _pt_add(p, q):
    return ((p[0] * q[0] - p[1] * q[1]) % P, (p[0] * q[1] + p[1] * q[0]) % P)


def index_to_point(index: int):
    r, g, i = (1, 0), _GEN, index & ((1 << 31) - 1)
    while i:
        if i & 1:
            r = _pt_add(r, g)
        g = _pt_add(g, g)
        i >>= 1
    return r


def _coset_vanishing(coset: Coset, px: Q, py: Q) -> Q:
    """coset_vanishing (crates/prover/src/core/constraints.rs:11-30) at a QM31 point."""
    init = index_to_point(coset.initial_index)
    half = index_to_point(coset.step_size >> 1)
    # p - initial + step/2, then log_size - 1 doublings of x.
    shift = _pt_add((init[0], (-init[1]) % P), half)
    x = q_sub(q_mul(px, q_m31(shift[0])), q_mul(py, q_m31(shift[1])))
    for _ in range(1, coset.log_size):
        x = q_sub(q_add(q_mul(x, x), q_mul(x, x)), q_m31(1))
    return x


# ------------------------------------------------------------------ Blake2s channel
_IV = [0x6A09E667, 0xBB67AE85, 0x3C6EF372, 0xA54FF53A, 0x510E527F, 0x9B05688C, 0x1F83D9AB, 0x5BE0CD19]
_SIGMA = [
    [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15], [14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3],
    [11, 8, 12, 0, 5, 2, 15, 13, 10, 14, 3, 6, 7, 1, 9, 4], [7, 9, 3, 1, 13, 12, 11, 14, 2, 6, 5, 10, 4, 0, 15, 8],
    [9, 0, 5, 7, 2, 4, 10, 15, 14, 1, 11, 12, 6, 8, 3, 13], [2, 12, 6, 10, 0, 11, 8, 3, 4, 13, 7, 5, 15, 14, 1, 9],
    [12, 5, 1, 15, 14, 13, 4, 10, 0, 7, 6, 3, 9, 2, 8, 11], [13, 11, 7, 14, 12, 1, 3, 9, 5, 0, 15, 4, 8, 6, 2, 10],
    [6, 15, 14, 9, 11, 3, 0, 8, 12, 2, 13, 7, 1, 4, 10, 5], [10, 2, 8, 4, 7, 6, 1, 5, 15, 11, 9, 14, 3, 12, 13, 0],
]


def blake2s_compress(h: Sequence[int], m: Sequence[int], t0=0, t1=0, f0=0, f1=0) -> List[int]:
    """The raw Blake2s compression function (RFC 7693 section 3.2), as the reference's
    crates/prover/src/core/vcs/blake2s_ref.rs:168-217 uses it for mix_u64."""
    M = 0xFFFFFFFF
    v = list(h) + _IV[:4] + [_IV[4] ^ t0, _IV[5] ^ t1, _IV[6] ^ f0, _IV[7] ^ f1]

    def rot(x, n):
        return ((x >> n) | (x << (32 - n))) & M

    def g(a, b, c, d, x, y):
        v[a] = (v[a] + v[b] + x) & M
        v[d] = rot(v[d] ^ v[a], 16)
        v[c] = (v[c] + v[d]) & M
        v[b] = rot(v[b] ^ v[c], 12)
        v[a] = (v[a] + v[b] + y) & M
        v[d] = rot(v[d] ^ v[a], 8)
        v[c] = (v[c] + v[d]) & M
        v[b] = rot(v[b] ^ v[c], 7)

    for r in range(10):
        s = _SIGMA[r]
        g(0, 4, 8, 12, m[s[0]], m[s[1]])
        g(1, 5, 9, 13, m[s[2]], m[s[3]])
        g(2, 6, 10, 14, m[s[4]], m[s[5]])
        g(3, 7, 11, 15, m[s[6]], m[s[7]])
        g(0, 5, 10, 15, m[s[8]], m[s[9]])
        g(1, 6, 11, 12, m[s[10]], m[s[11]])
        g(2, 7, 8, 13, m[s[12]], m[s[13]])
        g(3, 4, 9, 14, m[s[14]], m[s[15]])
    return [h[i] ^ v[i] ^ v[i + 8] for i in range(8)]


def _b2s(data: bytes) -> bytes:
    return hashlib.blake2s(data, digest_size=32).digest()


class Blake2sChannel:
    """Blake2sChannel (crates/prover/src/core/channel/blake2s.rs:15-110)."""

    def __init__(self):
        self.digest = bytes(32)
        self.n_sent = 0

    def _update(self, d: bytes):
        self.digest = d
        self.n_sent = 0

    def words(self) -> List[int]:
        return list(struct.unpack("<8I", self.digest))

    def mix_root(self, root: bytes):
        self._update(_b2s(self.digest + root))

    def mix_felts(self, felts: Sequence[Q]):
        self._update(_b2s(self.digest + b"".join(struct.pack("<4I", *f) for f in felts)))

    def mix_u64(self, v: int):
        m = [v & 0xFFFFFFFF, v >> 32] + [0] * 14
        self._update(struct.pack("<8I", *blake2s_compress(self.words(), m)))

    def draw_random_bytes(self) -> bytes:
        out = _b2s(self.digest + struct.pack("<Q", self.n_sent) + bytes(24))
        self.n_sent += 1
        return out

    def draw_base_felts(self) -> List[int]:
        while True:
            w = struct.unpack("<8I", self.draw_random_bytes())
            if all(x < 2 * P for x in w):
                return [x - P if x >= P else x for x in w]

    def draw_felt(self) -> Q:
        return tuple(self.draw_base_felts()[:4])

    def draw_felts(self, n: int) -> List[Q]:
        out: List[Q] = []
        while len(out) < n:
            f = self.draw_base_felts()
            out.append(tuple(f[:4]))
            if len(out) < n:
                out.append(tuple(f[4:]))
        return out

    def random_point(self) -> Tuple[Q, Q]:
        """CirclePoint::get_random_point (crates/prover/src/core/circle.rs:170-183)."""
        t = self.draw_felt()
        t2 = q_mul(t, t)
        d = q_inv(q_add(t2, q_m31(1)))
        return q_mul(q_sub(q_m31(1), t2), d), q_mul(q_add(t, t), d)


# ------------------------------------------------------------------ device columns
class Buf:
    """A device column from the column model (Column::zeros / uninitialized / at / to_cpu)."""

    def __init__(self, n_words: int, zero: bool = False):
        self.n = n_words
        p = C.c_void_p()
        call("stwo_buf_alloc", C.byref(p), max(n_words, 1) * 4, None)
        self.ptr = p.value
        if zero:
            call("stwo_buf_zero", self.ptr, n_words * 4, None)

    @classmethod
    def view(cls, owner: "Buf", word_offset: int, n_words: int) -> "Buf":
        """Words [word_offset, word_offset + n_words) of `owner`, which stays allocated while the
        view lives (the view frees nothing)."""
        v = cls.__new__(cls)
        v.n, v.ptr, v.owner = n_words, owner.ptr + 4 * word_offset, owner
        return v

    def __del__(self):
        if getattr(self, "owner", None) is not None:
            return
        try:
            _lib.load().stwo_buf_free(self.ptr, None)
        except Exception:
            pass

    def upload(self, words: Sequence[int]):
        arr = (C.c_uint32 * len(words))(*words)
        call("stwo_buf_upload", self.ptr, arr, len(words) * 4, None)

    def download(self) -> List[int]:
        arr = (C.c_uint32 * self.n)()
        call("stwo_buf_download", arr, self.ptr, self.n * 4, None)
        return list(arr)

    def at(self, idx: Sequence[int]) -> List[int]:
        if not idx:
            return []
        ia = (C.c_uint64 * len(idx))(*idx)
        out = (C.c_uint32 * len(idx))()
        call("stwo_read_words", self.ptr, ia, len(idx), out, None)
        return list(out)


def _read_cols(cols: Sequence[Buf], idx: Sequence[int]) -> List[List[int]]:
    """Column::at of the same indices in every column, one transfer (stwo_read_words_cols)."""
    if not cols or not idx:
        return [[] for _ in cols]
    n = len(idx)
    out = (C.c_uint32 * (len(cols) * n))()
    call("stwo_read_words_cols", _ptrs(cols), len(cols), (C.c_uint64 * n)(*idx), n, out, None)
    flat = list(out)
    return [flat[c * n:(c + 1) * n] for c in range(len(cols))]


def _block_views(sizes: Sequence[int]) -> List[Buf]:
    """Columns of the given word counts as views of one device block: one allocation for a tree's
    or a component's columns instead of one per column."""
    if not sizes:
        return []
    block = Buf(sum(sizes))
    out, at = [], 0
    for n in sizes:
        out.append(Buf.view(block, at, n))
        at += n
    return out


def _ptrs(bufs: Sequence[Buf]):
    return (C.c_void_p * max(1, len(bufs)))(*[b.ptr for b in bufs])


def _ptr4(bufs: Sequence[Buf]):
    return (C.c_void_p * 4)(*[b.ptr for b in bufs])


def _log2(n: int) -> int:
    return n.bit_length() - 1


class SecureCol:
    """SecureColumnByCoords: four coordinate columns."""

    def __init__(self, n: int, zero: bool = True, cols: Sequence[Buf] = None):
        self.cols = list(cols) if cols is not None else [Buf(n, zero) for _ in range(4)]
        self.n = n

    def at(self, idx: Sequence[int]) -> List[Q]:
        c = _read_cols(self.cols, idx)
        return [(c[0][i], c[1][i], c[2][i], c[3][i]) for i in range(len(idx))]


# ------------------------------------------------------------------ Merkle tree (vcs/prover.rs)
class MerkleTree:
    def __init__(self, columns: Sequence[Buf]):
        cols = sorted(columns, key=lambda c: -c.n)  # stable: equal sizes keep their order
        self.cols = cols
        max_log = _log2(cols[0].n) if cols else 0
        self.layers: Dict[int, Buf] = {}
        prev = None
        ci = 0
        for log in range(max_log, -1, -1):
            lc = []
            while ci < len(cols) and _log2(cols[ci].n) == log:
                lc.append(cols[ci])
                ci += 1
            out = Buf(8 << log)
            call("stwo_merkle_commit_layer", log, prev.ptr if prev else None, _ptrs(lc), len(lc), out.ptr, None)
            self.layers[log] = out
            prev = out
        self.max_log = max_log

    def root(self) -> bytes:
        return struct.pack("<8I", *self.layers[0].download())

    def _hashes(self, log: int, nodes: Sequence[int]) -> List[bytes]:
        w = self.layers[log].at([8 * n + k for n in nodes for k in range(8)])
        return [struct.pack("<8I", *w[8 * i:8 * i + 8]) for i in range(len(nodes))]

    def decommit(self, queries_per_log: Dict[int, List[int]]):
        """MerkleProver::decommit (vcs/prover.rs:80-149): (queried values, hash witness, column witness)."""
        queried, hash_witness, col_witness = [], [], []
        ci = 0
        last: List[int] = []
        for log in range(self.max_log, -1, -1):
            lc = []
            while ci < len(self.cols) and _log2(self.cols[ci].n) == log:
                lc.append(self.cols[ci])
                ci += 1
            cq = queries_per_log.get(log, [])
            has_prev = log + 1 <= self.max_log
            pi = qi = 0
            total = []
            wants = []  # (kind, node) in proof order: hash witness nodes of the layer below, values
            while True:
                cand = []
                if pi < len(last):
                    cand.append(last[pi] // 2)
                if qi < len(cq):
                    cand.append(cq[qi])
                if not cand:
                    break
                node = min(cand)
                if has_prev:
                    for child in (2 * node, 2 * node + 1):
                        if pi < len(last) and last[pi] == child:
                            pi += 1
                        else:
                            wants.append(("h", child))
                q = qi < len(cq) and cq[qi] == node
                if q:
                    qi += 1
                wants.append(("q" if q else "w", node))
                total.append(node)
            hnodes = [n for k, n in wants if k == "h"]
            hashes = dict(zip(hnodes, self._hashes(log + 1, hnodes))) if hnodes else {}
            vnodes = [n for k, n in wants if k != "h"]
            vals = _read_cols(lc, vnodes)
            vi = 0
            for kind, node in wants:
                if kind == "h":
                    hash_witness.append(hashes[node])
                else:
                    row = [vals[c][vi] for c in range(len(lc))]
                    (queried if kind == "q" else col_witness).extend(row)
                    vi += 1
            last = total
        return queried, hash_witness, col_witness


# ------------------------------------------------------------------ commitment scheme
class CommitmentTree:
    def __init__(self, polys: Sequence[Buf], evals: Sequence[Buf]):
        self.polys, self.evals = list(polys), list(evals)
        self.tree = MerkleTree(self.evals)


class CommitmentSchemeProver:
    def __init__(self, cfg: Tuple[int, int, int, int], max_log: int):
        self.pow_bits, self.log_blowup, self.log_last_layer, self.n_queries = cfg
        tw = C.c_void_p()
        call("stwo_twiddles_precompute", canonic_half_coset(max_log), C.byref(tw), None)
        self.tw = tw.value
        self.trees: List[CommitmentTree] = []

    def __del__(self):
        try:
            _lib.load().stwo_twiddles_free(self.tw)
        except Exception:
            pass

    def commit_polys(self, polys: Sequence[Buf], ch: Blake2sChannel):
        """TreeBuilder::extend_polys + commit (pcs/prover.rs:208-227)."""
        evals = _block_views([p.n << self.log_blowup for p in polys])
        by_log: Dict[int, List[int]] = {}
        for i, p in enumerate(polys):
            by_log.setdefault(_log2(p.n), []).append(i)
        for log in sorted(by_log):
            idx = by_log[log]
            call("stwo_evaluate_columns", self.tw, canonic_half_coset(log + self.log_blowup),
                 _ptrs([polys[i] for i in idx]), log, _ptrs([evals[i] for i in idx]), len(idx), None)
        t = CommitmentTree(polys, evals)
        ch.mix_root(t.tree.root())
        self.trees.append(t)

    def commit_evals(self, evals: Sequence[Buf], log_size: int, ch: Blake2sChannel):
        """TreeBuilder::extend_evals: the evaluations are interpolated in place (consumed)."""
        if evals:
            call("stwo_interpolate_columns", self.tw, canonic_half_coset(log_size), _ptrs(evals), len(evals), None)
        self.commit_polys(evals, ch)


def _pt_key(pt):
    return tuple(pt[0]) + tuple(pt[1])


def _accumulate_quotients(log: int, cols: Sequence[Buf], samples, rc: Q, log_blowup: int) -> SecureCol:
    """compute_fri_quotients for one log size (pcs/quotients.rs:49-101): ColumnSampleBatches grouped by
    point in CirclePoint's derived order, then QuotientOps::accumulate_quotients."""
    groups: Dict[tuple, list] = {}
    pts = {}
    for ci, smp in enumerate(samples):
        for pt, v in smp:
            groups.setdefault(_pt_key(pt), []).append((ci, v))
            pts[_pt_key(pt)] = pt
    keep = []
    batches = (SampleBatch * max(1, len(groups)))()
    for bi, key in enumerate(sorted(groups)):
        pt = pts[key]
        idx = (C.c_uint32 * len(groups[key]))(*[c for c, _ in groups[key]])
        vals = (QM31 * len(groups[key]))(*[QM31(v) for _, v in groups[key]])
        keep += [idx, vals]
        batches[bi] = SampleBatch(QM31Point(QM31(pt[0]), QM31(pt[1])), len(groups[key]), idx, vals)
    out = SecureCol(1 << log, zero=False)
    call("stwo_accumulate_quotients", log, _ptrs(cols), len(cols), QM31(rc), batches, len(groups), log_blowup,
         _ptr4(out.cols), None)
    return out


# ------------------------------------------------------------------ FRI (fri.rs:168-336)
def _queries(ch: Blake2sChannel, log_size: int, n_queries: int) -> List[int]:
    """Queries::generate (queries.rs:21-40)."""
    qs, cnt, mask = set(), 0, (1 << log_size) - 1
    while True:
        for w in struct.unpack("<8I", ch.draw_random_bytes()):
            qs.add(w & mask)
            cnt += 1
            if cnt == n_queries:
                return sorted(qs)


def _fold_queries(q: List[int], n: int) -> List[int]:
    out = []
    for p in q:
        v = p >> n
        if not out or out[-1] != v:
            out.append(v)
    return out


def _positions_and_witness(col: SecureCol, queries: List[int]):
    """fri.rs:943-976: the cosets of 2 around each query; values not queried become witness."""
    positions, wpos = [], []
    i = 0
    while i < len(queries):
        start = (queries[i] >> 1) << 1
        j = i
        while j < len(queries) and (queries[j] >> 1) == (queries[i] >> 1):
            j += 1
        qset = set(queries[i:j])
        for pos in (start, start + 1):
            positions.append(pos)
            if pos not in qset:
                wpos.append(pos)
        i = j
    return positions, col.at(wpos)


def _line_interpolate(dom: Coset, values: List[Q]) -> List[Q]:
    """LineEvaluation::interpolate's inverse FFT (poly/line.rs), coefficients in bit-reversed order."""
    n = len(values)
    lg = _log2(n)
    v = [values[int(format(i, f"0{lg}b")[::-1], 2) if lg else 0] for i in range(n)]
    d = dom
    while (1 << d.log_size) > 1:
        size = 1 << d.log_size
        half = size // 2
        xs = [index_to_point(d.initial_index + i * d.step_size)[0] for i in range(half)]
        for c in range(0, n, size):
            for i in range(half):
                it = pow(xs[i], P - 2, P)
                a, b = v[c + i], v[c + half + i]
                v[c + i] = q_add(a, b)
                v[c + half + i] = q_mul(q_sub(a, b), q_m31(it))
        d = double(d)
    inv_n = pow(n, P - 2, P)
    return [q_mul(x, q_m31(inv_n)) for x in v]


def _bit_reverse(v: list) -> list:
    n = len(v)
    lg = _log2(n)
    return [v[int(format(i, f"0{lg}b")[::-1], 2) if lg else 0] for i in range(n)]


class FriProver:
    def __init__(self, pcs: CommitmentSchemeProver, ch: Blake2sChannel, columns: Sequence[SecureCol]):
        self.pcs = pcs
        self.columns = list(columns)
        self.logs = [_log2(c.n) for c in columns]
        assert all(a > b for a, b in zip(self.logs, self.logs[1:])), "column sizes not decreasing"
        self.first_tree = MerkleTree([b for c in columns for b in c.cols])
        ch.mix_root(self.first_tree.root())
        first_log = self.logs[0] - 1
        dom = half_odds(first_log)
        layer = SecureCol(1 << first_log, zero=True)
        alpha = ch.draw_felt()
        self._fold_circle(layer, 0, alpha)
        nxt = 1
        self.inner = []
        last_size = 1 << (pcs.log_last_layer + pcs.log_blowup)
        while layer.n > last_size:
            tree = MerkleTree(layer.cols)
            ch.mix_root(tree.root())
            alpha = ch.draw_felt()
            folded = SecureCol(layer.n // 2, zero=False)
            call("stwo_fri_fold_line", pcs.tw, dom, _ptr4(layer.cols), QM31(alpha), _ptr4(folded.cols), None)
            self.inner.append((layer, dom, tree))
            dom = double(dom)
            layer = folded
            if nxt < len(columns) and columns[nxt].n // 2 == layer.n:
                self._fold_circle(layer, nxt, alpha)
                nxt += 1
        assert nxt == len(columns), "not all FRI columns consumed"
        vals = layer.at(list(range(layer.n)))
        coeffs = _bit_reverse(_line_interpolate(dom, vals))
        bound = 1 << pcs.log_last_layer
        if any(c != (0, 0, 0, 0) for c in coeffs[bound:]):
            raise RuntimeError("FRI last layer: invalid degree")
        self.last_layer_poly = _bit_reverse(coeffs[:bound])
        ch.mix_felts(self.last_layer_poly)

    def _fold_circle(self, dst: SecureCol, ci: int, alpha: Q):
        call("stwo_fri_fold_circle_into_line", self.pcs.tw, canonic_half_coset(self.logs[ci]), _ptr4(dst.cols),
             _ptr4(self.columns[ci].cols), QM31(alpha), None)

    def decommit(self, ch: Blake2sChannel):
        max_log = self.logs[0]
        q = _queries(ch, max_log, self.pcs.n_queries)
        by_log = {l: _fold_queries(q, max_log - l) for l in sorted(set(self.logs))}
        first_witness, dpos = [], {}
        for c, col in enumerate(self.columns):
            pos, wit = _positions_and_witness(col, _fold_queries(q, max_log - self.logs[c]))
            first_witness += wit
            dpos[self.logs[c]] = pos
        _, hw, cw = self.first_tree.decommit(dpos)
        first = (first_witness, hw, cw, self.first_tree.root())
        inner = []
        lq = _fold_queries(q, 1)
        for layer, dom, tree in self.inner:
            pos, wit = _positions_and_witness(layer, lq)
            _, hw, cw = tree.decommit({dom.log_size: pos})
            inner.append((wit, hw, cw, tree.root()))
            lq = _fold_queries(lq, 1)
        return first, inner, by_log


# ------------------------------------------------------------------ serialisation
class _Writer:
    def __init__(self):
        self.b = bytearray()

    def u32(self, v):
        self.b += struct.pack("<I", v)

    def u64(self, v):
        self.b += struct.pack("<Q", v)

    def qs(self, v):
        self.u64(len(v))
        for x in v:
            self.b += struct.pack("<4I", *x)

    def ms(self, v):
        self.u64(len(v))
        for x in v:
            self.u32(x)

    def dec(self, hw, cw):
        self.u64(len(hw))
        for h in hw:
            self.b += h
        self.ms(cw)

    def layer(self, lp):
        wit, hw, cw, root = lp
        self.qs(wit)
        self.dec(hw, cw)
        self.b += root


# ------------------------------------------------------------------ prove()
STWO_AIR_WIDE_FIB = 0


def _component(log_n: int, n_cols: int):
    return _lib.Component(STWO_AIR_WIDE_FIB, log_n, n_cols, QM31((0, 0, 0, 0)), None, 0)


def _wide_fib_oods(log_n: int, n_cols: int, mask: List[Q], rc: Q, px: Q, py: Q) -> Q:
    """The wide-Fibonacci constraints at the OODS point (PointEvaluator, constraint_framework/point.rs),
    each times 1 / coset_vanishing(trace coset, point), accumulated as acc * rc + value."""
    from .circle import coset, subgroup_gen

    dinv = q_inv(_coset_vanishing(coset(subgroup_gen(log_n + 1), log_n), px, py))
    acc = (0, 0, 0, 0)
    a, b = mask[0], mask[1]
    for i in range(2, n_cols):
        c = mask[i]
        cons = q_sub(c, q_add(q_mul(a, a), q_mul(b, b)))
        acc = q_add(q_mul(acc, rc), q_mul(dinv, cons))
        a, b = b, c
    return acc


def prove_wide_fib(log_n: int, n_cols: int, d_a: int, d_b: int, cfg=(5, 1, 0, 3), generated: bool = False) -> bytes:
    """test_wide_fib_prove_with_blake (wide_fibonacci/mod.rs:174-227) over the per-operation ABI:
    the trace of 2^log_n rows is generated on the device from the per-row pairs at device
    addresses d_a, d_b; returns the canonical proof bytes. With `generated`, the component's
    constraints come from its recorded expressions instead of the hand-written kernel: the domain
    evaluation is the generated kernel (stwo_eval_constraints_codegen) and the out-of-domain check
    evaluates the same expressions at the point (PointEvaluator)."""
    pow_bits, log_blowup, log_last, n_queries = cfg
    pcs = CommitmentSchemeProver(cfg, log_n + 1 + log_blowup)
    ch = Blake2sChannel()
    # Preprocessed tree (empty), then the trace.
    pcs.commit_polys([], ch)
    trace = [Buf(1 << log_n) for _ in range(n_cols)]
    call("stwo_gen_wide_fib_trace", log_n, n_cols, d_a, d_b, _ptrs(trace), None)
    pcs.commit_evals(trace, log_n, ch)

    # Composition polynomial (air/components.rs:122-137, accumulation.rs:49-149).
    rc = ch.draw_felt()
    comp = _component(log_n, n_cols)
    n_cons, eval_log, n_trees = C.c_uint32(), C.c_uint32(), C.c_uint32()
    tree_cols = (C.c_uint32 * 3)()
    call("stwo_component_info", C.byref(comp), C.byref(n_cons), C.byref(eval_log), C.byref(n_trees), tree_cols)
    n_cons, eval_log = n_cons.value, eval_log.value
    powers = (QM31 * n_cons)()
    call("stwo_generate_secure_powers", QM31(rc), n_cons, powers, None)
    acc = SecureCol(1 << eval_log, zero=True)
    t = pcs.trees[1]
    if log_n + log_blowup == eval_log:
        cols = t.evals
    else:  # the component's "Extension" step (constraint_framework/component.rs:305-322)
        cols = [Buf(1 << eval_log) for _ in t.polys]
        call("stwo_evaluate_columns", pcs.tw, canonic_half_coset(eval_log), _ptrs(t.polys), log_n, _ptrs(cols),
             len(cols), None)
    gen = None
    if generated:
        from .airs import WideFibonacciEval
        from .codegen import GeneratedComponent

        gen = GeneratedComponent(WideFibonacciEval(log_n, n_cols))
        gen.eval_constraints([c.ptr for c in cols], powers, [c.ptr for c in acc.cols])
    else:
        call("stwo_eval_constraints", C.byref(comp), _ptrs(cols), len(cols), powers, n_cons, _ptr4(acc.cols), None)
    call("stwo_interpolate_columns", pcs.tw, canonic_half_coset(eval_log), _ptr4(acc.cols), 4, None)
    pcs.commit_polys(acc.cols, ch)

    # Out-of-domain sampling (prover/mod.rs:51-68) and prove_values (pcs/prover.rs:83-148).
    px, py = ch.random_point()
    points = [[], [[(px, py)]] * n_cols, [[(px, py)]] * 4]
    polys = [p for tr in pcs.trees for p in tr.polys]
    poly_of, pts = [], []
    k = 0
    for ti, tr in enumerate(pcs.trees):
        for ci in range(len(tr.polys)):
            for pt in points[ti][ci]:
                poly_of.append(k)
                pts.append(pt)
            k += 1
    out = (QM31 * len(pts))()
    logs = (C.c_uint32 * len(polys))(*[_log2(p.n) for p in polys])
    call("stwo_eval_at_points", _ptrs(polys), logs, len(polys), (C.c_uint32 * len(pts))(*poly_of),
         (QM31Point * len(pts))(*[QM31Point(QM31(x), QM31(y)) for x, y in pts]), len(pts), out, None)
    vals = [tuple(out[i].v) for i in range(len(pts))]
    sampled, vi = [], 0
    for ti, tr in enumerate(pcs.trees):
        tv = []
        for ci in range(len(tr.polys)):
            tv.append(vals[vi:vi + len(points[ti][ci])])
            vi += len(points[ti][ci])
        sampled.append(tv)
    ch.mix_felts([v for tv in sampled for cv in tv for v in cv])
    comp_vals = [cv[0] for cv in sampled[2]]
    comp_at = q_add(q_add(comp_vals[0], q_mul(comp_vals[1], (0, 1, 0, 0))),
                    q_add(q_mul(comp_vals[2], (0, 0, 1, 0)), q_mul(comp_vals[3], (0, 0, 0, 1))))
    if gen is not None:
        from .circle import coset, subgroup_gen

        dinv = q_inv(_coset_vanishing(coset(subgroup_gen(log_n + 1), log_n), px, py))
        want_at = gen.eval_at_point([[], sampled[1], []], rc, dinv)
    else:
        want_at = _wide_fib_oods(log_n, n_cols, [cv[0] for cv in sampled[1]], rc, px, py)
    if comp_at != want_at:
        raise RuntimeError("ConstraintsNotSatisfied")

    return _finish_proof(pcs, ch, points, sampled, cfg)


def _finish_proof(pcs: "CommitmentSchemeProver", ch: Blake2sChannel, points, sampled, cfg) -> bytes:
    """prove_values after the sampled values are mixed (pcs/prover.rs:104-148): FRI quotients,
    the FRI commitment, proof of work, decommitment, and the canonical proof bytes."""
    pow_bits, log_blowup, log_last, n_queries = cfg
    # FRI quotients, stable-sorted by descending log size.
    cols = []
    for ti, tr in enumerate(pcs.trees):
        for ci, e in enumerate(tr.evals):
            cols.append((e, [(pt, v) for pt, v in zip(points[ti][ci], sampled[ti][ci])]))
    cols.sort(key=lambda x: -x[0].n)
    qrc = ch.draw_felt()
    quotients = []
    i = 0
    while i < len(cols):
        j = i
        while j < len(cols) and cols[j][0].n == cols[i][0].n:
            j += 1
        quotients.append(_accumulate_quotients(_log2(cols[i][0].n), [c for c, _ in cols[i:j]],
                                               [s for _, s in cols[i:j]], qrc, log_blowup))
        i = j
    fri = FriProver(pcs, ch, quotients)
    nonce = C.c_uint64()
    call("stwo_grind_blake2s", (C.c_uint32 * 8)(*ch.words()), pow_bits, C.byref(nonce), None)
    ch.mix_u64(nonce.value)
    first, inner, by_log = fri.decommit(ch)
    decs, queried, roots = [], [], []
    for tr in pcs.trees:
        q, hw, cw = tr.tree.decommit(by_log)
        queried.append(q)
        decs.append((hw, cw))
        roots.append(tr.tree.root())

    w = _Writer()
    w.u32(pow_bits)
    w.u32(log_blowup)
    w.u32(log_last)
    w.u64(n_queries)
    w.u64(len(roots))
    for r in roots:
        w.b += r
    w.u64(len(sampled))
    for tv in sampled:
        w.u64(len(tv))
        for cv in tv:
            w.qs(cv)
    w.u64(len(decs))
    for hw, cw in decs:
        w.dec(hw, cw)
    w.u64(len(queried))
    for q in queried:
        w.ms(q)
    w.u64(nonce.value)
    w.layer(first)
    w.u64(len(inner))
    for lp in inner:
        w.layer(lp)
    w.qs(fri.last_layer_poly)
    return bytes(w.b)
