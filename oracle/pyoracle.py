"""ORACLE — test infrastructure only.

ctypes wrapper of oracle/_build/liboracle.so, the C++ restatement of the reference's CPU
algorithms. Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg only;
the product (stwo_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
P = (1 << 31) - 1

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            import sys

            sys.path.insert(0, os.path.dirname(HERE))
            from stwo_gb300.build import build_oracle

            build_oracle()
        _lib = C.CDLL(LIB)
        _lib.oracle_grind.restype = C.c_uint64
        _lib.oracle_interpolate.restype = C.c_int
        _lib.oracle_evaluate.restype = C.c_int
    return _lib


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _c3(c):
    return (C.c_uint32 * 3)(*c)


def _arr4(cols):
    return (C.c_void_p * 4)(*[c.ctypes.data for c in cols])


def _ptr_table(cols):
    return (C.c_void_p * max(1, len(cols)))(*[c.ctypes.data for c in cols])


def twiddles(root):
    n = 1 << root[2]
    tw = np.zeros(n, np.uint32)
    itw = np.zeros(n, np.uint32)
    lib().oracle_twiddles(_c3(root), _p(tw), _p(itw))
    return tw, itw


def interpolate(half, tree_root, values):
    v = _u32(values).copy()
    rc = lib().oracle_interpolate(_c3(half), _c3(tree_root), _p(v))
    assert rc == 0, "oracle interpolate rejected its arguments"
    return v


def evaluate(half, tree_root, coeffs):
    c = _u32(coeffs)
    out = np.zeros(1 << (half[2] + 1), np.uint32)
    rc = lib().oracle_evaluate(_c3(half), _c3(tree_root), _p(c), C.c_uint32(c.size.bit_length() - 1), _p(out))
    assert rc == 0, "oracle evaluate rejected its arguments"
    return out


def eval_at_point(coeffs, point):
    c = _u32(coeffs)
    pt = _u32(list(point[0]) + list(point[1]))
    out = np.zeros(4, np.uint32)
    lib().oracle_eval_at_point(_p(c), C.c_uint32(c.size.bit_length() - 1), _p(pt), _p(out))
    return tuple(int(x) for x in out)


def commit_on_layer(log_size, prev, cols):
    cols = [_u32(c) for c in cols]
    out = np.zeros((1 << log_size) * 8, np.uint32)
    prev_p = _p(_u32(prev).reshape(-1)) if prev is not None else None
    keep = _u32(prev).reshape(-1) if prev is not None else None
    if keep is not None:
        prev_p = _p(keep)
    lib().oracle_commit_on_layer(C.c_uint32(log_size), prev_p, _ptr_table(cols), C.c_uint32(len(cols)), _p(out))
    return out.reshape(-1, 8)


def blake2s(data: bytes) -> bytes:
    out = (C.c_uint8 * 32)()
    buf = (C.c_uint8 * max(1, len(data))).from_buffer_copy(data if data else b"\0")
    lib().oracle_blake2s(buf, C.c_size_t(len(data)), out)
    return bytes(out)


def fold_line(domain, src4, alpha):
    src = [_u32(c) for c in src4]
    n = src[0].size
    out = [np.zeros(n // 2, np.uint32) for _ in range(4)]
    lib().oracle_fold_line(_c3(domain), _arr4(src), _p(_u32(alpha)), _arr4(out))
    return out


def fold_circle_into_line(half, dst4, src4, alpha):
    dst = [_u32(c).copy() for c in dst4]
    src = [_u32(c) for c in src4]
    lib().oracle_fold_circle_into_line(_c3(half), _arr4(dst), _arr4(src), _p(_u32(alpha)))
    return dst


def decompose(src4):
    src = [_u32(c) for c in src4]
    g = [np.zeros_like(c) for c in src]
    lam = np.zeros(4, np.uint32)
    lib().oracle_decompose(_arr4(src), C.c_uint32(src[0].size.bit_length() - 1), _arr4(g), _p(lam))
    return g, tuple(int(x) for x in lam)


def accumulate_quotients(log_n, cols, random_coeff, batches, log_blowup):
    cols = [_u32(c) for c in cols]
    pts, offs, ecols, evals = [], [0], [], []
    for (pt, cv) in batches:
        pts += list(pt[0]) + list(pt[1])
        for c, v in cv:
            ecols.append(c)
            evals += list(v)
        offs.append(len(ecols))
    pts, offs, ecols, evals = _u32(pts), _u32(offs), _u32(ecols + [0]), _u32(evals + [0, 0, 0, 0])
    n = 1 << log_n
    out = [np.zeros(n, np.uint32) for _ in range(4)]
    lib().oracle_accumulate_quotients(
        C.c_uint32(log_n), _ptr_table(cols), C.c_uint32(len(cols)), _p(_u32(random_coeff)),
        C.c_uint32(len(batches)), _p(pts), _p(offs), _p(ecols), _p(evals), C.c_uint32(log_blowup), _arr4(out))
    return out


def secure_powers(felt, n):
    out = np.zeros(4 * max(n, 1), np.uint32)
    lib().oracle_secure_powers(_p(_u32(felt)), C.c_uint32(n), _p(out))
    return [tuple(int(x) for x in out[4 * i:4 * i + 4]) for i in range(n)]


def grind(digest, pow_bits):
    return int(lib().oracle_grind(_p(_u32(digest)), C.c_uint32(pow_bits)))


def raw_compress(h, m, t0=0, t1=0, f0=0, f1=0):
    out = np.zeros(8, np.uint32)
    lib().oracle_raw_compress(_p(_u32(h)), _p(_u32(m)), C.c_uint32(t0), C.c_uint32(t1), C.c_uint32(f0),
                              C.c_uint32(f1), _p(out))
    return [int(x) for x in out]


def qm31_mul(a, b):
    out = np.zeros(4, np.uint32)
    lib().oracle_qm31_mul(_p(_u32(a)), _p(_u32(b)), _p(out))
    return tuple(int(x) for x in out)


def qm31_inv(a):
    out = np.zeros(4, np.uint32)
    lib().oracle_qm31_inv(_p(_u32(a)), _p(out))
    return tuple(int(x) for x in out)


def index_to_point(idx):
    out = np.zeros(2, np.uint32)
    lib().oracle_index_to_point(C.c_uint32(idx), _p(out))
    return int(out[0]), int(out[1])


def prove_wide_fib(log_n, n_cols, a, b, config=(5, 1, 0, 3)):
    """Canonical proof bytes of the wide-Fibonacci AIR (oracle prover)."""
    a, b = _u32(a), _u32(b)
    cap = 64 << 20
    out = np.zeros(cap, np.uint8)
    err = C.create_string_buffer(512)
    f = lib().oracle_prove_wide_fib
    f.restype = C.c_size_t
    n = f(C.c_uint32(log_n), C.c_uint32(n_cols), _p(a), _p(b), _p(_u32(config)), _p(out), C.c_size_t(cap), err,
          C.c_size_t(512))
    if n == 0:
        raise RuntimeError("oracle prove failed: " + err.value.decode())
    return bytes(out[:n])


def verify_wide_fib(log_n, n_cols, proof: bytes):
    """(accepted, reason) for canonical proof bytes of the wide-Fibonacci AIR."""
    buf = np.frombuffer(proof, dtype=np.uint8).copy()
    err = C.create_string_buffer(512)
    ok = lib().oracle_verify_wide_fib(C.c_uint32(log_n), C.c_uint32(n_cols), _p(buf), C.c_size_t(len(proof)), err,
                                      C.c_size_t(512))
    return bool(ok), err.value.decode()


def prove_poseidon(log_n, init=None, config=(5, 1, 0, 3)):
    """(proof bytes, claimed_sum) of the Poseidon2 AIR; init = None for the reference's inputs."""
    cap = 256 << 20
    out = np.zeros(cap, np.uint8)
    cs = np.zeros(4, np.uint32)
    err = C.create_string_buffer(512)
    f = lib().oracle_prove_poseidon
    f.restype = C.c_size_t
    ip = _p(_u32(init).reshape(-1)) if init is not None else None
    keep = _u32(init).reshape(-1) if init is not None else None
    if keep is not None:
        ip = _p(keep)
    n = f(C.c_uint32(log_n), ip, _p(_u32(config)), _p(out), C.c_size_t(cap), _p(cs), err, C.c_size_t(512))
    if n == 0:
        raise RuntimeError("oracle prove failed: " + err.value.decode())
    return bytes(out[:n]), tuple(int(x) for x in cs)


def prove_plonk(log_n, config=(5, 1, 0, 3)):
    """(proof bytes, claimed sum) of prove_fibonacci_plonk (plonk/mod.rs:153-266) with 2^log_n
    gates."""
    cap = 64 << 20
    out = np.zeros(cap, np.uint8)
    cs = np.zeros(4, np.uint32)
    err = C.create_string_buffer(512)
    f = lib().oracle_prove_plonk
    f.restype = C.c_size_t
    cfg = _u32(config)
    n = f(C.c_uint32(log_n), _p(cfg), _p(out), C.c_size_t(cap), _p(cs), err, C.c_size_t(512))
    if n == 0:
        raise RuntimeError("oracle prove failed: " + err.value.decode())
    return bytes(out[:n]), tuple(int(x) for x in cs)


def prove_state_machine(log_n, initial=(0, 0), config=(5, 1, 0, 3)):
    """(stark proof bytes, (claimed sum x, claimed sum y)) of prove_state_machine
    (state_machine/mod.rs:26-135)."""
    cap = 64 << 20
    out = np.zeros(cap, np.uint8)
    cs = np.zeros(8, np.uint32)
    err = C.create_string_buffer(512)
    f = lib().oracle_prove_state_machine
    f.restype = C.c_size_t
    init, cfg = _u32(initial), _u32(config)
    n = f(C.c_uint32(log_n), _p(init), _p(cfg), _p(out), C.c_size_t(cap), _p(cs), err, C.c_size_t(512))
    if n == 0:
        raise RuntimeError("oracle prove failed: " + err.value.decode())
    return bytes(out[:n]), (tuple(int(x) for x in cs[:4]), tuple(int(x) for x in cs[4:]))


def prove_blake(log_n, config=(5, 1, 0, 3)):
    """(stark proof bytes, eight claimed sums) of prove_blake (blake/air.rs:308-460) for 2^log_n
    instances: scheduler, round 0, round 1, XOR tables 12, 9, 8, 7, 4."""
    cap = 256 << 20
    out = np.zeros(cap, np.uint8)
    cs = np.zeros(32, np.uint32)
    err = C.create_string_buffer(512)
    f = lib().oracle_prove_blake
    f.restype = C.c_size_t
    cfg = _u32(config)
    n = f(C.c_uint32(log_n), _p(cfg), _p(out), C.c_size_t(cap), _p(cs), err, C.c_size_t(512))
    if n == 0:
        raise RuntimeError("oracle prove failed: " + err.value.decode())
    return bytes(out[:n]), [tuple(int(x) for x in cs[4 * i:4 * i + 4]) for i in range(8)]


def verify_blake(log_n, sums, proof: bytes):
    buf = np.frombuffer(proof, dtype=np.uint8).copy()
    err = C.create_string_buffer(512)
    cs = _u32([x for q in sums for x in q])
    ok = lib().oracle_verify_blake(C.c_uint32(log_n), _p(cs), _p(buf), C.c_size_t(len(proof)), err, C.c_size_t(512))
    return bool(ok), err.value.decode()


def blake2s_rounds(v, m, rounds=10):
    """The full Blake example's scheduler round function applied `rounds` times."""
    vv = _u32(v).copy()
    lib().oracle_blake2s_rounds(_p(vv), _p(_u32(m)), C.c_uint32(rounds))
    return [int(x) for x in vv]


def blake_traces(log_n):
    """The preprocessed and trace columns of prove_blake, in commit order, as one word array."""
    cap = 64 << 20
    out = np.zeros(cap, np.uint32)
    k = C.c_uint32(0)
    f = lib().oracle_blake_traces
    f.restype = C.c_size_t
    n = f(C.c_uint32(log_n), _p(out), C.c_size_t(cap), C.byref(k))
    if n == 0:
        raise RuntimeError("oracle blake_traces failed")
    return out[:n].copy(), k.value


def verify_plonk(log_n, claimed_sum, proof: bytes):
    buf = np.frombuffer(proof, dtype=np.uint8).copy()
    err = C.create_string_buffer(512)
    ok = lib().oracle_verify_plonk(C.c_uint32(log_n), _p(_u32(claimed_sum)), _p(buf), C.c_size_t(len(proof)), err,
                                   C.c_size_t(512))
    return bool(ok), err.value.decode()


def verify_state_machine(log_n, claimed_sums, proof: bytes):
    buf = np.frombuffer(proof, dtype=np.uint8).copy()
    err = C.create_string_buffer(512)
    cs = _u32(list(claimed_sums[0]) + list(claimed_sums[1]))
    ok = lib().oracle_verify_state_machine(C.c_uint32(log_n), _p(cs), _p(buf), C.c_size_t(len(proof)), err,
                                           C.c_size_t(512))
    return bool(ok), err.value.decode()


def verify_poseidon(log_n, claimed_sum, proof: bytes):
    buf = np.frombuffer(proof, dtype=np.uint8).copy()
    err = C.create_string_buffer(512)
    ok = lib().oracle_verify_poseidon(C.c_uint32(log_n), _p(_u32(claimed_sum)), _p(buf), C.c_size_t(len(proof)),
                                      err, C.c_size_t(512))
    return bool(ok), err.value.decode()


def prove_blake_round(log_n, inputs=None, config=(5, 1, 0, 3)):
    """(proof bytes, claimed_sum) of the Blake2s round AIR; inputs (per row 16 state + 16 message
    words) = None for the reference test's inputs."""
    cap = 256 << 20
    out = np.zeros(cap, np.uint8)
    cs = np.zeros(4, np.uint32)
    err = C.create_string_buffer(512)
    f = lib().oracle_prove_blake_round
    f.restype = C.c_size_t
    keep = _u32(inputs).reshape(-1) if inputs is not None else None
    ip = _p(keep) if keep is not None else None
    n = f(C.c_uint32(log_n), ip, _p(_u32(config)), _p(out), C.c_size_t(cap), _p(cs), err, C.c_size_t(512))
    if n == 0:
        raise RuntimeError("oracle prove failed: " + err.value.decode())
    return bytes(out[:n]), tuple(int(x) for x in cs)


def verify_blake_round(log_n, claimed_sum, proof: bytes):
    buf = np.frombuffer(proof, dtype=np.uint8).copy()
    err = C.create_string_buffer(512)
    ok = lib().oracle_verify_blake_round(C.c_uint32(log_n), _p(_u32(claimed_sum)), _p(buf), C.c_size_t(len(proof)),
                                         err, C.c_size_t(512))
    return bool(ok), err.value.decode()


# ---------------------------------------------------------------- GKR / MLE
GRAND_PRODUCT, LOGUP_GENERIC, LOGUP_MULTIPLICITIES, LOGUP_SINGLES = 0, 1, 2, 3


def gkr_pack(kind, cols):
    """Flat words of one layer: secure columns as (4, n) coordinate arrays, multiplicities (n,)."""
    return np.concatenate([_u32(c).reshape(-1) for c in cols])


def _layer_args(layers):
    kinds = _u32([k for k, _ in layers])
    logs = _u32([(np.asarray(cols[-1]).shape[-1]).bit_length() - 1 for _, cols in layers])
    data = np.concatenate([gkr_pack(k, cols) for k, cols in layers])
    return kinds, logs, data


def gkr_gen_eq_evals(y, v):
    y = _u32(y).reshape(-1, 4)
    out = np.zeros((4, 1 << len(y)), np.uint32)
    lib().oracle_gkr_gen_eq_evals(_p(y), C.c_uint32(len(y)), _p(_u32(v)), _p(out))
    return out


def gkr_next_layer(kind, cols):
    """Next layer's columns: [prod (4, n/2)] or [num (4, n/2), den (4, n/2)]."""
    n = np.asarray(cols[-1]).shape[-1]
    data = gkr_pack(kind, cols)
    ncols = 1 if kind == GRAND_PRODUCT else 2
    out = np.zeros((ncols, 4, n // 2), np.uint32)
    lib().oracle_gkr_next_layer(C.c_uint32(kind), C.c_uint32(n.bit_length() - 1), _p(data), _p(out))
    return [out[i] for i in range(ncols)]


def gkr_sum_as_poly(kind, cols, y, lam, correction, claim):
    n = np.asarray(cols[-1]).shape[-1]
    data = gkr_pack(kind, cols)
    y = _u32(y).reshape(-1, 4)
    coeffs = np.zeros((4, 4), np.uint32)
    f = lib().oracle_gkr_sum_as_poly
    f.restype = C.c_uint32
    k = f(C.c_uint32(kind), C.c_uint32(n.bit_length() - 1), _p(data), _p(y), C.c_uint32(len(y)), _p(_u32(lam)),
          _p(_u32(correction)), _p(_u32(claim)), _p(coeffs))
    return [tuple(int(x) for x in coeffs[i]) for i in range(k)]


def mle_fix_first_variable(col, a):
    col = _u32(col)
    is_base = col.ndim == 1
    n = col.shape[-1]
    out = np.zeros((4, n // 2), np.uint32)
    lib().oracle_mle_fix_first_variable(C.c_int(int(is_base)), C.c_uint32(n.bit_length() - 1), _p(col),
                                        _p(_u32(a)), _p(out))
    return out


def gkr_prove(layers, digest=None):
    """(proof+artifact bytes, final channel digest) of prove_batch over [(kind, cols), ...]."""
    kinds, logs, data = _layer_args(layers)
    cap = 16 << 20
    out = np.zeros(cap, np.uint8)
    dout = np.zeros(32, np.uint8)
    err = C.create_string_buffer(512)
    f = lib().oracle_gkr_prove
    f.restype = C.c_size_t
    dg = np.frombuffer(digest, np.uint8).copy() if digest is not None else None
    n = f(C.c_size_t(len(layers)), _p(kinds), _p(logs), _p(data), _p(dg) if dg is not None else None, _p(out),
          C.c_size_t(cap), _p(dout), err, C.c_size_t(512))
    if n == 0:
        raise RuntimeError("oracle GKR prove failed: " + err.value.decode())
    return bytes(out[:n]), bytes(dout)


def gkr_verify(layers, proof: bytes, digest=None, check_inputs=True):
    kinds, logs, data = _layer_args(layers)
    buf = np.frombuffer(proof, dtype=np.uint8).copy()
    err = C.create_string_buffer(512)
    dg = np.frombuffer(digest, np.uint8).copy() if digest is not None else None
    ok = lib().oracle_gkr_verify(C.c_size_t(len(layers)), _p(kinds), _p(logs), _p(data) if check_inputs else None,
                                 _p(dg) if dg is not None else None, _p(buf), C.c_size_t(len(proof)), err,
                                 C.c_size_t(512))
    return bool(ok), err.value.decode()


def channel_draw_felts(n):
    out = np.zeros((n, 4), np.uint32)
    lib().oracle_channel_draw_felts(C.c_size_t(n), _p(out))
    return out


def gen_words(k, c, n):
    """The benchmark input generator (word i of column c of workload k)."""
    out = np.zeros(n, np.uint32)
    lib().oracle_gen_words(C.c_uint64(k), C.c_uint64(c), C.c_uint64(n), _p(out))
    return out


def cfg2_outputs(n_cols, log, blowup, fri_log, threads=0):
    """The kernel-microbench pass on the oracle: (Merkle root words, [FRI layers as 4 columns each])."""
    root = np.zeros(8, np.uint32)
    last = np.zeros(64, np.uint32)
    sizes = [1 << (fri_log - 1)]
    while sizes[-1] > 16:
        sizes.append(sizes[-1] // 2)
    layers = np.zeros(4 * sum(sizes), np.uint32)
    f = lib().oracle_cfg2_outputs
    f.restype = C.c_double
    f(C.c_uint32(n_cols), C.c_uint32(log), C.c_uint32(blowup), C.c_uint32(fri_log), C.c_int(threads), _p(root),
      _p(last), _p(layers))
    out, off = [], 0
    for n in sizes:
        out.append(layers[off:off + 4 * n].reshape(4, n))
        off += 4 * n
    return root, out


def poseidon_linear(kind, state):
    """The Poseidon2 example's linear layers on a state: kind "m4" (4 words), "internal" or
    "external" (16 words)."""
    x = _u32(state).copy()
    getattr(lib(), f"oracle_poseidon_apply_{kind}")(_p(x))
    return [int(v) for v in x]


def eval_constraints(air, log_n, n_cols, claimed_sum, elements, cols, coeffs, acc):
    """The oracle's per-component constraint accumulation: returns acc (4 columns) after adding
    row_res / Z(row) on the evaluation domain. `cols` are the component's columns on that domain,
    tree by tree; `coeffs` the accumulator's powers in the order it hands them."""
    cs = _u32(claimed_sum)
    el = _u32(np.asarray(elements, np.uint32).reshape(-1)) if len(elements) else np.zeros(4, np.uint32)
    cl = [_u32(c) for c in cols]
    tbl = (C.c_void_p * max(1, len(cl)))(*[c.ctypes.data for c in cl])
    co = _u32(np.asarray(coeffs, np.uint32).reshape(-1))
    out = [_u32(a).copy() for a in acc]
    st = lib().oracle_eval_constraints(C.c_uint32(air), C.c_uint32(log_n), C.c_uint32(n_cols), _p(cs), _p(el),
                                       C.c_uint32(len(elements)), tbl, C.c_uint32(len(cl)), _p(co),
                                       C.c_uint32(len(coeffs)), _arr4(out))
    if st != 0:
        raise ValueError("oracle_eval_constraints: bad input")
    return out


# ---------------------------------------------------------------- Poseidon252
def _w8(x: int):
    return np.array([(x >> (32 * i)) & 0xFFFFFFFF for i in range(8)], np.uint32)


def _int8(w) -> int:
    return sum(int(v) << (32 * i) for i, v in enumerate(w))


def p252_hash(x: int, y: int) -> int:
    out = np.zeros(8, np.uint32)
    lib().oracle_p252_hash(_p(_w8(x)), _p(_w8(y)), _p(out))
    return _int8(out)


def p252_hash_many(vals) -> int:
    v = np.concatenate([_w8(x) for x in vals]) if len(vals) else np.zeros(8, np.uint32)
    out = np.zeros(8, np.uint32)
    lib().oracle_p252_hash_many(_p(v), C.c_size_t(len(vals)), _p(out))
    return _int8(out)


def p252_hash_node(children, vals) -> int:
    out = np.zeros(8, np.uint32)
    v = _u32(vals) if len(vals) else np.zeros(1, np.uint32)
    if children:
        l, r = _w8(children[0]), _w8(children[1])
        lib().oracle_p252_hash_node(_p(l), _p(r), _p(v), C.c_size_t(len(vals)), _p(out))
    else:
        lib().oracle_p252_hash_node(None, None, _p(v), C.c_size_t(len(vals)), _p(out))
    return _int8(out)


def p252_commit_on_layer(log_size, prev, cols):
    """prev: None or 2^(log+1) x 8 words; returns 2^log x 8 words."""
    cols = [_u32(c) for c in cols]
    out = np.zeros((1 << log_size) * 8, np.uint32)
    pv = _u32(prev).reshape(-1) if prev is not None else None
    lib().oracle_p252_commit_on_layer(C.c_uint32(log_size), _p(pv) if pv is not None else None, _ptr_table(cols),
                                      C.c_uint32(len(cols)), _p(out))
    return out.reshape(-1, 8)


def p252_grind(digest: int, pow_bits: int) -> int:
    f = lib().oracle_p252_grind
    f.restype = C.c_uint64
    return int(f(_p(_w8(digest)), C.c_uint32(pow_bits)))


def p252_trailing_zeros(digest: int) -> int:
    return int(lib().oracle_p252_trailing_zeros(_p(_w8(digest))))


def p252_channel(digest: int, felts, n_draw):
    """Mixes `felts` (QM31 tuples) into a channel at `digest`, then draws n_draw felts."""
    f = _u32(np.asarray(felts, np.uint32).reshape(-1)) if len(felts) else np.zeros(4, np.uint32)
    draws = np.zeros(max(1, n_draw) * 4, np.uint32)
    out = np.zeros(8, np.uint32)
    lib().oracle_p252_channel(_p(_w8(digest)), _p(f), C.c_size_t(len(felts)), C.c_size_t(n_draw), _p(draws), _p(out))
    return [tuple(int(x) for x in draws[4 * i:4 * i + 4]) for i in range(n_draw)], _int8(out)
