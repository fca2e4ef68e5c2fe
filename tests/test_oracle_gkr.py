"""GKR / MLE oracle checks, restating the reference's own GKR, sum-check and MLE tests:
crates/prover/src/core/backend/cpu/lookups/gkr.rs:298-470, lookups/gkr_verifier.rs:293-355,
lookups/sumcheck.rs:217-287 and backend/simd/lookups/mle.rs:105-131.
"""
import itertools

import numpy as np
import pytest

from tests import m31 as F

ONE = (1, 0, 0, 0)
ZERO = (0, 0, 0, 0)


def _col(rng, n):
    return rng.integers(0, F.P, (4, n), dtype=np.uint32)


def _q(col, i):
    return tuple(int(col[c][i]) for c in range(4))


def _felts_col(felts):
    return np.ascontiguousarray(np.asarray(felts, np.uint32).T)


def _eq(x, y):
    r = ONE
    for a, b in zip(x, y):
        r = F.q_mul(r, F.q_add(F.q_mul(a, b), F.q_mul(F.q_sub(ONE, a), F.q_sub(ONE, b))))
    return r


def _mle_eval(col, point):
    vals = [_q(col, i) for i in range(col.shape[-1])]
    for p in point:
        h = len(vals) // 2
        vals = [F.q_add(F.q_mul(p, F.q_sub(vals[i + h], vals[i])), vals[i]) for i in range(h)]
    return vals[0]


def _frac_sum(nums, dens):
    """Sequential Fraction sum from 0/1, as Iterator::sum does in the reference tests."""
    n, d = ZERO, ONE
    for a, b in zip(nums, dens):
        n, d = F.q_add(F.q_mul(b, n), F.q_mul(d, a)), F.q_mul(d, b)
    return n, d


def _claims(proof: bytes):
    """Output claims of instance 0 parsed from the canonical bytes (layout of write_gkr)."""
    w = np.frombuffer(proof, np.uint8)
    pos = 0

    def u64():
        nonlocal pos
        v = int(w[pos:pos + 8].view(np.uint64)[0])
        pos += 8
        return v

    def q():
        nonlocal pos
        v = tuple(int(x) for x in w[pos:pos + 16].view(np.uint32))
        pos += 16
        return v

    for _ in range(u64()):
        for _ in range(u64()):
            for _ in range(u64()):
                q()
    for _ in range(u64()):
        for _ in range(u64()):
            for _ in range(u64()):
                q(), q()
    out = []
    for _ in range(u64()):
        out.append([q() for _ in range(u64())])
    return out


def test_gen_eq_evals_kat(oracle):
    # cpu/lookups/gkr.rs:298-316: y = [7, 3], v = 2.
    y = [F.q(7), F.q(3)]
    got = oracle.gkr_gen_eq_evals(y, F.q(2))
    for i, bits in enumerate(itertools.product([ZERO, ONE], repeat=2)):
        assert _q(got, i) == F.q_mul(_eq(list(bits), y), F.q(2))


def test_gen_eq_evals_first_variable_is_most_significant(oracle):
    rng = np.random.default_rng(1)
    y = [tuple(int(v) for v in rng.integers(0, F.P, 4)) for _ in range(4)]
    v = tuple(int(x) for x in rng.integers(0, F.P, 4))
    got = oracle.gkr_gen_eq_evals(y, v)
    for i in range(16):
        bits = [ONE if (i >> (3 - j)) & 1 else ZERO for j in range(4)]
        assert _q(got, i) == F.q_mul(_eq(bits, y), v)


def test_grand_product_works(oracle):
    values = oracle.channel_draw_felts(32)
    col = _felts_col(values)
    product = ONE
    for v in values:
        product = F.q_mul(product, tuple(int(x) for x in v))
    proof, _ = oracle.gkr_prove([(oracle.GRAND_PRODUCT, [col])])
    ok, why = oracle.gkr_verify([(oracle.GRAND_PRODUCT, [col])], proof)
    assert ok, why
    assert _claims(proof) == [[product]]


@pytest.mark.parametrize("kind", ["generic", "singles", "multiplicities"])
def test_logup_works(oracle, kind):
    rng = np.random.default_rng(0)
    n = 32
    dens = _col(rng, n)
    if kind == "generic":
        layer = (oracle.LOGUP_GENERIC, [_col(rng, n), dens])
        nums = [_q(layer[1][0], i) for i in range(n)]
    elif kind == "singles":
        layer = (oracle.LOGUP_SINGLES, [dens])
        nums = [ONE] * n
    else:
        mult = rng.integers(0, F.P, n, dtype=np.uint32)
        layer = (oracle.LOGUP_MULTIPLICITIES, [mult, dens])
        nums = [F.q(int(m)) for m in mult]
    proof, _ = oracle.gkr_prove([layer])
    ok, why = oracle.gkr_verify([layer], proof)
    assert ok, why
    assert _claims(proof) == [list(_frac_sum(nums, [_q(dens, i) for i in range(n)]))]


@pytest.mark.parametrize("logs", [(5, 5), (5, 7)])
def test_prove_batch_works(oracle, logs):
    # gkr_verifier.rs:293-355: two grand products drawn from one channel.
    felts = oracle.channel_draw_felts(sum(1 << l for l in logs))
    cols = [_felts_col(felts[:1 << logs[0]]), _felts_col(felts[1 << logs[0]:])]
    layers = [(oracle.GRAND_PRODUCT, [c]) for c in cols]
    proof, _ = oracle.gkr_prove(layers)
    ok, why = oracle.gkr_verify(layers, proof)
    assert ok, why


def test_mixed_batch_and_channel_state(oracle):
    rng = np.random.default_rng(5)
    layers = [
        (oracle.LOGUP_GENERIC, [_col(rng, 64), _col(rng, 64)]),
        (oracle.GRAND_PRODUCT, [_col(rng, 8)]),
        (oracle.LOGUP_SINGLES, [_col(rng, 128)]),
        (oracle.LOGUP_MULTIPLICITIES, [rng.integers(0, F.P, 16, dtype=np.uint32), _col(rng, 16)]),
    ]
    digest = bytes(range(32))
    proof, d1 = oracle.gkr_prove(layers, digest)
    ok, why = oracle.gkr_verify(layers, proof, digest)
    assert ok, why
    proof2, d2 = oracle.gkr_prove(layers)
    assert proof2 != proof and d1 != d2
    ok, _ = oracle.gkr_verify(layers, proof, None)
    assert not ok


def test_tampered_proof_rejected(oracle):
    rng = np.random.default_rng(3)
    layer = (oracle.LOGUP_GENERIC, [_col(rng, 32), _col(rng, 32)])
    proof, _ = oracle.gkr_prove([layer])
    for off in (8 + 8 + 8 + 4, len(proof) // 2, len(proof) - 200):
        bad = bytearray(proof)
        bad[off] ^= 1
        ok, _ = oracle.gkr_verify([layer], bytes(bad))
        assert not ok


def test_fix_first_variable_matches_mle_eval(oracle):
    # simd/lookups/mle.rs:105-131 compare against the CPU fold; here the fold chain must equal
    # the multilinear evaluation and base columns must fold as their secure embedding does.
    rng = np.random.default_rng(9)
    col = _col(rng, 16)
    point = [tuple(int(v) for v in rng.integers(0, F.P, 4)) for _ in range(4)]
    cur = col
    for p in point:
        cur = oracle.mle_fix_first_variable(cur, p)
    assert _q(cur, 0) == _mle_eval(col, point)
    base = rng.integers(0, F.P, 16, dtype=np.uint32)
    emb = np.zeros((4, 16), np.uint32)
    emb[0] = base
    a = point[0]
    assert np.array_equal(oracle.mle_fix_first_variable(base, a), oracle.mle_fix_first_variable(emb, a))


def test_next_layer_matches_definition(oracle):
    rng = np.random.default_rng(11)
    num, den = _col(rng, 8), _col(rng, 8)
    (prod,) = oracle.gkr_next_layer(oracle.GRAND_PRODUCT, [num])
    for i in range(4):
        assert _q(prod, i) == F.q_mul(_q(num, 2 * i), _q(num, 2 * i + 1))
    nn, nd = oracle.gkr_next_layer(oracle.LOGUP_GENERIC, [num, den])
    sn, sd = oracle.gkr_next_layer(oracle.LOGUP_SINGLES, [den])
    for i in range(4):
        a, b = _q(num, 2 * i), _q(num, 2 * i + 1)
        c, d = _q(den, 2 * i), _q(den, 2 * i + 1)
        assert _q(nn, i) == F.q_add(F.q_mul(d, a), F.q_mul(c, b))
        assert _q(nd, i) == F.q_mul(c, d) == _q(sd, i)
        assert _q(sn, i) == F.q_add(c, d)


def test_sum_as_poly_round_consistency(oracle):
    rng = np.random.default_rng(13)
    num, den = _col(rng, 32), _col(rng, 32)
    y = [tuple(int(v) for v in rng.integers(0, F.P, 4)) for _ in range(6)]
    lam, corr, claim = (tuple(int(v) for v in rng.integers(0, F.P, 4)) for _ in range(3))
    coeffs = oracle.gkr_sum_as_poly(oracle.LOGUP_GENERIC, [num, den], y, lam, corr, claim)
    assert 1 <= len(coeffs) <= 4

    def ev(x):
        acc = ZERO
        for c in reversed(coeffs):
            acc = F.q_add(F.q_mul(acc, x), c)
        return acc

    assert F.q_add(ev(ZERO), ev(ONE)) == claim
