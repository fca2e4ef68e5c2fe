"""Pins the oracle to the reference's known-answer tests (CPU only).

Each test restates a reference test or a published vector:
  Blake2s:  crates/prover/src/core/vcs/blake2_hash.rs:112-131 (single_hash_test, hash_state_test)
            and RFC 7693 Appendix B (BLAKE2s-256("abc")).
  Fields:   crates/prover/src/core/fields/qm31.rs:150-170, cm31.rs:95-115 (test_ops).
  Circle:   crates/prover/src/core/circle.rs:185-200 (generator order), :527 (secure generator).
  CPU FFT:  crates/prover/src/core/backend/cpu/circle.rs:257-340 (eval_at_point, evaluate n coeffs,
            interpolate round trips).
  FRI:      crates/prover/src/core/fri.rs:1224-1253 (fold_line_works).
  Twiddles: crates/prover/src/core/poly/utils.rs:104-113 (test_domain_line_twiddles_works).
  Quotients: crates/prover/src/core/backend/simd/quotients.rs:296-344 (SIMD == CPU on low-degree input).
  Poseidon2: crates/prover/src/examples/poseidon/mod.rs:427-461 (test_apply_m4, test_apply_internal).
"""
import numpy as np
import pytest

from tests import m31 as F


def test_blake2s_known_answers(oracle):
    assert oracle.blake2s(b"a").hex() == "4a0d129873403037c2cd9b9048203687f6233fb6738956e0349bd4320fec3e90"
    assert oracle.blake2s(b"abc").hex() == "508c5e8c327c14e2e1a72ba34eeb452f37458b209ed63a294d999b4c86675982"
    assert oracle.blake2s(b"").hex() == "69217a3079908094e11121d042354a7c1f55b6482ca1a51e1b250dfd1ed0eef9"
    # hash_state_test: incremental "a" then "b" equals hash("ab").
    assert oracle.blake2s(b"ab") == oracle.blake2s(b"a" + b"b")


def test_blake2s_multiblock_boundaries(oracle):
    import hashlib

    for n in [0, 1, 63, 64, 65, 127, 128, 129, 1000]:
        data = bytes((i * 7 + 3) & 0xFF for i in range(n))
        assert oracle.blake2s(data) == hashlib.blake2s(data).digest(), n


def test_qm31_cm31_ops(oracle):
    P = F.P
    assert oracle.qm31_mul((1, 2, 3, 4), (4, 5, 6, 7)) == (P - 71, 93, P - 16, 50)
    assert F.q_mul((1, 2, 3, 4), (4, 5, 6, 7)) == (P - 71, 93, P - 16, 50)
    assert F.cm_mul((1, 2), (4, 5)) == (P - 6, 13)
    a = (1, 2, 3, 4)
    assert oracle.qm31_mul(a, oracle.qm31_inv(a)) == (1, 0, 0, 0)


def test_circle_generator_order(oracle):
    p = F.GEN
    for _ in range(30):
        p = F.padd(p, p)
    assert p != (1, 0)
    assert F.padd(p, p) == (1, 0)
    assert oracle.index_to_point(1 << 30) == (F.P - 1, 0)
    for i in [0, 1, 2, 3, 12345, (1 << 31) - 1]:
        assert oracle.index_to_point(i) == F.index_to_point(i)


def test_twiddle_tree_layout(oracle):
    # The tree of a canonic half coset: per level, x of the first half of the coset in
    # bit-reversed order, then the doubled coset, padded with 1.
    half = F.canonic_half(4)
    tw, itw = oracle.twiddles(half)
    assert len(tw) == 8 and tw[-1] == 1
    init, step, log = half
    xs = [F.index_to_point(init + step * F.brev(j, 2))[0] for j in range(4)]
    assert list(tw[:4]) == xs
    assert all(F.mul(int(a), int(b)) == 1 for a, b in zip(tw, itw))


def test_eval_at_point_4_coeffs(oracle):
    # 1 + 2y + 3x + 4xy, coefficients bit reversed: [1, 3, 2, 4]; x = 5, y = 8.
    x, y = F.q(5), F.q(8)
    got = oracle.eval_at_point([1, 3, 2, 4], (x, y))
    want = F.q(1 + 3 * 8 + 2 * 5 + 4 * 5 * 8)
    assert got == want
    assert oracle.eval_at_point([1, 2], (x, y)) == F.q(1 + 2 * 8)
    assert oracle.eval_at_point([1], (x, y)) == F.q(1)


@pytest.mark.parametrize("log", [1, 2, 3, 4, 5])
def test_evaluate_matches_eval_at_point(oracle, log):
    half = F.canonic_half(log)
    coeffs = list(range(1, (1 << log) + 1))
    ev = oracle.evaluate(half, half, coeffs)
    pts = F.domain_points_bitrev(half)
    for i, p in enumerate(pts):
        assert (int(ev[i]), 0, 0, 0) == oracle.eval_at_point(coeffs, (F.q(p[0]), F.q(p[1]))), i


@pytest.mark.parametrize("log", [1, 2, 3, 6, 9])
def test_interpolate_roundtrip(oracle, log):
    rng = np.random.default_rng(log)
    half = F.canonic_half(log)
    vals = F.rand_m31(rng, 1 << log)
    coeffs = oracle.interpolate(half, half, vals)
    assert np.array_equal(oracle.evaluate(half, half, coeffs), vals)


def test_fold_line_works(oracle):
    # Restates fri.rs:1224-1253: fold of even/odd line polys equals 2 * (f_e + alpha f_o).
    even, odd = [1, 2, 1, 3], [3, 5, 4, 1]
    coeffs = [F.q(c) for c in even + odd]
    alpha = F.q(19283)
    init, step = 1 << (31 - 5), 1 << (31 - 3)  # Coset::half_odds(3)
    domain = (init, step, 3)

    def line_eval(cs, x):
        n = len(cs)
        log = n.bit_length() - 1
        facts = []
        for _ in range(log):
            facts.append(x)
            x = F.q_sub(F.q_add(F.q_mul(x, x), F.q_mul(x, x)), F.q(1))

        def fold(vals, fs):
            if len(vals) == 1:
                return vals[0]
            h = len(vals) // 2
            return F.q_add(fold(vals[:h], fs[1:]), F.q_mul(fold(vals[h:], fs[1:]), fs[0]))

        return fold(cs, facts)

    xs = [F.index_to_point(init + step * i)[0] for i in range(8)]
    vals = [line_eval(coeffs, F.q(x)) for x in xs]
    vals_br = [vals[F.brev(i, 3)] for i in range(8)]
    cols = [np.array([v[k] for v in vals_br], np.uint32) for k in range(4)]
    out = oracle.fold_line(domain, cols, alpha)
    folded = [tuple(int(out[k][i]) for k in range(4)) for i in range(4)]
    folded_nat = [folded[F.brev(i, 2)] for i in range(4)]
    dinit, dstep = (2 * init) & F.P, (2 * step) & F.P
    for i in range(4):
        x = F.q(F.index_to_point(dinit + dstep * i)[0])
        fe = line_eval([F.q(c) for c in even], x)
        fo = line_eval([F.q(c) for c in odd], x)
        want = F.q_add(fe, F.q_mul(alpha, fo))
        assert folded_nat[i] == F.q_add(want, want), i


def test_quotients_simd_route_equals_cpu_route_on_low_degree(oracle):
    # Low-degree columns sampled at their true values: the sub-domain + extension route of the
    # SIMD backend equals direct row evaluation (the reference's test_accumulate_quotients).
    log_n, blowup = 8, 1
    rng = np.random.default_rng(7)
    trace_half = F.canonic_half(log_n - blowup)
    dom_half = F.canonic_half(log_n)
    cols = []
    for _ in range(3):
        coeffs = F.rand_m31(rng, 1 << (log_n - blowup))
        cols.append(oracle.evaluate(dom_half, dom_half, coeffs))
    # Two random circle points over QM31 (CirclePoint::get_random_point, circle.rs:170-183).
    pts = []
    for _ in range(2):
        t = tuple(int(v) for v in rng.integers(0, F.P, 4))
        t2 = F.q_mul(t, t)
        d = oracle.qm31_inv(F.q_add(t2, F.q(1)))
        pts.append((F.q_mul(F.q_sub(F.q(1), t2), d), F.q_mul(F.q_add(t, t), d)))
    coeff_polys = [oracle.interpolate(dom_half, dom_half, c) for c in cols]
    batches = []
    for pt in sorted(pts):
        batches.append((pt, [(i, oracle.eval_at_point(coeff_polys[i], pt)) for i in range(3)]))
    rc = (5, 6, 7, 8)
    simd = oracle.accumulate_quotients(log_n, cols, rc, batches, blowup)
    direct = oracle.accumulate_quotients(log_n, cols, rc, batches, 0)
    for k in range(4):
        assert np.array_equal(simd[k], direct[k])
    del trace_half


def test_grind_minimum_nonce(oracle):
    digest = list(range(1, 9))
    n = oracle.grind(digest, 6)
    for k in range(n):
        assert oracle.raw_compress(digest, [k & 0xFFFFFFFF, k >> 32] + [0] * 14)[0] % 64 != 0
    assert oracle.raw_compress(digest, [n, 0] + [0] * 14)[0] % 64 == 0


def _matmul(rows, state):
    return [sum(r * s for r, s in zip(row, state)) % F.P for row in rows]


def test_poseidon_apply_m4(oracle):
    """test_apply_m4 (crates/prover/src/examples/poseidon/mod.rs:427-440): apply_m4 equals the
    row-major matrix [5 7 1 3; 4 6 1 1; 1 3 5 7; 1 1 4 6] on the state (0, 1, 2, 3)."""
    m4 = [[5, 7, 1, 3], [4, 6, 1, 1], [1, 3, 5, 7], [1, 1, 4, 6]]
    state = [0, 1, 2, 3]
    assert oracle.poseidon_linear("m4", state) == _matmul(m4, state)
    # The same matrix on a state of large words (wrap-around of the additions).
    big = [F.P - 1, F.P - 2, 12345, F.P - 7]
    assert oracle.poseidon_linear("m4", big) == _matmul(m4, big)


def test_poseidon_apply_internal(oracle):
    """test_apply_internal (poseidon/mod.rs:442-461): the internal round matrix is the all-ones
    matrix plus diag(2^(i+1)), on the state (3i + 187)."""
    state = [3 * i + 187 for i in range(16)]
    mat = [[1 + ((1 << (i + 1)) if i == j else 0) for j in range(16)] for i in range(16)]
    assert oracle.poseidon_linear("internal", state) == _matmul(mat, state)


def test_poseidon_apply_external(oracle):
    """The external round matrix (poseidon/mod.rs apply_external_round_matrix): circ(2 M4, M4, M4,
    M4) as blocks, i.e. M4 on each quarter followed by adding the column sums of the quarters."""
    m4 = [[5, 7, 1, 3], [4, 6, 1, 1], [1, 3, 5, 7], [1, 1, 4, 6]]
    mat = [[m4[i % 4][j % 4] * (2 if i // 4 == j // 4 else 1) for j in range(16)] for i in range(16)]
    state = [(i * 0x1234567 + 99) % F.P for i in range(16)]
    assert oracle.poseidon_linear("external", state) == _matmul(mat, state)
