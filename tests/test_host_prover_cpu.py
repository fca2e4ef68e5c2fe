"""The host-side pieces of stwo_gb300/host_prover.py against the oracle, without a GPU: the raw
Blake2s compression, the channel's draws, QM31 products and inverses, circle points and the line
interpolation of the last FRI layer."""
import numpy as np

from tests import m31 as F


def test_blake2s_compress_matches_oracle(oracle):
    from stwo_gb300.host_prover import blake2s_compress

    rng = np.random.default_rng(10)
    for t0, t1, f0, f1 in [(0, 0, 0, 0), (64, 0, 0xFFFFFFFF, 0), (123456, 7, 0, 0xFFFFFFFF)]:
        h = [int(x) for x in rng.integers(0, 1 << 32, 8)]
        m = [int(x) for x in rng.integers(0, 1 << 32, 16)]
        assert blake2s_compress(h, m, t0, t1, f0, f1) == oracle.raw_compress(h, m, t0, t1, f0, f1)


def test_channel_draws_match_oracle(oracle):
    from stwo_gb300.host_prover import Blake2sChannel

    ch = Blake2sChannel()
    want = oracle.channel_draw_felts(9)
    assert ch.draw_felts(9) == [tuple(int(x) for x in r) for r in want]


def test_field_and_circle_ops_match_oracle(oracle):
    from stwo_gb300.host_prover import index_to_point, q_inv, q_mul

    rng = np.random.default_rng(11)
    for _ in range(20):
        a = tuple(int(x) for x in rng.integers(0, F.P, 4))
        b = tuple(int(x) for x in rng.integers(0, F.P, 4))
        assert q_mul(a, b) == oracle.qm31_mul(a, b)
        assert q_inv(a) == oracle.qm31_inv(a)
        assert q_mul(a, q_inv(a)) == (1, 0, 0, 0)
    for idx in [0, 1, 2, 12345, (1 << 30) + 7, (1 << 31) - 1]:
        assert index_to_point(idx) == oracle.index_to_point(idx)


def test_line_interpolate_inverts_line_evaluation(oracle):
    """The last-layer interpolation recovers a polynomial of degree < 2 in the x-coordinate from
    its evaluations on a line domain of 4 points: f(x) = c0 + c1 * x has bit-reversed coefficients
    [c0, c1] (the line FFT basis of degree 1 is 1, x), the two other coefficients zero."""
    from stwo_gb300.circle import half_odds
    from stwo_gb300.host_prover import _bit_reverse, _line_interpolate, index_to_point, q_add, q_m31, q_mul

    dom = half_odds(2)
    c0, c1 = (5, 6, 7, 8), (1, 2, 3, 4)
    xs = [index_to_point(dom.initial_index + i * dom.step_size)[0] for i in range(4)]
    vals = _bit_reverse([q_add(c0, q_mul(c1, q_m31(x))) for x in xs])
    coeffs = _bit_reverse(_line_interpolate(dom, vals))
    assert coeffs[0] == c0 and coeffs[1] == c1 and coeffs[2:] == [(0, 0, 0, 0)] * 2
