"""Parity of every CUDA backend op with the oracle, bit for bit, through the C ABI.

Sizes cover the reference's branch boundaries (log <= 2 special cases, the SIMD backend's
MIN_FFT_LOG_SIZE = 5 and CACHED_FFT_LOG_SIZE = 16 boundaries, the 2^13 shared-memory tile of
this backend, multi-pass logs) and edge inputs (0 and P-1 words, empty column sets).
"""
import numpy as np
import pytest

from tests import m31 as F

pytestmark = pytest.mark.gpu


def dev(x):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, np.uint32)).view(np.int32)).cuda()


def host(t):
    return t.cpu().numpy().view(np.uint32)


def rq(rng):
    return tuple(int(v) for v in rng.integers(0, F.P, 4))


def rand_point(oracle, rng):
    t = rq(rng)
    t2 = F.q_mul(t, t)
    d = oracle.qm31_inv(F.q_add(t2, F.q(1)))
    return (F.q_mul(F.q_sub(F.q(1), t2), d), F.q_mul(F.q_add(t, t), d))


@pytest.mark.parametrize("root", [F.canonic_half(1), F.canonic_half(5), F.canonic_half(14),
                                  (12345, 1 << 22, 9), (3 << 18, 1 << 22, 9)])
def test_twiddle_tree(cuda, oracle, root):
    import ctypes as C

    from stwo_gb300 import _lib
    from stwo_gb300.backend import TwiddleTree

    t = TwiddleTree(_lib.Coset(*root))
    tw_p, itw_p, n = t.arrays()
    import torch

    torch.cuda.synchronize()
    got = np.zeros(n, np.uint32)
    igot = np.zeros(n, np.uint32)
    _lib.call("stwo_buf_download", got.ctypes.data_as(C.c_void_p), tw_p, n * 4, None)
    _lib.call("stwo_buf_download", igot.ctypes.data_as(C.c_void_p), itw_p, n * 4, None)
    tw, itw = oracle.twiddles(root)
    assert np.array_equal(got, tw)
    assert np.array_equal(igot, itw)


@pytest.mark.parametrize("log", [1, 2, 3, 4, 5, 6, 7, 8, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22])
def test_interpolate(cuda, oracle, log):
    from stwo_gb300 import _lib
    from stwo_gb300.backend import TwiddleTree

    rng = np.random.default_rng(100 + log)
    half = F.canonic_half(log)
    ncols = 3
    vals = [F.rand_m31(rng, 1 << log) for _ in range(ncols)]
    vals[0][:4] = [0, F.P - 1, 1, F.P - 1][: min(4, 1 << log)]
    # The domain's own tree, and the tree of a bigger canonic tower (H_{L+2} doubles into H_L).
    for root in (half, F.canonic_half(log + 2)):
        t = TwiddleTree(_lib.Coset(*root))
        cols = [dev(v) for v in vals]
        cuda.interpolate_columns(cols, _lib.Coset(*half), t)
        for c, v in zip(cols, vals):
            assert np.array_equal(host(c), oracle.interpolate(half, half, v))


@pytest.mark.parametrize("coeff_log,log", [(1, 1), (1, 3), (2, 2), (3, 5), (5, 5), (4, 9), (10, 11), (12, 14),
                                           (13, 13), (14, 16), (16, 17), (17, 19), (18, 20), (16, 20), (20, 22)])
def test_evaluate(cuda, oracle, coeff_log, log):
    from stwo_gb300 import _lib
    from stwo_gb300.backend import TwiddleTree

    rng = np.random.default_rng(200 + coeff_log * 31 + log)
    half = F.canonic_half(log)
    coeffs = [F.rand_m31(rng, 1 << coeff_log) for _ in range(2)]
    t = TwiddleTree(_lib.Coset(*F.canonic_half(log + 1)))
    out = cuda.evaluate_polynomials([dev(c) for c in coeffs], _lib.Coset(*half), t)
    for o, c in zip(out, coeffs):
        assert np.array_equal(host(o), oracle.evaluate(half, half, c))


def test_interpolate_non_canonic_domain(cuda, oracle):
    # A sub-domain as used by the quotient extension: half coset (init of log 12, log 10).
    from stwo_gb300 import _lib
    from stwo_gb300.backend import TwiddleTree

    rng = np.random.default_rng(5)
    dom = F.canonic_half(12)
    half = (dom[0], 1 << (31 - 10), 10)
    v = F.rand_m31(rng, 1 << 11)
    t = TwiddleTree(_lib.Coset(*half))
    c = dev(v)
    cuda.interpolate_columns([c], _lib.Coset(*half), t)
    assert np.array_equal(host(c), oracle.interpolate(half, half, v))


@pytest.mark.parametrize("log", [0, 1, 3, 8, 9, 13, 15, 16, 17, 18, 20])
def test_eval_at_points(cuda, oracle, log):
    rng = np.random.default_rng(300 + log)
    polys = [F.rand_m31(rng, 1 << log) for _ in range(3)]
    queries = [(i % 3, rand_point(oracle, rng)) for i in range(5)]
    got = cuda.eval_at_points([dev(p) for p in polys], queries)
    for (pi, pt), g in zip(queries, got):
        assert g == oracle.eval_at_point(polys[pi], pt)


# Layers of at most 2^13 nodes take the latency kernel, larger ones (log 14, 17, 19) the throughput
# kernel.
@pytest.mark.parametrize("log,ncols,prev", [(0, 0, False), (0, 0, True), (3, 1, False), (4, 15, True),
                                            (5, 16, False), (5, 17, True), (7, 100, False), (10, 0, True),
                                            (9, 256, True), (2, 33, False), (6, 1300, False), (12, 4, True),
                                            (3, 3100, True), (2, 6200, False), (14, 37, True), (17, 20, False),
                                            (19, 3, True)])
def test_merkle_layer(cuda, oracle, log, ncols, prev):
    import torch

    rng = np.random.default_rng(400 + log * 7 + ncols)
    n = 1 << log
    cols = [F.rand_m31(rng, n) for _ in range(ncols)]
    prev_np = rng.integers(0, 1 << 32, size=(2 * n, 8), dtype=np.uint64).astype(np.uint32) if prev else None
    got = cuda.commit_on_layer(log, dev(prev_np) if prev else None, [dev(c) for c in cols])
    torch.cuda.synchronize()
    want = oracle.commit_on_layer(log, prev_np, cols)
    assert np.array_equal(host(got).reshape(-1, 8), want)


@pytest.mark.parametrize("log", [1, 2, 3, 4, 5, 10, 15, 21, 22])
def test_fold_line(cuda, oracle, log):
    from stwo_gb300 import _lib
    from stwo_gb300.backend import SecureColumn, TwiddleTree

    rng = np.random.default_rng(500 + log)
    # Line domain: the half coset of the canonic domain of log+1; tree rooted at a bigger tower.
    line = F.canonic_half(log + 1)
    t = TwiddleTree(_lib.Coset(*F.canonic_half(log + 3)))
    src = [F.rand_m31(rng, 1 << log) for _ in range(4)]
    alpha = rq(rng)
    out = cuda.fold_line(SecureColumn([dev(c) for c in src]), _lib.Coset(*line), alpha, t)
    want = oracle.fold_line(line, src, alpha)
    for k in range(4):
        assert np.array_equal(host(out.cols[k]), want[k])


@pytest.mark.parametrize("log", [1, 2, 3, 4, 6, 12, 16, 21, 22])
def test_fold_circle_into_line(cuda, oracle, log):
    from stwo_gb300 import _lib
    from stwo_gb300.backend import SecureColumn, TwiddleTree

    rng = np.random.default_rng(600 + log)
    half = F.canonic_half(log)
    t = TwiddleTree(_lib.Coset(*F.canonic_half(log + 1)))
    src = [F.rand_m31(rng, 1 << log) for _ in range(4)]
    dst = [F.rand_m31(rng, 1 << (log - 1)) for _ in range(4)]
    alpha = rq(rng)
    d = SecureColumn([dev(c) for c in dst])
    cuda.fold_circle_into_line(d, SecureColumn([dev(c) for c in src]), _lib.Coset(*half), alpha, t)
    want = oracle.fold_circle_into_line(half, dst, src, alpha)
    for k in range(4):
        assert np.array_equal(host(d.cols[k]), want[k])


@pytest.mark.parametrize("log", [4, 5, 11])
def test_decompose(cuda, oracle, log):
    from stwo_gb300.backend import SecureColumn

    rng = np.random.default_rng(700 + log)
    src = [F.rand_m31(rng, 1 << log) for _ in range(4)]
    g, lam = cuda.decompose(SecureColumn([dev(c) for c in src]))
    wg, wlam = oracle.decompose(src)
    assert lam == wlam
    for k in range(4):
        assert np.array_equal(host(g.cols[k]), wg[k])


# Sub-domains below 4 x 128 rows per SM take two rows per lane, larger ones four (log 18, blowup 1);
# sub-domains of 2^13..2^16 rows interpolate and extend with the shared pass fused (log 15).
@pytest.mark.parametrize("log_n,blowup,ncols,npts", [(3, 1, 2, 1), (6, 1, 3, 2), (7, 1, 5, 2), (8, 2, 4, 3),
                                                      (10, 1, 40, 2), (12, 1, 7, 1), (13, 3, 9, 2), (15, 1, 3, 2),
                                                      (18, 1, 3, 2)])
def test_accumulate_quotients(cuda, oracle, log_n, blowup, ncols, npts):
    rng = np.random.default_rng(800 + log_n * 13 + ncols)
    cols = [F.rand_m31(rng, 1 << log_n) for _ in range(ncols)]
    pts = sorted(rand_point(oracle, rng) for _ in range(npts))
    batches = []
    for bi, pt in enumerate(pts):
        sel = [c for c in range(ncols) if (c + bi) % 2 == 0 or npts == 1]
        batches.append((pt, [(c, rq(rng)) for c in sel]))
    rc = rq(rng)
    out = cuda.accumulate_quotients(log_n, [dev(c) for c in cols], rc, batches, blowup)
    want = oracle.accumulate_quotients(log_n, cols, rc, batches, blowup)
    for k in range(4):
        assert np.array_equal(host(out.cols[k]), want[k])


def test_secure_powers_and_accumulate(cuda, oracle):
    from stwo_gb300.backend import SecureColumn

    rng = np.random.default_rng(900)
    felt = rq(rng)
    assert cuda.generate_secure_powers(felt, 1000) == oracle.secure_powers(felt, 1000)
    a = [F.rand_m31(rng, 1000) for _ in range(4)]
    b = [F.rand_m31(rng, 1000) for _ in range(4)]
    A = SecureColumn([dev(x) for x in a])
    cuda.accumulate(A, SecureColumn([dev(x) for x in b]))
    for k in range(4):
        assert np.array_equal(host(A.cols[k]), ((a[k].astype(np.uint64) + b[k]) % F.P).astype(np.uint32))


@pytest.mark.parametrize("pow_bits", [0, 1, 5, 10, 16])
def test_grind(cuda, oracle, pow_bits):
    digest = [0x12345678 * (i + 1) & 0xFFFFFFFF for i in range(8)]
    assert cuda.grind(digest, pow_bits) == oracle.grind(digest, pow_bits)


def test_bit_reverse_and_extend(cuda):
    rng = np.random.default_rng(1000)
    v = F.rand_m31(rng, 1 << 10)
    c = dev(v)
    cuda.bit_reverse_column(c)
    idx = [F.brev(i, 10) for i in range(1 << 10)]
    assert np.array_equal(host(c), v[idx])
    e = cuda.extend(dev(v), 12)
    assert np.array_equal(host(e)[: 1 << 10], v) and not host(e)[1 << 10:].any()


def test_invalid_arguments_return_status(cuda):
    from stwo_gb300 import _lib
    from stwo_gb300.backend import TwiddleTree

    # A coset containing a point with x = 0 has no inverse twiddles (the reference panics).
    with pytest.raises(_lib.StwoError) as e:
        TwiddleTree(_lib.Coset(1 << 20, 1 << 21, 10))
    assert e.value.status == 1

    t = TwiddleTree(_lib.Coset(*F.canonic_half(5)))
    # A domain that is not a doubling of the tree's root is rejected, not computed.
    with pytest.raises(_lib.StwoError) as e:
        cuda.interpolate_columns([dev(np.zeros(1 << 7, np.uint32))], _lib.Coset(*F.canonic_half(7)), t)
    assert e.value.status == 1
    with pytest.raises(_lib.StwoError):
        cuda.grind([0] * 8, 33)


@pytest.mark.parametrize("shift", [1, 2])
def test_accumulate_quotients_unaligned_columns(cuda, oracle, shift):
    """Columns that start 4 bytes past a 16-byte boundary take the one-row-per-lane kernel, and 8
    bytes past it the two-rows-per-lane kernel; the result is the same."""
    rng = np.random.default_rng(811)
    log_n, blowup, ncols = 12, 1, 9
    cols = [F.rand_m31(rng, 1 << log_n) for _ in range(ncols)]
    pts = sorted(rand_point(oracle, rng) for _ in range(2))
    batches = [(pts[0], [(c, rq(rng)) for c in range(ncols)]), (pts[1], [(c, rq(rng)) for c in range(0, ncols, 3)])]
    rc = rq(rng)
    shifted = [dev(np.concatenate([np.zeros(shift, np.uint32), c]))[shift:] for c in cols]
    assert all(t.data_ptr() % 16 == 4 * shift for t in shifted)
    out = cuda.accumulate_quotients(log_n, shifted, rc, batches, blowup)
    want = oracle.accumulate_quotients(log_n, cols, rc, batches, blowup)
    for k in range(4):
        assert np.array_equal(host(out.cols[k]), want[k])


def test_butterfly_rate_diagnostic(cuda):
    """The butterfly probe reports a positive event-timed rate and an issue cost in SM cycles that
    is consistent with it: the rate cannot exceed what every scheduler issuing one warp-butterfly
    per that many cycles at the maximum SM clock allows."""
    import ctypes as C

    import torch
    from stwo_gb300 import _lib

    rate, cyc, mhz = C.c_double(), C.c_double(), C.c_double()
    _lib.call("stwo_butterfly_rate", 64, C.byref(rate), C.byref(cyc), C.byref(mhz), None)
    assert rate.value > 0 and 4.0 < cyc.value < 200.0 and 100.0 < mhz.value < 3000.0
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert rate.value <= 4 * sms * mhz.value * 1.05e6 * 32 / cyc.value
    with pytest.raises(_lib.StwoError):
        _lib.call("stwo_butterfly_rate", 0, C.byref(rate), None, None, None)


def test_blake2s_rate_diagnostic(cuda):
    """The BLAKE2s probe: a positive rate, an issue cost per warp-wide compression of at least its
    ~1,100 integer operations spread over the scheduler's pipes, and a consistent clock."""
    import ctypes as C

    import torch
    from stwo_gb300 import _lib

    rate, cyc, mhz = C.c_double(), C.c_double(), C.c_double()
    _lib.call("stwo_blake2s_rate", 16, C.byref(rate), C.byref(cyc), C.byref(mhz), None)
    assert rate.value > 0 and 100.0 < cyc.value < 20000.0 and 100.0 < mhz.value < 3000.0
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert rate.value <= 4 * sms * mhz.value * 1.05e6 * 32 / cyc.value


def test_autotuned_shapes_give_the_same_results(cuda, oracle):
    """In tune mode the Merkle layer and the quotient row pass time their candidate shapes on the
    call's own data; the results still equal the oracle's, and the table records one of the
    candidates for each size."""
    import torch
    from stwo_gb300 import autotune

    autotune.clear()
    autotune.set_mode(autotune.TUNE)
    try:
        rng = np.random.default_rng(4242)
        for log, ncols in [(11, 20), (14, 5)]:
            n = 1 << log
            cols = [F.rand_m31(rng, n) for _ in range(ncols)]
            got = cuda.commit_on_layer(log, None, [dev(c) for c in cols])
            torch.cuda.synchronize()
            assert np.array_equal(host(got).reshape(-1, 8), oracle.commit_on_layer(log, None, cols))
        log_n, blowup = 13, 1
        cols = [F.rand_m31(rng, 1 << log_n) for _ in range(6)]
        pts = sorted(rand_point(oracle, rng) for _ in range(2))
        batches = [(pts[0], [(c, rq(rng)) for c in range(6)]), (pts[1], [(c, rq(rng)) for c in range(0, 6, 2)])]
        rc = rq(rng)
        out = cuda.accumulate_quotients(log_n, [dev(c) for c in cols], rc, batches, blowup)
        want = oracle.accumulate_quotients(log_n, cols, rc, batches, blowup)
        for k in range(4):
            assert np.array_equal(host(out.cols[k]), want[k])
        table = autotune.entries()
        merkle = [e for e in table if e["site"] == 1]
        quot = [e for e in table if e["site"] == 2]
        assert len(merkle) == 2 and all(e["choice"] in (0, 1, 2, 3, 4) for e in merkle)
        assert len(quot) == 1 and quot[0]["choice"] in (1, 2, 4)
        # With the table in use, the same calls give the same results again.
        autotune.set_mode(autotune.USE)
        out2 = cuda.accumulate_quotients(log_n, [dev(c) for c in cols], rc, batches, blowup)
        for k in range(4):
            assert np.array_equal(host(out2.cols[k]), want[k])
    finally:
        autotune.set_mode(autotune.OFF)
        autotune.clear()
