"""GKR / MLE on the GPU against the oracle: GkrOps::{gen_eq_evals, next_layer,
sum_as_poly_in_first_variable}, MleOps::fix_first_variable and the batch prover
(crates/prover/src/core/lookups/gkr_prover.rs:22-42, :401-516; lookups/mle.rs:9-14), bit-exact,
mirroring the SIMD backend's `*_matches_cpu` and `*_works` tests
(crates/prover/src/core/backend/simd/lookups/gkr.rs:529-690, simd/lookups/mle.rs:105-131).
"""
import numpy as np
import pytest

from tests import m31 as F

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.uint32)).view(np.int32)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint32)


def _sec(a):
    from stwo_gb300.backend import SecureColumn

    return SecureColumn([_dev(a[c]) for c in range(4)])


def _sec_host(col):
    return np.stack([_host(c) for c in col.cols])


def _rq(rng):
    return tuple(int(v) for v in rng.integers(0, F.P, 4))


def _rand(rng, n):
    return rng.integers(0, F.P, (4, n), dtype=np.uint32)


def _layer(rng, kind, log_n):
    n = 1 << log_n
    if kind == 0:
        return [_rand(rng, n)]
    if kind == 1:
        return [_rand(rng, n), _rand(rng, n)]
    if kind == 2:
        return [rng.integers(0, F.P, n, dtype=np.uint32), _rand(rng, n)]
    return [_rand(rng, n)]


def _gpu_layer(kind, cols):
    from stwo_gb300.backend import GkrLayer

    if kind == 0:
        return GkrLayer(0, _sec(cols[0]))
    if kind == 1:
        return GkrLayer(1, _sec(cols[0]), _sec(cols[1]))
    if kind == 2:
        return GkrLayer(2, _dev(cols[0]), _sec(cols[1]))
    return GkrLayer(3, None, _sec(cols[0]))


@pytest.mark.parametrize("n_y", [0, 1, 3, 8, 9, 12, 17])
def test_gen_eq_evals_matches_oracle(cuda, oracle, n_y):
    from stwo_gb300.backend import GkrOps

    rng = np.random.default_rng(n_y)
    y = [_rq(rng) for _ in range(n_y)]
    v = _rq(rng)
    got = _sec_host(GkrOps.gen_eq_evals(y, v))
    assert np.array_equal(got, oracle.gkr_gen_eq_evals(y, v))


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
@pytest.mark.parametrize("log_n", [1, 2, 5, 11, 16])
def test_next_layer_matches_oracle(cuda, oracle, kind, log_n):
    from stwo_gb300.backend import GkrOps

    rng = np.random.default_rng(100 * kind + log_n)
    cols = _layer(rng, kind, log_n)
    nxt = GkrOps.next_layer(_gpu_layer(kind, cols))
    want = oracle.gkr_next_layer(kind, cols)
    assert np.array_equal(_sec_host(nxt.num), want[0])
    if kind != 0:
        assert np.array_equal(_sec_host(nxt.den), want[1])


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
@pytest.mark.parametrize("log_n,extra", [(2, 0), (3, 2), (7, 0), (12, 3), (17, 1)])
def test_sum_as_poly_matches_oracle(cuda, oracle, kind, log_n, extra):
    from stwo_gb300.backend import GkrOps

    rng = np.random.default_rng(1000 + 10 * kind + log_n)
    cols = _layer(rng, kind, log_n)
    y = [_rq(rng) for _ in range(log_n - 1 + extra)]
    lam, corr, claim = _rq(rng), _rq(rng), _rq(rng)
    # EqEvals::generate(y) (gkr_prover.rs:58-69): gen_eq_evals(y[1..], eq([0], [y0])).
    eq = GkrOps.gen_eq_evals(y[1:], F.q_sub((1, 0, 0, 0), y[0]))
    got = GkrOps.sum_as_poly_in_first_variable(_gpu_layer(kind, cols), eq, y, lam, corr, claim)
    want = oracle.gkr_sum_as_poly(kind, cols, y, lam, corr, claim)
    assert got == want


@pytest.mark.parametrize("log_n", [1, 2, 6, 13, 19])
def test_fix_first_variable_matches_oracle(cuda, oracle, log_n):
    from stwo_gb300.backend import GkrOps

    rng = np.random.default_rng(log_n)
    a = _rq(rng)
    sec = _rand(rng, 1 << log_n)
    base = rng.integers(0, F.P, 1 << log_n, dtype=np.uint32)
    assert np.array_equal(_sec_host(GkrOps.fix_first_variable(_sec(sec), a)), oracle.mle_fix_first_variable(sec, a))
    assert np.array_equal(_sec_host(GkrOps.fix_first_variable(_dev(base), a)), oracle.mle_fix_first_variable(base, a))


def test_fix_first_variable_in_place(cuda, oracle):
    import ctypes as C

    from stwo_gb300 import _lib
    from stwo_gb300.backend import _ptrs, _q, _stream

    rng = np.random.default_rng(77)
    sec = _rand(rng, 1 << 10)
    a = _rq(rng)
    col = _sec(sec)
    _lib.call("stwo_mle_fix_first_variable_secure", 10, _ptrs(col.cols), _q(a), _ptrs(col.cols), _stream())
    got = _sec_host(col)[:, : 1 << 9]
    assert np.array_equal(got, oracle.mle_fix_first_variable(sec, a))
    del C


def _prove_both(oracle, layers_np, digest=None):
    from stwo_gb300.backend import GkrOps

    gpu = [_gpu_layer(k, cols) for k, cols in layers_np]
    got, dg = GkrOps.prove_batch(gpu, digest)
    want, dw = oracle.gkr_prove(layers_np, digest)
    return got, want, dg, dw


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
@pytest.mark.parametrize("log_n", [1, 2, 3, 6, 10])
def test_prove_batch_matches_oracle(cuda, oracle, kind, log_n):
    if kind == 2 and log_n == 1:
        pytest.skip("a one-variable multiplicities layer has no mask (gkr_prover.rs:336-337)")
    rng = np.random.default_rng(10 * kind + log_n)
    layers = [(kind, _layer(rng, kind, log_n))]
    got, want, dg, dw = _prove_both(oracle, layers)
    assert got == want and dg == dw
    ok, why = oracle.gkr_verify(layers, got)
    assert ok, why


def test_grand_product_from_channel_felts(cuda, oracle):
    # cpu/lookups/gkr.rs:318-336: the input is test_channel().draw_felts(32).
    felts = oracle.channel_draw_felts(32)
    layers = [(0, [np.ascontiguousarray(felts.T)])]
    got, want, _, _ = _prove_both(oracle, layers)
    assert got == want
    assert oracle.gkr_verify(layers, got)[0]


def test_mixed_batch_with_digest(cuda, oracle):
    rng = np.random.default_rng(31)
    layers = [(1, _layer(rng, 1, 9)), (0, _layer(rng, 0, 4)), (3, _layer(rng, 3, 11)), (2, _layer(rng, 2, 6)),
              (1, _layer(rng, 1, 2))]
    digest = bytes((7 * i + 3) % 256 for i in range(32))
    got, want, dg, dw = _prove_both(oracle, layers, digest)
    assert got == want and dg == dw
    ok, why = oracle.gkr_verify(layers, got, digest)
    assert ok, why


def test_inputs_unchanged_and_repeatable(cuda, oracle):
    from stwo_gb300.backend import GkrOps

    rng = np.random.default_rng(41)
    cols = _layer(rng, 1, 12)
    layer = _gpu_layer(1, cols)
    a, _ = GkrOps.prove_batch([layer])
    assert np.array_equal(_sec_host(layer.num), cols[0]) and np.array_equal(_sec_host(layer.den), cols[1])
    b, _ = GkrOps.prove_batch([layer])
    assert a == b


def test_logup_generic_2_18_matches_oracle(cuda, oracle):
    rng = np.random.default_rng(18)
    layers = [(1, _layer(rng, 1, 18))]
    got, want, _, _ = _prove_both(oracle, layers)
    assert got == want


def test_logup_generic_2_20_verifies(cuda, oracle):
    # The 2^20-leaf workload (16 Poseidon relation fractions per row at 2^16 rows): the oracle
    # verifier accepts the GPU proof and its claims match the input layer at the GKR point.
    rng = np.random.default_rng(20)
    layers = [(1, _layer(rng, 1, 20))]
    from stwo_gb300.backend import GkrOps

    got, _ = GkrOps.prove_batch([_gpu_layer(1, layers[0][1])])
    ok, why = oracle.gkr_verify(layers, got)
    assert ok, why


def test_rejects_bad_arguments(cuda):
    from stwo_gb300 import _lib
    from stwo_gb300.backend import GkrLayer, GkrOps

    rng = np.random.default_rng(1)
    with pytest.raises(_lib.StwoError):
        GkrOps.prove_batch([GkrLayer(2, _dev(rng.integers(0, F.P, 2, dtype=np.uint32)), _sec(_rand(rng, 2)))])
    with pytest.raises(_lib.StwoError):
        GkrOps.prove_batch([GkrLayer(7, None, _sec(_rand(rng, 4)))])


def test_large_mixed_batch(cuda, oracle):
    # 66 instances of three kinds and sizes 2..4 in one batch.
    rng = np.random.default_rng(65)
    layers = [(k % 4 if k % 4 != 2 else 1, _layer(rng, k % 4 if k % 4 != 2 else 1, 2 + k % 3)) for k in range(66)]
    got, want, dg, dw = _prove_both(oracle, layers)
    assert got == want and dg == dw
