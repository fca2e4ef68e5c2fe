"""Whole proofs on the GPU are byte-identical to the oracle's and accepted by its verifier."""
import numpy as np
import pytest

from tests import m31 as F

pytestmark = pytest.mark.gpu


def dev(x):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, np.uint32)).view(np.int32)).cuda()


# Traces of 2^13..2^16 rows interpolate and extend with the shared pass fused (one to four
# layers in it: 13, 14 with blowup 2, 15); smaller ones run the two transforms apart.
@pytest.mark.parametrize("log_n,n_cols,cfg", [(2, 100, (5, 1, 0, 3)), (3, 100, (5, 1, 0, 3)),
                                              (5, 100, (5, 1, 0, 3)), (6, 100, (5, 1, 0, 3)),
                                              (8, 100, (5, 1, 0, 3)), (10, 32, (10, 1, 0, 3)),
                                              (7, 20, (3, 2, 1, 5)), (9, 50, (0, 1, 2, 8)),
                                              (12, 100, (5, 1, 0, 3)), (13, 20, (5, 1, 0, 3)),
                                              (14, 8, (3, 2, 1, 5)), (15, 4, (5, 1, 0, 3))])
def test_wide_fib_proof_bytes_match_oracle(cuda, oracle, log_n, n_cols, cfg):
    from stwo_gb300.prover import prove_wide_fib, wide_fib_trace

    rng = np.random.default_rng(log_n * 1000 + n_cols)
    a = F.rand_m31(rng, 1 << log_n)
    b = F.rand_m31(rng, 1 << log_n)
    want = oracle.prove_wide_fib(log_n, n_cols, a, b, cfg)
    got = prove_wide_fib(log_n, wide_fib_trace(log_n, n_cols, dev(a), dev(b)), cfg)
    assert len(got) == len(want)
    assert got == want
    ok, why = oracle.verify_wide_fib(log_n, n_cols, got)
    assert ok, why


def _random_cases(n, seed):
    """Seeded (log_n, n_cols, (pow_bits, log_blowup, log_last_layer, n_queries)) combinations that
    the reference's FRI verifier accepts: every column's line degree bound (log_n - 1 for the trace)
    above the last layer's (FriVerifier::commit, crates/prover/src/core/fri.rs:356-420)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        log_n = int(rng.integers(2, 13))
        out.append((log_n, int(rng.integers(4, 151)),
                    (int(rng.integers(0, 13)), int(rng.integers(1, 4)), int(rng.integers(0, min(3, log_n - 1))),
                     int(rng.integers(1, 21)))))
    return out


@pytest.mark.parametrize("log_n,n_cols,cfg", _random_cases(8, 2026))
def test_wide_fib_random_configurations_match_oracle(cuda, oracle, log_n, n_cols, cfg):
    """Seeded random sizes, widths and PcsConfigs: bytes equal to the oracle's, verifier accepts."""
    from stwo_gb300.prover import prove_wide_fib, wide_fib_trace

    rng = np.random.default_rng(log_n * 7919 + n_cols)
    a = F.rand_m31(rng, 1 << log_n)
    b = F.rand_m31(rng, 1 << log_n)
    want = oracle.prove_wide_fib(log_n, n_cols, a, b, cfg)
    assert prove_wide_fib(log_n, wide_fib_trace(log_n, n_cols, dev(a), dev(b)), cfg) == want
    ok, why = oracle.verify_wide_fib(log_n, n_cols, want)
    assert ok, why


def test_wide_fib_reference_inputs(cuda, oracle):
    # The reference test's inputs (a = 1, b = row index) at log 2..6.
    from stwo_gb300.prover import prove_wide_fib, wide_fib_trace

    for log_n in range(2, 7):
        n = 1 << log_n
        a, b = np.ones(n, np.uint32), np.arange(n, dtype=np.uint32)
        got = prove_wide_fib(log_n, wide_fib_trace(log_n, 100, dev(a), dev(b)))
        assert got == oracle.prove_wide_fib(log_n, 100, a, b)


@pytest.mark.parametrize("log_n,seeded,cfg", [(4, False, (5, 1, 0, 3)), (5, False, (10, 1, 0, 3)),
                                              (6, True, (5, 1, 0, 3)), (8, True, (3, 2, 1, 4)),
                                              (10, False, (10, 1, 0, 3))])
def test_poseidon_proof_bytes_match_oracle(cuda, oracle, log_n, seeded, cfg):
    from stwo_gb300.prover import prove_poseidon

    init = None
    if seeded:
        rng = np.random.default_rng(log_n)
        init = F.rand_m31(rng, (1 << log_n) * 8 * 16)
    want, want_cs = oracle.prove_poseidon(log_n, init, cfg)
    got, cs = prove_poseidon(log_n, dev(init) if seeded else None, cfg)
    assert cs == want_cs
    assert len(got) == len(want)
    assert got == want
    ok, why = oracle.verify_poseidon(log_n, cs, got)
    assert ok, why


def _random_poseidon_cases(n, seed):
    """Seeded (log_n, cfg) for Poseidon2 proofs within the verifier's rule (last layer bound below
    log_n - 1)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        log_n = int(rng.integers(4, 10))
        out.append((log_n, (int(rng.integers(0, 13)), int(rng.integers(1, 4)), int(rng.integers(0, 3)),
                            int(rng.integers(1, 21)))))
    return out


@pytest.mark.parametrize("log_n,cfg", _random_poseidon_cases(4, 2027))
def test_poseidon_random_configurations_match_oracle(cuda, oracle, log_n, cfg):
    """Seeded random sizes and PcsConfigs over seeded initial states: bytes and claimed sum equal to
    the oracle's, verifier accepts."""
    from stwo_gb300.prover import prove_poseidon

    init = F.rand_m31(np.random.default_rng(log_n * 31 + cfg[3]), (1 << log_n) * 8 * 16)
    want, want_cs = oracle.prove_poseidon(log_n, init, cfg)
    got, cs = prove_poseidon(log_n, dev(init), cfg)
    assert (got, cs) == (want, want_cs)
    ok, why = oracle.verify_poseidon(log_n, cs, got)
    assert ok, why


@pytest.mark.parametrize("log_n", [4, 9])
def test_poseidon_initial_states_from_pinned_host_memory(cuda, oracle, log_n):
    # The trace kernel reads the initial states straight from pinned host memory (16 rows: half a
    # block of 32); the proof equals the one from device memory and the oracle's.
    import torch
    from stwo_gb300.prover import prove_poseidon

    rng = np.random.default_rng(70 + log_n)
    init = F.rand_m31(rng, (1 << log_n) * 8 * 16)
    host = torch.from_numpy(init.view(np.int32)).pin_memory()
    cfg = (5, 1, 0, 3)
    want, want_cs = oracle.prove_poseidon(log_n, init, cfg)
    got_host, cs_host = prove_poseidon(log_n, host, cfg)
    got_dev, cs_dev = prove_poseidon(log_n, dev(init), cfg)
    assert cs_host == cs_dev == want_cs
    assert got_host == got_dev == want


def test_poseidon_headline_size_matches_oracle(cuda, oracle):
    # The benchmarked proof itself: 2^16 rows, seeded states, pow_bits 10 (the same generator as
    # bench.py's workload), byte-identical to the oracle's and accepted by its verifier.
    from stwo_gb300.prover import prove_poseidon
    from tests.golden.cases import words

    log_n, cfg = 16, (10, 1, 0, 3)
    init = words(3, (1 << log_n) * 8 * 16)
    want, want_cs = oracle.prove_poseidon(log_n, init, cfg)
    got, cs = prove_poseidon(log_n, dev(init), cfg)
    assert cs == want_cs
    assert got == want
    ok, why = oracle.verify_poseidon(log_n, cs, got)
    assert ok, why
