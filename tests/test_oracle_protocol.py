"""The oracle's prover and verifier agree (CPU): wide-Fibonacci proofs at the reference test's
sizes (crates/prover/src/examples/wide_fibonacci/mod.rs:174-227, log 2..6 with inputs a = 1,
b = row index) are accepted, and tampered proofs are rejected."""
import numpy as np
import pytest


@pytest.mark.parametrize("log_n", [2, 3, 4, 5, 6, 8])
def test_wide_fib_prove_verify(oracle, log_n):
    n = 1 << log_n
    a = np.ones(n, np.uint32)
    b = np.arange(n, dtype=np.uint32)
    proof = oracle.prove_wide_fib(log_n, 100, a, b)
    ok, why = oracle.verify_wide_fib(log_n, 100, proof)
    assert ok, why


def test_wide_fib_tampered_proofs_rejected(oracle):
    n = 1 << 5
    proof = oracle.prove_wide_fib(5, 100, np.ones(n, np.uint32), np.arange(n, dtype=np.uint32))
    rng = np.random.default_rng(0)
    for pos in rng.integers(0, len(proof), size=12):
        bad = bytearray(proof)
        bad[int(pos)] ^= 0x04
        ok, _ = oracle.verify_wide_fib(5, 100, bytes(bad))
        assert not ok, int(pos)
    assert not oracle.verify_wide_fib(5, 100, proof[:-1])[0]


def test_wide_fib_other_configs(oracle):
    n = 1 << 6
    a = np.full(n, 7, np.uint32)
    b = (np.arange(n, dtype=np.uint32) * 13) % ((1 << 31) - 1)
    for cfg in [(0, 1, 0, 3), (8, 2, 1, 5), (5, 1, 2, 10)]:
        proof = oracle.prove_wide_fib(6, 40, a, b, cfg)
        ok, why = oracle.verify_wide_fib(6, 40, proof)
        assert ok, (cfg, why)


@pytest.mark.parametrize("log_n", [3, 4, 5, 7])
def test_poseidon_prove_verify(oracle, log_n):
    proof, claimed_sum = oracle.prove_poseidon(log_n)
    ok, why = oracle.verify_poseidon(log_n, claimed_sum, proof)
    assert ok, why
    # A wrong claimed sum is rejected by the constraint check at the OODS point.
    bad = ((claimed_sum[0] + 1) % ((1 << 31) - 1),) + claimed_sum[1:]
    assert not oracle.verify_poseidon(log_n, bad, proof)[0]


def test_poseidon_seeded_inputs(oracle):
    rng = np.random.default_rng(3)
    init = rng.integers(0, (1 << 31) - 1, size=(1 << 5) * 8 * 16, dtype=np.int64).astype(np.uint32)
    proof, cs = oracle.prove_poseidon(5, init)
    assert oracle.verify_poseidon(5, cs, proof)[0]


@pytest.mark.parametrize("log_n", [4, 5, 7, 10])
def test_blake_round_prove_verify(oracle, log_n):
    # The reference round test's inputs (crates/prover/src/examples/blake/round/mod.rs:60-110: v_i = i,
    # m_i = i + 1 on every row); prove() itself checks the constraints at the OODS point.
    proof, cs = oracle.prove_blake_round(log_n)
    ok, why = oracle.verify_blake_round(log_n, cs, proof)
    assert ok, why


def test_blake_round_seeded_inputs_and_tampering(oracle):
    rng = np.random.default_rng(3)
    inputs = rng.integers(0, 2**32, (1 << 6) * 32, dtype=np.uint64).astype(np.uint32)
    proof, cs = oracle.prove_blake_round(6, inputs, (3, 2, 1, 5))
    assert oracle.verify_blake_round(6, cs, proof)[0]
    # A different claimed sum changes the transcript (it is mixed before the interaction tree).
    wrong = (cs[0] ^ 1,) + tuple(cs[1:])
    assert not oracle.verify_blake_round(6, wrong, proof)[0]
    for pos in rng.integers(0, len(proof), size=8):
        bad = bytearray(proof)
        bad[int(pos)] ^= 0x10
        assert not oracle.verify_blake_round(6, cs, bytes(bad))[0], int(pos)
    # Other inputs give another claimed sum.
    other = inputs.copy()
    other[5] ^= 1
    assert oracle.prove_blake_round(6, other, (3, 2, 1, 5))[1] != cs
