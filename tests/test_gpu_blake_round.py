"""The Blake2s round AIR on the GPU: proofs byte-identical to the oracle's and accepted by its
verifier, with the reference round test's inputs (crates/prover/src/examples/blake/round/mod.rs:
60-110) and with seeded inputs; the same proofs through the batch server."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(x):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, np.uint32)).view(np.int32)).cuda()


# Up to 2^15 rows the interaction trace runs one warp per G-function, above it one thread per row:
# 2^16 covers the second schedule.
@pytest.mark.parametrize("log_n,seeded,cfg", [(4, False, (5, 1, 0, 3)), (5, True, (5, 1, 0, 3)),
                                              (7, True, (3, 2, 1, 5)), (10, False, (10, 1, 0, 3)),
                                              (12, True, (10, 1, 0, 3)), (16, True, (5, 1, 0, 3))])
def test_blake_round_proof_bytes_match_oracle(cuda, oracle, log_n, seeded, cfg):
    from stwo_gb300.prover import prove_blake_round

    inputs = None
    if seeded:
        rng = np.random.default_rng(100 + log_n)
        inputs = rng.integers(0, 2**32, (1 << log_n) * 32, dtype=np.uint64).astype(np.uint32)
    want, want_cs = oracle.prove_blake_round(log_n, inputs, cfg)
    got, cs = prove_blake_round(log_n, dev(inputs) if seeded else None, cfg)
    assert cs == want_cs
    assert len(got) == len(want)
    assert got == want
    ok, why = oracle.verify_blake_round(log_n, cs, got)
    assert ok, why


def test_blake_round_jobs_in_a_batch(cuda, oracle):
    from stwo_gb300.prover import AIR_BLAKE_ROUND, Job, prove_batch, prove_blake_round

    rng = np.random.default_rng(7)
    jobs, singles = [], []
    for log_n in (6, 9, 8):
        inputs = dev(rng.integers(0, 2**32, (1 << log_n) * 32, dtype=np.uint64).astype(np.uint32))
        jobs.append(Job(AIR_BLAKE_ROUND, log_n, (5, 1, 0, 3), init=inputs))
        singles.append(prove_blake_round(log_n, inputs, (5, 1, 0, 3)))
    res = prove_batch(jobs, n_workers=3)
    for r, (proof, cs) in zip(res, singles):
        assert r.proof == proof
        assert tuple(r.claimed_sum) == cs
