"""Batched and served proving (stwo_prove_batch, stwo_server_*): proofs made concurrently on a
worker pool are byte-identical to single-call proofs and accepted by the oracle verifier; the
HBM-budget admission and the wait order do not change results; a failing job reports its error
without disturbing the others."""
import numpy as np
import pytest

from tests.golden import cases

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.uint32)).view(np.int32)).cuda()


def _jobs():
    from stwo_gb300.prover import AIR_POSEIDON, AIR_WIDE_FIB, Job

    specs = [("wf", 5, 16, 21, (5, 1, 0, 3)), ("ps", 4, None, None, (5, 1, 0, 3)), ("wf", 8, 100, 22, (5, 1, 0, 3)),
             ("ps", 5, None, 23, (10, 1, 0, 3)), ("wf", 6, 16, 24, (3, 2, 1, 5)), ("ps", 6, None, 25, (5, 1, 0, 3))]
    jobs = []
    for kind, log, cols, seed, cfg in specs:
        n = 1 << log
        if kind == "wf":
            jobs.append(Job(AIR_WIDE_FIB, log, cfg, n_cols=cols, a=_dev(cases.words(seed, n)),
                            b=_dev(cases.words(seed + 1, n))))
        else:
            init = _dev(cases.words(seed, n * 128)) if seed else None
            jobs.append(Job(AIR_POSEIDON, log, cfg, init=init))
    return jobs


def _single(job):
    from stwo_gb300.prover import AIR_WIDE_FIB, prove_poseidon, prove_wide_fib, wide_fib_trace

    if job.air == AIR_WIDE_FIB:
        return prove_wide_fib(job.log_n_rows, wide_fib_trace(job.log_n_rows, job.n_cols, job.a, job.b), job.cfg)
    return prove_poseidon(job.log_n_rows, job.init, job.cfg)[0]


def test_batch_matches_single_calls_and_verifies(cuda, oracle):
    from stwo_gb300.prover import AIR_WIDE_FIB, prove_batch

    jobs = _jobs()
    results = prove_batch(jobs, n_workers=4)
    for job, r in zip(jobs, results):
        assert r.proof == _single(job)
        if job.air == AIR_WIDE_FIB:
            a = job.a.cpu().numpy().view(np.uint32)
            b = job.b.cpu().numpy().view(np.uint32)
            assert r.proof == oracle.prove_wide_fib(job.log_n_rows, job.n_cols, a, b, job.cfg)
        else:
            ok, why = oracle.verify_poseidon(job.log_n_rows, r.claimed_sum, r.proof)
            assert ok, why


def test_server_wait_order_and_tiny_budget(cuda):
    from stwo_gb300.prover import Server

    jobs = _jobs()
    want = [_single(j) for j in jobs]
    with Server(n_workers=3) as srv:
        tickets = [srv.submit(j) for j in jobs]
        got = {t: srv.wait(t).proof for t in reversed(tickets)}
    assert [got[t] for t in tickets] == want
    # A 1-byte budget admits one job at a time; results are unchanged.
    jobs = _jobs()
    with Server(n_workers=4, hbm_budget=1) as srv:
        rs = [srv.wait(t) for t in [srv.submit(j) for j in jobs]]
    assert [r.proof for r in rs] == want
    assert all(r.latency_ms >= r.run_ms >= 0 for r in rs)


def test_failing_job_reports_error(cuda):
    from stwo_gb300 import _lib
    from stwo_gb300.prover import AIR_WIDE_FIB, Job, Server

    jobs = _jobs()
    bad = Job(AIR_WIDE_FIB, 5, n_cols=2, a=jobs[0].a, b=jobs[0].b)
    with Server(n_workers=2) as srv:
        t_bad = srv.submit(bad)
        t_ok = srv.submit(jobs[0])
        with pytest.raises(_lib.StwoError):
            srv.wait(t_bad)
        assert srv.wait(t_ok).proof == _single(jobs[0])


def test_admission_estimate_grows_with_size(cuda):
    from stwo_gb300.prover import AIR_POSEIDON, Job

    small, big = Job(AIR_POSEIDON, 8), Job(AIR_POSEIDON, 16)
    assert 0 < small.hbm_bytes() < big.hbm_bytes()
    assert big.hbm_bytes() > 2 << 30  # a 2^16-row Poseidon2 proof holds ~3 GB


def test_server_priority_levels_keep_results(cuda):
    """Jobs of every stream-priority class at once (under 256 MB, under 2 GB, and two large ones
    that overlap) give the same proofs as single calls."""
    from stwo_gb300.prover import AIR_POSEIDON, AIR_WIDE_FIB, Job, Server

    jobs = [Job(AIR_POSEIDON, 16, (10, 1, 0, 3), init=_dev(cases.words(31, (1 << 16) * 128))),
            Job(AIR_POSEIDON, 6, (5, 1, 0, 3), init=_dev(cases.words(32, (1 << 6) * 128))),
            Job(AIR_POSEIDON, 13, (10, 1, 0, 3), init=_dev(cases.words(33, (1 << 13) * 128))),
            Job(AIR_POSEIDON, 16, (10, 1, 0, 3), init=_dev(cases.words(34, (1 << 16) * 128))),
            Job(AIR_WIDE_FIB, 8, (5, 1, 0, 3), n_cols=100, a=_dev(cases.words(35, 256)), b=_dev(cases.words(36, 256)))]
    sizes = [j.hbm_bytes() for j in jobs]
    assert sizes[1] < 256 << 20 and sizes[4] < 256 << 20
    assert 256 << 20 <= sizes[2] < 2 << 30
    assert sizes[0] >= 2 << 30 and sizes[3] >= 2 << 30
    want = [_single(j) for j in jobs]
    with Server(n_workers=5) as srv:
        rs = [srv.wait(t) for t in [srv.submit(j) for j in jobs]]
    assert [r.proof for r in rs] == want
