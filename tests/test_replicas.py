"""The multi-GPU path is independent replicas: two gloo ranks on the CPU check the timing
collectives (barrier, max over ranks) and the whole-job rate that bench.py reports for N > 1."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    from stwo_gb300 import replicas

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ranks = replicas.Ranks.from_env()
        replicas.barrier(ranks, cuda=False)
        step_s = 0.010 + 0.005 * rank  # rank 1 is the slower replica
        slowest = replicas.max_over_ranks(step_s, ranks, device="cpu")
        out.put((rank, slowest, replicas.whole_job_rate(84934656, ranks, slowest)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_agree_on_timing():
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    assert [r for r, _, _ in res] == [0, 1]
    for _, slowest, rate in res:
        assert slowest == pytest.approx(0.015)
        assert rate == pytest.approx(84934656 * 2 / 0.015)


def test_single_rank_needs_no_process_group():
    from stwo_gb300 import replicas

    ranks = replicas.Ranks(1, 0, 0)
    assert replicas.max_over_ranks(0.5, ranks) == 0.5
    assert replicas.whole_job_rate(10, ranks, 2.0) == 5.0
