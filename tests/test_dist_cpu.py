"""The multi-rank path of bench.py on CPU: two gloo ranks (world size 2).

Pairs are independent, so ranks share no data: each registers its own batch (its
own seed) and the only collectives are the barriers around the timed region and the
max-reduce of the step time (weak scaling: value = world x pairs / max time).  The
reference arm runs on rank 0 only."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    import torch.distributed as dist

    r, w = bench.dist_init("gloo")
    bench.barrier()
    step_ms = 10.0 + 5.0 * rank  # rank 1 is the slower one
    ms = bench.reduce_max(step_ms)
    total = bench.reduce_sum(1.0)
    value = w * 64 / (ms / 1000.0)
    # the reference arm does nothing on ranks other than 0
    ran_reference = None
    if rank != 0:
        class A:
            pairs, seed, steps, warmup = 64, 0, 1, 0

        bench.run_reference(A())
        ran_reference = False
    bench.barrier()
    q.put((r, w, ms, total, value, bench.rank_seed(0, r), ran_reference))
    dist.destroy_process_group()


def test_two_gloo_ranks_weak_scaling():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, ms0, tot0, v0, s0, _), (r1, w1, ms1, tot1, v1, s1, ref1) = out
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert ms0 == ms1 == 15.0          # the max over ranks
    assert tot0 == tot1 == 2.0
    assert v0 == v1 == 2 * 64 / 0.015  # whole-job pairs/s
    assert s0 != s1                    # every rank registers its own batch
    assert ref1 is False


def test_single_rank_helpers_are_local():
    import bench

    assert bench.reduce_max(3.0) == 3.0
    assert bench.reduce_sum(3.0) == 3.0
    bench.barrier()
    assert bench.dist_env()[1] >= 1


@pytest.fixture(autouse=True)
def _clean_env(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
