"""The multi-GPU form of the bench is N independent replicas (the per-step path has no
data-parallel exchange): the host logic that aggregates them — max-over-ranks time,
whole-job throughput, rank-0-only reference arm — runs here as two gloo ranks on CPU."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, dist = bench.dist_setup(world)
    seconds = 2.0 if r == 1 else 1.0  # rank 1 is the slow one
    value, slowest = bench.replicas_value(dist, w, 10, seconds)
    q.put((r, w, value, slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_aggregate_over_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, value, slowest) in enumerate(out):
        assert rank == r and world == 2
        assert slowest == 2.0          # every rank sees the slowest rank's time
        assert value == pytest.approx(2 * 10 / 2.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(bench, "dist_setup", lambda n: (1, 2, None))
    monkeypatch.setattr(bench, "cpu_leg", lambda *a, **k: pytest.fail("a rank other than 0 timed the reference"))

    class A:
        gpus, steps, warmup = 2, 3, 3
    bench.reference_arm(A())
    assert capsys.readouterr().out == ""
