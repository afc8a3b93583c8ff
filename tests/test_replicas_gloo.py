"""The N > 1 host logic of bench.py on CPU: two gloo ranks (127.0.0.1), each timing its own
replica job; the job time is the slowest rank's, every rank sees the same maxima, and the
whole-job rate counts every replica's steps.  No GPU: the step is not sharded across GPUs,
so these reductions are the only cross-rank traffic the bench has."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out) -> None:
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "measured" (100 + 10 r) ms of device time and (2 + r) s end to end
        t_max, e2e = bench.max_over_ranks([100.0 + 10 * rank, 2.0 + rank])
        dist.barrier()
        out.put((rank, t_max, e2e, bench.replica_value(world, 20, t_max)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_replica_rate_with_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    for rank, t_max, e2e, value in got:
        assert t_max == 110.0 and e2e == 3.0
        assert value == pytest.approx(2 * 20 / 0.110)


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks([1.5, 2.5]) == [1.5, 2.5]
    assert bench.replica_value(1, 20, 250.0) == pytest.approx(80.0)
