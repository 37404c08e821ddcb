"""bench.py's multi-GPU path on the CPU: replicas with no data exchange,
the job time as the maximum over ranks (gloo, world size 2), whole-job
throughput summed over replicas."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    t = bench.max_over_ranks(1.5 + rank, dist, "cpu")
    out.put((rank, t, bench.aggregate_mpix_s(1_000_000, world, 2, t)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world_2():
    import torch.multiprocessing as tmp

    ctx = tmp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in res] == [0, 1]
    for _, t, v in res:
        assert t == 2.5  # the slower rank's time on every rank
        assert v == pytest.approx(1_000_000 * 2 * 2 / 2.5 / 1e6)


def test_single_process_needs_no_group():
    import bench

    assert bench.max_over_ranks(3.0, None, "cpu") == 3.0
    assert bench.aggregate_mpix_s(2_000_000, 1, 4, 2.0) == pytest.approx(4.0)
