"""The benchmark's multi-rank path on CPU: two gloo ranks, each timing its own
replica; the job time is the slowest rank's and the throughput counts every
rank's bytes. (Multi-GPU runs use the same code over NCCL.)"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(1.0 + rank, world, "cpu")  # rank 1 is the slow one
    out.put((rank, ms, bench.whole_job_gbs(4e9, ms, world)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_report_max_time_and_total_bytes():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks agree on the slowest time (2 ms) and on 2 x 4 GB / 2 ms
    assert [r[1] for r in res] == [2.0, 2.0]
    assert all(abs(r[2] - 4000.0) < 1e-9 for r in res)


def test_single_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.5, 1, "cpu") == 1.5
    assert bench.whole_job_gbs(3e9, 1.5, 1) == pytest.approx(2000.0)
