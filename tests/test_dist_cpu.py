"""bench.py's multi-rank plumbing (one process per GPU, replicas only) on CPU:
world_size 2 over gloo on 127.0.0.1 -- rank discovery, the barrier and the
max-over-ranks timing reduction that the bench applies to its step times."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    ws, r, local = bench.dist_setup()
    assert (ws, r, local) == (world, rank, rank)
    bench.barrier(ws)
    got = bench.max_over_ranks(10.0 + rank, ws)
    import torch.distributed as dist
    dist.destroy_process_group()
    out.put((rank, got))


def test_two_ranks_gloo_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _ in res] == [0, 1]
    assert all(got == 11.0 for _, got in res)   # every rank sees the slowest rank's time


def test_reference_arm_prints_on_rank0_only():
    import bench

    class A:
        steps, warmup = 1, 3
    assert bench.run_reference(A(), 2, 1) is None   # ranks other than 0 do no work
