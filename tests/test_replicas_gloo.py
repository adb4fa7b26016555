"""The multi-GPU path of the benchmark is independent replicas (the lifting-line step has no
exchange between GPUs): one process per GPU, a barrier around the timed region, and rank 0
reporting the whole job as (interactions of all ranks) / (slowest rank's time). This checks
that plumbing of bench.py (dist_init, barrier, allreduce_max, allreduce_sum) with two gloo
ranks on the CPU, as torchrun would start them (RANK / WORLD_SIZE / MASTER_* in the
environment, rendezvous on 127.0.0.1)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench

    ws, r, local = bench.dist_info()
    assert (ws, r, local) == (world, rank, rank)
    bench.dist_init(ws, "gloo")
    bench.barrier(ws)
    # each replica's own figures: interactions done and time taken
    inter = 1.0e9 * (rank + 1)
    ms = 100.0 + 25.0 * rank
    total_ms = bench.allreduce_max(ws, ms)
    all_inter = bench.allreduce_sum(ws, inter)
    bench.barrier(ws)
    out[rank] = (total_ms, all_inter, all_inter / (total_ms * 1e-3))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_replicas_report_the_whole_job():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        codes = [p.exitcode for p in procs]
        res = dict(out)
    assert codes == [0, 0], codes
    for r in range(world):
        total_ms, all_inter, value = res[r]
        assert total_ms == 125.0  # the slowest replica
        assert all_inter == 3.0e9  # every replica's interactions
        assert value == pytest.approx(3.0e9 / 0.125)


def test_one_process_needs_no_process_group():
    import bench

    assert bench.allreduce_max(1, 7.0) == 7.0
    assert bench.allreduce_sum(1, 7.0) == 7.0
    bench.barrier(1)
    bench.dist_init(1, "gloo")  # a no-op for one process
