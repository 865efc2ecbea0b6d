"""CPU tests of the multi-rank path of bench.py with two gloo ranks: the
barrier and the max-over-ranks time of the replica runs, the whole-job value
the replicas report, and that the reference arm runs on rank 0 only."""
import io
import os
import socket
from contextlib import redirect_stdout

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        barrier, max_over_ranks = bench.rank_collectives(dist, torch.device("cpu"))
        barrier()
        local_ms = [1.5, 2.5][rank]                 # rank 1 is the slower replica
        ms = max_over_ranks(local_ms)
        out.put((rank, ms, bench.replica_value(world, 1000, ms)))
        barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [2.5, 2.5]
    # whole job: 2 replicas x 1000 particles per 2.5 ms
    assert all(g[2] == pytest.approx(2 * 1000 / 2.5e-3) for g in got)


def test_one_process_needs_no_collective():
    barrier, max_over_ranks = bench.rank_collectives(None, torch.device("cpu"))
    barrier()
    assert max_over_ranks(3.25) == 3.25
    assert bench.replica_value(1, 4_194_304, 3.2) == pytest.approx(4_194_304 / 3.2e-3)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    """Under torchrun the other ranks exit 0 without work and print nothing."""
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = bench.parse_args(["--impl", "reference", "--gpus", "2"])
    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference(args) == 0
    assert buf.getvalue() == ""
