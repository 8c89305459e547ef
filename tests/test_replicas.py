"""The multi-GPU form of the benchmark is replicas only: each rank runs its own scene, and
ranks meet only at a barrier and a max-reduction of their timed region.  This runs that
coordination with two gloo ranks on the CPU."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    barrier, allmax = bench.replica_sync(world, "cpu")
    barrier()
    ms = allmax(100.0 * (rank + 1))          # rank r's timed region took 100 (r + 1) ms
    q.put((rank, ms, bench.job_rate(world, 10, ms)))
    barrier()
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's 200 ms; 2 ranks x 10 substeps in 0.2 s
    assert [o[1] for o in out] == [200.0, 200.0]
    assert all(abs(o[2] - 100.0) < 1e-9 for o in out)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    barrier, allmax = bench.replica_sync(1, "cpu")
    barrier()
    assert allmax(3.5) == 3.5 and bench.job_rate(1, 4, 500.0) == 8.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    bench.run_reference(bench.parse(["--impl", "reference"]))
    assert capsys.readouterr().out == ""
