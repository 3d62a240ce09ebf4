"""The N>1 path of bench.py on CPU: two gloo ranks on 127.0.0.1.  Each replica images its own
visibilities (no data-path collective); the only cross-rank steps are the barriers around the
timed region and the max over ranks of the elapsed time, from which the whole-job value is
the units of all ranks over the slowest rank's time.  The reference arm runs on rank 0 only.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as tdist
    import bench
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        tdist.barrier()
        # rank r took 10 + 5 r ms per step for 1000 visibilities
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, tdist)
        value = bench.whole_job_mvis(1000, world, ms / 1e3)
        alone = bench.max_over_ranks(7.0)  # no process group: the value itself
        out.put((rank, ms, value, alone))
        tdist.barrier()
    finally:
        tdist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time_and_the_whole_job_value():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    slowest = 10.0 + 5.0 * (world - 1)
    for rank, ms, value, alone in got:
        assert ms == slowest  # every rank sees the slowest rank's time
        assert value == pytest.approx(1000 * world / (slowest / 1e3) / 1e6)
        assert alone == 7.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Under torchrun the reference (CPU) arm does its work and prints on rank 0 alone; the
    other ranks return at once with nothing printed."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    assert bench.run_reference(bench.parse()) is None
    assert capsys.readouterr().out == ""
