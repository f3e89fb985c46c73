"""The benchmark's multi-rank path on CPU: two gloo ranks (127.0.0.1) take the
maximum of their timings and report the whole-job throughput of independent
replicas; the reference arm does no work on ranks other than 0."""

import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [30.0, 42.5][rank]  # ms: rank 1 is the slow replica
        t_max = bench.max_over_ranks(local, world, device="cpu")
        out[rank] = (t_max, bench.job_value(1000, world, t_max / 1e3))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_replica():
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    for rank in (0, 1):
        t_max, value = out[rank]
        assert t_max == 42.5
        assert value == pytest.approx(2 * 1000 / 0.0425)


def test_single_rank_is_identity():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(12.0, 1) == 12.0
    assert bench.job_value(10, 1, 0.5) == 20.0


def test_reference_arm_other_ranks_do_nothing(monkeypatch, capsys):
    sys.path.insert(0, REPO)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        gpus, steps, warmup = 2, 1, 0
    assert bench.run_reference(Args()) == 0
    assert capsys.readouterr().out == ""


def test_reference_arm_line_on_rank0(monkeypatch, capsys):
    """Rank 0 of the reference arm times the oracle port (small sector here)
    and prints one line with the reference-arm keys."""
    import json
    sys.path.insert(0, REPO)
    import bench
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("WORLD_SIZE", "1")
    saved = (bench.NORB, bench.NALPHA, bench.NBETA, bench.NCHOL, bench.METRIC)
    bench.set_workload(8, 4, 4, 16)

    class Args:
        gpus, steps, warmup = 1, 1, 0
    try:
        assert bench.run_reference(Args()) == 0
    finally:
        bench.NORB, bench.NALPHA, bench.NBETA, bench.NCHOL, bench.METRIC = saved
    lines = [x for x in capsys.readouterr().out.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["unit"] == "det/s"
    assert line["config"]["determinants"] == 70 * 70
    assert line["value"] > 0 and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["e2e"]["d2h_bytes_per_step"] == 0
