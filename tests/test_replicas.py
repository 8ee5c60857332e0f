"""Multi-GPU is replicas only: frames are independent, every rank runs its own
frames and the job's throughput is all ranks' frames over the slowest rank's
time. The host logic runs here as world_size-2 gloo ranks on the CPU."""
import io
import os
import sys
import contextlib

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, ws, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    secs = 2.0 + rank                                   # rank 1 is the slow one
    slowest = bench.max_over_ranks(secs, dist, "cpu")
    value = bench.replica_value(ws, 100, slowest)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, slowest, value))


def test_replica_throughput_uses_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    sys.path.insert(0, ROOT)
    import bench
    for rank, slowest, value in res:
        assert slowest == 3.0
        assert value == pytest.approx(2 * 100 * 1920 * 1080 * 64 / 3.0 / 1e6)
    assert bench.max_over_ranks(1.25, None, "cpu") == 1.25


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup, gpus = 5, 3, 2
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        assert bench.run_reference(A()) == 0
    assert buf.getvalue() == ""                         # no work, no line on the other ranks


def test_reference_arm_line_matches_the_gpu_arm_config(monkeypatch):
    """The reference arm prints one line on rank 0 with the GPU arm's `config`
    (the driver compares the two), its CPU baseline and a zero-copy e2e; a
    small frame stands in for configuration A so the test runs in seconds."""
    sys.path.insert(0, ROOT)
    import json
    import bench
    monkeypatch.setattr(bench, "W", 96)
    monkeypatch.setattr(bench, "H", 40)
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("WORLD_SIZE", "1")

    class A:
        steps, warmup, gpus = 2, 1, 1
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        assert bench.run_reference(A()) == 0
    line = json.loads(buf.getvalue())
    assert line["impl"] == "reference" and line["steps"] == 2 and line["warmup"] == 1
    assert line["config"] == bench.workload_config(1)
    assert line["cpu_baseline"]["value"] == line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert "what" in line["reference_gpu"]             # the reference's CUDA programs, or why not
