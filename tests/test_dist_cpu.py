"""The bench's multi-process path on CPU: two gloo ranks (world size 2).

The path does not shard (one PLR matrix per GPU, replicas only), so what the
ranks share is the timing contract: a barrier around the timed region, the
slowest rank's time (max over ranks) and rank 0 alone reporting.  These run
bench.py's own helpers under torch.distributed with the gloo backend.
"""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as dist
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = bench.dist_init()
        bench.barrier(w)
        # each rank's "timed region" differs; the report takes the slowest
        ms = bench.max_over_ranks(10.0 + 5.0 * r, w, "cpu")
        bench.barrier(w)
        # the reference arm runs on rank 0 only: other ranks return at once
        skipped = bench.run_reference(type("A", (), {"steps": 1, "warmup": 0})()) is None if r != 0 else None
        with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
            json.dump({"world": w, "rank": r, "local": local, "ms": ms, "skipped": skipped}, f)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_share_the_timing_contract(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    assert [x["rank"] for x in res] == [0, 1]
    assert all(x["world"] == 2 and x["local"] == x["rank"] for x in res)
    assert all(x["ms"] == 15.0 for x in res)          # max over ranks, seen by every rank
    assert res[1]["skipped"] is True                   # reference arm: rank 1 does no work


def test_single_process_defaults(monkeypatch):
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    sys.path.insert(0, ROOT)
    import bench
    assert bench.dist_init() == (1, 0, 0)
    assert bench.max_over_ranks(7.5, 1, "cpu") == 7.5
    bench.barrier(1)


def test_clock_sampler_child_never_outlives_the_run(monkeypatch):
    """A workload that raises still stops the sampler's child process."""
    import subprocess
    sys.path.insert(0, ROOT)
    import bench
    real = subprocess.Popen
    started = []

    def fake(cmd, **kw):
        p = real(["sleep", "30"], **kw)
        started.append(p)
        return p

    monkeypatch.setattr(bench.subprocess, "Popen", fake)
    s = bench.ClockSampler(0)
    try:
        s.start()
        raise RuntimeError("workload failed")
    except RuntimeError:
        pass
    finally:
        out = s.stop()
    assert started and started[0].poll() is not None
    assert out["reasons"] == ["no samples"]


@pytest.mark.parametrize("workload,fn", [("ppmm", "ppmm_reference_arm"), ("compress", "compress_reference")])
def test_reference_arm_follows_the_workload(monkeypatch, capsys, workload, fn):
    """--impl reference with a secondary workload prints that workload's
    line (host cores only), marked impl=reference."""
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    sys.path.insert(0, ROOT)
    import bench
    from dplr_gb300 import workloads
    seen = {}

    def stub(steps, warmup):
        seen["args"] = (steps, warmup)
        return {"metric": workload, "value": 1.0, "unit": "x/s", "impl": "reference"}

    monkeypatch.setattr(bench if fn == "ppmm_reference_arm" else workloads, fn, stub)
    args = type("A", (), {"steps": 2, "warmup": 1, "workload": workload})()
    bench.run_reference(args)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert seen["args"] == (2, 1)
    assert line["impl"] == "reference" and line["metric"] == workload and line["warmup"] == 1
