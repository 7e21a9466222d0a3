"""The multi-GPU path of bench.py is replicas only: every rank transforms its
own copy of the batch, with no data-path collective; the only exchange is the
max-over-ranks step time.  Covered here with two gloo ranks on the CPU."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist)      # rank 1 is the slowest
    value = bench.whole_job_value(16384, world, ms)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out, f"r{rank}"), "w") as f:
        f.write(f"{ms} {value}")


def test_max_over_ranks_and_whole_job_value(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    mp.spawn(_rank, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    for r in range(world):
        ms, value = map(float, (tmp_path / f"r{r}").read_text().split())
        assert ms == 15.0                                   # every rank sees the slowest time
        assert value == pytest.approx(2 * 16384 / 0.015)


def test_single_process_value():
    import bench
    assert bench.max_over_ranks(12.5) == 12.5
    assert bench.whole_job_value(16384, 1, 40.0) == pytest.approx(16384 / 0.04)


def test_reference_arm_only_on_rank0():
    """Under torchrun the reference arm runs on rank 0 alone; other ranks exit 0 without output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_line(orc):
    """rank 0: one JSON line with the same metric, unit and workload config as the GPU arm."""
    import json

    import bench
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == "NTT/s"
    assert line["higher_is_better"] is True and line["value"] > 0
    # the GPU arm's config is the same dict (same keys and values): the
    # driver's same-config check compares the two
    assert line["config"] == bench.workload_config("canonical", 1)
    assert line["coefficients_per_s"] > line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
