"""The multi-rank side of bench.py on CPU: two gloo ranks on 127.0.0.1 take the slowest
rank's time and report the whole-job rate (the same helpers run over NCCL on GPUs)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        seconds = 1.5 + rank  # rank 1 is the slow one
        slowest = bench.max_over_ranks(seconds, "cpu")
        assert slowest == 1.5 + (world - 1)
        assert bench.job_rate(64 * 5, slowest, world) == pytest.approx(world * 64 * 5 / slowest)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    if not torch.distributed.is_available():
        pytest.skip("torch.distributed unavailable")
    mp.spawn(_rank_main, args=(2, _free_port()), nprocs=2, join=True)


def test_single_rank_helpers():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(2.25, "cpu") == 2.25
    assert bench.job_rate(320, 4.0, 1) == 80.0


def test_hbm_roofline(tmp_path):
    sys.path.insert(0, ROOT)
    import bench

    pk = tmp_path / "peaks.json"
    pk.write_text('{"hbm_gbs": 6000.0}')
    r = bench.hbm_roofline(3.0e9, 0.5, str(pk))
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == 6.0 and r["peak"] == 6000.0 and abs(r["frac"] - 1e-3) < 1e-15
    assert r["peak_source"].startswith("measured")
    r = bench.hbm_roofline(3.0e9, 0.5, str(tmp_path / "absent.json"))
    assert r["peak"] == 6800.0 and r["peak_source"] == "fallback"


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the CPU oracle on the host cores) prints one JSON line
    with the keys of the benchmark contract, on the same metric, unit and workload."""
    import json
    import subprocess

    sys.path.insert(0, ROOT)
    import bench

    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] > 0 and line["cpu_baseline"]["cores"] >= 1 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    # the same workload description as the GPU arm prints (sizes of the D=6 L=8 problem)
    assert line["config"] == bench.workload_config(40081, 2975, 37769167)
