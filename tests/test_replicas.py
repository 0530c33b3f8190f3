"""Multi-GPU form of bench.py (replicas: rays are independent given a replicated scene, so there is
no data-path collective) on the CPU with world_size-2 gloo ranks: each rank times its own
replica, the job time is the max over ranks, the whole-job rate counts every rank's units, ranks
render different views, and the reference arm runs on rank 0 only."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, torch.device("cpu"))
        rate = bench.whole_job_rate(30, ms, world)
        a = bench.parse_args([])
        cam = bench.make_camera(a, rank)
        ref = bench.reference_arm(a, rank, world) if rank != 0 else "rank0"
        out.put((rank, ms, rate, tuple(float(x) for x in cam.origin), ref))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, rate0, o0, ref0), (r1, ms1, rate1, o1, ref1) = res
    assert ms0 == ms1 == 15.0                      # max over ranks
    assert rate0 == rate1 == pytest.approx(30 * 2 / 0.015)
    assert o0 != o1                                # each replica renders its own view
    assert ref1 is None                            # the reference arm runs on rank 0 only


def test_single_rank_is_unchanged():
    assert bench.max_over_ranks(12.5, 1, torch.device("cpu")) == 12.5
    assert bench.whole_job_rate(10, 100.0, 1) == pytest.approx(100.0)


def test_reference_arm_json_line():
    """The reference arm (the CPU restatement timed on the host) prints one JSON line with the
    bench contract's keys, on the same metric, unit and workload as the GPU arm."""
    import json
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--scene", "small",
                          "--steps", "2", "--warmup", "1", "--cpu-sample-stride", "4"],
                         capture_output=True, text=True, check=True, cwd=root, timeout=600).stdout
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "train-steps/s"
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1 and d["higher_is_better"] is True
    assert d["config"]["workload"] == "train step, 64 uniform [-1,1]^3 Gaussians, 256x256"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    # the line says that its steps were samples of the full step, how large, and what it spent
    assert d["extrapolated"] is True and d["cpu_baseline"]["extrapolated"] is True
    assert 0 < d["cpu_baseline"]["sampled_fraction"]["rays"] <= 1
    assert d["timed_seconds"] > 0 and d["cpu_baseline"]["cpu"]
    assert d["config"]["parallelism"] == "replicas x1"
    assert d["e2e"] == {"value": d["value"], "unit": "train-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
