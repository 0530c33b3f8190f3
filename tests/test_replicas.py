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
