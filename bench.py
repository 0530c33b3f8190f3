#!/usr/bin/env python
"""Benchmark: one training step of the Gaussian ray tracer at 3M Gaussians, 1920x1080.

A step is what the reference's training loop does per image (train.py:245-287 minus the loss's
SSIM term): SH colour + forward trace, L1 loss against a target image, reverse-replay backward +
SH backward, fused Adam, BVH refit.  Synthetic, seeded inputs: 3M Gaussians drawn from 200
anisotropic clusters inside a radius-10 sphere (log-scales N(-4.5, 0.5)), camera on a radius-8
orbit, fx = fy = 1440, seeded random target image.  Inputs (3 GB of parameters and optimiser
state) are far larger than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  `value` is train-steps/s with the target image resident in HBM;
`e2e` is the same step through the public Raytracer API with the target copied from pinned host
memory and the loss read back every step (the upload of step i+1 runs on a copy stream during step
i; `e2e.serial_value` is the same with upload and step in series; each of the three timed loops starts
from the same training state, since training moves the Gaussians and their cost).  `roofline` is for the kernel with the largest share of
the step, from CUDA events recorded around each launch inside the timed region.  `--impl
reference` times the CPU restatement of the reference's algorithm (oracle/, the reference itself
needs OptiX and does not build here) on a bounded sample of rays per step, extrapolated.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "rays/s and train-steps/s at 3M Gaussians 1080p; served p50/p99 latency vs plain"
LR = dict(mean=1.6e-4, scale=5e-3, rotation=1e-3, opacity=2.5e-2, sh=2.5e-3)


def parse():
    return apply_scene(parse_args(None))


def parse_args(argv):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-gaussians", type=int, default=3_000_000)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-stride", type=int, default=24, help="1 ray in stride^2 pixels for the CPU sample")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and served measurements")
    ap.add_argument("--serve-requests", type=int, default=2000)
    ap.add_argument("--no-served", action="store_true", help="skip the served measurement only")
    ap.add_argument("--trace-variant", type=int, default=0, help="forward-kernel variant (0 = library default)")
    ap.add_argument("--view", type=int, default=-1,
                    help="clustered scene: train on the pose of view K of the batched form's 16 jittered orbit "
                         "views (at --width x --height) instead of the default orbit camera")
    ap.add_argument("--record-traffic", nargs="+", metavar="ARG",
                    help="CSV KEY KERNEL [UNITS_SCALE]: store the per-launch DRAM bytes of KERNEL in an ncu CSV "
                         "capture under KEY in profiles/ncu_traffic.json, with the digest of the current kernel "
                         "sources, and exit")
    ap.add_argument("--scene", default="clustered", choices=["clustered", "small", "gradcheck"],
                    help="clustered: --n-gaussians clustered Gaussians on a radius-8 orbit; small: 64 Gaussians in "
                         "[-1,1]^3, 256x256 camera at distance 4 (fx = 256); gradcheck: 1000 Gaussians in [-2,2]^3, "
                         "128x128 camera")
    return ap.parse_args(argv)


def apply_scene(a):
    """The small and gradcheck scenes fix their own size and resolution."""
    if a.scene == "small":
        a.n_gaussians, a.width, a.height = 64, 256, 256
    elif a.scene == "gradcheck":
        a.n_gaussians, a.width, a.height = 1000, 128, 128
    return a


def workload_config(a, rank=0):
    kind = {"clustered": "clustered", "small": "uniform [-1,1]^3", "gradcheck": "uniform [-2,2]^3"}[a.scene]
    count = f"{a.n_gaussians / 1e6:g}M" if a.n_gaussians >= 100_000 else f"{a.n_gaussians}"
    view = f", jittered view {a.view}" if a.view >= 0 and a.scene == "clustered" else ""
    return {"workload": f"train step, {count} {kind} Gaussians, {a.width}x{a.height}{view}",
            "n_gaussians": a.n_gaussians, "width": a.width, "height": a.height, "rays_per_step": a.width * a.height,
            "sh_degree": 3, "t_threshold": 0.03, "alpha_threshold": 0.01, "exp_power": 2.0,
            "l2": "inputs larger than L2 (no flush)" if a.scene == "clustered" and a.n_gaussians >= 1_000_000
            else "inputs smaller than L2, resident between steps (no flush)", "seed": 0}


def make_scene(a):
    from gray_gb300 import synthetic

    if a.scene == "small":
        return synthetic.small_scene(seed=0)
    if a.scene == "gradcheck":
        return synthetic.gradcheck_scene(seed=0)
    return synthetic.clustered_scene(a.n_gaussians, seed=0)


def make_camera(a, rank):
    from gray_gb300 import synthetic

    if a.scene == "small":
        return synthetic.camera_small(a.width, a.height)
    if a.scene == "gradcheck":
        return synthetic.camera_small(a.width, a.height, focal=float(a.width))
    if a.view >= 0:
        return synthetic.uneven_view(a.view, a.width, a.height)
    return synthetic.orbit_camera(0.3 + 0.7 * rank, a.width, a.height)


# ----------------------------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 20 ms; stop() keeps the samples whose
    timestamps fall inside the marked window (mark_begin .. mark_end)."""
    FIELDS = "timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu_index):
        self.proc = None
        self.gpu = gpu_index
        import tempfile

        self.path = os.path.join(tempfile.gettempdir(), f"gray_bench_clocks_{os.getpid()}.csv")
        self.t0 = self.t1 = None

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            # wait (at most 3 s) until sampling has begun
            deadline = time.time() + 3.0
            while time.time() < deadline and os.path.getsize(self.path) == 0:
                time.sleep(0.02)
        except Exception:
            self.proc = None

    def mark_begin(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    @staticmethod
    def _epoch(stamp):
        from datetime import datetime

        for fmt in ("%Y/%m/%d %H:%M:%S.%f", "%Y/%m/%d %H:%M:%S"):
            try:
                return datetime.strptime(stamp.strip(), fmt).timestamp()
            except ValueError:
                pass
        return None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 10:
                rows.append(parts)
        if self.t0 is not None and self.t1 is not None:
            inside = [r for r in rows if (lambda t: t is not None and self.t0 - 0.05 <= t <= self.t1 + 0.05)(
                self._epoch(r[0]))]
            rows = inside or rows[-1:]
        if not rows:
            return None
        sm = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        mx = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[6 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak_gbs():
    try:
        m = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def max_over_ranks(ms, world, device):
    """The job's time is the slowest replica's: MAX all-reduce over the ranks (no-op for one rank)."""
    if world <= 1:
        return ms
    import torch

    t = torch.tensor([ms], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, ms, world):
    """Units per second of all replicas together: every rank processes units_per_rank in the
    (max-over-ranks) time ms (weak scaling)."""
    return units_per_rank * world / (ms / 1000.0)


def kernel_source_hash() -> str:
    """Digest of the CUDA sources (gray_gb300/csrc), to tie a captured DRAM figure to the kernels it
    was measured on."""
    import hashlib

    h = hashlib.sha256()
    csrc = os.path.join(ROOT, "gray_gb300", "csrc")
    for name in sorted(os.listdir(csrc)):
        if name.endswith((".cu", ".cuh", ".h")):
            h.update(name.encode())
            h.update(open(os.path.join(csrc, name), "rb").read())
    return h.hexdigest()[:16]


TRAFFIC_FILE = os.path.join(ROOT, "profiles", "ncu_traffic.json")


def ncu_traffic(kernel, a):
    """DRAM bytes (read + write) of one launch of `kernel` on this workload, from an ncu capture
    summarised in profiles/ncu_traffic.json (key "<kernel> <gaussians> <width>x<height>"); None when
    the capture was made on other kernel sources than the ones built now."""
    try:
        entry = json.load(open(TRAFFIC_FILE)).get(f"{kernel} {a.n_gaussians} {a.width}x{a.height}")
    except Exception:
        return None
    if not isinstance(entry, dict) or entry.get("sources") != kernel_source_hash():
        return None
    return entry.get("bytes")


def record_traffic(csv_path, key, kernel, per_launch_units=1.0):
    """Add the DRAM bytes of the launches of `kernel` (a substring of the kernel name) in an ncu CSV
    (--metrics dram__bytes_read.sum,dram__bytes_write.sum --csv) to profiles/ncu_traffic.json under
    `key`, averaged per launch and scaled by per_launch_units (a capture of a smaller case scaled to
    the full launch), together with the digest of the kernel sources it was captured on."""
    import csv

    per_launch = {}
    with open(csv_path) as f:
        rows = [r for r in csv.reader(f) if r]
    head = next(i for i, r in enumerate(rows) if "Metric Name" in r)
    cols = rows[head]
    mi, vi, ii, ki = cols.index("Metric Name"), cols.index("Metric Value"), cols.index("ID"), cols.index("Kernel Name")
    units = rows[head + 1] if rows[head + 1][mi] == "" else None
    for r in rows[head + 1 + (1 if units else 0):]:
        if kernel in r[ki] and r[mi] in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
            v = float(r[vi].replace(",", ""))
            unit = r[cols.index("Metric Unit")] if "Metric Unit" in cols else "byte"
            v *= {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "KB": 1e3, "MB": 1e6, "GB": 1e9}.get(unit, 1)
            per_launch[r[ii]] = per_launch.get(r[ii], 0.0) + v
    avg = sum(per_launch.values()) / max(len(per_launch), 1) * per_launch_units
    try:
        table = json.load(open(TRAFFIC_FILE))
    except Exception:
        table = {}
    if not per_launch:
        raise ValueError(f"no launch of a kernel named like {kernel!r} in {csv_path}")
    table[key] = {"bytes": int(avg), "launches": len(per_launch), "kernel": kernel, "sources": kernel_source_hash()}
    json.dump(table, open(TRAFFIC_FILE, "w"), indent=1, sort_keys=True)
    return table[key]


def gpu_arm(a, rank, world, local_rank):
    import numpy as np
    import torch
    import torch.nn.functional as F

    from gray_gb300 import RaytracerConfig, Raytracer, _lib

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    sc = make_scene(a)
    cam = make_camera(a, rank)
    cfg = RaytracerConfig(sh=True, sh_max_degree=3, lr_mean_init=LR["mean"], lr_scale_init=LR["scale"],
                          lr_rotation_init=LR["rotation"], lr_opacity_init=LR["opacity"], lr_sh_dc_init=LR["sh"],
                          lr_sh_rest=LR["sh"], ppll_backward_size=160_000_000)
    rt = Raytracer(cfg, sc.n, a.width, a.height)
    g = rt.cuda_module.get_gaussians()
    with torch.no_grad():
        g.mean.copy_(torch.from_numpy(sc.mean))
        g.rotation.copy_(torch.from_numpy(sc.rotation))
        g.scale.copy_(torch.from_numpy(sc.scale))
        g.opacity.copy_(torch.from_numpy(sc.opacity))
        g.sh_coeffs_dc.copy_(torch.from_numpy(sc.sh_dc))
        g.sh_coeffs_rest.copy_(torch.from_numpy(sc.sh_rest))
        g.current_sh_degree.fill_(3)
    rt.cuda_module.rebuild_bvh()
    if a.trace_variant:
        rt.cuda_module.set_trace_variant(a.trace_variant)
    gen = torch.Generator().manual_seed(1234 + rank)
    target_host = torch.rand(3, a.height, a.width, generator=gen).pin_memory()
    target_dev = target_host.to(dev)
    loss_host = torch.zeros(1).pin_memory()
    stream = torch.cuda.current_stream()

    def train_step(target):
        render = rt(cam)
        loss = F.l1_loss(render, target)
        rt.backward(loss)
        rt.step()
        return loss

    def e2e_step():
        target_dev.copy_(target_host, non_blocking=True)
        loss = train_step(target_dev)
        loss_host.copy_(loss.detach().reshape(1), non_blocking=True)

    # end to end with the input upload of step i+1 on a copy stream while step i computes (double
    # buffered, as a training loop with a prefetching loader runs); every step still uploads its
    # target from pinned host memory and reads its loss back inside the timed region
    copy_stream = torch.cuda.Stream()
    bufs = [torch.empty_like(target_dev), torch.empty_like(target_dev)]
    uploaded = [torch.cuda.Event(), torch.cuda.Event()]
    consumed = [torch.cuda.Event(), torch.cuda.Event()]

    def e2e_run(k):
        bufs[0].copy_(target_host, non_blocking=True)
        uploaded[0].record(stream)
        for i in range(k):
            if i + 1 < k:
                j = (i + 1) % 2
                copy_stream.wait_stream(stream) if i == 0 else copy_stream.wait_event(consumed[j])
                with torch.cuda.stream(copy_stream):
                    bufs[j].copy_(target_host, non_blocking=True)
                    uploaded[j].record(copy_stream)
            stream.wait_event(uploaded[i % 2])
            loss = train_step(bufs[i % 2])
            loss_host.copy_(loss.detach().reshape(1), non_blocking=True)
            consumed[i % 2].record(stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def timed(fn, k):
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return max_over_ranks(e0.elapsed_time(e1), world, dev)

    for _ in range(a.warmup):
        train_step(target_dev)
    torch.cuda.synchronize()
    rt.cuda_module.check_status()

    # Every train step moves the Gaussians (Adam on a random target), and their cost per step moves
    # with them (about 7% over 150 steps of this workload).  Each timed segment below therefore starts
    # from the same training state, restored before it: parameters, gradients, Adam moments, pruning
    # statistics, SH degree, step counter, and the snapshot + refit that follow from them.
    state_names = [k + n for k in ("", "grad_", "first_moment_", "second_moment_")
                   for n in ("mean", "rotation", "scale", "opacity", "channels", "sh_coeffs_dc", "sh_coeffs_rest")]
    state_names += ["pruning_weight", "pruning_counter", "was_visible", "marked", "current_sh_degree"]
    gh, meta = rt.cuda_module.get_gaussians(), rt.cuda_module.get_metadata()
    start_state = {n: getattr(gh, n).clone() for n in state_names}
    start_steps = meta.total_num_steps.clone()

    def restore_start_state():
        with torch.no_grad():
            for n, t in start_state.items():
                getattr(gh, n).copy_(t)
            meta.total_num_steps.copy_(start_steps)
        rt.cuda_module.update_bvh()
        torch.cuda.synchronize()

    # ---- timed region: device-resident inputs ----
    st = rt.cuda_module.get_stats()
    st.reset()
    clocks = ClockSampler(local_rank)
    clocks.start()
    clocks.mark_begin()
    with _lib.Profiler(capacity=64 * (a.steps + 1)) as prof:
        ms = timed(lambda: train_step(target_dev), a.steps)
    clocks.mark_end()
    clk = clocks.stop()
    rt.cuda_module.check_status()
    V = float(rt.cuda_module.get_gaussians().was_visible.sum().item())  # Gaussians the last backward touched
    H = float(st.num_gaussians_hit.sum().item()) / a.steps
    A = float(st.num_gaussians_accumulated.sum().item()) / a.steps
    R = a.width * a.height
    ms_step = ms / a.steps
    steps_per_s = whole_job_rate(a.steps, ms, world)

    # ---- e2e through the public API with host buffers (from the same training state) ----
    for _ in range(max(1, a.warmup // 2)):
        e2e_step()
    e2e_run(2)
    restore_start_state()
    ms_e2e_serial = timed(e2e_step, a.steps)
    restore_start_state()
    ms_e2e = timed(lambda: e2e_run(a.steps), 1)
    e2e_steps_per_s = whole_job_rate(a.steps, ms_e2e, world)

    # ---- render-only throughput (inference-style forward, no grads) ----
    with torch.no_grad():
        for _ in range(2):
            rt(cam, skip_copy=True)
        ms_render = timed(lambda: rt(cam, skip_copy=True), a.steps)
    rays_per_s = whole_job_rate(R * a.steps, ms_render, world)

    # ---- roofline of the dominant kernel ----
    res = prof.results
    n = sc.n
    algo = {
        "trace_forward": 44.0 * H + 12.0 * A + 60.0 * R,
        "trace_backward": 120.0 * A + 72.0 * R,
        "forward_prep": 228.0 * n,
        # every accumulator row is read (64 B); rows of Gaussians the replay touched are cleared (64 B),
        # folded into the gradients (read + write of 60 B), flagged visible (1 B), and run through the
        # SH backward (mean 12, coefficients 180 + colour 12 read; grad_dc 12 + grad_rest 180 written)
        "fold_sh_backward": 64.0 * n + (64.0 + 120.0 + 1.0 + 12.0 + 180.0 + 12.0 + 12.0 + 180.0) * V,
        "adam": (59 * 32.0 + 12.0) * n,  # 59 Adam floats x (p, m, v, g) read + written; channel grads zeroed
        "snapshot": (44.0 + 48 + 48 + 32) * n,
        "refit": 44.0 * n + 24.0 * (2 * n - 1),
    }
    total_ms = sum(v[0] for v in res.values())
    dominant = max(res, key=lambda k: res[k][0])
    dom_ms = res[dominant][0] / res[dominant][1]
    peak, peak_kind = measured_peak_gbs()
    achieved = algo.get(dominant, 0.0) / (dom_ms / 1000.0) / 1e9
    # kernels behind one profiled scope: adam = step count + update; trace_backward = backward
    # record + replay; tile_schedule = super-tile walk + tile walk + bucket scan + scatter (on the
    # library's side stream, beside forward_prep), then trace_forward = the trace: with the default
    # variant the narrow and the wide kernel, one of which returns at once (all in trace_forward
    # when no side stream could be had); refit = block-local climb + upper tree.  The snapshot, the
    # forward preparation and the backward record run a bulk-copy kernel over whole tiles (128, 64
    # and 128 Gaussians) and a plain one over the rest.
    def tiled(tile):
        return int(n >= tile) + int(n % tile != 0)

    traces = 2 if not a.trace_variant else 1
    kernels_per_group = {"adam": 2, "trace_backward": 1 + tiled(128), "refit": 2, "tile_schedule": 4,
                         "trace_forward": traces if "tile_schedule" in res else 4 + traces, "snapshot": tiled(128),
                         "forward_prep": tiled(64)}
    launches = sum(cnt * kernels_per_group.get(name, 1) for name, (_, cnt) in res.items())
    roofline = {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "traffic": ncu_traffic(dominant, a), "traffic_sources": kernel_source_hash(),
                "algorithmic_bytes": algo.get(dominant),
                "avg_launch_ms": round(dom_ms, 4),
                "shares": {k: round(v[0] / total_ms, 4) for k, v in sorted(res.items(), key=lambda kv: -kv[1][0])},
                "hits_per_ray": round(H / R, 2), "composited_per_ray": round(A / R, 2)}

    batched = None if a.no_extras else batched_form(a, rt.cuda_module)
    differentiation = None if a.no_extras else differentiation_form(a, rt.cuda_module, cam, target_dev)
    served = None
    if not (a.no_extras or a.no_served):
        served = served_form(a, rank)  # the serving configuration's precision (fp32)
        # the reference's inference mode (fp16 SH coefficients), continuous batching only
        served["fp16_sh_variant"] = served_form(a, rank, sh_fp16=True, plain=False,
                                                requests=max(a.serve_requests // 2, 1))

    cpu = None
    if rank == 0 and not a.no_cpu_baseline:
        cpu = cpu_baseline(a)

    line = {"metric": METRIC, "value": round(steps_per_s, 3), "unit": "train-steps/s", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": f"synthetic (seeded {a.scene} scene)",
            "config": dict(workload_config(a), parallelism=f"replicas x{world}"),
            "rays_per_s": round(rays_per_s, 1), "train_rays_per_s": round(R * steps_per_s, 1),
            "e2e": {"value": round(e2e_steps_per_s, 3), "unit": "train-steps/s",
                    "h2d_bytes_per_step": int(target_host.numel() * 4), "d2h_bytes_per_step": 4,
                    "upload": "pinned host -> device on a copy stream, overlapped with the previous step",
                    "serial_value": round(whole_job_rate(a.steps, ms_e2e_serial, world), 3)},
            "gpu_launches": launches, "roofline": roofline, "clocks": clk, "cpu_baseline": cpu,
            "batched": batched, "differentiation": differentiation, "served": served}
    return line


def batched_form(a, tracer):
    """16 views of uneven resolution ({640x480, 1280x720, 1600x1040, 1920x1080}, radius-8 orbit, +-15
    degree jitter) of the benchmark scene: one persistent launch replayed from a CUDA graph with an
    autotuned kernel variant, against 16 plain one-view launches (forward_pass_display)."""
    import torch

    from gray_gb300 import synthetic
    from gray_gb300.batch import BatchRenderer

    cams = synthetic.uneven_cameras(16, seed=0)
    rays = sum(c.image_width * c.image_height for c in cams)

    def plain():
        for c in cams:
            t = tracer.get_camera()
            t.znear.fill_(0.0)
            t.zfar.fill_(99999.9)
            t.vertical_fov_radians.fill_(float(c.fov_y))
            t.set_pose(c.origin_cuda(), c.rotation_c2w_blender_cuda())
            tracer.get_config().rays_from_python.fill_(False)
            tracer.set_render_resolution(c.image_width, c.image_height)
            with torch.no_grad():
                tracer.forward_pass_display()

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    ms_plain = timed(plain, 3)
    br = BatchRenderer([tracer], use_graph=True, autotune=True)
    reqs = [(0, c) for c in cams]
    ms_batch = timed(lambda: br.render(reqs), 5)
    tracer.set_render_resolution(a.width, a.height)
    return {"views": 16, "rays": rays, "plain_ms": round(ms_plain, 3), "batched_ms": round(ms_batch, 3),
            "plain_rays_per_s": round(rays / ms_plain * 1000.0, 1),
            "batched_rays_per_s": round(rays / ms_batch * 1000.0, 1),
            "speedup": round(ms_plain / ms_batch, 3), "tuned": [list(v) for v in br.tuned.values()]}


def differentiation_form(a, tracer, cam, target):
    """The hand-written backward behind torch.autograd.Function (gray_gb300.autograd.render) on the
    benchmark view: render + L1 + backward with the hit lists kept from the forward, and with them
    recomputed by a second forward inside the backward (nothing kept between the two)."""
    import torch
    import torch.nn.functional as F

    from gray_gb300.autograd import render

    g = tracer.get_gaussians()
    params = {k: getattr(g, k).detach().clone().requires_grad_() for k in
              ("mean", "rotation", "scale", "opacity", "sh_coeffs_dc", "sh_coeffs_rest")}

    def step(recompute):
        img = render(tracer, cam, params["mean"], params["rotation"], params["scale"], params["opacity"],
                     sh_dc=params["sh_coeffs_dc"], sh_rest=params["sh_coeffs_rest"], recompute=recompute)
        F.l1_loss(img, target).backward()

    out = {}
    for mode, rc in (("stored_ms", False), ("recompute_ms", True)):
        for _ in range(2):
            step(rc)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            step(rc)
        e1.record()
        torch.cuda.synchronize()
        out[mode] = round(e0.elapsed_time(e1) / 5, 3)
    out["hitlist_mb"] = round(float(tracer.get_ppll_backward_data().total_hits.item()) * 4 / 1e6, 1)
    tracer.check_status()
    return out


# serving knobs: three execution slots, at most 16 requests and 12M rays (about 1.5 4K views) per
# batch; a sweep on the serving configuration (slots 2-4, batch 8-16, budgets 8.3M-20M rays or none)
# kept throughput at 576 M rays/s everywhere and this choice had the lowest p50 with a low p99
SERVE_SLOTS, SERVE_MAX_BATCH, SERVE_RAY_BUDGET = 3, 16, 12_000_000


def served_form(a, rank, sh_fp16=False, plain=True, requests=None, slots=None, max_batch=None, ray_budget=-1):
    """Four resident inference scenes (0.5M, 1M, 3M, 6M clustered Gaussians, different seeds; fp32 SH,
    or fp16 SH as the reference's inference mode stores it); Poisson arrivals at 200 req/s, each naming
    a scene, a random orbit pose and a resolution uniform in {640x480, 1280x720, 1920x1080, 3840x2160};
    continuous batching vs the plain one-request-per-launch loop on the same schedule."""
    import numpy as np
    import torch

    from gray_gb300 import classes, synthetic
    from gray_gb300.serve import RenderServer, plain_loop, poisson_arrivals, run_served

    sizes = [500_000, 1_000_000, 3_000_000, 6_000_000]
    tracers = []
    for i, n in enumerate(sizes):
        sc = synthetic.clustered_scene(n, seed=100 + i)
        t = classes.Raytracer(3840, 2160, n, 3, 1, 1, inference_only=True, inference_sh_fp16=sh_fp16)
        t.get_config().t_threshold.fill_(0.03)
        g = t.get_gaussians()
        with torch.no_grad():
            for k, v in (("mean", sc.mean), ("rotation", sc.rotation), ("scale", sc.scale),
                         ("opacity", sc.opacity), ("sh_coeffs_dc", sc.sh_dc), ("sh_coeffs_rest", sc.sh_rest)):
                getattr(g, k).copy_(torch.from_numpy(v))
            g.current_sh_degree.fill_(3)
        t.rebuild_bvh()
        tracers.append(t)
        del sc
    rng = np.random.default_rng(7 + rank)
    res = [(640, 480), (1280, 720), (1920, 1080), (3840, 2160)]
    count = requests or a.serve_requests
    sched = []
    for t_arr in poisson_arrivals(200.0, count, seed=3 + rank):
        w, h = res[int(rng.integers(0, 4))]
        sched.append((float(t_arr), int(rng.integers(0, 4)),
                      synthetic.orbit_camera(float(rng.uniform(0, 2 * np.pi)), w, h,
                                             jitter_rad=tuple(rng.uniform(-0.26, 0.26, 2)))))
    # warm-up (autotune-free eager launches; first-touch allocations)
    warm = RenderServer(tracers, slots=2, max_batch=16)
    for s_, cam in [(i, synthetic.orbit_camera(0.1, 640, 480)) for i in range(4)]:
        warm.submit(s_, cam)
    warm.drain()
    torch.cuda.synchronize()
    slots = slots or SERVE_SLOTS
    max_batch = max_batch or SERVE_MAX_BATCH
    ray_budget = SERVE_RAY_BUDGET if ray_budget == -1 else ray_budget
    srv = RenderServer(tracers, slots=slots, max_batch=max_batch, ray_budget=ray_budget)
    tuned = srv.tune([(s_, cam) for _, s_, cam in sched[:16]])
    reqs, wall = run_served(srv, sched)
    lat = np.array([r.latency for r in reqs]) * 1000.0
    rays = sum(r.rays for r in reqs)
    out = {"dtype": "f16 SH" if sh_fp16 else "f32", "requests": count, "rate_hz": 200.0, "scenes": sizes,
           "slots": slots, "max_batch": max_batch, "ray_budget": ray_budget,
           "p50_ms": round(float(np.percentile(lat, 50)), 2), "p99_ms": round(float(np.percentile(lat, 99)), 2),
           "rays_per_s": round(rays / wall, 1), "offered_rays_per_s": round(rays / sched[-1][0], 1),
           "tuned": list(tuned),
           "by_resolution": {f"{w}x{h}": {"p50_ms": round(float(np.percentile(v, 50)), 2),
                                          "p99_ms": round(float(np.percentile(v, 99)), 2), "requests": len(v)}
                             for (w, h) in res
                             for v in [[r.latency * 1000.0 for r in reqs if r.camera.image_width == w]] if v}}
    if plain:
        plain_lat, wall_p = plain_loop(tracers, sched)
        lat_p = np.array([l for l, _ in plain_lat]) * 1000.0
        out.update(plain_p50_ms=round(float(np.percentile(lat_p, 50)), 2),
                   plain_p99_ms=round(float(np.percentile(lat_p, 99)), 2), plain_rays_per_s=round(rays / wall_p, 1))
    del tracers
    torch.cuda.empty_cache()
    return out


# ----------------------------------------------------------------------------------------------
# CPU restatement (oracle): baseline leg and reference arm
# ----------------------------------------------------------------------------------------------
def cpu_model() -> str:
    """The host CPU's model name (x86 'model name', or lscpu's 'Model name' on Arm)."""
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform

    return platform.processor() or platform.machine()


class CpuScene:
    """The oracle's view of the benchmark scene: snapshot, BVH, SH colours, sample rays, and a slice
    of the Gaussians with its own BVH for the per-Gaussian passes."""

    SLICE = 200_000

    def __init__(self, a, sc, cam):
        import numpy as np

        from oracle import oracle as O

        O.build()
        self.O = O
        self.a = a
        self.threads = O.hardware_threads()
        self.sc = sc
        self.origin = cam.origin.astype(np.float32)
        self.geom, self.l2w, self.aabb, self.vis = O.snapshot(sc.mean, sc.rotation, sc.scale, sc.opacity[:, 0])
        self.live = O.forward_prep(sc.opacity[:, 0])
        self.chan = O.sh_forward(3, sc.mean, self.origin, sc.sh_dc[:, 0, :], sc.sh_rest)
        self.bvh = O.Bvh(self.aabb, self.vis)
        ro, rd = O.camera_rays(a.width, a.height, cam.fov_y, self.origin, cam.rotation_c2w_blender())
        s = a.cpu_sample_stride
        ys, xs = np.meshgrid(np.arange(s // 2, a.height, s), np.arange(s // 2, a.width, s), indexing="ij")
        idx = (ys * a.width + xs).ravel()
        self.ro, self.rd = ro[idx], rd[idx]
        self.cfg = O.TraceConfig(t_threshold=0.03)
        m = self.m = min(sc.n, self.SLICE)
        self.slice_bvh = O.Bvh(self.aabb[:m], self.vis[:m])
        self.state = {}
        for name, width in (("channels", 3), ("opacity", 1), ("mean", 3), ("rotation", 4), ("scale", 3),
                            ("sh_dc", 3), ("sh_rest", 45)):
            for pre in ("", "g_", "m_", "v_"):
                self.state[pre + name] = np.zeros(m * width, np.float32)
        self.ray_fraction = self.ro.shape[0] / float(a.width * a.height)
        self.gauss_fraction = m / float(sc.n)

    def step_seconds(self):
        """One extrapolated CPU train step: trace forward + backward on the ray sample (all threads)
        scaled to the full image, plus SH forward and backward, Adam, snapshot and refit over a slice
        of the Gaussians (one thread, as the oracle runs them) scaled to N.  Returns (extrapolated
        seconds, seconds actually spent, forward result)."""
        import numpy as np

        O, a, sc, m = self.O, self.a, self.sc, self.m
        R_full = a.width * a.height
        t0 = time.perf_counter()
        fwd = O.trace_forward(self.ro, self.rd, self.geom, self.live, self.chan, self.vis, self.cfg, bvh=self.bvh,
                              nthreads=self.threads)
        gout = np.sign(fwd["rgb"] - 0.5).astype(np.float32) / np.float32(3 * R_full)
        O.trace_backward(a.width, a.height, self.ro, self.rd, fwd, gout, self.geom, self.l2w, sc.opacity, sc.scale,
                         sc.rotation, self.chan, self.cfg, nthreads=self.threads)
        t_trace = time.perf_counter() - t0
        t1 = time.perf_counter()
        chan = O.sh_forward(3, sc.mean[:m], self.origin, sc.sh_dc[:m, 0, :], sc.sh_rest[:m])
        O.sh_backward(3, sc.mean[:m], self.origin, sc.sh_rest[:m], chan, chan, np.ones(m, np.uint8),
                      np.zeros((m, 3), np.float32))
        O.adam_step(self.state, {"mean": 1e-4}, m, 15, 1)
        _, _, aabb2, _ = O.snapshot(sc.mean[:m], sc.rotation[:m], sc.scale[:m], sc.opacity[:m, 0])
        self.slice_bvh.refit(aabb2)
        t_gauss = time.perf_counter() - t1
        spent = time.perf_counter() - t0
        return t_trace / self.ray_fraction + t_gauss / self.gauss_fraction, spent, fwd

    def measure(self, steps, warmup):
        """The protocol both CPU figures use: `warmup` untimed steps, then the median of `steps`."""
        for _ in range(warmup):
            self.step_seconds()
        runs = [self.step_seconds() for _ in range(steps)]
        ext = statistics.median(r[0] for r in runs)
        return ext, sum(r[1] for r in runs), runs[-1][2]

    def describe(self, steps, timed_s):
        a = self.a
        return {"cores": self.threads, "cpu": cpu_model(), "kind": "port", "extrapolated": True,
                "sampled_fraction": {"rays": round(self.ray_fraction, 6), "gaussians": round(self.gauss_fraction, 6)},
                "timed_seconds": round(timed_s, 4), "timed_steps": steps,
                "sample": f"per step: {self.ro.shape[0]} rays (1 per {a.cpu_sample_stride}^2 pixels) traced forward + "
                          f"backward with the oracle's BVH on {self.threads} threads, scaled to {a.width}x{a.height}; "
                          f"SH forward + backward, Adam, snapshot and refit on a {self.m}-Gaussian slice (1 thread), "
                          f"scaled to {a.n_gaussians}; median of {steps} steps after warm-up"}


CPU_BASELINE_STEPS, CPU_BASELINE_WARMUP = 3, 1


def cpu_baseline(a):
    """The reference arm's measurement (--impl reference) on this workload, run in a process of its own:
    inside the GPU arm's process the CUDA context and torch's worker threads share the host cores
    with the oracle's threads and slowed it by half; a separate process measures the same thing the
    reference arm does."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--steps", str(CPU_BASELINE_STEPS),
           "--warmup", str(CPU_BASELINE_WARMUP), "--scene", a.scene, "--n-gaussians", str(a.n_gaussians),
           "--width", str(a.width), "--height", str(a.height), "--cpu-sample-stride", str(a.cpu_sample_stride)]
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0", CUDA_VISIBLE_DEVICES="")
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=1800)
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    if r.returncode != 0 or not lines:
        return {"value": None, "error": (r.stderr or r.stdout)[-300:]}
    out = json.loads(lines[-1])["cpu_baseline"]
    out["process"] = "separate (bench.py --impl reference)"
    return out


def reference_arm(a, rank, world):
    """The reference's algorithm on the host cores (the CPU restatement in oracle/; the reference
    itself needs OptiX 8 and RT cores, which GB300 does not have), on the GPU arm's workload, under
    the same protocol as the GPU arm's cpu_baseline.  Each step is a bounded sample of the step,
    extrapolated: ms_per_step is the extrapolated full step, timed_seconds what the run spent."""
    if rank != 0:
        return None
    sc = make_scene(a)
    cam = make_camera(a, 0)
    cs = CpuScene(a, sc, cam)
    t, spent, fwd = cs.measure(a.steps, a.warmup)
    v = round(1.0 / t, 5)
    base = {"value": v, "unit": "train-steps/s"}
    base.update(cs.describe(a.steps, spent))
    base["hits_per_ray_sample"] = round(float(fwd["nhit"].mean()), 2)
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "train-steps/s", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(1000 * t, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": f"synthetic (seeded {a.scene} scene)",
            "config": dict(workload_config(a), parallelism=f"replicas x{world}"), "extrapolated": True,
            "timed_seconds": round(spent, 4),
            "note": "ms_per_step is the extrapolated full step; each timed step traced a sample of it "
                    "(sampled_fraction), so steps x ms_per_step exceeds timed_seconds",
            "cpu_baseline": base,
            "e2e": {"value": v, "unit": "train-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    a = parse()
    if a.record_traffic:
        if len(a.record_traffic) < 3:
            sys.exit("--record-traffic CSV KEY KERNEL [UNITS_SCALE]")
        csv_path, key, kernel = a.record_traffic[:3]
        scale = float(a.record_traffic[3]) if len(a.record_traffic) > 3 else 1.0
        print(json.dumps({key: record_traffic(csv_path, key, kernel, scale)}))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and a.impl == "gb300":
        import torch

        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    if a.impl == "reference":
        line = reference_arm(a, rank, world)
    else:
        line = gpu_arm(a, rank, world, local_rank)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1 and a.impl == "gb300":
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
