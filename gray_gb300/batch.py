"""Batched rendering: many views of resident scenes in one persistent launch, replayed from a CUDA
graph, with the kernel variant and persistent-grid size picked by an autotuner.

    br = BatchRenderer([tracer_a, tracer_b])             # gray_gb300.classes.Raytracer per scene
    images = br.render([(0, cam0), (1, cam1), (0, cam2)])  # list of [3, h, w] views

Per pixel the result is bit-identical to rendering the same view alone with forward_pass_display
(same ray arithmetic, same traversal and selection); the batch only changes how work is scheduled:
one launch whose warps pull 32-ray packets of every view from a global counter.  The first render of
a batch signature (the scenes and resolutions of its views) autotunes and captures a CUDA graph;
later renders with the same signature update the camera poses in pinned host memory and replay.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .camera import CameraInfo


class BatchSceneC(ctypes.Structure):
    _fields_ = [("geom", ctypes.c_void_p), ("live", ctypes.c_void_p), ("nodes", ctypes.c_void_p),
                ("root_box", ctypes.c_void_p), ("l2w", ctypes.c_void_p), ("n", ctypes.c_int32), ("exp_power", ctypes.c_float),
                ("alpha_threshold", ctypes.c_float), ("t_threshold", ctypes.c_float), ("bg", ctypes.c_float * 3),
                ("pad", ctypes.c_int32)]


class BatchViewC(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("w2c", ctypes.c_float * 9), ("fov_y", ctypes.c_float),
                ("znear", ctypes.c_float), ("zfar", ctypes.c_float), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("scene", ctypes.c_uint32), ("packet_offset", ctypes.c_uint32),
                ("group_offset", ctypes.c_uint32), ("out_offset", ctypes.c_uint64), ("channels", ctypes.c_void_p)]


def _bind():
    L = _lib.load()
    if not getattr(L, "_batch_bound", False):
        L.gray_batch_packets.restype = ctypes.c_uint32
        L.gray_batch_packets.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32]
        L.gray_batch_groups.restype = ctypes.c_uint32
        L.gray_batch_groups.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32]
        L.gray_frontier_words.restype = ctypes.c_uint32
        L.gray_frontier_words.argtypes = []
        L.gray_batch_prep.restype = ctypes.c_int
        L.gray_batch_prep.argtypes = [ctypes.POINTER(_lib.ParamsC), ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                      ctypes.c_void_p]
        L.gray_render_batch.restype = ctypes.c_int
        L.gray_render_batch.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                        ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
        L._batch_bound = True
    return L


def _check(L, rc, what):
    if rc != 0:
        raise _lib.GrayError(f"{what}: {L.gray_last_error().decode()} (code {rc})")


# untuned choice: 4x8 packets with a 16-entry k-buffer (the library's default variant), as many
# blocks per SM as its register cap allows (6)
DEFAULT_VARIANT, DEFAULT_BLOCKS_PER_SM = 7, 6
# candidates the autotuner tries: (kernel variant, persistent blocks per SM), each variant with the
# block counts around its residency limit (32-entry buffers: 4 per SM; 16 entries uncapped: 3;
# 16 entries capped: 6)
TUNE_CANDIDATES = [(1, 4), (5, 4), (2, 3), (6, 3), (3, 5), (3, 6), (7, 5), (7, 6)]


@dataclass
class _Plan:
    """Buffers and descriptors of one batch signature."""
    signature: tuple
    variant: int
    blocks_per_sm: int
    views_host: torch.Tensor       # pinned bytes of the view array
    views_dev: torch.Tensor
    origins_host: torch.Tensor     # pinned [V,3]
    origins_dev: torch.Tensor
    channels: list                 # per scene: [V_s, N_s, 3] or None
    view_rows: list                # per view: (scene, row inside that scene's channel block)
    out: torch.Tensor
    offsets: list
    total_packets: int
    counter: torch.Tensor
    frontier: torch.Tensor         # per packet group: its BVH frontier (GRAY_FRONTIER_WORDS words)
    total_groups: int
    graph: object = None


class BatchRenderer:
    def __init__(self, tracers, use_graph: bool = True, autotune: bool = True, variant: int | None = None,
                 blocks_per_sm: int | None = None, znear: float = 0.0, zfar: float = 99999.9,
                 cache_plans: bool = True):
        self.L = _bind()
        self.tracers = list(tracers)
        self.device = self.tracers[0].device
        self.use_graph = use_graph
        self.autotune = autotune and variant is None
        self.fixed = (variant or DEFAULT_VARIANT, blocks_per_sm or DEFAULT_BLOCKS_PER_SM)
        self.znear, self.zfar = float(znear), float(zfar)
        self.status = torch.zeros(1, device=self.device, dtype=torch.int32)
        self.plans = {}
        self.cache_plans = cache_plans or use_graph
        self.tuned = {}
        self._scenes_dev = None
        self._scene_ptrs = None

    # ---------------- scene table ----------------
    def _scene_table(self):
        ptrs = []
        for t in self.tracers:
            ws = t.scene_workspace()
            ptrs.append((ws.geom.data_ptr(), ws.live.data_ptr(), ws.nodes.data_ptr(), ws.root_box.data_ptr(),
                         ws.l2w.data_ptr(), t.get_gaussians().count))
        if self._scenes_dev is not None and ptrs == self._scene_ptrs:
            return self._scenes_dev
        arr = (BatchSceneC * len(self.tracers))()
        for i, t in enumerate(self.tracers):
            cfg = t.get_config()
            g, lv, nd, rb, lw, n = ptrs[i]
            arr[i].geom, arr[i].live, arr[i].nodes, arr[i].root_box, arr[i].l2w, arr[i].n = g, lv, nd, rb, lw, n
            arr[i].exp_power = float(cfg.exp_power.item())
            arr[i].alpha_threshold = float(cfg.alpha_threshold.item())
            arr[i].t_threshold = float(cfg.t_threshold.item())
            for k in range(3):
                arr[i].bg[k] = float(cfg.background_channels[k].item())
        raw = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8)
        self._scenes_dev = raw.to(self.device)
        self._scene_ptrs = ptrs
        self.plans.clear()
        return self._scenes_dev

    # ---------------- planning ----------------
    def _plan(self, reqs, variant, bps):
        sig = tuple((s, c.image_width, c.image_height) for s, c in reqs)
        V = len(reqs)
        per_scene = {}
        view_rows = []
        for s, _ in reqs:
            view_rows.append((s, per_scene.get(s, 0)))
            per_scene[s] = per_scene.get(s, 0) + 1
        channels = [None] * len(self.tracers)
        for s, cnt in per_scene.items():
            n = self.tracers[s].get_gaussians().count
            channels[s] = torch.empty(cnt, max(n, 1), 3, device=self.device)
        offsets, total, packets = [], 0, 0
        for s, c in reqs:
            offsets.append(total)
            total += 3 * c.image_width * c.image_height
        out = torch.empty(max(total, 1), device=self.device)
        vh = torch.zeros(V * ctypes.sizeof(BatchViewC), dtype=torch.uint8).pin_memory()
        oh = torch.zeros(V, 3, dtype=torch.float32).pin_memory()
        groups = sum(int(self.L.gray_batch_groups(c.image_width, c.image_height, variant)) for _, c in reqs)
        frontier = torch.empty(max(groups, 1) * int(self.L.gray_frontier_words()), device=self.device,
                               dtype=torch.int32)
        plan = _Plan(sig, variant, bps, vh, torch.zeros_like(vh, device=self.device), oh,
                     torch.zeros(V, 3, device=self.device), channels, view_rows, out, offsets, 0,
                     torch.zeros(1, device=self.device, dtype=torch.int32), frontier, groups)
        self._write_views(plan, reqs)
        return plan

    def _write_views(self, plan, reqs):
        arr = (BatchViewC * len(reqs)).from_buffer(plan.views_host.numpy())
        packets = groups = 0
        for i, (s, cam) in enumerate(reqs):
            rot = cam.rotation_c2w_blender()
            w2c = rot.T.astype(np.float32)
            v = arr[i]
            for k in range(3):
                v.origin[k] = float(cam.origin[k])
            for k in range(9):
                v.w2c[k] = float(w2c.reshape(-1)[k])
            v.fov_y = float(cam.fov_y)
            v.znear, v.zfar = self.znear, self.zfar
            v.width, v.height = cam.image_width, cam.image_height
            v.scene = s
            v.packet_offset = packets
            packets += int(self.L.gray_batch_packets(cam.image_width, cam.image_height, plan.variant))
            v.group_offset = groups
            groups += int(self.L.gray_batch_groups(cam.image_width, cam.image_height, plan.variant))
            v.out_offset = plan.offsets[i]
            sc, row = plan.view_rows[i]
            v.channels = plan.channels[sc][row].data_ptr()
            plan.origins_host[i] = torch.from_numpy(np.asarray(cam.origin, np.float32))
        plan.total_packets = packets

    def _launch(self, plan):
        stream = torch.cuda.current_stream(self.device)
        plan.views_dev.copy_(plan.views_host, non_blocking=True)
        plan.origins_dev.copy_(plan.origins_host, non_blocking=True)
        rows = {}
        for i, (s, row) in enumerate(plan.view_rows):
            rows.setdefault(s, []).append(i)
        for s, idx in rows.items():
            t = self.tracers[s]
            if t._params is None:
                t._params = t._build_params()
            first = idx[0]
            rc = self.L.gray_batch_prep(ctypes.byref(t._params),
                                        ctypes.c_void_p(plan.origins_dev[first:].data_ptr()), len(idx),
                                        ctypes.c_void_p(plan.channels[s].data_ptr()), ctypes.c_void_p(stream.cuda_stream))
            _check(self.L, rc, "gray_batch_prep")
        rc = self.L.gray_render_batch(ctypes.c_void_p(self._scenes_dev.data_ptr()),
                                      ctypes.c_void_p(plan.views_dev.data_ptr()), len(plan.view_rows),
                                      plan.total_packets, ctypes.c_void_p(plan.out.data_ptr()),
                                      ctypes.c_void_p(plan.counter.data_ptr()),
                                      ctypes.c_void_p(plan.frontier.data_ptr()), plan.total_groups,
                                      plan.variant, plan.blocks_per_sm,
                                      ctypes.c_void_p(self.status.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        _check(self.L, rc, "gray_render_batch")

    def _tune(self, reqs):
        sig = tuple((s, c.image_width, c.image_height) for s, c in reqs)
        if sig in self.tuned:
            return self.tuned[sig]
        if not self.autotune:
            self.tuned[sig] = self.fixed
            return self.fixed
        best, best_ms = None, float("inf")
        for variant, bps in TUNE_CANDIDATES:
            plan = self._plan(reqs, variant, bps)
            self._launch(plan)
            torch.cuda.synchronize(self.device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(2):
                self._launch(plan)
            e1.record()
            torch.cuda.synchronize(self.device)
            ms = e0.elapsed_time(e1) / 2
            if ms < best_ms:
                best, best_ms = (variant, bps), ms
        self.tuned[sig] = best
        return best

    # ---------------- public ----------------
    def render(self, reqs):
        """reqs: list of (scene_index, CameraInfo); views must have contiguous same-scene groups
        in any order.  Returns a list of [3, h, w] tensors (views into one output buffer)."""
        reqs = [(int(s), c) for s, c in reqs]
        # views of one scene must be adjacent for the per-scene colour prep (origins slice)
        order = sorted(range(len(reqs)), key=lambda i: reqs[i][0])
        sreqs = [reqs[i] for i in order]
        self._scene_table()
        sig = tuple((s, c.image_width, c.image_height) for s, c in sreqs)
        plan = self.plans.get(sig)
        if plan is None:
            variant, bps = self._tune(sreqs)
            plan = self._plan(sreqs, variant, bps)
            if self.cache_plans:
                self.plans[sig] = plan
            if self.use_graph:
                self._launch(plan)  # warm-up outside capture
                torch.cuda.synchronize(self.device)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._launch(plan)
                plan.graph = g
        else:
            self._write_views(plan, sreqs)
        if plan.graph is not None:
            plan.graph.replay()
        else:
            self._launch(plan)
        outs = [None] * len(reqs)
        for k, i in enumerate(order):
            s, cam = reqs[i]
            off = plan.offsets[k]
            outs[i] = plan.out[off:off + 3 * cam.image_width * cam.image_height].view(
                cam.image_height, cam.image_width, 3).permute(2, 0, 1)
        return outs

    def check_status(self):
        v = int(self.status.item())
        if v:
            self.status.zero_()
            raise _lib.GrayError(f"batch render device status {v:#x}")
