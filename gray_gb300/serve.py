"""Serving: a continuous-batching render loop over several resident scenes.

    srv = RenderServer([tracer_0, tracer_1, ...])      # inference tracers, BVHs built
    srv.submit(scene_index, camera, arrival_time)
    srv.poll()                                         # admit / launch / retire; call in a loop
    srv.completed                                      # finished requests with latencies

Requests wait in a queue.  Whenever an execution slot (a CUDA stream) is free, every waiting request
whose output and per-view colour buffers fit in the free device memory (cudaMemGetInfo minus a
reserve) is admitted -- requests that arrived while earlier batches were running join the next
batch -- and the whole batch, across scenes and resolutions, is rendered in one persistent launch
(gray_gb300.batch).  With two slots, one batch can be prepared and launched while the other is still
on the GPU, so their work overlaps on the device.  A request's pixels are bit-identical whether it
is rendered alone or in any mix (each ray is traced independently; nothing is shared across rays).

`plain_loop` is the baseline: one request per launch, in arrival order, through the reference's
forward_pass_display path.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .batch import DEFAULT_BLOCKS_PER_SM, DEFAULT_VARIANT, BatchRenderer, _bind
from .camera import CameraInfo


@dataclass
class Request:
    rid: int
    scene: int
    camera: CameraInfo
    arrival: float
    admitted: float = 0.0
    finished: float = 0.0
    image: torch.Tensor | None = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival

    @property
    def rays(self) -> int:
        return self.camera.image_width * self.camera.image_height


@dataclass
class _Slot:
    stream: torch.cuda.Stream
    renderer: BatchRenderer
    event: torch.cuda.Event | None = None
    batch: list = field(default_factory=list)
    bytes: int = 0


class RenderServer:
    def __init__(self, tracers, slots: int = 2, max_batch: int = 32, reserve_bytes: int = 4 << 30,
                 keep_images: bool = False, variant: int | None = None, blocks_per_sm: int | None = None,
                 ray_budget: int | None = None):
        self.tracers = list(tracers)
        self.device = self.tracers[0].device
        self.slots = [_Slot(torch.cuda.Stream(self.device),
                            BatchRenderer(self.tracers, use_graph=False, autotune=False,
                                          variant=variant or DEFAULT_VARIANT,
                                          blocks_per_sm=blocks_per_sm or DEFAULT_BLOCKS_PER_SM, cache_plans=False)) for _ in range(slots)]
        self.max_batch = max_batch
        # at most this many rays per batch (a batch always takes its first request): a batch's
        # requests finish together, so an unbounded batch makes its small requests wait for its
        # largest ones and holds its slot for long
        self.ray_budget = ray_budget
        self.reserve = reserve_bytes
        self.keep_images = keep_images
        self.queue: list[Request] = []
        self.completed: list[Request] = []
        self.inflight_bytes = 0
        self._next = 0

    def tune(self, sample):
        """Pick the kernel variant and persistent grid size once, with the batch autotuner, on a
        representative list of (scene, camera) requests; every later batch uses the choice (a
        per-batch tuning would cost more than it saves, since served batches rarely repeat)."""
        probe = BatchRenderer(self.tracers, use_graph=False, autotune=True, cache_plans=False)
        reqs = sorted(((int(s), c) for s, c in sample), key=lambda r: r[0])
        probe._scene_table()
        choice = probe._tune(reqs)
        torch.cuda.synchronize(self.device)
        for sl in self.slots:
            sl.renderer.fixed = choice
            sl.renderer.tuned.clear()
        return choice

    def submit(self, scene: int, camera: CameraInfo, arrival: float | None = None) -> Request:
        r = Request(self._next, scene, camera, time.perf_counter() if arrival is None else arrival)
        self._next += 1
        self.queue.append(r)
        return r

    def _request_bytes(self, r: Request) -> int:
        """Output image, the view's colour buffer and its packet groups' BVH frontiers (at most one
        group per 128 pixels, rounded up per 8x16 or 16x8 pixel group)."""
        n = self.tracers[r.scene].get_gaussians().count
        w, h = r.camera.image_width, r.camera.image_height
        groups = max(-(-w // 8) * -(-h // 16), -(-w // 16) * -(-h // 8))
        return 3 * 4 * r.rays + 12 * n + 4 * int(_bind().gray_frontier_words()) * groups + 256

    def _retire(self):
        now = time.perf_counter()
        for sl in self.slots:
            if sl.event is not None and sl.event.query():
                for r, img in sl.batch:
                    r.finished = now
                    if self.keep_images:
                        r.image = img
                    self.completed.append(r)
                self.inflight_bytes -= sl.bytes
                sl.event, sl.batch, sl.bytes = None, [], 0

    def _admit(self, free_bytes: int):
        batch, need, rays = [], 0, 0
        budget = free_bytes - self.reserve
        while self.queue and len(batch) < self.max_batch:
            r = self.queue[0]
            b = self._request_bytes(r)
            if batch and need + b > budget:
                break
            if not batch and b > budget:
                break  # wait for memory to free up
            if batch and self.ray_budget is not None and rays + r.rays > self.ray_budget:
                break
            batch.append(self.queue.pop(0))
            need += b
            rays += r.rays
        return batch, need

    def poll(self) -> int:
        """Retire finished batches, then fill every free slot with a new batch.  Returns the
        number of requests launched."""
        self._retire()
        launched = 0
        for sl in self.slots:
            if sl.event is not None or not self.queue:
                continue
            free, _ = torch.cuda.mem_get_info(self.device)
            # memory the caching allocator holds but does not use is free for our purposes too
            free += torch.cuda.memory_reserved(self.device) - torch.cuda.memory_allocated(self.device)
            batch, need = self._admit(free)
            if not batch:
                break
            now = time.perf_counter()
            for r in batch:
                r.admitted = now
            with torch.cuda.stream(sl.stream):
                imgs = sl.renderer.render([(r.scene, r.camera) for r in batch])
                if self.keep_images:
                    imgs = [im.clone() for im in imgs]
                ev = torch.cuda.Event()
                ev.record(sl.stream)
            sl.event, sl.batch, sl.bytes = ev, list(zip(batch, imgs)), need
            self.inflight_bytes += need
            launched += len(batch)
        return launched

    def idle(self) -> bool:
        return not self.queue and all(sl.event is None for sl in self.slots)

    def drain(self):
        while not self.idle():
            self.poll()
            time.sleep(0.0002)


def poisson_arrivals(rate_hz: float, count: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_hz, count))


def run_served(server: RenderServer, schedule):
    """schedule: list of (arrival_offset_s, scene, camera).  Submits each request when its arrival
    time has passed and polls until all are done.  Returns (requests, wall seconds)."""
    t0 = time.perf_counter()
    i = 0
    reqs = []
    while i < len(schedule) or not server.idle():
        now = time.perf_counter() - t0
        while i < len(schedule) and schedule[i][0] <= now:
            off, s, cam = schedule[i]
            reqs.append(server.submit(s, cam, t0 + off))
            i += 1
        server.poll()
        time.sleep(0.0001)
    return reqs, time.perf_counter() - t0


def plain_loop(tracers, schedule, znear=0.0, zfar=99999.9):
    """One request per launch through forward_pass_display, in arrival order.  Returns a list of
    (latency_s, rays) and the wall seconds."""
    t0 = time.perf_counter()
    out = []
    for off, s, cam in schedule:
        while time.perf_counter() - t0 < off:
            time.sleep(0.0001)
        t = tracers[s]
        c = t.get_camera()
        c.znear.fill_(znear)
        c.zfar.fill_(zfar)
        c.vertical_fov_radians.fill_(float(cam.fov_y))
        c.set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
        t.get_config().rays_from_python.fill_(False)
        t.set_render_resolution(cam.image_width, cam.image_height)
        with torch.no_grad():
            t.forward_pass_display()
        torch.cuda.synchronize(t.device)
        out.append((time.perf_counter() - (t0 + off), cam.image_width * cam.image_height))
    return out, time.perf_counter() - t0
