"""Python mirror of the reference's torch custom classes (torch.classes.gray.*).

graphdeco-inria/gray registers, in cuda/raytracer.cpp:3-13, the classes CameraDataHolder,
ConfigDataHolder, Framebuffer, GaussianDataHolder, MetaDataHolder, StatsDataHolder,
PPLLDataHolder and Raytracer.  This module provides the same class names, constructor
arguments, methods and tensor attributes (same shapes and dtypes, mutated in place), backed by
libgray_gb300.so through its C ABI instead of OptiX.  Code written against
`torch.classes.gray.Raytracer(...)` works against `gray_gb300.classes.Raytracer(...)`.

Differences a caller can observe: no forward per-pixel linked list is materialised (hits are
selected during traversal), and the backward hit list stores gaussian ids only.
"""
from __future__ import annotations

import torch

from . import _lib

CHANNELS = 3
MAX_ALPHA = 0.9999
NULL_PTR = 0xFFFFFFFF


def _dev():
    if not torch.cuda.is_available():
        raise _lib.GrayError("gray_gb300 needs a CUDA device (there is no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def _p(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


class CameraDataHolder:
    """cuda/core/camera.h:39-77"""

    def __init__(self, device):
        f = dict(device=device, dtype=torch.float32)
        self.origin = torch.zeros(3, **f)
        self.vertical_fov_radians = torch.zeros(1, **f)
        self.rotation_c2w = torch.zeros(3, 3, **f)
        self.rotation_w2c = torch.zeros(3, 3, **f)
        self.znear = torch.zeros(1, **f)
        self.zfar = torch.zeros(1, **f)

    def set_pose(self, c2w_origin: torch.Tensor, c2w_rotation: torch.Tensor):
        if tuple(c2w_rotation.shape) != (3, 3):
            raise RuntimeError("c2w_rotation must be 3x3")
        if tuple(c2w_origin.shape) != (3,):
            raise RuntimeError("c2w_origin must be 3")
        self.rotation_c2w.copy_(c2w_rotation)
        self.origin.copy_(c2w_origin)
        self.rotation_w2c.copy_(c2w_rotation.transpose(0, 1))


class ConfigDataHolder:
    """cuda/core/config.h:27-86 (same defaults)"""

    def __init__(self, device):
        f = dict(device=device, dtype=torch.float32)
        b = dict(device=device, dtype=torch.bool)
        self.exp_power = torch.tensor([2.0], **f)
        self.alpha_threshold = torch.tensor([0.01], **f)
        self.t_threshold = torch.tensor([0.01], **f)
        self.jitter_primary_rays = torch.tensor([False], **b)
        self.global_scale_factor = torch.ones(1, **f)
        self.eps_forward_normalization = torch.tensor([1e-12], **f)
        self.eps_scale_grad = torch.tensor([1e-12], **f)
        self.background_channels = torch.zeros(CHANNELS, **f)
        self.render_depth = torch.tensor([False], **b)
        self.render_ellipsoids = torch.tensor([False], **b)
        self.ellipsoid_min_opacity = torch.tensor([0.0], **f)
        self.rays_from_python = torch.tensor([False], **b)
        self.zero_grads = torch.tensor([True], **b)
        self.enable_sh = torch.tensor([True], **b)
        self.has_pre_mlp = torch.tensor([False], **b)
        self.needs_ray_output = torch.tensor([False], **b)
        self.update_channels = torch.tensor([True], **b)


class Framebuffer:
    """cuda/core/framebuffer.h:72-122 (registered as "Framebuffer")"""

    def __init__(self, width: int, height: int, device):
        f = dict(device=device, dtype=torch.float32)
        self.output_channels = torch.zeros(height, width, CHANNELS, **f)
        self.output_depth = torch.zeros(height, width, 1, **f)
        self.transmittance = torch.zeros(height, width, 1, **f)
        self.full_transmittance = torch.zeros(height, width, 1, **f)
        self.remaining_channels_estimate = torch.zeros(height, width, CHANNELS, **f)
        self.ray_origin = torch.zeros(height, width, 3, **f)
        self.ray_direction = torch.zeros(height, width, 3, **f)
        self.grad_output_channels = torch.zeros(height, width, CHANNELS, **f)


FramebufferDataHolder = Framebuffer

_PARAM_NAMES = ("mean", "rotation", "scale", "opacity", "channels", "sh_coeffs_dc", "sh_coeffs_rest")
_WIDTH = dict(mean=3, rotation=4, scale=3, opacity=1, channels=CHANNELS)


class GaussianDataHolder:
    """cuda/core/gaussians.h:70-419: parameters, gradients, Adam moments and pruning statistics.

    All tensors start with one row and are grown or shrunk in place by resize(); gradients are
    also exposed as the parameters' `.grad` like the reference's mutable_grad()."""

    def __init__(self, max_sh_degree: int, inference_only: bool, device, inference_sh_fp16: bool = True):
        self.device = device
        self.count = 1
        self.max_sh_degree = int(max_sh_degree)
        self.num_sh_coeffs = (self.max_sh_degree + 1) ** 2 - 1
        self.inference_only = bool(inference_only)
        f = dict(device=device, dtype=torch.float32)
        # the reference stores SH in fp16 for inference (cuda/core/gaussians.h:132); inference_sh_fp16=False
        # keeps fp32 coefficients in an inference holder (no gradients or optimiser state either way)
        sh_dtype = torch.float16 if inference_only and inference_sh_fp16 else torch.float32
        self.current_sh_degree = torch.tensor([0], device=device, dtype=torch.int32)
        self.mean = torch.zeros(1, 3, **f)
        self.rotation = torch.zeros(1, 4, **f)
        self.scale = torch.zeros(1, 3, **f)
        self.opacity = torch.zeros(1, 1, **f)
        self.channels = torch.zeros(1, CHANNELS, **f)
        self.sh_coeffs_dc = torch.zeros(1, 1, CHANNELS, device=device, dtype=sh_dtype)
        self.sh_coeffs_rest = torch.zeros(1, self.num_sh_coeffs, CHANNELS, device=device, dtype=sh_dtype)
        for name in ("lr_mean", "lr_rotation", "lr_scale", "lr_opacity", "lr_channels", "lr_sh_dc", "lr_sh_rest"):
            setattr(self, name, torch.ones(1, **f))
        self.beta_1 = torch.tensor([0.9], **f)
        self.beta_2 = torch.tensor([0.999], **f)
        self.epsilon = torch.tensor([1e-15], **f)
        self.sh_update_laziness = torch.tensor([1], device=device, dtype=torch.int32)
        for kind in ("grad_", "first_moment_", "second_moment_"):
            for name in _PARAM_NAMES:
                like = getattr(self, name)
                setattr(self, kind + name, torch.zeros(like.shape, **f))
        self.pruning_weight = torch.zeros(1, 1, **f)
        self.pruning_counter = torch.zeros(1, 1, device=device, dtype=torch.int32)
        self.was_visible = torch.zeros(1, 1, device=device, dtype=torch.bool)
        self.marked = torch.zeros(1, 1, **f)
        self._link_grads()

    def _link_grads(self):
        if self.inference_only:
            return
        for name in _PARAM_NAMES:
            getattr(self, name).grad = getattr(self, "grad_" + name)

    def _shape(self, name, n):
        if name in _WIDTH:
            return (n, _WIDTH[name])
        if name == "sh_coeffs_dc":
            return (n, 1, CHANNELS)
        return (n, self.num_sh_coeffs, CHANNELS)

    def resize(self, n: int):
        """cuda/core/gaussians.h:198-263: only shrinking is allowed once populated; the leading
        rows keep their values (torch resize_ semantics)."""
        n = int(n)
        if self.count > 1 and n > self.count:
            raise RuntimeError("The new number of Gaussians must not be larger than the current count.")
        if n < 0:
            raise RuntimeError("negative Gaussian count")
        old = self.count
        with torch.no_grad():
            self.count = n
            for name in _PARAM_NAMES:
                getattr(self, name).grad = None
                self._resize(getattr(self, name), self._shape(name, n), old)
            for name in ("lr_mean", "lr_rotation", "lr_scale", "lr_opacity", "lr_channels", "lr_sh_dc", "lr_sh_rest"):
                t = getattr(self, name)
                first = t.reshape(-1)[:1].clone()
                t.resize_(n, 1)
                if n > old:
                    t[old:] = first  # only element 0 is read; keep the rows consistent
            if not self.inference_only:  # inference keeps one-row gradient/optimiser tensors (gaussians.h:226)
                for kind in ("grad_", "first_moment_", "second_moment_"):
                    for name in _PARAM_NAMES:
                        self._resize(getattr(self, kind + name), self._shape(name, n), old)
                for name in ("pruning_weight", "pruning_counter", "marked"):
                    self._resize(getattr(self, name), (n, 1), old)
            self._resize(self.was_visible, (n, 1), old)
        self._link_grads()

    @staticmethod
    def _resize(t: torch.Tensor, shape, old: int):
        """resize_ keeping the leading rows; rows added by growing are zeroed (torch leaves them
        uninitialised, so gradients and moments would otherwise start from stale memory)."""
        t.resize_(shape)
        if shape[0] > old:
            t[old:].zero_()

    def increment_sh_degree(self):
        with torch.no_grad():
            if int(self.current_sh_degree.item()) < self.max_sh_degree:
                self.current_sh_degree += 1

    def struct(self) -> _lib.GaussiansC:
        g = _lib.GaussiansC()
        g.count = self.count
        g.max_sh_degree = self.max_sh_degree
        g.num_sh_coeffs = self.num_sh_coeffs
        g.sh_is_fp16 = int(self.sh_coeffs_dc.dtype == torch.float16)
        g.current_sh_degree = _p(self.current_sh_degree)
        for name in _PARAM_NAMES:
            setattr(g, name, _p(getattr(self, name)))
        for name in ("lr_mean", "lr_rotation", "lr_scale", "lr_opacity", "lr_channels", "lr_sh_dc", "lr_sh_rest",
                     "beta_1", "beta_2", "epsilon", "sh_update_laziness", "pruning_weight", "pruning_counter",
                     "was_visible", "marked"):
            setattr(g, name, _p(getattr(self, name)))
        if not self.inference_only:
            for kind in ("grad_", "first_moment_", "second_moment_"):
                for name in _PARAM_NAMES:
                    setattr(g, kind + name, _p(getattr(self, kind + name)))
        return g


class MetaDataHolder:
    """cuda/core/metadata.h:14-46"""

    def __init__(self, device):
        b = dict(device=device, dtype=torch.bool)
        self.run_forward_pass = torch.ones(1, **b)
        self.run_backward_pass = torch.ones(1, **b)
        self.grads_enabled = torch.ones(1, **b)
        self.total_num_calls = torch.zeros(1, device=device, dtype=torch.int32)
        self.total_num_steps = torch.zeros(1, device=device, dtype=torch.int32)

    def update(self):
        self.grads_enabled.fill_(torch.is_grad_enabled())
        self.total_num_calls += 1


class StatsDataHolder:
    """cuda/core/stats.h:11-38"""

    def __init__(self, width: int, height: int, device):
        self.num_gaussians_hit = torch.zeros(height, width, device=device, dtype=torch.int32)
        self.num_gaussians_accumulated = torch.zeros(height, width, device=device, dtype=torch.int32)

    def reset(self):
        self.num_gaussians_hit.zero_()
        self.num_gaussians_accumulated.zero_()


class PPLLDataHolder:
    """Per-pixel hit list (cuda/core/per_pixel_linked_list.h:64-118).

    The backward list holds, per pixel, a chain of segments [prev, count, ids...] in `pool`
    (u32 words); `total_hits` counts words used.  The forward list of the reference is not
    materialised (hits are selected during traversal), so its holder keeps empty buffers."""

    def __init__(self, name: str, width: int, height: int, size: int, device):
        self.name = name[:8]
        self.size = int(max(size, 1))
        self.head_per_pixel = torch.full((height, width), -1, device=device, dtype=torch.int32)
        self.total_hits = torch.zeros(1, device=device, dtype=torch.int32)
        self.pool = torch.zeros(self.size, device=device, dtype=torch.int32)
        self.gaussian_ids = self.pool
        self.distances = torch.zeros(0, device=device, dtype=torch.float16)
        self.alphas = torch.zeros(0, device=device, dtype=torch.float16)
        self.previous_entries = torch.zeros(0, device=device, dtype=torch.int32)

    @staticmethod
    def NULL_PTR() -> int:
        return NULL_PTR

    def reset(self):
        self.total_hits.zero_()
        self.head_per_pixel.fill_(-1)


class _SceneWorkspace:
    """Device buffers of the instance snapshot and the LBVH for n Gaussians."""

    def __init__(self, n: int, device, training: bool = True):
        n = max(int(n), 0)
        m = max(n - 1, 1)
        nn = max(n, 1)
        f = dict(device=device, dtype=torch.float32)
        i32 = dict(device=device, dtype=torch.int32)
        self.n = n
        self.geom = torch.zeros(nn, 12, **f)
        self.l2w = torch.zeros(nn, 12, **f)
        self.aabb = torch.zeros(nn, 8, **f)
        self.visible = torch.zeros(nn, device=device, dtype=torch.uint8)
        self.live = torch.zeros(nn, 2, **f)
        self.grad_acc = torch.zeros(nn, 16, **f)
        self.nodes = torch.zeros(m, 16, **f)
        self.int_parent = torch.zeros(m, **i32)
        self.leaf_parent = torch.zeros(nn, **i32)
        self.order = torch.zeros(nn, **i32)
        self.codes = torch.zeros(nn, **i32)
        self.refit_flags = torch.zeros(m, **i32)
        words = int(_lib.load().gray_sort_tmp_words(n))
        self.sort_tmp = torch.zeros(max(words, 1), **i32)
        self.root_box = torch.zeros(8, **f)
        self.bounds = torch.zeros(8, **i32)
        self.bwd_rec = torch.zeros(nn if training else 1, 24, **f)
        self.bvh_valid = False

    def struct(self) -> _lib.SceneC:
        s = _lib.SceneC()
        for name in ("geom", "l2w", "aabb", "visible", "live", "grad_acc", "nodes", "int_parent", "leaf_parent",
                     "order", "codes", "refit_flags", "sort_tmp", "root_box", "bounds", "bwd_rec"):
            setattr(s, name, _p(getattr(self, name)))
        s.bvh_valid = int(self.bvh_valid)
        return s


class Raytracer:
    """cuda/raytracer.h:29-184: torch.classes.gray.Raytracer over libgray_gb300.so."""

    def __init__(self, width: int, height: int, num_gaussians: int, sh_max_degree: int, ppll_forward_size: int,
                 ppll_backward_size: int, inference_only: bool = False, inference_sh_fp16: bool = True):
        _lib.load()
        dev = _dev()
        self.device = dev
        self.width = int(width)
        self.height = int(height)
        self.alloc_width = int(width)
        self.alloc_height = int(height)
        self.inference_only = bool(inference_only)
        self.camera_data = CameraDataHolder(dev)
        self.config_data = ConfigDataHolder(dev)
        self.framebuffer_data = Framebuffer(self.width, self.height, dev)
        self.gaussian_data = GaussianDataHolder(sh_max_degree, inference_only, dev, inference_sh_fp16)
        self.meta_data = MetaDataHolder(dev)
        self.stats_data = StatsDataHolder(self.width, self.height, dev)
        self.ppll_forward_data = PPLLDataHolder("forward", self.width, self.height, 1, dev)
        self.ppll_backward_data = PPLLDataHolder("backward", self.width, self.height,
                                                 1 if inference_only else ppll_backward_size, dev)
        self.status = torch.zeros(1, device=dev, dtype=torch.int32)
        # work order of the forward's pixel tiles (densest first), rebuilt by every forward
        self.schedule = torch.zeros(int(_lib.load().gray_schedule_words(self.width, self.height)), device=dev,
                                    dtype=torch.int32)
        self.trace_variant = 0  # forward-kernel variant (0 = automatic choice); results do not depend on it
        # counts forwards: each one overwrites the colours, saved state and hit lists a backward replays
        self.generation = 0
        self._scene = _SceneWorkspace(1, dev, not self.inference_only)
        self._params = None
        if num_gaussians > 0:
            self.resize(num_gaussians)

    # ---- state plumbing ----
    def _build_params(self) -> _lib.ParamsC:
        p = _lib.ParamsC()
        p.image_width = self.alloc_width
        p.image_height = self.alloc_height
        p.render_width = self.width
        p.render_height = self.height
        c = self.camera_data
        for name in ("origin", "vertical_fov_radians", "rotation_c2w", "rotation_w2c", "znear", "zfar"):
            setattr(p.camera, name, _p(getattr(c, name)))
        cf = self.config_data
        for name, _ in _lib.ConfigC._fields_:
            setattr(p.config, name, _p(getattr(cf, name)))
        fb = self.framebuffer_data
        for name, _ in _lib.FramebufferC._fields_:
            setattr(p.framebuffer, name, _p(getattr(fb, name)))
        p.gaussians = self.gaussian_data.struct()
        m = self.meta_data
        for name, _ in _lib.MetadataC._fields_:
            setattr(p.metadata, name, _p(getattr(m, name)))
        p.stats.num_gaussians_hit = _p(self.stats_data.num_gaussians_hit)
        p.stats.num_gaussians_accumulated = _p(self.stats_data.num_gaussians_accumulated)
        h = self.ppll_backward_data
        p.hitlist.head_per_pixel = _p(h.head_per_pixel)
        p.hitlist.total_words = _p(h.total_hits)
        p.hitlist.pool = _p(h.pool)
        p.hitlist.size = h.size
        p.hitlist.schedule = _p(self.schedule)
        p.scene = self._scene.struct()
        p.status = _p(self.status)
        p.trace_variant = int(self.trace_variant)
        return p

    def _call(self, name: str):
        if self._params is None:
            self._params = self._build_params()
        _lib.call(name, self._params, torch.cuda.current_stream(self.device).cuda_stream)

    def _invalidate(self):
        self._params = None

    # ---- reference methods ----
    def forward_pass(self):
        self.meta_data.grads_enabled.fill_(torch.is_grad_enabled())
        self.generation += 1
        self._call("gray_forward_pass")

    def forward_pass_display(self):
        self.generation += 1
        self._call("gray_forward_pass_display")

    def backward_pass(self):
        self._call("gray_backward_pass")

    def step(self):
        self._call("gray_step")

    def update_bvh(self):
        self._call("gray_update_bvh")

    def rebuild_bvh(self):
        self._scene.bvh_valid = True
        self._invalidate()
        try:
            self._call("gray_rebuild_bvh")
        except Exception:
            self._scene.bvh_valid = False
            self._invalidate()
            raise

    def resize(self, new_num_gaussians: int):
        self.gaussian_data.resize(new_num_gaussians)
        self._scene = _SceneWorkspace(self.gaussian_data.count, self.device, not self.inference_only)
        self._invalidate()

    def set_trace_variant(self, variant: int):
        """Select the forward-trace kernel variant (0 = automatic choice); every variant gives identical
        results."""
        self.trace_variant = int(variant)
        self._invalidate()

    def set_render_resolution(self, new_width: int, new_height: int):
        if new_width < 1 or new_height < 1:
            raise RuntimeError("render resolution must be positive")
        if new_width > self.alloc_width or new_height > self.alloc_height:
            raise RuntimeError("render resolution cannot exceed the allocated framebuffer size")
        self.width = int(new_width)
        self.height = int(new_height)
        self._invalidate()

    def get_camera(self):
        return self.camera_data

    def get_config(self):
        return self.config_data

    def get_framebuffer(self):
        return self.framebuffer_data

    def get_gaussians(self):
        return self.gaussian_data

    def get_metadata(self):
        return self.meta_data

    def get_stats(self):
        return self.stats_data

    def get_ppll_forward_data(self):
        return self.ppll_forward_data

    def get_ppll_backward_data(self):
        return self.ppll_backward_data

    def get_num_channels(self) -> int:
        return CHANNELS

    def get_max_alpha(self) -> float:
        return MAX_ALPHA

    # ---- device-side error reporting (replaces the reference's __trap on overflow) ----
    def check_status(self):
        """Synchronise and raise if a kernel reported a device-side condition."""
        v = int(self.status.item())
        if v:
            self.status.zero_()
            raise _lib.GrayError(f"device status {v:#x}: " + ", ".join(
                n for bit, n in ((1, "backward hit list overflow (increase ppll_backward_size)"),
                                 (2, "BVH traversal limit exceeded"), (4, "refit budget exhausted"),
                                 (8, "render_ellipsoids=True is only supported for no-grad display renders"),
                                 (16, "a bulk copy did not complete (streaming kernel stopped early)"))
                if v & bit))

    def scene_workspace(self):
        return self._scene
