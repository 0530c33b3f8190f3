"""torch.autograd.Function around the hand-written backward.

    img = gray_gb300.autograd.render(tracer, camera, mean, rotation, scale, opacity,
                                     channels=None, sh_dc=None, sh_rest=None, recompute=None)

`tracer` is a gray_gb300.classes.Raytracer sized for the Gaussians.  The parameters are copied into
the tracer's holders (a no-op when they already are the holder tensors), the instance snapshot is
refreshed (the reference's update_bvh) and the forward trace runs; the returned [3, h, w] image is
differentiable with respect to every parameter passed in.  The backward of the autograd graph calls
the library's reverse-replay backward (reference: cuda/backward_pass.cu) and the SH backward.

What a backward replays -- the composited hit lists, the per-pixel saved state (transmittance, full
transmittance, tail estimate, rays) and the view's SH colours -- lives in the tracer and is
overwritten by the tracer's next forward.  The reference has the same rule (a backward needs its
forward's state unmodified, README.md:143-154) and leaves it to the caller; here each render keeps
track of it:

* while no other forward has run on the tracer, the backward replays the state in place (no copy);
* when another render is about to overwrite it, the state is evicted: copied out of the tracer
  ("stored") if the copy fits in free device memory, otherwise dropped, and the backward then re-runs
  this render's forward first ("recomputed": deterministic, so the hit lists are identical);
* a forward made outside this module (forward_pass / forward_pass_display on the tracer) gives no
  notice, so a render whose state it overwrote is recomputed;
* renders on one tracer from different parameter tensors: a backward whose render is no longer
  resident reloads its own tensors, refreshes the snapshot and recomputes.  The values of the
  parameters must not change between a render and its backward (the reference's rule too).

recompute=None (default) chooses by free memory as above; recompute=False always stores on eviction
(an allocation failure then raises); recompute=True never keeps the state and always re-runs the
forward in the backward, so many renders share one hit-list pool at the cost of a second forward.
"""
from __future__ import annotations

import weakref

import torch

from .camera import CameraInfo

# device memory left free when deciding whether an evicted render's state may be copied
_RESERVE_BYTES = 1 << 30

_FB_STATE = ("transmittance", "full_transmittance", "remaining_channels_estimate", "ray_origin", "ray_direction")
_CAM_STATE = ("origin", "vertical_fov_radians", "rotation_c2w", "rotation_w2c", "znear", "zfar")


def _set_camera(tracer, camera: CameraInfo, znear=0.0, zfar=99999.9):
    c = tracer.get_camera()
    c.znear.fill_(znear)
    c.zfar.fill_(zfar)
    c.vertical_fov_radians.fill_(float(camera.fov_y))
    c.set_pose(camera.origin_cuda(), camera.rotation_c2w_blender_cuda())
    tracer.get_config().rays_from_python.fill_(False)


def _load(tracer, names, tensors):
    g = tracer.get_gaussians()
    with torch.no_grad():
        for name, t in zip(names, tensors):
            if t is None:
                continue
            dst = getattr(g, name)
            if t.data_ptr() != dst.data_ptr():
                dst.copy_(t.detach().reshape(dst.shape))


def free_device_bytes(device) -> int:
    """Free device memory plus what the caching allocator holds unused."""
    free, _ = torch.cuda.mem_get_info(device)
    unused = torch.cuda.memory_reserved(device) - torch.cuda.memory_allocated(device)
    return int(free + max(unused, 0))


class _TraceState:
    """The state one render's forward left in its tracer, and where it is now: resident in the
    tracer (generation matches), saved in copies, or to be recomputed."""

    def __init__(self, tracer, camera, policy, params):
        self.tracer, self.camera, self.policy = tracer, camera, policy
        self.params = params
        self.params_key = _params_key(params)
        self.use_sh = params[5] is not None
        self.generation = tracer.generation
        self.saved = None
        self.recompute = policy == "recompute"
        self.consumed = False

    def resident(self) -> bool:
        ref = getattr(self.tracer, "_gray_resident", None)
        return ref is not None and ref() is self and self.generation == self.tracer.generation

    def copy_bytes(self) -> int:
        t = self.tracer
        fb, hl = t.get_framebuffer(), t.get_ppll_backward_data()
        used = int(hl.total_hits.item())
        n = sum(getattr(fb, k).numel() for k in _FB_STATE) + hl.head_per_pixel.numel() + used
        return 4 * (n + t.get_gaussians().channels.numel())

    def evict(self):
        """Called before another forward overwrites this render's state in the tracer."""
        if self.saved is not None or self.recompute or not self.resident():
            self.recompute = self.saved is None
            return
        if self.consumed:  # its backward ran; a second one (retain_graph) recomputes
            self.recompute = True
            return
        need = self.copy_bytes()
        if self.policy == "auto" and need + _RESERVE_BYTES > free_device_bytes(self.tracer.device):
            self.recompute = True
            return
        t = self.tracer
        fb, hl, cam = t.get_framebuffer(), t.get_ppll_backward_data(), t.get_camera()
        used = int(hl.total_hits.item())
        self.saved = {
            "fb": {k: getattr(fb, k).clone() for k in _FB_STATE},
            "head": hl.head_per_pixel.clone(),
            "total": hl.total_hits.clone(),
            "pool": hl.pool[:used].clone(),
            "channels": t.get_gaussians().channels.clone(),
            "cam": {k: getattr(cam, k).clone() for k in _CAM_STATE},
        }

    def make_resident(self):
        """Put this render's forward state back in the tracer before its backward."""
        if self.resident() and not self.recompute:
            return
        t = self.tracer
        _evict_resident(t)
        t.get_config().enable_sh.fill_(self.use_sh)
        if getattr(t, "_gray_params_key", None) != self.params_key:
            _load(t, _PARAM_NAMES, self.params)
            t.update_bvh()
            t._gray_params_key = self.params_key
            self.recompute = True  # the tracer's per-forward values (opacity, scaling factor) changed too
        if self.saved is not None and not self.recompute:
            sv = self.saved
            fb, hl, cam = t.get_framebuffer(), t.get_ppll_backward_data(), t.get_camera()
            with torch.no_grad():
                for k, v in sv["fb"].items():
                    getattr(fb, k).copy_(v)
                for k, v in sv["cam"].items():
                    getattr(cam, k).copy_(v)
                hl.head_per_pixel.copy_(sv["head"])
                hl.total_hits.copy_(sv["total"])
                hl.pool[: sv["pool"].numel()].copy_(sv["pool"])
                t.get_gaussians().channels.copy_(sv["channels"])
                t.get_gaussians().was_visible.zero_()
            t.generation += 1
        else:
            _set_camera(t, self.camera)
            with torch.enable_grad():
                t.forward_pass()
        self.generation = t.generation
        self.saved = None
        self.recompute = self.policy == "recompute"
        t._gray_resident = weakref.ref(self)


_PARAM_NAMES = ("mean", "rotation", "scale", "opacity", "channels", "sh_coeffs_dc", "sh_coeffs_rest")


def _params_key(params):
    return tuple(None if t is None else (t.data_ptr(), tuple(t.shape)) for t in params)


def _evict_resident(tracer):
    ref = getattr(tracer, "_gray_resident", None)
    st = ref() if ref is not None else None
    if st is not None:
        st.evict()
    tracer._gray_resident = None


class RayTraceFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, tracer, camera, policy, mean, rotation, scale, opacity, channels, sh_dc, sh_rest):
        _evict_resident(tracer)
        params = tuple(None if t is None else t.detach() for t in (mean, rotation, scale, opacity, channels, sh_dc,
                                                                   sh_rest))
        _load(tracer, _PARAM_NAMES, params)
        tracer._gray_params_key = _params_key(params)
        use_sh = sh_dc is not None
        tracer.get_config().enable_sh.fill_(use_sh)
        tracer.update_bvh()
        _set_camera(tracer, camera)
        with torch.enable_grad():
            tracer.forward_pass()
        h, w = tracer.height, tracer.width
        out = tracer.get_framebuffer().output_channels[:h, :w].detach().clone().moveaxis(-1, 0)
        st = _TraceState(tracer, camera, policy, params)
        tracer._gray_resident = weakref.ref(st)
        ctx.state, ctx.use_sh = st, use_sh
        ctx.shapes = [None if t is None else t.shape for t in (mean, rotation, scale, opacity, channels, sh_dc,
                                                             sh_rest)]
        return out

    @staticmethod
    def backward(ctx, grad_out):
        st = ctx.state
        st.make_resident()
        tracer = st.tracer
        g = tracer.get_gaussians()
        with torch.no_grad():
            for name in ("grad_mean", "grad_rotation", "grad_scale", "grad_opacity", "grad_channels",
                         "grad_sh_coeffs_dc", "grad_sh_coeffs_rest"):
                getattr(g, name).zero_()
            h, w = tracer.height, tracer.width
            tracer.get_framebuffer().grad_output_channels[:h, :w].copy_(grad_out.moveaxis(0, -1))
        tracer.backward_pass()
        st.consumed = True
        grads = [g.grad_mean, g.grad_rotation, g.grad_scale, g.grad_opacity, g.grad_channels, g.grad_sh_coeffs_dc,
                 g.grad_sh_coeffs_rest]
        out = []
        for gr, shape in zip(grads, ctx.shapes):
            out.append(None if shape is None else gr.clone().reshape(shape))
        return (None, None, None, *out)


def render(tracer, camera: CameraInfo, mean, rotation, scale, opacity, channels=None, sh_dc=None, sh_rest=None,
           recompute: bool | None = None):
    """Differentiable render of `camera` ([3, h, w]) through the hand-written backward.

    recompute: None = keep the forward's state while it fits in free device memory, else re-run the
    forward in the backward; False = always keep it; True = always re-run."""
    if channels is None and sh_dc is None:
        raise ValueError("pass either channels or sh_dc/sh_rest")
    policy = "auto" if recompute is None else ("recompute" if recompute else "store")
    return RayTraceFunction.apply(tracer, camera, policy, mean, rotation, scale, opacity, channels, sh_dc, sh_rest)
