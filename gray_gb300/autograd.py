"""torch.autograd.Function around the hand-written backward.

    img = gray_gb300.autograd.render(tracer, camera, mean, rotation, scale, opacity,
                                     channels=None, sh_dc=None, sh_rest=None, recompute=False)

`tracer` is a gray_gb300.classes.Raytracer sized for the Gaussians.  The parameters are copied into
the tracer's holders (a no-op when they already are the holder tensors), the instance snapshot is
refreshed (the reference's update_bvh) and the forward trace runs; the returned [3, h, w] image is
differentiable with respect to every parameter passed in.  The backward of the autograd graph calls
the library's reverse-replay backward (reference: cuda/backward_pass.cu) and the SH backward.

recompute=True does not keep the forward's hit lists alive between forward and backward: the
backward re-runs the forward trace (deterministic, so the lists are identical) right before the
reverse replay.  This lets many renders share one hit-list pool (memory of one view instead of
all views) at the cost of a second forward.
"""
from __future__ import annotations

import torch

from .camera import CameraInfo


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


class RayTraceFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, tracer, camera, recompute, mean, rotation, scale, opacity, channels, sh_dc, sh_rest):
        names = ("mean", "rotation", "scale", "opacity", "channels", "sh_coeffs_dc", "sh_coeffs_rest")
        _load(tracer, names, (mean, rotation, scale, opacity, channels, sh_dc, sh_rest))
        use_sh = sh_dc is not None
        tracer.get_config().enable_sh.fill_(use_sh)
        tracer.update_bvh()
        _set_camera(tracer, camera)
        with torch.enable_grad():
            tracer.forward_pass()
        h, w = tracer.height, tracer.width
        out = tracer.get_framebuffer().output_channels[:h, :w].detach().clone().moveaxis(-1, 0)
        ctx.tracer, ctx.camera, ctx.recompute, ctx.use_sh = tracer, camera, recompute, use_sh
        ctx.shapes = [None if t is None else t.shape for t in (mean, rotation, scale, opacity, channels, sh_dc,
                                                             sh_rest)]
        return out

    @staticmethod
    def backward(ctx, grad_out):
        tracer = ctx.tracer
        if ctx.recompute:
            _set_camera(tracer, ctx.camera)
            with torch.enable_grad():
                tracer.forward_pass()
        g = tracer.get_gaussians()
        with torch.no_grad():
            for name in ("grad_mean", "grad_rotation", "grad_scale", "grad_opacity", "grad_channels",
                         "grad_sh_coeffs_dc", "grad_sh_coeffs_rest"):
                getattr(g, name).zero_()
            h, w = tracer.height, tracer.width
            tracer.get_framebuffer().grad_output_channels[:h, :w].copy_(grad_out.moveaxis(0, -1))
        tracer.backward_pass()
        grads = [g.grad_mean, g.grad_rotation, g.grad_scale, g.grad_opacity, g.grad_channels, g.grad_sh_coeffs_dc,
                 g.grad_sh_coeffs_rest]
        out = []
        for gr, shape in zip(grads, ctx.shapes):
            out.append(None if shape is None else gr.clone().reshape(shape))
        return (None, None, None, *out)


def render(tracer, camera: CameraInfo, mean, rotation, scale, opacity, channels=None, sh_dc=None, sh_rest=None,
           recompute: bool = False):
    """Differentiable render of `camera` ([3, h, w]) through the hand-written backward."""
    if channels is None and sh_dc is None:
        raise ValueError("pass either channels or sh_dc/sh_rest")
    return RayTraceFunction.apply(tracer, camera, recompute, mean, rotation, scale, opacity, channels, sh_dc,
                                  sh_rest)
