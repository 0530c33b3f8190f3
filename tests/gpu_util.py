"""Helpers shared by the GPU parity tests: load a scene into gray_gb300.classes.Raytracer, trace
given rays through the C ABI, and decode the backward hit lists."""
from __future__ import annotations

import numpy as np
import torch

from gray_gb300 import classes


def make_tracer(width, height, mean, rotation, scale, opacity, channels=None, sh_dc=None, sh_rest=None,
                sh_degree=0, alpha_threshold=0.01, t_threshold=0.03, bg=(0.0, 0.0, 0.0), exp_power=2.0,
                pool_words=4_000_000, render_depth=False, inference_only=False):
    n = mean.shape[0]
    max_deg = 3 if sh_dc is not None else 0
    rt = classes.Raytracer(width, height, n, max_deg, 1, pool_words, inference_only)
    cfg = rt.get_config()
    cfg.alpha_threshold.fill_(alpha_threshold)
    cfg.t_threshold.fill_(t_threshold)
    cfg.exp_power.fill_(exp_power)
    cfg.background_channels.copy_(torch.tensor(bg, dtype=torch.float32))
    cfg.render_depth.fill_(render_depth)
    cfg.enable_sh.fill_(sh_dc is not None)
    cfg.zero_grads.fill_(False)
    rt.get_camera().znear.fill_(0.0)
    rt.get_camera().zfar.fill_(99999.9)
    g = rt.get_gaussians()
    with torch.no_grad():
        g.mean.copy_(torch.from_numpy(np.asarray(mean, np.float32)))
        g.rotation.copy_(torch.from_numpy(np.asarray(rotation, np.float32)))
        g.scale.copy_(torch.from_numpy(np.asarray(scale, np.float32)))
        g.opacity.copy_(torch.from_numpy(np.asarray(opacity, np.float32).reshape(n, 1)))
        if channels is not None:
            g.channels.copy_(torch.from_numpy(np.asarray(channels, np.float32)))
        if sh_dc is not None:
            g.sh_coeffs_dc.copy_(torch.from_numpy(np.asarray(sh_dc, np.float32)).reshape(n, 1, 3))
            g.sh_coeffs_rest.copy_(torch.from_numpy(np.asarray(sh_rest, np.float32)).reshape(n, 15, 3))
            g.current_sh_degree.fill_(sh_degree)
    rt.rebuild_bvh()
    return rt


def trace_rays(rt, ray_o, ray_d, grads=True):
    """Trace the given rays (one per framebuffer pixel, row-major) with rays_from_python."""
    fb = rt.get_framebuffer()
    H, W = fb.ray_origin.shape[:2]
    fb.ray_origin.copy_(torch.from_numpy(np.asarray(ray_o, np.float32)).reshape(H, W, 3))
    fb.ray_direction.copy_(torch.from_numpy(np.asarray(ray_d, np.float32)).reshape(H, W, 3))
    rt.get_config().rays_from_python.fill_(True)
    with torch.set_grad_enabled(grads):
        rt.forward_pass()
    torch.cuda.synchronize()
    rt.check_status()


def hit_lists(rt):
    """Per-pixel composited gaussian ids, front to back."""
    h = rt.get_ppll_backward_data()
    head = h.head_per_pixel.reshape(-1).cpu().numpy().view(np.uint32)
    pool = h.pool.cpu().numpy().view(np.uint32)
    out = []
    for seg in head:
        segs = []
        while seg != 0xFFFFFFFF:
            cnt = int(pool[seg + 1])
            segs.append(pool[seg + 2:seg + 2 + cnt].copy())
            seg = int(pool[seg])
        out.append(np.concatenate(segs[::-1]) if segs else np.zeros(0, np.uint32))
    return out


def oracle_lists(fwd):
    o, ids = fwd["offsets"], fwd["ids"]
    return [ids[o[i]:o[i + 1]] for i in range(len(o) - 1)]


def fb_numpy(rt):
    fb = rt.get_framebuffer()
    return {k: getattr(fb, k).detach().reshape(-1, getattr(fb, k).shape[-1]).cpu().numpy()
            for k in ("output_channels", "output_depth", "transmittance", "full_transmittance",
                      "remaining_channels_estimate", "ray_origin", "ray_direction")}
