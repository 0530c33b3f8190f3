"""Raytracer: the reference's nn.Module surface (gray/raytracer.py:30-438) on libgray_gb300.

Same constructor, __call__ / backward / step / set_render_resolution / prune /
update_pruning_stats / from_point_cloud / from_safetensors / save_safetensors, and the same
`cuda_module` attribute, which here is gray_gb300.classes.Raytracer instead of
torch.classes.gray.Raytracer.  The post-processing MLP (the consumer of the ray and depth outputs)
is gray_gb300.mlp.PostMLP; the pre-processing MLP and exposure compensation of the reference are
outside the ray tracing path and not provided (their flags must stay False).
"""
from __future__ import annotations

import os
from typing import Optional

import numpy as np
import torch

from . import classes
from .camera import CameraInfo
from .config import RaytracerConfig


class Raytracer(torch.nn.Module):
    def __init__(self, cfg: RaytracerConfig, num_points: int, image_width: int, image_height: int,
                 inference_only: bool = False):
        super().__init__()
        if cfg.pre_mlp or cfg.exposure_comp_enabled:
            raise NotImplementedError("the pre-MLP and exposure compensation are not part of gray_gb300")
        self.cfg = cfg
        self.image_width = image_width
        self.image_height = image_height
        self.render_width = image_width
        self.render_height = image_height
        self.cuda_module = classes.Raytracer(image_width, image_height, num_points, cfg.sh_max_degree,
                                             cfg.ppll_forward_size, cfg.ppll_backward_size, inference_only)
        self.bg_color = torch.tensor(cfg.bg_color)
        config = self.cuda_module.get_config()
        config.alpha_threshold.fill_(cfg.alpha_threshold)
        config.t_threshold.fill_(cfg.t_threshold)
        config.exp_power.fill_(cfg.exp_power)
        config.render_depth.fill_(cfg.render_depth)
        config.background_channels.copy_(self.bg_color)
        config.enable_sh.fill_(cfg.sh)
        config.needs_ray_output.fill_(cfg.post_mlp)
        config.update_channels.fill_(not cfg.pre_mlp and not cfg.sh)
        g = self.cuda_module.get_gaussians()
        g.lr_rotation.fill_(cfg.lr_rotation_init)
        g.lr_scale.fill_(cfg.lr_scale_init)
        g.lr_mean.fill_(cfg.lr_mean_init)
        g.lr_opacity.fill_(cfg.lr_opacity_init)
        g.lr_channels.fill_(cfg.lr_channels)
        g.lr_sh_dc.fill_(cfg.lr_sh_dc_init)
        g.lr_sh_rest.fill_(cfg.lr_sh_rest)
        g.beta_1.fill_(cfg.beta_1)
        g.beta_2.fill_(cfg.beta_2)
        g.epsilon.fill_(cfg.epsilon)
        g.sh_update_laziness.fill_(cfg.sh_update_laziness)
        num_channels = self.cuda_module.get_num_channels()
        if num_channels != 3 and not cfg.post_mlp:
            raise ValueError("the post-processing MLP must be enabled when the tracer has other than 3 channels")
        self.post_mlp = None
        if cfg.post_mlp:
            from .mlp import PostMLP

            self.post_mlp = PostMLP(cfg, num_channels)
        self.output_channels = None

    def __call__(self, cam_info: CameraInfo, znear=0.0, zfar=99999.9, skip_copy=False):
        camera = self.cuda_module.get_camera()
        camera.znear.fill_(znear)
        camera.zfar.fill_(zfar)
        config = self.cuda_module.get_config()
        config.rays_from_python.fill_(False)
        camera.vertical_fov_radians.fill_(cam_info.fov_y)
        camera.set_pose(cam_info.origin_cuda(), cam_info.rotation_c2w_blender_cuda())
        framebuffer = self.cuda_module.get_framebuffer()
        grad_enabled = torch.is_grad_enabled()
        assert not (skip_copy and grad_enabled), "skip_copy=True is not supported with gradients enabled"
        self.cuda_module.forward_pass()
        h, w = self.render_height, self.render_width
        out = framebuffer.output_channels.detach()[:h, :w]
        if not skip_copy or grad_enabled:
            out = out.clone()
        out = out.moveaxis(-1, 0)
        if grad_enabled:
            assert self.output_channels is None, "Called the forward pass multiple times without a backward pass"
            out.requires_grad_()
            self.output_channels = out
        if self.post_mlp is not None:
            # gray/raytracer.py:163-167: hit points from the depth along each ray
            ray_direction = framebuffer.ray_direction.detach()[:h, :w].moveaxis(-1, 0)
            depth = framebuffer.output_depth.detach()[:h, :w].moveaxis(-1, 0)
            hit_point = cam_info.origin_cuda()[:, None, None] + depth * ray_direction
            return self.post_mlp(out, hit_point, ray_direction)
        return out

    def backward(self, loss):
        loss.backward()
        with torch.no_grad():
            fb = self.cuda_module.get_framebuffer()
            h, w = self.render_height, self.render_width
            fb.grad_output_channels[:h, :w].copy_(self.output_channels.grad.moveaxis(0, -1))
            self.output_channels = None
        self.cuda_module.backward_pass()

    def step(self):
        self.update_pruning_stats()
        self.cuda_module.step()
        self.cuda_module.update_bvh()
        if self.post_mlp is not None:
            self.post_mlp.step()

    def set_render_resolution(self, width: int, height: int):
        self.render_width = width
        self.render_height = height
        self.cuda_module.set_render_resolution(width, height)

    @staticmethod
    def from_point_cloud(cfg: RaytracerConfig, points: np.ndarray, colors: np.ndarray, distances_to_cam: np.ndarray,
                         image_width: int, image_height: int, inference_only: bool = False, radius: float = 1.0):
        """gray/raytracer.py:205-294 with the point cloud given as arrays (binning included)."""
        points = np.asarray(points, np.float32)
        colors = np.asarray(colors, np.float32)
        distances_to_cam = np.asarray(distances_to_cam, np.float32)
        if cfg.init_binning:
            pts = torch.from_numpy(points).cuda()
            cols = torch.from_numpy(colors).cuda()
            dist = torch.from_numpy(distances_to_cam).cuda().unsqueeze(1)
            rounded = (pts / (cfg.init_bin_size * radius)).round()
            uniq, inverse, counts = rounded.unique(dim=0, sorted=True, return_counts=True, return_inverse=True)
            m = uniq.shape[0]
            cs = torch.zeros((m, 3), device=pts.device).index_add_(0, inverse, cols)
            ps = torch.zeros((m, 3), device=pts.device).index_add_(0, inverse, pts)
            ds = torch.zeros((m, 1), device=pts.device).index_add_(0, inverse, dist)
            points = (ps / counts.unsqueeze(1)).cpu().numpy()
            colors = (cs / counts.unsqueeze(1)).cpu().numpy()
            distances_to_cam = (ds / counts.unsqueeze(1)).squeeze(1).cpu().numpy()
        n = points.shape[0]
        rt = Raytracer(cfg, n, image_width, image_height, inference_only=inference_only)
        g = rt.cuda_module.get_gaussians()
        with torch.no_grad():
            g.rotation.copy_(torch.tensor([[1.0, 0.0, 0.0, 0.0]]).repeat(n, 1))
            g.scale.copy_(torch.from_numpy(distances_to_cam * cfg.init_scale).cuda().unsqueeze(1).log())
            g.mean.copy_(torch.from_numpy(points).cuda())
            g.opacity.copy_(torch.logit(cfg.init_opacity * torch.ones(n, 1)))
            g.channels.copy_(torch.from_numpy(colors).cuda())
            g.sh_coeffs_dc.copy_(((torch.from_numpy(colors).cuda().unsqueeze(1) - 0.5) / 0.28209479177387814))
        rt.cuda_module.rebuild_bvh()
        return rt

    @torch.no_grad()
    def prune(self, iteration: int, mask: Optional[torch.Tensor] = None):
        """gray/raytracer.py:296-359: keep the Gaussians selected by `mask` (default: average
        pruning weight >= pruning_min_weight), with their Adam moments."""
        g = self.cuda_module.get_gaussians()
        keep = {}
        for name in ("mean", "channels", "opacity", "rotation", "scale", "sh_coeffs_dc", "sh_coeffs_rest"):
            keep[name] = getattr(g, name).clone()
            keep["first_moment_" + name] = getattr(g, "first_moment_" + name).clone()
            keep["second_moment_" + name] = getattr(g, "second_moment_" + name).clone()
        if mask is None:
            denom = g.pruning_counter.squeeze(1).clamp(min=1)
            mask = g.pruning_weight.squeeze(1) / denom >= self.cfg.pruning_min_weight
        self.cuda_module.resize(int(mask.sum().item()))
        for name, t in keep.items():
            getattr(g, name).copy_(t[mask])
        g.pruning_weight.zero_()
        g.pruning_counter.zero_()

    @torch.no_grad()
    def update_pruning_stats(self):
        g = self.cuda_module.get_gaussians()
        g.pruning_counter.add_(g.was_visible)  # one kernel: the bool flags are promoted in place

    @staticmethod
    def from_safetensors(cfg: RaytracerConfig, path: str, image_width: int, image_height: int,
                         inference_only: bool = False):
        """gray/raytracer.py:368-420."""
        from .safetensors_io import load_file

        sd = load_file(path)
        for k in ("bg_color", "image_width", "image_height"):
            sd.pop(k, None)
        n = sd["mean"].shape[0]
        rt = Raytracer(cfg, n, image_width, image_height, inference_only=inference_only)
        g = rt.cuda_module.get_gaussians()
        with torch.no_grad():
            g.mean.copy_(sd.pop("mean"))
            g.rotation.copy_(sd.pop("rotation"))
            g.scale.copy_(sd.pop("scale"))
            g.opacity.copy_(sd.pop("opacity"))
            if cfg.sh:
                g.channels.zero_()
                g.sh_coeffs_dc.copy_(sd.pop("sh_coeffs_dc"))
                g.sh_coeffs_rest.copy_(sd.pop("sh_coeffs_rest"))
                g.current_sh_degree.copy_(sd.pop("current_sh_degree"))
            else:
                g.channels.copy_(sd.pop("channels"))
                g.sh_coeffs_dc.zero_()
                g.sh_coeffs_rest.zero_()
                g.current_sh_degree.zero_()
        rt.cuda_module.rebuild_bvh()
        for k in ("channels", "sh_coeffs_dc", "sh_coeffs_rest", "current_sh_degree"):
            sd.pop(k, None)
        rt.load_state_dict(sd)
        return rt

    def save_safetensors(self, model_path: str, iteration: int):
        """gray/raytracer.py:422-438: gaussians_{iteration:05d}.safetensors."""
        from .safetensors_io import save_file

        g = self.cuda_module.get_gaussians()
        tensors = {"mean": g.mean, "rotation": g.rotation, "scale": g.scale, "opacity": g.opacity}
        if self.cfg.sh:
            tensors["sh_coeffs_dc"] = g.sh_coeffs_dc
            tensors["sh_coeffs_rest"] = g.sh_coeffs_rest
            tensors["current_sh_degree"] = g.current_sh_degree
        else:
            tensors["channels"] = g.channels
        path = os.path.join(model_path, f"gaussians_{iteration:05d}.safetensors")
        save_file({**self.state_dict(), **tensors}, path)
        return path
