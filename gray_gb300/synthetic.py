"""Seeded synthetic scenes and cameras for the benchmark workloads (no datasets are needed).

Workloads (Gaussian parameters follow the reference's storage: log-scales, logit opacities,
unnormalised quaternions, SH degree 3):
  small     64 Gaussians, means U[-1,1]^3, log-scales N(-3, 0.3), quaternions N(0,1)^4,
            opacity logits N(0,1), SH DC N(0.5, 0.2), rest N(0, 0.05); one 256x256 camera
            (fx = fy = 256) at distance 4 looking at the origin.
  clustered N Gaussians with means from 200 anisotropic Gaussian clusters (sigma 0.05-0.5 per
            axis, random orientation) inside a radius-10 sphere, log-scales N(-4.5, 0.5), other
            parameters as `small`.  Cameras on a radius-8 orbit looking at the origin, fx = fy =
            0.75 * width, optional +-15 degree pose jitter.
  gradcheck 1000 Gaussians as `small` but means U[-2,2]^3; one 128x128 camera.
Random numbers come from numpy's PCG64 generator, so scenes are identical on every machine.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .camera import CameraInfo, look_at


@dataclass
class Scene:
    mean: np.ndarray       # [N,3] float32
    rotation: np.ndarray   # [N,4]
    scale: np.ndarray      # [N,3] log
    opacity: np.ndarray    # [N,1] logit
    sh_dc: np.ndarray      # [N,1,3]
    sh_rest: np.ndarray    # [N,15,3]

    @property
    def n(self) -> int:
        return self.mean.shape[0]


def _params(rng, mean, log_scale_mu, log_scale_sigma):
    n = mean.shape[0]
    rot = rng.standard_normal((n, 4))
    rot /= np.linalg.norm(rot, axis=1, keepdims=True)
    return Scene(
        mean=mean.astype(np.float32),
        rotation=rot.astype(np.float32),
        scale=rng.normal(log_scale_mu, log_scale_sigma, (n, 3)).astype(np.float32),
        opacity=rng.standard_normal((n, 1)).astype(np.float32),
        sh_dc=rng.normal(0.5, 0.2, (n, 1, 3)).astype(np.float32),
        sh_rest=rng.normal(0.0, 0.05, (n, 15, 3)).astype(np.float32),
    )


def small_scene(seed: int = 0, n: int = 64) -> Scene:
    rng = np.random.default_rng(seed)
    return _params(rng, rng.uniform(-1.0, 1.0, (n, 3)), -3.0, 0.3)


def gradcheck_scene(seed: int = 0, n: int = 1000) -> Scene:
    rng = np.random.default_rng(seed)
    return _params(rng, rng.uniform(-2.0, 2.0, (n, 3)), -3.0, 0.3)


def clustered_scene(n: int, seed: int = 0, clusters: int = 200, radius: float = 10.0) -> Scene:
    rng = np.random.default_rng(seed)
    sig = rng.uniform(0.05, 0.5, (clusters, 3))
    # cluster centres uniform in the ball, pulled in so each cluster stays inside it
    dirs = rng.standard_normal((clusters, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    r = (radius - 2.0 * sig.max(axis=1)) * rng.uniform(0.0, 1.0, clusters) ** (1.0 / 3.0)
    centres = dirs * r[:, None]
    q = rng.standard_normal((clusters, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)
    member = rng.integers(0, clusters, n)
    local = rng.standard_normal((n, 3)) * sig[member]
    mean = centres[member] + np.einsum("nij,nj->ni", R[member], local)
    return _params(rng, mean, -4.5, 0.5)


def camera_small(width: int = 256, height: int = 256, focal: float = 256.0) -> CameraInfo:
    fov_y = 2.0 * math.atan(0.5 * height / focal)
    return look_at((0.0, -4.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), fov_y, width, height)


def orbit_camera(angle: float, width: int, height: int, radius: float = 8.0, elevation: float = 0.3,
                 jitter_rad: tuple[float, float] = (0.0, 0.0), uid: int = 0) -> CameraInfo:
    focal = 0.75 * width
    fov_y = 2.0 * math.atan(0.5 * height / focal)
    el = elevation + jitter_rad[1]
    az = angle + jitter_rad[0]
    o = radius * np.array([math.cos(el) * math.cos(az), math.cos(el) * math.sin(az), math.sin(el)])
    # +-15 degree jitter of the viewing direction: look slightly off the origin
    target = np.array([0.0, 0.0, 0.0]) + radius * np.array([math.sin(jitter_rad[0]), math.sin(jitter_rad[1]), 0.0])
    return look_at(o, target, (0.0, 0.0, 1.0), fov_y, width, height, uid=uid)


RESOLUTIONS = [(640, 480), (1280, 720), (1600, 1040), (1920, 1080)]


def uneven_cameras(count: int = 16, seed: int = 0, resolutions=None) -> list[CameraInfo]:
    rng = np.random.default_rng(seed + 7919)
    resolutions = resolutions or RESOLUTIONS
    cams = []
    for i in range(count):
        w, h = resolutions[int(rng.integers(0, len(resolutions)))]
        jit = tuple(rng.uniform(-math.radians(15), math.radians(15), 2))
        cams.append(orbit_camera(2 * math.pi * i / count, w, h, jitter_rad=jit, uid=i))
    return cams


def uneven_view(k: int, width: int, height: int, count: int = 16, seed: int = 0) -> CameraInfo:
    """The pose of uneven_cameras(count, seed)[k] at width x height."""
    c = uneven_cameras(count, seed)[k % count]
    fov_y = 2.0 * math.atan(0.5 * height / (0.75 * width))
    return CameraInfo(uid=c.uid, R=c.R, T=c.T, origin=c.origin, fov_y=fov_y,
                      fov_x=2.0 * math.atan(math.tan(fov_y / 2.0) * width / height), image_width=width,
                      image_height=height)
