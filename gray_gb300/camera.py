"""CameraInfo with the reference's pose convention (gray/camera.py:9-119).

Only the fields and helpers the ray tracer reads are kept: origin, R (world-from-camera
rotation in COLMAP convention), fov_y, image size.  rotation_c2w_blender_cuda() applies the
reference's conversion (negate R, then flip the x column) that Raytracer.__call__ feeds to
CameraDataHolder.set_pose.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class CameraInfo:
    uid: int = 0
    R: np.ndarray = field(default_factory=lambda: np.eye(3))
    T: np.ndarray = field(default_factory=lambda: np.zeros(3))
    origin: np.ndarray = field(default_factory=lambda: np.zeros(3))
    fov_y: float = 1.0
    fov_x: float = 1.0
    image_path: str = ""
    image_name: str = ""
    image_width: int = 0
    image_height: int = 0
    is_test: bool = False

    def origin_cuda(self):
        import torch

        tensor = getattr(self, "_origin_cuda", None)
        if tensor is None:
            tensor = torch.from_numpy(np.asarray(self.origin, dtype=np.float32)).cuda()
            self._origin_cuda = tensor
        return tensor

    def rotation_c2w_blender_cuda(self):
        import torch

        tensor = getattr(self, "_rotation_c2w_blender_cuda", None)
        if tensor is None:
            tensor = torch.from_numpy(self.rotation_c2w_blender()).cuda()
            self._rotation_c2w_blender_cuda = tensor
        return tensor

    def rotation_c2w_blender(self) -> np.ndarray:
        rotation = -np.asarray(self.R, dtype=np.float32).copy()
        rotation[:, 0] *= -1
        return rotation

    def to_json(self):
        out = {}
        for k in self.__dataclass_fields__:
            v = getattr(self, k)
            out[k] = v.tolist() if isinstance(v, np.ndarray) else v
        return out

    @staticmethod
    def from_json(d: dict) -> "CameraInfo":
        kw = {}
        for k in CameraInfo.__dataclass_fields__:
            v = d.get(k)
            kw[k] = np.array(v) if isinstance(v, list) else v
        return CameraInfo(**kw)


def look_at(origin, target=(0.0, 0.0, 0.0), up=(0.0, 0.0, 1.0), fov_y=0.8, width=64, height=64, uid=0):
    """CameraInfo at `origin` looking at `target` (COLMAP-style R with +z forward, -y up).

    With the reference's conversion the ray for the image centre points from origin to target."""
    o = np.asarray(origin, np.float64)
    f = np.asarray(target, np.float64) - o
    f = f / np.linalg.norm(f)
    u = np.asarray(up, np.float64)
    if abs(float(np.dot(u, f))) > 0.999:
        u = np.array([0.0, 1.0, 0.0]) if abs(f[1]) < 0.9 else np.array([1.0, 0.0, 0.0])
    r = np.cross(f, u)
    r = r / np.linalg.norm(r)
    d = np.cross(f, r)  # camera "down"
    R = np.stack([r, d, f], axis=1)  # columns: x right, y down, z forward (world from camera)
    fov_x = 2.0 * math.atan(math.tan(fov_y / 2.0) * width / height)
    return CameraInfo(uid=uid, R=R, T=-R.T @ o, origin=o, fov_y=fov_y, fov_x=fov_x, image_width=width,
                      image_height=height)


def save_cameras_json(model_path: str, cameras) -> str:
    """Write `cameras` as the scene's cameras.json: a list of CameraInfo.to_json() records (the file
    gray/scene.py:156-170 and render.py read back)."""
    import json
    import os

    path = os.path.join(model_path, "cameras.json")
    with open(path, "w") as f:
        json.dump([c.to_json() for c in cameras], f)
    return path


def load_cameras_json(model_path: str):
    """gray/scene.py:156-170 without the images: cameras.json next to `model_path` (a directory, or
    a file inside it), sorted by image_name and split into (train, test) by is_test."""
    import json
    import os

    model_dir = os.path.dirname(model_path) if os.path.isfile(model_path) else model_path
    path = os.path.join(model_dir, "cameras.json")
    if not os.path.exists(path):
        raise FileNotFoundError(f"No colmap dataset and no cameras.json found at '{path}'")
    with open(path) as f:
        payload = json.load(f)
    cams = sorted((CameraInfo.from_json(e) for e in payload), key=lambda c: c.image_name)
    return [c for c in cams if not c.is_test], [c for c in cams if c.is_test]
