"""gray_gb300 -- GB300-native (sm_103a) differentiable Gaussian ray tracer.

Drop-in for the ray tracing path of graphdeco-inria/gray: `gray_gb300.classes.Raytracer` mirrors
torch.classes.gray.Raytracer and `gray_gb300.Raytracer` mirrors gray.raytracer.Raytracer; both
run hand-written CUDA kernels from libgray_gb300.so (built by `python -m gray_gb300.build`).
"""
from . import classes
from .cadence import TrainCadence
from .camera import CameraInfo, load_cameras_json, look_at, save_cameras_json
from .config import RaytracerConfig
from .raytracer import Raytracer

__all__ = ["CameraInfo", "RaytracerConfig", "Raytracer", "TrainCadence", "classes", "load_cameras_json", "look_at",
           "save_cameras_json"]
