"""ctypes view of libgray_gb300.so (include/gray_gb300.h).

The structures below mirror the C structs field for field; every pointer is carried as a
c_void_p holding a device address taken from a torch tensor's data_ptr().
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libgray_gb300.so")

P = ctypes.c_void_p


def _ptrs(*names):
    return [(n, P) for n in names]


class GaussiansC(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int32), ("max_sh_degree", ctypes.c_int32), ("num_sh_coeffs", ctypes.c_int32),
                ("sh_is_fp16", ctypes.c_int32), ("current_sh_degree", P)] + _ptrs(
        "mean", "rotation", "scale", "opacity", "channels", "sh_coeffs_dc", "sh_coeffs_rest",
        "lr_mean", "lr_rotation", "lr_scale", "lr_opacity", "lr_channels", "lr_sh_dc", "lr_sh_rest",
        "beta_1", "beta_2", "epsilon", "sh_update_laziness",
        "grad_mean", "grad_rotation", "grad_scale", "grad_opacity", "grad_channels", "grad_sh_coeffs_dc",
        "grad_sh_coeffs_rest",
        "first_moment_mean", "first_moment_rotation", "first_moment_scale", "first_moment_opacity",
        "first_moment_channels", "first_moment_sh_coeffs_dc", "first_moment_sh_coeffs_rest",
        "second_moment_mean", "second_moment_rotation", "second_moment_scale", "second_moment_opacity",
        "second_moment_channels", "second_moment_sh_coeffs_dc", "second_moment_sh_coeffs_rest",
        "pruning_weight", "pruning_counter", "was_visible", "marked")


class CameraC(ctypes.Structure):
    _fields_ = _ptrs("origin", "vertical_fov_radians", "rotation_c2w", "rotation_w2c", "znear", "zfar")


class ConfigC(ctypes.Structure):
    _fields_ = _ptrs("exp_power", "alpha_threshold", "t_threshold", "jitter_primary_rays", "global_scale_factor",
                     "eps_forward_normalization", "eps_scale_grad", "background_channels", "render_depth",
                     "render_ellipsoids", "ellipsoid_min_opacity", "rays_from_python", "zero_grads", "enable_sh",
                     "needs_ray_output", "update_channels")


class FramebufferC(ctypes.Structure):
    _fields_ = _ptrs("output_channels", "output_depth", "transmittance", "full_transmittance",
                     "remaining_channels_estimate", "ray_origin", "ray_direction", "grad_output_channels")


class MetadataC(ctypes.Structure):
    _fields_ = _ptrs("run_forward_pass", "run_backward_pass", "grads_enabled", "total_num_calls", "total_num_steps")


class StatsC(ctypes.Structure):
    _fields_ = _ptrs("num_gaussians_hit", "num_gaussians_accumulated")


class HitlistC(ctypes.Structure):
    _fields_ = _ptrs("head_per_pixel", "total_words", "pool") + [("size", ctypes.c_uint32)] + _ptrs("schedule")


class SceneC(ctypes.Structure):
    _fields_ = _ptrs("geom", "l2w", "aabb", "visible", "live", "grad_acc", "nodes", "int_parent", "leaf_parent",
                     "order", "codes", "refit_flags", "sort_tmp", "root_box", "bounds", "bwd_rec") + [
        ("bvh_valid", ctypes.c_int32)]


class ParamsC(ctypes.Structure):
    _fields_ = [("image_width", ctypes.c_uint32), ("image_height", ctypes.c_uint32),
                ("render_width", ctypes.c_uint32), ("render_height", ctypes.c_uint32),
                ("camera", CameraC), ("config", ConfigC), ("framebuffer", FramebufferC), ("gaussians", GaussiansC),
                ("metadata", MetadataC), ("stats", StatsC), ("hitlist", HitlistC), ("scene", SceneC),
                ("status", P), ("trace_variant", ctypes.c_int32)]


ENTRY_POINTS = ("gray_forward_pass", "gray_forward_pass_display", "gray_backward_pass", "gray_step",
                "gray_update_bvh", "gray_rebuild_bvh", "gray_sort_tmp_words", "gray_profiler_enable",
                "gray_profiler_collect", "gray_last_error", "gray_version")

_lib = None


class GrayError(RuntimeError):
    pass


def load(path: str | None = None):
    """Load the CUDA library; raises if it has not been built (there is no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise GrayError(f"libgray_gb300.so not found at {path}; run `python -m gray_gb300.build`")
    L = ctypes.CDLL(path)
    for name in ("gray_forward_pass", "gray_forward_pass_display", "gray_backward_pass", "gray_step",
                 "gray_update_bvh", "gray_rebuild_bvh"):
        f = getattr(L, name)
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.POINTER(ParamsC), ctypes.c_void_p]
    L.gray_sort_tmp_words.restype = ctypes.c_size_t
    L.gray_sort_tmp_words.argtypes = [ctypes.c_int32]
    L.gray_schedule_words.restype = ctypes.c_size_t
    L.gray_schedule_words.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    L.gray_profiler_enable.restype = ctypes.c_int
    L.gray_profiler_enable.argtypes = [ctypes.c_int, ctypes.c_int]
    L.gray_profiler_collect.restype = ctypes.c_int
    L.gray_profiler_collect.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.gray_last_error.restype = ctypes.c_char_p
    L.gray_version.restype = ctypes.c_char_p
    _lib = L
    return L


def call(name: str, params: ParamsC, stream: int):
    L = load()
    rc = getattr(L, name)(ctypes.byref(params), ctypes.c_void_p(stream))
    if rc != 0:
        raise GrayError(f"{name}: {L.gray_last_error().decode()} (code {rc})")


class Profiler:
    """Per-launch CUDA-event timing of the library's kernel groups (gray_profiler_* in the C ABI).

        with Profiler() as prof:
            ...                      # calls into the library
        prof.results                 # {name: (total_ms, launches)}
    """

    def __init__(self, capacity: int = 8192):
        self.capacity = capacity
        self.results = {}

    def __enter__(self):
        L = load()
        if L.gray_profiler_enable(1, self.capacity) != 0:
            raise GrayError(L.gray_last_error().decode())
        return self

    def __exit__(self, *exc):
        L = load()
        L.gray_profiler_enable(0, 0)
        buf = ctypes.create_string_buffer(1 << 16)
        n = L.gray_profiler_collect(buf, len(buf))
        if n < 0:
            raise GrayError(L.gray_last_error().decode())
        self.results = {}
        for line in buf.value.decode().strip().splitlines():
            name, ms, cnt = line.split()
            self.results[name] = (float(ms), int(cnt))
        return False
