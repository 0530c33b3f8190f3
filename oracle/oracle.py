"""ctypes front end of the CPU oracle (oracle/gray_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / reference arm as the checker.  The product (gray_gb300) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libgray_oracle.so")
_lib = None

F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
U8P = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
I64P = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
U32P = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


def build() -> str:
    """Compile the oracle with make (gcc, no cmake)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class _TraceCfg(ctypes.Structure):
    _fields_ = [
        ("exp_power", ctypes.c_float),
        ("alpha_threshold", ctypes.c_float),
        ("t_threshold", ctypes.c_float),
        ("znear", ctypes.c_float),
        ("zfar", ctypes.c_float),
        ("eps_forward_normalization", ctypes.c_float),
        ("bg", ctypes.c_float * 3),
        ("render_depth", ctypes.c_int),
        ("pass_slots", ctypes.c_int),
        ("max_passes", ctypes.c_int),
    ]


class _Bvh(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int),
        ("nodes", ctypes.POINTER(ctypes.c_float)),
        ("codes", ctypes.POINTER(ctypes.c_uint32)),
        ("order", ctypes.POINTER(ctypes.c_uint32)),
        ("int_parent", ctypes.POINTER(ctypes.c_int32)),
        ("leaf_parent", ctypes.POINTER(ctypes.c_int32)),
        ("root_box", ctypes.c_float * 8),
    ]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_expf.restype = ctypes.c_float
        L.orc_expf.argtypes = [ctypes.c_float]
        L.orc_logf.restype = ctypes.c_float
        L.orc_logf.argtypes = [ctypes.c_float]
        L.orc_f2h.restype = ctypes.c_uint16
        L.orc_f2h.argtypes = [ctypes.c_float]
        L.orc_h2f.restype = ctypes.c_float
        L.orc_h2f.argtypes = [ctypes.c_uint16]
        L.orc_maxalpha_mul.restype = ctypes.c_float
        L.orc_eval_gaussian.restype = ctypes.c_float
        L.orc_eval_gaussian.argtypes = [ctypes.c_float, ctypes.c_float]
        L.orc_maxalpha_mul.argtypes = [ctypes.c_float, ctypes.c_float]
        L.orc_adam_pow.restype = ctypes.c_float
        L.orc_adam_pow.argtypes = [ctypes.c_float, ctypes.c_int]
        L.orc_scaling_factor.restype = ctypes.c_float
        L.orc_scaling_factor.argtypes = [ctypes.c_float] * 3
        L.orc_snapshot.argtypes = [ctypes.c_int, F32P, F32P, F32P, F32P, ctypes.c_float, ctypes.c_float,
                                   ctypes.c_float, F32P, F32P, F32P, U8P]
        L.orc_forward_prep.argtypes = [ctypes.c_int, F32P, ctypes.c_float, ctypes.c_float, F32P]
        L.orc_camera_rays.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, F32P, F32P, F32P, F32P]
        L.orc_sh_forward.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, F32P, F32P, F32P, F32P, F32P]
        L.orc_sh_backward.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, F32P, F32P, F32P, F32P, F32P,
                                      U8P, F32P, F32P, F32P]
        L.orc_lbvh_build.argtypes = [ctypes.c_int, F32P, U8P, ctypes.POINTER(_Bvh)]
        L.orc_lbvh_refit.argtypes = [ctypes.POINTER(_Bvh), F32P]
        L.orc_lbvh_refit_climb.argtypes = [ctypes.POINTER(_Bvh), F32P]
        L.orc_lbvh_refit_climb.restype = ctypes.c_int
        L.orc_lbvh_free.argtypes = [ctypes.POINTER(_Bvh)]
        L.orc_trace_forward.argtypes = [
            ctypes.c_int, F32P, F32P, ctypes.c_int, F32P, F32P, F32P, U8P, ctypes.c_void_p,
            ctypes.POINTER(_TraceCfg), F32P, F32P, F32P, F32P, F32P, I32P, I32P, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_int]
        L.orc_trace_backward.argtypes = [
            ctypes.c_int, ctypes.c_int, ctypes.c_int, F32P, F32P, F32P, F32P, F32P, F32P, I64P, U32P,
            ctypes.c_int, F32P, F32P, F32P, F32P, F32P, F32P, ctypes.POINTER(_TraceCfg), ctypes.c_float, F64P,
            ctypes.c_int]
        L.orc_ellipsoids.argtypes = [ctypes.c_int, F32P, F32P, ctypes.c_int, F32P, F32P, F32P, ctypes.c_float,
                                     ctypes.c_float, ctypes.c_float, F32P, F32P, F32P, I32P, ctypes.c_int]
        L.orc_hardware_threads.restype = ctypes.c_int
        L.orc_pretest_check.argtypes = [ctypes.c_int, F32P, F32P, I64P]
        L.orc_cull_check.argtypes = [ctypes.c_int, F32P, F32P, F32P, F64P, I64P]
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def pretest_check(lo, ld):
    """(accepted, kept, dropped) pair counts of the exact hit decision and of the CUDA path's
    division-free pretest on object-space rays lo, ld (n x 3)."""
    lo, ld = _f32(lo).reshape(-1, 3), _f32(ld).reshape(-1, 3)
    counts = np.zeros(3, dtype=np.int64)
    lib().orc_pretest_check(len(lo), lo, ld, counts)
    return tuple(int(c) for c in counts)


def cull_check(normals, l2w, thresholds, planes):
    """(culled, wrong) counts of the CUDA path's ellipsoid-plane cull against FP64 on n planes
    (normals n x 3, the cull's thresholds n, the planes' exact offsets n) and ellipsoids (l2w rows
    n x 12)."""
    normals, l2w, thresholds = _f32(normals).reshape(-1, 3), _f32(l2w).reshape(-1, 12), _f32(thresholds).reshape(-1)
    planes = np.ascontiguousarray(planes, dtype=np.float64).reshape(-1)
    counts = np.zeros(2, dtype=np.int64)
    lib().orc_cull_check(len(normals), normals, l2w, thresholds, planes, counts)
    return tuple(int(c) for c in counts)


@dataclass
class TraceConfig:
    exp_power: float = 2.0
    alpha_threshold: float = 0.01
    t_threshold: float = 0.03
    znear: float = 0.0
    zfar: float = 99999.9
    eps_forward_normalization: float = 1e-12
    bg: tuple = (0.0, 0.0, 0.0)
    render_depth: bool = False
    pass_slots: int = 32
    max_passes: int = 99

    def c(self) -> _TraceCfg:
        c = _TraceCfg()
        c.exp_power = self.exp_power
        c.alpha_threshold = self.alpha_threshold
        c.t_threshold = self.t_threshold
        c.znear = self.znear
        c.zfar = self.zfar
        c.eps_forward_normalization = self.eps_forward_normalization
        for i in range(3):
            c.bg[i] = float(self.bg[i])
        c.render_depth = int(bool(self.render_depth))
        c.pass_slots = int(self.pass_slots)
        c.max_passes = int(self.max_passes)
        return c


def expf(x: float) -> float:
    return lib().orc_expf(x)


def logf(x: float) -> float:
    return lib().orc_logf(x)


def eval_gaussian(d: float, exp_power=2.0) -> float:
    """Response at squared local radius d, as the GPU evaluates it."""
    return float(lib().orc_eval_gaussian(d, exp_power))


def maxalpha_mul(a: float, b: float) -> float:
    return float(lib().orc_maxalpha_mul(a, b))


def scaling_factor(opacity: float, alpha_threshold=0.01, exp_power=2.0) -> float:
    return float(lib().orc_scaling_factor(opacity, alpha_threshold, exp_power))


def snapshot(mean, rotation, scale, opacity, alpha_threshold=0.01, exp_power=2.0, global_scale_factor=1.0):
    mean, rotation, scale, opacity = map(_f32, (mean, rotation, scale, opacity))
    n = mean.shape[0]
    geom = np.zeros((n, 12), np.float32)
    l2w = np.zeros((n, 12), np.float32)
    aabb = np.zeros((n, 8), np.float32)
    vis = np.zeros(n, np.uint8)
    lib().orc_snapshot(n, mean, rotation, scale, opacity, alpha_threshold, exp_power, global_scale_factor, geom,
                       l2w, aabb, vis)
    return geom, l2w, aabb, vis


def forward_prep(opacity, alpha_threshold=0.01, exp_power=2.0):
    opacity = _f32(opacity)
    live = np.zeros((opacity.shape[0], 2), np.float32)
    lib().orc_forward_prep(opacity.shape[0], opacity, alpha_threshold, exp_power, live)
    return live


def camera_rays(width, height, fov_y, origin, c2w):
    ro = np.zeros((height * width, 3), np.float32)
    rd = np.zeros((height * width, 3), np.float32)
    lib().orc_camera_rays(width, height, fov_y, _f32(origin), _f32(c2w), ro, rd)
    return ro, rd


def sh_forward(degree, mean, cam_origin, sh_dc, sh_rest):
    mean = _f32(mean)
    n = mean.shape[0]
    sh_rest = _f32(sh_rest).reshape(n, -1, 3)
    out = np.zeros((n, 3), np.float32)
    lib().orc_sh_forward(n, degree, sh_rest.shape[1], mean, _f32(cam_origin), _f32(sh_dc), sh_rest, out)
    return out


def sh_backward(degree, mean, cam_origin, sh_rest, channels, grad_channels, was_visible, grad_mean):
    mean = _f32(mean)
    n = mean.shape[0]
    sh_rest = _f32(sh_rest).reshape(n, -1, 3)
    gdc = np.zeros((n, 3), np.float32)
    grest = np.zeros_like(sh_rest)
    gm = _f32(grad_mean).copy()
    lib().orc_sh_backward(n, degree, sh_rest.shape[1], mean, _f32(cam_origin), sh_rest, _f32(channels),
                          _f32(grad_channels), np.ascontiguousarray(was_visible, dtype=np.uint8), gdc, grest, gm)
    return gdc, grest, gm


class Bvh:
    def __init__(self, aabb, visible):
        self._c = _Bvh()
        aabb = _f32(aabb)
        lib().orc_lbvh_build(aabb.shape[0], aabb, np.ascontiguousarray(visible, dtype=np.uint8),
                             ctypes.byref(self._c))
        self.n = aabb.shape[0]

    def refit(self, aabb):
        lib().orc_lbvh_refit(ctypes.byref(self._c), _f32(aabb))

    def refit_climb(self, aabb) -> int:
        """Bottom-up refit by the GPU's climbing protocol; returns its status bits."""
        return int(lib().orc_lbvh_refit_climb(ctypes.byref(self._c), _f32(aabb)))

    @property
    def int_parent(self):
        m = max(self.n - 1, 0)
        return np.ctypeslib.as_array(self._c.int_parent, shape=(max(m, 1),))[:m]

    @property
    def leaf_parent(self):
        return np.ctypeslib.as_array(self._c.leaf_parent, shape=(self.n,))

    @property
    def nodes(self):
        m = max(self.n - 1, 0)
        return np.ctypeslib.as_array(self._c.nodes, shape=(max(m, 1), 16))[:m].copy()

    @property
    def order(self):
        return np.ctypeslib.as_array(self._c.order, shape=(self.n,)).copy()

    @property
    def codes(self):
        return np.ctypeslib.as_array(self._c.codes, shape=(self.n,)).copy()

    @property
    def root_box(self):
        return np.array(self._c.root_box[:], np.float32)

    def ptr(self):
        return ctypes.cast(ctypes.byref(self._c), ctypes.c_void_p)

    def __del__(self):
        try:
            lib().orc_lbvh_free(ctypes.byref(self._c))
        except Exception:
            pass


def trace_forward(ray_o, ray_d, geom, live, channels, visible, cfg: TraceConfig, bvh: Bvh | None = None,
                  want_lists=True, nthreads=0):
    """Returns a dict with rgb, depth, T, fullT, rem, nhit, nacc and (optionally) the composited
    gaussian id lists as CSR (offsets, ids)."""
    ray_o, ray_d, geom, live, channels = map(_f32, (ray_o, ray_d, geom, live, channels))
    visible = np.ascontiguousarray(visible, dtype=np.uint8)
    R = ray_o.shape[0]
    n = geom.shape[0]
    out = dict(rgb=np.zeros((R, 3), np.float32), depth=np.zeros(R, np.float32), T=np.zeros(R, np.float32),
               fullT=np.zeros(R, np.float32), rem=np.zeros((R, 3), np.float32), nhit=np.zeros(R, np.int32),
               nacc=np.zeros(R, np.int32))
    c = cfg.c()
    bptr = bvh.ptr() if bvh is not None else None

    def run(offsets, ids):
        lib().orc_trace_forward(R, ray_o, ray_d, n, geom, live, channels, visible, bptr, ctypes.byref(c),
                                out["rgb"], out["depth"], out["T"], out["fullT"], out["rem"], out["nhit"],
                                out["nacc"], offsets, ids, nthreads)

    run(None, None)
    if want_lists:
        offsets = np.zeros(R + 1, np.int64)
        offsets[1:] = np.cumsum(out["nacc"])
        ids = np.zeros(max(int(offsets[-1]), 1), np.uint32)
        run(offsets.ctypes.data_as(ctypes.c_void_p), ids.ctypes.data_as(ctypes.c_void_p))
        out["offsets"] = offsets
        out["ids"] = ids[: offsets[-1]]
    return out


def trace_backward(launch_w, launch_h, ray_o, ray_d, fwd, grad_out, geom, l2w, opacity, scale, rotation, channels,
                   cfg: TraceConfig, eps_scale_grad=1e-12, nthreads=1):
    """Per-Gaussian gradient accumulators (double) laid out as
    (rot4 | mean3, opacity | scale3, pruning | channels3, count)."""
    n = geom.shape[0]
    grad = np.zeros((n, 16), np.float64)
    ids = np.ascontiguousarray(fwd["ids"], dtype=np.uint32)
    if ids.size == 0:
        ids = np.zeros(1, np.uint32)
    lib().orc_trace_backward(
        ray_o.shape[0], launch_w, launch_h, _f32(ray_o), _f32(ray_d), _f32(fwd["T"]), _f32(fwd["fullT"]),
        _f32(fwd["rem"]), _f32(grad_out), np.ascontiguousarray(fwd["offsets"], dtype=np.int64), ids, n, _f32(geom),
        _f32(l2w), _f32(opacity).reshape(-1), _f32(scale), _f32(rotation), _f32(channels), ctypes.byref(cfg.c()),
        eps_scale_grad, grad, nthreads)
    return grad


def ellipsoids(ray_o, ray_d, geom, live, channels, znear=0.0, zfar=99999.9, min_opacity=0.0, bg=(0.0, 0.0, 0.0),
               nthreads=0):
    """Ellipsoid view (cuda/ellipsoid_viewer.cu:1-94), brute force.  Returns rgb [R,3], depth [R]
    and the winning gaussian per ray (-1 miss, -2 inactive ray whose outputs stay as given: zeros)."""
    ray_o, ray_d, geom, live, channels = map(_f32, (ray_o, ray_d, geom, live, channels))
    R = ray_o.shape[0]
    rgb = np.zeros((R, 3), np.float32)
    depth = np.zeros(R, np.float32)
    ids = np.zeros(R, np.int32)
    lib().orc_ellipsoids(R, ray_o, ray_d, geom.shape[0], geom, live, channels, znear, zfar, min_opacity,
                         _f32(np.asarray(bg, np.float32)), rgb, depth, ids, nthreads)
    return rgb, depth, ids


def hardware_threads() -> int:
    return lib().orc_hardware_threads()


class _AdamState(ctypes.Structure):
    _fields_ = ([("n", ctypes.c_int), ("num_rest", ctypes.c_int)]
                + [(k, ctypes.POINTER(ctypes.c_float)) for k in (
                    "channels", "opacity", "mean", "rotation", "scale", "sh_dc", "sh_rest",
                    "g_channels", "g_opacity", "g_mean", "g_rotation", "g_scale", "g_sh_dc", "g_sh_rest",
                    "m_channels", "m_opacity", "m_mean", "m_rotation", "m_scale", "m_sh_dc", "m_sh_rest",
                    "v_channels", "v_opacity", "v_mean", "v_rotation", "v_scale", "v_sh_dc", "v_sh_rest")]
                + [(k, ctypes.c_float) for k in ("lr_channels", "lr_opacity", "lr_mean", "lr_rotation", "lr_scale",
                                                 "lr_sh_dc", "lr_sh_rest")])


ADAM_GROUPS = ("channels", "opacity", "mean", "rotation", "scale", "sh_dc", "sh_rest")


def adam_step(state: dict, lrs: dict, n: int, num_rest: int, step: int, zero_grads=True, update_channels=True,
              beta1=0.9, beta2=0.999, eps=1e-15, enable_sh=True, laziness=1):
    """In-place fused Adam on float32 numpy arrays: state[name], state['g_'+name], state['m_'+name],
    state['v_'+name] for name in ADAM_GROUPS (flat or shaped, contiguous)."""
    s = _AdamState()
    s.n = n
    s.num_rest = num_rest
    keep = []
    for name in ADAM_GROUPS:
        for pre in ("", "g_", "m_", "v_"):
            a = state[pre + name]
            assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
            keep.append(a)
            setattr(s, pre + name, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        setattr(s, "lr_" + name, float(lrs.get(name, 0.0)))
    L = lib()
    L.orc_adam_step.argtypes = [ctypes.POINTER(_AdamState), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int]
    L.orc_adam_step(ctypes.byref(s), step, int(zero_grads), int(update_channels), beta1, beta2, eps, int(enable_sh),
                    laziness)
    return state
