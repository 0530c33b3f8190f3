"""Launches the reference's own SH, Adam and Gaussian-response kernels on the GPU.

TEST INFRASTRUCTURE ONLY (tests/ and the fixture generator under tests/golden/): the reference's
cuda/utils/sh.cu, cuda/opt/adam.cu and cuda/utils/kernel.cu, compiled unchanged with the
reference's flags into oracle/_ref/gray_ref.cubin (`make -C oracle ref REF=<checkout>`, see
oracle/ref_kernels.cu), are loaded with the CUDA driver API (libcuda through ctypes) into the
context torch uses and launched on torch's current stream, with the same launch shapes as the
reference's host launchers (cuda/utils/sh.cu:290-304, cuda/opt/adam.cu:70-83).  The package never
imports this module.

The kernels take the reference's parameter structs by value; RefGaussians / RefCamera / RefAdam
mirror them, and tests/test_reference_kernels.py checks the mirrors against oracle/ref_layout.json
(the offsets nvcc gives the reference's own struct definitions).
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(_HERE, "_ref", "gray_ref.cubin")
LAYOUT = os.path.join(_HERE, "ref_layout.json")

P = ctypes.c_void_p

_GAUSSIAN_PTRS = (
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


class RefGaussians(ctypes.Structure):
    """struct Gaussians (cuda/core/gaussians.h:7-65) with CHANNELS=3."""
    _fields_ = ([("count", ctypes.c_int), ("max_sh_degree", ctypes.c_int), ("num_sh_coeffs", ctypes.c_int),
                 ("current_sh_degree", P)] + [(n, P) for n in _GAUSSIAN_PTRS] + [("sh_is_fp16", ctypes.c_bool)])


class RefCamera(ctypes.Structure):
    """struct Camera (cuda/core/camera.h:8-15)."""
    _fields_ = [(n, P) for n in ("origin", "vertical_fov_radians", "rotation_c2w", "rotation_w2c", "znear", "zfar")]


class RefAdam(ctypes.Structure):
    """struct Adam (cuda/opt/adam.cu:5-11)."""
    _fields_ = [("step", ctypes.c_int), ("zero_grads", ctypes.c_bool), ("beta1", ctypes.c_float),
                ("beta2", ctypes.c_float), ("epsilon", ctypes.c_float)]


def available() -> bool:
    return os.path.exists(CUBIN)


# (key, substring of the kernel's symbol): Itanium names of the reference's kernels; the SH kernels
# sit in an anonymous namespace, so their full names carry a per-file prefix and are found by search.
_KERNELS = (
    ("sh_forward_f32", "17sh_forward_kernelI6float3E"),
    ("sh_forward_f16", "17sh_forward_kernelI5half3E"),
    ("sh_backward", "18sh_backward_kernel"),
    ("adam_base", "21adam_step_base_kernel"),
    ("adam_sh", "19adam_step_sh_kernel"),
    ("kernel_functions", "gray_ref_kernel_functions"),
)


def _ptr(t):
    return None if t is None else t.data_ptr()


class RefKernels:
    def __init__(self):
        import torch

        if not available():
            raise FileNotFoundError(f"{CUBIN} is missing: run `make -C oracle ref REF=<reference checkout>`")
        torch.zeros(1, device="cuda")  # the runtime's primary context is current on this thread from here on
        self._torch = torch
        cu = ctypes.CDLL("libcuda.so.1")
        self._cu = cu
        cu.cuCtxGetCurrent.argtypes = [ctypes.POINTER(P)]
        cu.cuModuleLoad.argtypes = [ctypes.POINTER(P), ctypes.c_char_p]
        cu.cuModuleGetFunctionCount.argtypes = [ctypes.POINTER(ctypes.c_uint), P]
        cu.cuModuleEnumerateFunctions.argtypes = [ctypes.POINTER(P), ctypes.c_uint, P]
        cu.cuFuncGetName.argtypes = [ctypes.POINTER(ctypes.c_char_p), P]
        cu.cuLaunchKernel.argtypes = [P, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                      ctypes.c_uint, ctypes.c_uint, P, ctypes.POINTER(P), ctypes.POINTER(P)]
        ctx = P()
        self._check(cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        mod = P()
        self._check(cu.cuModuleLoad(ctypes.byref(mod), CUBIN.encode()), "cuModuleLoad")
        self._mod = mod
        count = ctypes.c_uint()
        self._check(cu.cuModuleGetFunctionCount(ctypes.byref(count), mod), "cuModuleGetFunctionCount")
        funcs = (P * count.value)()
        self._check(cu.cuModuleEnumerateFunctions(funcs, count.value, mod), "cuModuleEnumerateFunctions")
        names = {}
        for f in funcs:
            name = ctypes.c_char_p()
            self._check(cu.cuFuncGetName(ctypes.byref(name), f), "cuFuncGetName")
            names[name.value.decode()] = f
        self.fn = {}
        for key, pattern in _KERNELS:
            hits = [f for n, f in names.items() if pattern in n]
            if len(hits) != 1:
                raise RuntimeError(f"kernel {key!r} ({pattern}) not found once in the cubin: {sorted(names)}")
            self.fn[key] = hits[0]

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def _launch(self, key, blocks, threads, args, smem=0):
        if blocks == 0:
            return
        params = (P * len(args))(*[P(ctypes.addressof(a)) for a in args])
        stream = P(self._torch.cuda.current_stream().cuda_stream)
        self._check(self._cu.cuLaunchKernel(self.fn[key], blocks, 1, 1, threads, 1, 1, smem, stream, params, None),
                    f"cuLaunchKernel({key})")

    # ---- structs ----
    @staticmethod
    def gaussians(count, num_sh_coeffs, tensors: dict, sh_is_fp16=False, max_sh_degree=3):
        g = RefGaussians()
        g.count = int(count)
        g.max_sh_degree = int(max_sh_degree)
        g.num_sh_coeffs = int(num_sh_coeffs)
        g.current_sh_degree = _ptr(tensors.get("current_sh_degree"))
        for n in _GAUSSIAN_PTRS:
            setattr(g, n, _ptr(tensors.get(n)))
        g.sh_is_fp16 = bool(sh_is_fp16)
        return g

    @staticmethod
    def camera(origin):
        c = RefCamera()
        c.origin = _ptr(origin)
        return c

    # ---- kernels ----
    def sh_forward(self, mean, cam_origin, sh_dc, sh_rest, degree):
        """cuda/utils/sh.cu:290-296 sh_forward_pass: channels [N,3] from dc [N,1,3] and rest [N,K,3]
        (float32, or float16 = the reference's inference mode)."""
        torch = self._torch
        n, k = mean.shape[0], sh_rest.shape[1]
        fp16 = sh_dc.dtype == torch.float16
        channels = torch.zeros(n, 3, device=mean.device, dtype=torch.float32)
        deg = torch.tensor([degree], device=mean.device, dtype=torch.int32)
        g = self.gaussians(n, k, {"current_sh_degree": deg, "mean": mean, "channels": channels,
                                  "sh_coeffs_dc": sh_dc, "sh_coeffs_rest": sh_rest}, sh_is_fp16=fp16)
        cam = self.camera(cam_origin)
        self._launch("sh_forward_f16" if fp16 else "sh_forward_f32", (n + 127) // 128, 128, [g, cam])
        return channels

    def sh_backward(self, mean, cam_origin, sh_rest, channels, grad_channels, was_visible, grad_mean, degree):
        """cuda/utils/sh.cu:298-304 sh_backward_pass: (grad_dc, grad_rest, grad_mean); grad_mean is
        updated in place (+=), grad_dc / grad_rest are written for visible Gaussians only (zeros
        elsewhere here)."""
        torch = self._torch
        n, k = mean.shape[0], sh_rest.shape[1]
        grad_dc = torch.zeros(n, 1, 3, device=mean.device, dtype=torch.float32)
        grad_rest = torch.zeros(n, k, 3, device=mean.device, dtype=torch.float32)
        deg = torch.tensor([degree], device=mean.device, dtype=torch.int32)
        g = self.gaussians(n, k, {"current_sh_degree": deg, "mean": mean, "channels": channels,
                                  "sh_coeffs_rest": sh_rest, "grad_channels": grad_channels,
                                  "was_visible": was_visible, "grad_mean": grad_mean,
                                  "grad_sh_coeffs_dc": grad_dc, "grad_sh_coeffs_rest": grad_rest})
        self._launch("sh_backward", (n + 127) // 128, 128, [g, self.camera(cam_origin)])
        return grad_dc, grad_rest, grad_mean

    def adam_step(self, t: dict, n, num_sh_coeffs, step, zero_grads, update_channels, beta_1, beta_2, epsilon,
                  enable_sh, sh_update_laziness):
        """cuda/opt/adam.cu:70-83 adam_step over the tensors in t (reference names: mean, grad_mean,
        first_moment_mean, ..., lr_mean, ...), updated in place."""
        groups = ("channels", "opacity", "mean", "rotation", "scale", "sh_coeffs_dc", "sh_coeffs_rest")
        short = {"sh_coeffs_dc": "sh_dc", "sh_coeffs_rest": "sh_rest"}
        need = [k for grp in groups for k in (grp, "grad_" + grp, "first_moment_" + grp, "second_moment_" + grp,
                                              "lr_" + short.get(grp, grp))]
        missing = [k for k in need if t.get(k) is None]
        if missing:  # the kernels dereference every one of these
            raise ValueError(f"adam_step needs {missing}")
        g = self.gaussians(n, num_sh_coeffs, t)
        adam = RefAdam()
        adam.step, adam.zero_grads = int(step), bool(zero_grads)
        adam.beta1, adam.beta2, adam.epsilon = float(beta_1), float(beta_2), float(epsilon)
        self._launch("adam_base", (n + 255) // 256, 256, [g, adam, ctypes.c_bool(bool(update_channels))])
        if enable_sh and step % sh_update_laziness == 0:
            total = n * (num_sh_coeffs + 1)
            self._launch("adam_sh", (total + 255) // 256, 256, [g, adam], smem=1)

    def kernel_functions(self, opacity, local_hit, alpha_threshold, exp_power):
        """cuda/utils/kernel.cu:3-42 per element: (scaling factor, response, alpha)."""
        torch = self._torch
        n = opacity.shape[0]
        out = [torch.zeros(n, device=opacity.device, dtype=torch.float32) for _ in range(3)]
        args = [ctypes.c_int(n), P(opacity.data_ptr()), P(local_hit.data_ptr()), ctypes.c_float(alpha_threshold),
                ctypes.c_float(exp_power)] + [P(o.data_ptr()) for o in out]
        self._launch("kernel_functions", (n + 255) // 256, 256, args)
        return tuple(out)
