"""Generate tests/golden/reference_kernels.npz: inputs and outputs of the reference's own SH, Adam
and Gaussian-response kernels, run on a GPU.

    make -C oracle ref REF=<graphdeco-inria/gray checkout>     # once, where the checkout is
    python tests/golden/make_reference_kernels.py <out.npz>     # on a machine with the GPU

The kernels are graphdeco-inria/gray's cuda/utils/sh.cu (sh_forward_kernel for float3 and half3
coefficients, sh_backward_kernel), cuda/opt/adam.cu (adam_step_base_kernel, adam_step_sh_kernel) and
cuda/utils/kernel.cu (compute_scaling_factor, eval_gaussian, compute_alpha), compiled unchanged with
the reference's fast-math flags (oracle/ref_kernels.cu) and launched by oracle/ref_kernels.py.
Every input is seeded and stored beside the outputs, so the tests that read the file (the oracle on
the CPU, gray_gb300's kernels on the GPU) need neither the reference nor its cubin.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import ref_kernels as R  # noqa: E402

N_SH = 256
N_ADAM = 64
N_KERNEL = 4096
NUM_REST = 15
EXP_POWERS = (1.0, 2.0, 3.0, 2.5)
# (step, zero_grads, update_channels, sh_update_laziness): the SH groups are updated when
# step % laziness == 0 (cuda/opt/adam.cu:79)
ADAM_CASES = ((1, True, True, 1), (7, False, False, 2), (8, True, False, 2))
ADAM_LR = {"mean": 1.6e-4, "scale": 5e-3, "rotation": 1e-3, "opacity": 2.5e-2, "channels": 2.5e-3, "sh_dc": 2.5e-3,
           "sh_rest": 2.5e-3}
ADAM_SHAPES = {"mean": (3,), "rotation": (4,), "scale": (3,), "opacity": (1,), "channels": (3,),
               "sh_coeffs_dc": (1, 3), "sh_coeffs_rest": (NUM_REST, 3)}


def sh_inputs(rng):
    mean = rng.uniform(-2, 2, (N_SH, 3)).astype(np.float32)
    origin = np.array([0.3, -4.0, 1.0], np.float32)
    dc = rng.normal(0.5, 0.2, (N_SH, 1, 3)).astype(np.float32)
    dc[:16, 0, np.arange(16) % 3] = -3.0  # colours clamped at zero on one channel (the backward masks them)
    rest = rng.normal(0.0, 0.05, (N_SH, NUM_REST, 3)).astype(np.float32)
    return mean, origin, dc, rest


def main(out_path: str) -> None:
    dev = torch.device("cuda")
    K = R.RefKernels()
    rng = np.random.default_rng(2024)
    out = {}
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731

    # ---- SH forward (fp32 and fp16 coefficients) and backward, degrees 0..3 ----
    mean, origin, dc, rest = sh_inputs(rng)
    out.update(sh_mean=mean, sh_origin=origin, sh_dc=dc, sh_rest=rest)
    dc16, rest16 = dc.astype(np.float16), rest.astype(np.float16)
    out.update(sh_dc16=dc16, sh_rest16=rest16)
    grad_ch = rng.standard_normal((N_SH, 3)).astype(np.float32)
    visible = rng.uniform(size=N_SH) < 0.8
    grad_mean_in = rng.normal(0.0, 0.1, (N_SH, 3)).astype(np.float32)
    out.update(sh_grad_channels=grad_ch, sh_visible=visible, sh_grad_mean_in=grad_mean_in)
    for deg in range(4):
        col = K.sh_forward(t(mean), t(origin), t(dc), t(rest), deg)
        out[f"sh_deg{deg}_colour"] = col.cpu().numpy()
        out[f"sh_deg{deg}_colour16"] = K.sh_forward(t(mean), t(origin), t(dc16), t(rest16), deg).cpu().numpy()
        gdc, grest, gmean = K.sh_backward(t(mean), t(origin), t(rest), col, t(grad_ch), t(visible), t(grad_mean_in),
                                          deg)
        out[f"sh_deg{deg}_grad_dc"] = gdc.cpu().numpy()
        out[f"sh_deg{deg}_grad_rest"] = grest.cpu().numpy()
        out[f"sh_deg{deg}_grad_mean"] = gmean.cpu().numpy()

    # ---- Adam ----
    short = {"sh_coeffs_dc": "sh_dc", "sh_coeffs_rest": "sh_rest"}
    init = {}
    for grp, shp in ADAM_SHAPES.items():
        init[grp] = rng.standard_normal((N_ADAM, *shp)).astype(np.float32)
        init["grad_" + grp] = rng.normal(0.0, 0.01, (N_ADAM, *shp)).astype(np.float32)
        init["first_moment_" + grp] = rng.normal(0.0, 0.005, (N_ADAM, *shp)).astype(np.float32)
        init["second_moment_" + grp] = (rng.normal(0.0, 0.01, (N_ADAM, *shp)) ** 2).astype(np.float32)
    for k, v in init.items():
        out["adam_in_" + k] = v
    for ci, (step, zero_grads, update_channels, lazy) in enumerate(ADAM_CASES):
        st = {k: t(v.copy()) for k, v in init.items()}
        for grp in ADAM_SHAPES:
            st["lr_" + short.get(grp, grp)] = torch.tensor([ADAM_LR[short.get(grp, grp)]], device=dev)
        K.adam_step(st, N_ADAM, NUM_REST, step, zero_grads, update_channels, 0.9, 0.999, 1e-15, True, lazy)
        for k in init:
            out[f"adam_case{ci}_{k}"] = st[k].cpu().numpy()
    out["adam_cases"] = np.array(ADAM_CASES, np.int64)

    # ---- Gaussian response, scaling factor and alpha ----
    opac = (1.0 / (1.0 + np.exp(-rng.normal(0.0, 2.0, N_KERNEL)))).astype(np.float32)
    dirs = rng.standard_normal((N_KERNEL, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    hit = (dirs * rng.uniform(0.0, 2.2, (N_KERNEL, 1))).astype(np.float32)
    out.update(kf_opacity=opac, kf_local_hit=hit, kf_exp_powers=np.array(EXP_POWERS, np.float32))
    for p in EXP_POWERS:
        sf, g, a = K.kernel_functions(t(opac), t(hit), 0.01, p)
        out[f"kf_p{p}_scaling"] = sf.cpu().numpy()
        out[f"kf_p{p}_response"] = g.cpu().numpy()
        out[f"kf_p{p}_alpha"] = a.cpu().numpy()
    torch.cuda.synchronize()
    np.savez_compressed(out_path, **out)
    print("wrote", out_path, f"({os.path.getsize(out_path)} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_reference_kernels.py <out.npz>")
    main(sys.argv[1])
