"""gray_gb300's SH, SH-backward and Adam kernels against the reference's own kernels (needs a GB300).

Two sources for the reference side:
* tests/golden/reference_kernels.npz: outputs of graphdeco-inria/gray's cuda/utils/sh.cu and
  cuda/opt/adam.cu (compiled unchanged with the reference's fast-math flags) on seeded inputs,
  stored with those inputs (tests/golden/make_reference_kernels.py);
* oracle/_ref/gray_ref.cubin, when present: the same kernels launched live on larger inputs
  (oracle/ref_kernels.py).
Our side runs through the C ABI: forward_pass_display for the SH colour (forward_prep_kernel),
backward_pass with an empty hit list for the SH backward (fold_sh_backward_kernel), step for Adam.
Bars: colours within 1e-4 absolute, SH gradients within 1e-3 relative, Adam moments within 1e-6 and
parameters within 3e-4 of the update size (adam_close says why).
"""
import os

import numpy as np
import pytest
import torch

from gray_gb300 import classes
from tests import gpu_util as G

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURE = os.path.join(ROOT, "tests", "golden", "reference_kernels.npz")
SHORT = {"sh_coeffs_dc": "sh_dc", "sh_coeffs_rest": "sh_rest"}
LRS = {"mean": 1.6e-4, "scale": 5e-3, "rotation": 1e-3, "opacity": 2.5e-2, "channels": 2.5e-3, "sh_dc": 2.5e-3,
       "sh_rest": 2.5e-3}


@pytest.fixture(scope="module", autouse=True)
def _cuda(gray_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.fixture(scope="module")
def refk():
    if not os.path.exists(FIXTURE):
        pytest.skip("tests/golden/reference_kernels.npz not generated yet")
    return np.load(FIXTURE)


@pytest.fixture(scope="module")
def live():
    from oracle import ref_kernels as R

    if not R.available():
        pytest.skip("oracle/_ref/gray_ref.cubin not built (make -C oracle ref REF=<reference checkout>)")
    return R.RefKernels()


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def adam_close(kind, got, ref, before):
    """Adam bar.  Moments: within 1e-6 of the group's largest moment (measured <= 1e-7).
    Gradients: identical (zeroed or left as they were).  Parameters: within 3e-4 of the group's
    largest update plus 2 ulp of the parameter (measured <= 1.5e-4): the reference's fast-math powf
    in the bias correction (cuda/opt/adam.cu:15-16) has about 2^-22 relative error in beta^t, which
    1 - beta_2^t ~ 0.002 at the first steps turns into up to ~1e-4 relative error in every update;
    parameter-relative, that is below 1e-6 whenever an update is below ~1% of its parameter."""
    if kind == "first_moment_" or kind == "second_moment_":
        return float(np.abs(got - ref).max()) <= 1e-6 * float(np.abs(ref).max()) + 1e-30
    if kind == "grad_":
        return bool(np.array_equal(got, ref))
    upd = float(np.abs(ref - before).max())
    return bool(np.all(np.abs(got - ref) <= 3e-4 * upd + 2 * np.spacing(np.abs(ref).astype(np.float32))))


def _sh_tracer(mean, origin, dc, rest, deg, inference_only=False):
    n = mean.shape[0]
    rot = np.tile(np.array([1.0, 0.0, 0.0, 0.0], np.float32), (n, 1))
    rt = G.make_tracer(1, 1, mean, rot, np.full((n, 3), -3.0, np.float32), np.zeros(n, np.float32),
                       sh_dc=dc.astype(np.float32), sh_rest=rest.astype(np.float32), sh_degree=deg,
                       inference_only=inference_only)
    c = rt.get_camera()
    c.vertical_fov_radians.fill_(0.7)
    c.set_pose(torch.from_numpy(np.asarray(origin, np.float32)).cuda(), torch.eye(3).cuda())
    return rt


def our_sh_colour(mean, origin, dc, rest, deg, fp16):
    rt = _sh_tracer(mean, origin, dc, rest, deg, inference_only=fp16)
    rt.forward_pass_display()
    torch.cuda.synchronize()
    rt.check_status()
    return rt.get_gaussians().channels.cpu().numpy()


def our_sh_backward(mean, origin, rest, channels, grad_channels, visible, grad_mean_in, deg):
    """fold_sh_backward_kernel on given colours and colour gradients: a forward fills the state, the
    hit list is emptied (the replay adds nothing), and each visible Gaussian's accumulator row gets a
    hit count of one, so the fold runs the SH backward on exactly these inputs."""
    n = mean.shape[0]
    rt = _sh_tracer(mean, origin, np.zeros((n, 1, 3), np.float32), rest, deg)
    with torch.enable_grad():
        rt.forward_pass()
    torch.cuda.synchronize()
    g = rt.get_gaussians()
    h = rt.get_ppll_backward_data()
    with torch.no_grad():
        h.head_per_pixel.fill_(-1)
        h.total_hits.zero_()
        g.channels.copy_(torch.from_numpy(channels))
        g.grad_channels.copy_(torch.from_numpy(grad_channels))
        g.grad_mean.copy_(torch.from_numpy(grad_mean_in))
        g.grad_sh_coeffs_dc.zero_()
        g.grad_sh_coeffs_rest.zero_()
        acc = rt.scene_workspace().grad_acc
        acc.zero_()
        acc.view(-1, 16)[torch.from_numpy(np.asarray(visible, bool)).cuda(), 15] = 1.0
    rt.backward_pass()
    torch.cuda.synchronize()
    rt.check_status()
    return (g.grad_sh_coeffs_dc.cpu().numpy(), g.grad_sh_coeffs_rest.cpu().numpy(), g.grad_mean.cpu().numpy(),
            g.was_visible.cpu().numpy().reshape(-1))


def our_adam(init: dict, n, step, zero_grads, update_channels, lazy):
    rt = classes.Raytracer(1, 1, n, 3, 1, 1024)
    g = rt.get_gaussians()
    cfg = rt.get_config()
    cfg.zero_grads.fill_(bool(zero_grads))
    cfg.update_channels.fill_(bool(update_channels))
    cfg.enable_sh.fill_(True)
    g.sh_update_laziness.fill_(int(lazy))
    with torch.no_grad():
        for k, v in init.items():
            getattr(g, k).copy_(torch.from_numpy(v).reshape(getattr(g, k).shape))
        for name, lr in LRS.items():
            getattr(g, "lr_" + name).fill_(lr)
    rt.get_metadata().total_num_steps.fill_(step - 1)  # step() counts the call first, like the reference
    rt.step()
    torch.cuda.synchronize()
    return {k: getattr(g, k).cpu().numpy() for k in init}


@pytest.mark.parametrize("deg", [0, 1, 2, 3])
@pytest.mark.parametrize("fp16", [False, True])
def test_sh_colour_matches_reference_kernel(refk, deg, fp16):
    dc = refk["sh_dc16"] if fp16 else refk["sh_dc"]
    rest = refk["sh_rest16"] if fp16 else refk["sh_rest"]
    col = our_sh_colour(refk["sh_mean"], refk["sh_origin"], dc, rest, deg, fp16)
    ref = refk[f"sh_deg{deg}_colour16" if fp16 else f"sh_deg{deg}_colour"]
    err = np.abs(col - ref).max()
    assert err <= 1e-4 and err <= 2e-6, err


@pytest.mark.parametrize("deg", [0, 1, 2, 3])
def test_sh_backward_matches_reference_kernel(refk, deg):
    gdc, grest, gm, vis = our_sh_backward(refk["sh_mean"], refk["sh_origin"], refk["sh_rest"],
                                          refk[f"sh_deg{deg}_colour"], refk["sh_grad_channels"], refk["sh_visible"],
                                          refk["sh_grad_mean_in"], deg)
    assert np.array_equal(vis.astype(bool), refk["sh_visible"])
    assert rel_err(gdc, refk[f"sh_deg{deg}_grad_dc"]) <= 1e-6
    assert rel_err(grest, refk[f"sh_deg{deg}_grad_rest"]) <= 1e-6
    e = rel_err(gm, refk[f"sh_deg{deg}_grad_mean"])
    assert e <= 1e-3 and e <= 1e-5, e


@pytest.mark.parametrize("case", [0, 1, 2])
def test_adam_matches_reference_kernel(refk, case):
    step, zero_grads, update_channels, lazy = (int(v) for v in refk["adam_cases"][case])
    init = {k[len("adam_in_"):]: refk[k] for k in refk.files if k.startswith("adam_in_")}
    n = init["mean"].shape[0]
    got = our_adam(init, n, step, zero_grads, update_channels, lazy)
    for k in init:
        ref = refk[f"adam_case{case}_{k}"]
        g = got[k].reshape(ref.shape)
        kind = next((p for p in ("grad_", "first_moment_", "second_moment_") if k.startswith(p)), "")
        assert adam_close(kind, g, ref, init[k]), k


# ---- live: the reference's kernels launched on the same (larger) inputs as ours ----

@pytest.mark.parametrize("fp16", [False, True])
def test_sh_colour_matches_reference_kernel_live(live, fp16):
    rng = np.random.default_rng(77)
    n = 200_000
    mean = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
    origin = np.array([1.5, -8.0, 0.5], np.float32)
    dc = rng.normal(0.5, 0.2, (n, 1, 3)).astype(np.float32)
    rest = rng.normal(0.0, 0.05, (n, 15, 3)).astype(np.float32)
    if fp16:
        dc, rest = dc.astype(np.float16), rest.astype(np.float16)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    for deg in (1, 3):
        ref = live.sh_forward(t(mean), t(origin), t(dc), t(rest), deg).cpu().numpy()
        col = our_sh_colour(mean, origin, dc, rest, deg, fp16)
        err = np.abs(col - ref).max()
        assert err <= 1e-4 and err <= 4e-6, (deg, err)


def test_sh_backward_matches_reference_kernel_live(live):
    rng = np.random.default_rng(78)
    n = 100_000
    mean = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
    origin = np.array([1.5, -8.0, 0.5], np.float32)
    dc = rng.normal(0.5, 0.2, (n, 1, 3)).astype(np.float32)
    rest = rng.normal(0.0, 0.05, (n, 15, 3)).astype(np.float32)
    gch = rng.standard_normal((n, 3)).astype(np.float32)
    vis = rng.uniform(size=n) < 0.7
    gm_in = rng.normal(0.0, 0.1, (n, 3)).astype(np.float32)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    col = live.sh_forward(t(mean), t(origin), t(dc), t(rest), 3)
    rdc, rrest, rgm = live.sh_backward(t(mean), t(origin), t(rest), col, t(gch), t(vis), t(gm_in), 3)
    gdc, grest, gm, _ = our_sh_backward(mean, origin, rest, col.cpu().numpy(), gch, vis, gm_in, 3)
    assert rel_err(gdc, rdc.cpu().numpy()) <= 1e-6
    assert rel_err(grest, rrest.cpu().numpy()) <= 1e-6
    assert rel_err(gm, rgm.cpu().numpy()) <= 1e-5
