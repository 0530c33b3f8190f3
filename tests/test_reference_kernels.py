"""The CPU oracle against the reference's own SH, Adam and Gaussian-response kernels (CPU only).

tests/golden/reference_kernels.npz holds seeded inputs and the outputs of graphdeco-inria/gray's
cuda/utils/sh.cu, cuda/opt/adam.cu and cuda/utils/kernel.cu, compiled unchanged with the
reference's fast-math flags and run on a GB300 (tests/golden/make_reference_kernels.py).  The oracle
restates gray_gb300's kernels bit-exactly (tests/test_gpu_parity.py), so these bars pin both to the
reference: colours within 1e-4, SH gradients within 1e-3 relative, Adam moments within 1e-6 and
parameters within 3e-4 of the update size (adam_close says why).  The measured differences (fast
math, and a closed-form SH basis in place of the reference's complex recurrence) are far below the
colour and gradient bars; those tests assert a tighter bound too.
"""
import ctypes
import json
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURE = os.path.join(ROOT, "tests", "golden", "reference_kernels.npz")
SHORT = {"sh_coeffs_dc": "sh_dc", "sh_coeffs_rest": "sh_rest"}


@pytest.fixture(scope="module")
def refk():
    if not os.path.exists(FIXTURE):
        pytest.skip("tests/golden/reference_kernels.npz not generated yet")
    return np.load(FIXTURE)


def rel_err(a, b):
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


def test_ref_struct_mirrors_match_the_reference_layout():
    """The ctypes mirrors used to launch the reference's kernels have the byte layout nvcc gives the
    reference's own struct definitions (oracle/ref_layout.json, written by `make -C oracle ref`)."""
    from oracle import ref_kernels as R

    layout = json.load(open(R.LAYOUT))
    for name, cls in (("Gaussians", R.RefGaussians), ("Camera", R.RefCamera), ("Adam", R.RefAdam)):
        want = layout[name]
        got = {f: getattr(cls, f).offset for f, _ in cls._fields_}
        assert set(got) == set(want) - {"__size__"}, name
        assert all(got[f] == want[f] for f in got), name
        assert ctypes.sizeof(cls) == want["__size__"], name


@pytest.mark.parametrize("deg", [0, 1, 2, 3])
@pytest.mark.parametrize("fp16", [False, True])
def test_oracle_sh_colour_matches_reference_kernel(oracle, refk, deg, fp16):
    dc = refk["sh_dc16"].astype(np.float32) if fp16 else refk["sh_dc"]
    rest = refk["sh_rest16"].astype(np.float32) if fp16 else refk["sh_rest"]
    col = oracle.sh_forward(deg, refk["sh_mean"], refk["sh_origin"], dc[:, 0, :], rest)
    ref = refk[f"sh_deg{deg}_colour16" if fp16 else f"sh_deg{deg}_colour"]
    err = np.abs(col - ref).max()
    assert err <= 1e-4 and err <= 2e-6, err
    assert np.array_equal(col == 0.0, ref == 0.0)  # the same colours are clamped


@pytest.mark.parametrize("deg", [0, 1, 2, 3])
def test_oracle_sh_backward_matches_reference_kernel(oracle, refk, deg):
    gdc, grest, gm = oracle.sh_backward(deg, refk["sh_mean"], refk["sh_origin"], refk["sh_rest"],
                                        refk[f"sh_deg{deg}_colour"], refk["sh_grad_channels"], refk["sh_visible"],
                                        refk["sh_grad_mean_in"])
    assert rel_err(gdc, refk[f"sh_deg{deg}_grad_dc"][:, 0, :]) <= 1e-6
    assert rel_err(grest, refk[f"sh_deg{deg}_grad_rest"]) <= 1e-6
    e = rel_err(gm, refk[f"sh_deg{deg}_grad_mean"])
    assert e <= 1e-3 and e <= 1e-5, e


@pytest.mark.parametrize("case", [0, 1, 2])
def test_oracle_adam_matches_reference_kernel(oracle, refk, case):
    step, zero_grads, update_channels, lazy = (int(v) for v in refk["adam_cases"][case])
    groups = ("channels", "opacity", "mean", "rotation", "scale", "sh_coeffs_dc", "sh_coeffs_rest")
    n = refk["adam_in_mean"].shape[0]
    st, lrs = {}, {}
    for grp in groups:
        o = SHORT.get(grp, grp)
        st[o] = refk["adam_in_" + grp].copy()
        st["g_" + o] = refk["adam_in_grad_" + grp].copy()
        st["m_" + o] = refk["adam_in_first_moment_" + grp].copy()
        st["v_" + o] = refk["adam_in_second_moment_" + grp].copy()
    lrs = {"mean": 1.6e-4, "scale": 5e-3, "rotation": 1e-3, "opacity": 2.5e-2, "channels": 2.5e-3, "sh_dc": 2.5e-3,
           "sh_rest": 2.5e-3}
    oracle.adam_step(st, lrs, n, 15, step, zero_grads=bool(zero_grads), update_channels=bool(update_channels),
                     enable_sh=True, laziness=lazy)
    for grp in groups:
        o = SHORT.get(grp, grp)
        for pre_o, pre_r in (("", ""), ("g_", "grad_"), ("m_", "first_moment_"), ("v_", "second_moment_")):
            ref = refk[f"adam_case{case}_{pre_r}{grp}"]
            got = st[pre_o + o].reshape(ref.shape)
            assert adam_close(pre_r, got, ref, refk[f"adam_in_{pre_r}{grp}"]), (grp, pre_r)


@pytest.mark.parametrize("p", [1.0, 2.0, 3.0, 2.5])
def test_oracle_gaussian_response_matches_reference_kernel(oracle, refk, p):
    opac, hit = refk["kf_opacity"], refk["kf_local_hit"]
    sf = np.array([oracle.scaling_factor(float(o), 0.01, p) for o in opac], np.float32)
    d = (hit.astype(np.float32) ** 2).sum(1, dtype=np.float32)
    g = np.array([oracle.eval_gaussian(float(x), p) for x in d], np.float32)
    a = np.array([oracle.maxalpha_mul(float(x), float(o)) for x, o in zip(g, opac)], np.float32)
    ref_sf, ref_g, ref_a = (refk[f"kf_p{p}_{k}"] for k in ("scaling", "response", "alpha"))
    assert np.array_equal(sf == 0.0, ref_sf == 0.0)
    assert rel_err(sf, ref_sf) <= 1e-5
    assert np.abs(g - ref_g).max() <= 1e-6
    assert np.abs(a - ref_a).max() <= 1e-6


def test_fp16_alpha_keys_equal_the_reference_kernel(oracle, refk):
    """The reference composites with alpha stored in fp16 (cuda/core/per_pixel_linked_list.h:29-31)
    and computes alpha with fast-math expf; our alpha (the oracle's, bit-exact with the GPU's) rounds
    to the same fp16 key as the reference kernel's for every live sample here, so the images' 3e-4
    distance from the reference tests' FP64 loops is the reference's own fp16 storage."""
    opac, hit = refk["kf_opacity"], refk["kf_local_hit"]
    d = (hit.astype(np.float32) ** 2).sum(1, dtype=np.float32)
    g = np.array([oracle.eval_gaussian(float(x), 2.0) for x in d], np.float32)
    a = np.array([oracle.maxalpha_mul(float(x), float(o)) for x, o in zip(g, opac)], np.float32)
    ref = refk["kf_p2.0_alpha"]
    live = a > 0.01
    assert live.sum() > 3000
    assert np.array_equal(a[live].astype(np.float16), ref[live].astype(np.float16))
