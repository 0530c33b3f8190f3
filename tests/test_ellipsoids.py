"""Ellipsoid view (reference: cuda/ellipsoid_viewer.cu:1-94): the oracle's restatement pinned by
closed-form cases on the CPU, and the CUDA kernel (closest-hit traversal of the LBVH) checked bit for
bit against the oracle's brute force on the GPU."""
import math

import numpy as np
import pytest
import torch

from gray_gb300 import synthetic
from tests import gpu_util as G


def _one_sphere(oracle, radius_scale, opacity_logit, centre=(0.0, 0.0, 5.0)):
    mean = np.array([centre], np.float32)
    rot = np.array([[1.0, 0.0, 0.0, 0.0]], np.float32)
    scale = np.full((1, 3), math.log(radius_scale), np.float32)
    opac = np.array([opacity_logit], np.float32)
    geom, _, _, vis = oracle.snapshot(mean, rot, scale, opac)
    live = oracle.forward_prep(opac)
    live[vis == 0, 0] = -np.inf
    return geom, live, oracle.scaling_factor(1.0 / (1.0 + math.exp(-opacity_logit)), 0.01, 2.0)


def test_oracle_ellipsoid_sphere_closed_form(oracle):
    """Sphere of radius r = s * sf centred at distance 5 on the ray: hit at 5 - r, normal facing the
    ray (align 1: colour + 0.15); from inside the sphere the far root at 5 + r with align 0.5; a
    znear beyond the near root selects the far root; min_opacity above the opacity hides it."""
    geom, live, sf = _one_sphere(oracle, 0.5, 2.0)
    r = 0.5 * sf
    chan = np.array([[0.2, 0.4, 0.6]], np.float32)
    ro = np.zeros((1, 3), np.float32)
    rd = np.array([[0.0, 0.0, 1.0]], np.float32)
    rgb, depth, ids = oracle.ellipsoids(ro, rd, geom, live, chan)
    assert ids[0] == 0
    assert abs(depth[0] - (5.0 - r)) < 1e-5
    np.testing.assert_allclose(rgb[0], chan[0] + 0.15, rtol=0, atol=1e-6)
    # znear past the near root: far root, normal along the ray -> clamp 0.5
    rgb, depth, ids = oracle.ellipsoids(ro, rd, geom, live, chan, znear=5.0)
    assert ids[0] == 0 and abs(depth[0] - (5.0 + r)) < 1e-5
    np.testing.assert_allclose(rgb[0], 0.5 * (chan[0] + 0.15), rtol=0, atol=1e-6)
    # zfar before the near root: miss -> background, depth 0
    rgb, depth, ids = oracle.ellipsoids(ro, rd, geom, live, chan, zfar=5.0 - r - 0.01, bg=(0.1, 0.2, 0.3))
    assert ids[0] == -1 and depth[0] == 0.0
    np.testing.assert_allclose(rgb[0], [0.1, 0.2, 0.3])
    # opacity sigmoid(2) = 0.881 < 0.9: hidden
    _, _, ids = oracle.ellipsoids(ro, rd, geom, live, chan, min_opacity=0.9)
    assert ids[0] == -1
    # centre behind the ray origin: rejected (cuda/ellipsoid_viewer.cu:34-36)
    _, _, ids = oracle.ellipsoids(np.array([[0.0, 0.0, 5.2]], np.float32), rd, geom, live, chan)
    assert ids[0] == -1
    # grazing ray offset by 0.9 r: hit at 5 - r cos(asin 0.9); oblique normal -> align = cos
    off = 0.9 * r
    rgb, depth, ids = oracle.ellipsoids(np.array([[off, 0.0, 0.0]], np.float32), rd, geom, live, chan)
    c = math.sqrt(1.0 - 0.81)
    assert ids[0] == 0 and abs(depth[0] - (5.0 - r * c)) < 1e-5
    np.testing.assert_allclose(rgb[0], max(0.5, c) * (chan[0] + 0.15), atol=1e-5)
    # inactive ray (zero direction): outputs untouched
    _, _, ids = oracle.ellipsoids(ro, np.zeros((1, 3), np.float32), geom, live, chan)
    assert ids[0] == -2


def test_oracle_ellipsoid_nearest_and_ties(oracle):
    """Two spheres on the ray: the nearer wins; two identical spheres: the smaller id wins."""
    mean = np.array([[0, 0, 8.0], [0, 0, 4.0], [0, 0, 4.0]], np.float32)
    rot = np.tile(np.array([[1.0, 0, 0, 0]], np.float32), (3, 1))
    scale = np.full((3, 3), math.log(0.3), np.float32)
    opac = np.full(3, 1.0, np.float32)
    geom, _, _, vis = oracle.snapshot(mean, rot, scale, opac)
    live = oracle.forward_prep(opac)
    chan = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    _, _, ids = oracle.ellipsoids(np.zeros((1, 3), np.float32), np.array([[0, 0, 1.0]], np.float32), geom, live,
                                  chan)
    assert ids[0] == 1


# ------------------------------------------------------------------------------------------------
# GPU
# ------------------------------------------------------------------------------------------------
def _render(rt, ray_o=None, ray_d=None, min_opacity=0.0):
    cfg = rt.get_config()
    cfg.render_ellipsoids.fill_(True)
    cfg.ellipsoid_min_opacity.fill_(min_opacity)
    fb = rt.get_framebuffer()
    if ray_o is not None:
        H, W = fb.ray_origin.shape[:2]
        fb.ray_origin.copy_(torch.from_numpy(ray_o).reshape(H, W, 3))
        fb.ray_direction.copy_(torch.from_numpy(ray_d).reshape(H, W, 3))
    cfg.rays_from_python.fill_(ray_o is not None)
    with torch.no_grad():
        rt.forward_pass_display()
    torch.cuda.synchronize()
    rt.check_status()
    rgb = fb.output_channels.reshape(-1, 3).cpu().numpy()
    depth = fb.output_depth.reshape(-1).cpu().numpy()
    cfg.render_ellipsoids.fill_(False)
    return rgb, depth


def _oracle_inputs(oracle, sc):
    geom, _, _, vis = oracle.snapshot(sc.mean, sc.rotation, sc.scale, sc.opacity.reshape(-1))
    live = oracle.forward_prep(sc.opacity.reshape(-1))
    live[vis == 0, 0] = -np.inf
    return geom, live


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["small", "clustered"])
def test_ellipsoid_view_bit_exact(oracle, gray_lib, which):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rng = np.random.default_rng(11)
    if which == "small":
        sc = synthetic.small_scene(seed=3, n=300)
        W, H = 96, 64
        cam_o = np.array([0.0, -4.0, 0.3], np.float32)
    else:
        sc = synthetic.clustered_scene(20_000, seed=8)
        sc.scale[:] += np.float32(1.0)
        W, H = 80, 60
        cam_o = np.array([0.0, -14.0, 1.0], np.float32)
    n = sc.mean.shape[0]
    chan = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    rt = G.make_tracer(W, H, sc.mean, sc.rotation, sc.scale, sc.opacity, channels=chan, bg=(0.05, 0.1, 0.15))
    geom, live = _oracle_inputs(oracle, sc)
    # rays from python: a fan from one origin plus random origins; a few inactive rays
    R = W * H
    d = rng.standard_normal((R, 3)).astype(np.float32) * np.float32(0.25)
    d[:, 1] += 1.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.tile(cam_o, (R, 1))
    o[R // 2:] += rng.uniform(-1, 1, (R - R // 2, 3)).astype(np.float32)
    d[::97] = 0.0
    for minop in (0.0, 0.6):
        rgb, depth = _render(rt, o, d, minop)
        orgb, odepth, oid = oracle.ellipsoids(o, d, geom, live, chan, min_opacity=minop, bg=(0.05, 0.1, 0.15))
        act = oid != -2
        assert (oid >= 0).sum() > R // 10
        assert np.array_equal(rgb[act], orgb[act])
        assert np.array_equal(depth[act], odepth[act])
    # camera rays (the GPU's own primary rays, read back from a forward with gradients)
    cam = synthetic.look_at(cam_o, (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0.9, W, H)
    c = rt.get_camera()
    c.vertical_fov_radians.fill_(cam.fov_y)
    c.set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
    rt.get_config().rays_from_python.fill_(False)
    with torch.enable_grad():
        rt.forward_pass()
    torch.cuda.synchronize()
    f = G.fb_numpy(rt)
    co, cd = f["ray_origin"].copy(), f["ray_direction"].copy()
    rgb, depth = _render(rt)
    orgb, odepth, oid = oracle.ellipsoids(co, cd, geom, live, chan, bg=(0.05, 0.1, 0.15))
    assert np.array_equal(rgb, orgb) and np.array_equal(depth, odepth)


@pytest.mark.gpu
def test_ellipsoids_with_gradients_are_reported(gray_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    sc = synthetic.small_scene(seed=1, n=50)
    rt = G.make_tracer(32, 32, sc.mean, sc.rotation, sc.scale, sc.opacity,
                       channels=np.full((50, 3), 0.5, np.float32))
    cam = synthetic.camera_small(32, 32, 32.0)
    c = rt.get_camera()
    c.vertical_fov_radians.fill_(cam.fov_y)
    c.set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
    rt.get_config().render_ellipsoids.fill_(True)
    with torch.enable_grad():
        rt.forward_pass()
    torch.cuda.synchronize()
    with pytest.raises(RuntimeError, match="render_ellipsoids"):
        rt.check_status()
    rt.get_config().render_ellipsoids.fill_(False)
