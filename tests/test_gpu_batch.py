"""Batched form: many views of several resident scenes in one persistent launch (eager, autotuned,
and replayed from a CUDA graph) must give, per pixel, exactly the bits of rendering each view alone
with the plain one-view-per-launch path.  Needs a GB300."""
import numpy as np
import pytest
import torch

from gray_gb300 import synthetic
from gray_gb300.batch import BatchRenderer
from tests import gpu_util as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda(gray_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _scenes(maxw, maxh):
    a = synthetic.clustered_scene(60_000, seed=31)
    b = synthetic.small_scene(seed=4, n=200)
    ta = G.make_tracer(maxw, maxh, a.mean, a.rotation, a.scale + np.float32(0.8), a.opacity, sh_dc=a.sh_dc,
                       sh_rest=a.sh_rest, sh_degree=3)
    tb = G.make_tracer(maxw, maxh, b.mean, b.rotation, b.scale, b.opacity, sh_dc=b.sh_dc, sh_rest=b.sh_rest,
                       sh_degree=2, bg=(0.1, 0.2, 0.3))
    return ta, tb


def _plain(tracer, cam):
    c = tracer.get_camera()
    c.znear.fill_(0.0)
    c.zfar.fill_(99999.9)
    c.vertical_fov_radians.fill_(float(cam.fov_y))
    c.set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
    tracer.get_config().rays_from_python.fill_(False)
    tracer.set_render_resolution(cam.image_width, cam.image_height)
    with torch.no_grad():
        tracer.forward_pass_display()
    h, w = cam.image_height, cam.image_width
    return tracer.get_framebuffer().output_channels[:h, :w].clone().permute(2, 0, 1)


def _cams():
    return [(0, synthetic.orbit_camera(0.2, 96, 64)), (1, synthetic.camera_small(80, 72, 80.0)),
            (0, synthetic.orbit_camera(2.1, 40, 56)), (0, synthetic.orbit_camera(4.0, 128, 80)),
            (1, synthetic.look_at((0.5, -3.0, 1.0), (0, 0, 0), (0, 0, 1), 0.9, 64, 64))]


@pytest.mark.parametrize("use_graph,autotune", [(False, False), (True, True)])
def test_batch_equals_plain_per_view(use_graph, autotune):
    ta, tb = _scenes(128, 96)
    tracers = [ta, tb]
    reqs = _cams()
    br = BatchRenderer(tracers, use_graph=use_graph, autotune=autotune)
    outs = [o.clone() for o in br.render(reqs)]
    torch.cuda.synchronize()
    br.check_status()
    for (s, cam), got in zip(reqs, outs):
        ref = _plain(tracers[s], cam)
        assert torch.equal(got, ref), (s, cam.image_width, cam.image_height, (got - ref).abs().max().item())
    # same signature, new poses: the graph (or eager launch) replays with updated cameras
    reqs2 = [(s, synthetic.orbit_camera(0.7 + i, c.image_width, c.image_height) if s == 0 else c)
             for i, (s, c) in enumerate(reqs)]
    outs2 = [o.clone() for o in br.render(reqs2)]
    torch.cuda.synchronize()
    for (s, cam), got in zip(reqs2, outs2):
        assert torch.equal(got, _plain(tracers[s], cam))


def test_request_alone_equals_request_in_mix():
    ta, tb = _scenes(128, 96)
    reqs = _cams()
    mix = BatchRenderer([ta, tb], use_graph=False, autotune=False).render(reqs)
    mix = [m.clone() for m in mix]
    for k, req in enumerate(reqs):
        alone = BatchRenderer([ta, tb], use_graph=False, autotune=False, variant=3).render([req])[0]
        assert torch.equal(alone, mix[k])


def test_grazing_rays_batched_equal_plain_for_every_candidate_variant():
    """One Gaussian per pixel whose support sphere the pixel's camera ray grazes (within 2e-4,
    both sides): every kernel variant the autotuner may pick renders it in the batch kernel with
    exactly the bits of the plain path (whose hit lists equal the oracle's on the same scene)."""
    import math

    from gray_gb300.batch import TUNE_CANDIDATES

    W, H = 64, 48
    n = W * H
    rot = np.tile(np.array([1.0, 0.0, 0.0, 0.0], np.float32), (n, 1))
    scale = np.full((n, 3), math.log(0.02), np.float32)
    opac = np.full((n, 1), 2.0, np.float32)
    cam = synthetic.look_at((0.0, -5.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0.9, W, H)
    rng = np.random.default_rng(12)
    chan = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    probe = G.make_tracer(W, H, rng.uniform(-1.0, 1.0, (n, 3)).astype(np.float32), rot, scale, opac, channels=chan)
    c = probe.get_camera()
    c.vertical_fov_radians.fill_(cam.fov_y)
    c.set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
    probe.get_config().rays_from_python.fill_(False)
    with torch.enable_grad():
        probe.forward_pass()
    torch.cuda.synchronize()
    f = G.fb_numpy(probe)
    ro, rd = f["ray_origin"].astype(np.float64), f["ray_direction"].astype(np.float64)
    radius = 0.02 * math.sqrt(math.sqrt(4.0 * math.log((1.0 / (1.0 + math.exp(-2.0))) / 0.01)))
    side = rng.standard_normal((n, 3))
    side -= np.sum(side * rd, axis=1, keepdims=True) * rd / np.sum(rd * rd, axis=1, keepdims=True)
    side /= np.linalg.norm(side, axis=1, keepdims=True)
    eps = rng.uniform(-2e-4, 2e-4, n)
    mean = (ro + rng.uniform(3.5, 6.5, (n, 1)) * rd + (radius * (1.0 + eps))[:, None] * side).astype(np.float32)
    tracer = G.make_tracer(W, H, mean, rot, scale, opac, channels=chan)
    ref = _plain(tracer, cam)
    assert ref.abs().sum().item() > 0
    for variant, bps in TUNE_CANDIDATES:
        br = BatchRenderer([tracer], use_graph=False, autotune=False, variant=variant, blocks_per_sm=bps)
        got = br.render([(0, cam)])[0].clone()
        torch.cuda.synchronize()
        br.check_status()
        assert torch.equal(got, ref), (variant, bps, (got - ref).abs().max().item())
