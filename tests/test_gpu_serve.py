"""Serving form: continuous batching over resident scenes; each request's image is the same alone
and in the mix.  Needs a GB300."""
import numpy as np
import pytest
import torch

from gray_gb300 import classes, synthetic
from gray_gb300.serve import RenderServer, plain_loop, poisson_arrivals, run_served

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda(gray_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _scene_tracer(n, seed, maxw, maxh, sh_fp16=False):
    """A resident inference scene: fp32 SH (the serving configuration's precision) or fp16 SH (the
    reference's inference mode, cuda/core/gaussians.h:132)."""
    sc = synthetic.clustered_scene(n, seed=seed)
    rt = classes.Raytracer(maxw, maxh, sc.n, 3, 1, 1, inference_only=True, inference_sh_fp16=sh_fp16)
    rt.get_config().t_threshold.fill_(0.03)
    g = rt.get_gaussians()
    with torch.no_grad():
        for k, v in (("mean", sc.mean), ("rotation", sc.rotation), ("scale", sc.scale), ("opacity", sc.opacity),
                     ("sh_coeffs_dc", sc.sh_dc), ("sh_coeffs_rest", sc.sh_rest)):
            getattr(g, k).copy_(torch.from_numpy(v))
        g.current_sh_degree.fill_(3)
    rt.rebuild_bvh()
    return rt


@pytest.mark.parametrize("sh_fp16", [False, True])
def test_served_results_equal_alone_and_in_mix(sh_fp16):
    tracers = [_scene_tracer(40_000, 1, 160, 120, sh_fp16), _scene_tracer(90_000, 2, 160, 120, sh_fp16)]
    assert tracers[0].get_gaussians().sh_coeffs_rest.dtype == (torch.float16 if sh_fp16 else torch.float32)
    rng = np.random.default_rng(0)
    res = [(64, 48), (160, 120), (96, 96)]
    sched = []
    for i, t in enumerate(poisson_arrivals(400.0, 24, seed=1)):
        w, h = res[int(rng.integers(0, 3))]
        sched.append((float(t), int(rng.integers(0, 2)), synthetic.orbit_camera(float(rng.uniform(0, 6.28)), w, h)))
    srv = RenderServer(tracers, slots=2, max_batch=8, reserve_bytes=0, keep_images=True)
    reqs, wall = run_served(srv, sched)
    torch.cuda.synchronize()
    assert len(srv.completed) == len(sched)
    assert all(r.latency >= 0 for r in reqs)
    for r in reqs:
        alone = RenderServer(tracers, slots=1, reserve_bytes=0, keep_images=True)
        alone.submit(r.scene, r.camera)
        alone.drain()
        assert torch.equal(alone.completed[0].image, r.image), r.rid
    # the plain one-request-per-launch loop renders the same pixels
    for off, s, cam in sched[:4]:
        lat, _ = plain_loop(tracers, [(0.0, s, cam)])
        h, w = cam.image_height, cam.image_width
        ref = tracers[s].get_framebuffer().output_channels[:h, :w].permute(2, 0, 1)
        got = next(r.image for r in reqs if r.camera is cam)
        assert torch.equal(got, ref)


def test_tuned_server_renders_the_same_pixels():
    """A server whose kernel variant was picked once by the autotuner renders exactly what the
    untuned server renders (every variant gives the same pixels)."""
    tracers = [_scene_tracer(40_000, 1, 160, 120), _scene_tracer(90_000, 2, 160, 120)]
    cams = [(0, synthetic.orbit_camera(0.5, 160, 120)), (1, synthetic.orbit_camera(2.0, 96, 96)),
            (0, synthetic.orbit_camera(4.0, 64, 48))]
    tuned = RenderServer(tracers, slots=2, reserve_bytes=0, keep_images=True)
    choice = tuned.tune(cams)
    assert len(choice) == 2
    plain = RenderServer(tracers, slots=1, reserve_bytes=0, keep_images=True)
    for s, cam in cams:
        tuned.submit(s, cam)
        plain.submit(s, cam)
    tuned.drain()
    plain.drain()
    torch.cuda.synchronize()
    a = sorted(tuned.completed, key=lambda r: r.rid)
    b = sorted(plain.completed, key=lambda r: r.rid)
    for x, y in zip(a, b):
        assert torch.equal(x.image, y.image)
