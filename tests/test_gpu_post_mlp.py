"""The post-processing MLP on the ray tracer's outputs (gray/raytracer.py:157-195 with
gray/mlp.py:143-215), needs a GB300: the network reads the rendered colour with the encoded ray
direction and hit point (origin + depth * direction), its loss gradient reaches the tracer's
backward through the colour, and step() updates both the Gaussians and the network."""
import numpy as np
import pytest
import torch

from gray_gb300 import Raytracer, RaytracerConfig, mlp, synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda(gray_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_post_mlp_consumes_rays_and_depth_and_trains():
    sc = synthetic.clustered_scene(30_000, seed=5)
    cfg = RaytracerConfig(sh=False, post_mlp=True, render_depth=True, post_mlp_freq_bands=2,
                          ppll_backward_size=8_000_000)
    W, H = 96, 72
    rt = Raytracer(cfg, sc.n, W, H)
    g = rt.cuda_module.get_gaussians()
    with torch.no_grad():
        for k, v in (("mean", sc.mean), ("rotation", sc.rotation), ("scale", sc.scale), ("opacity", sc.opacity)):
            getattr(g, k).copy_(torch.from_numpy(v))
        g.channels.copy_(torch.from_numpy(np.random.default_rng(1).uniform(0.1, 0.9, (sc.n, 3)).astype(np.float32)))
    rt.cuda_module.rebuild_bvh()
    assert bool(rt.cuda_module.get_config().needs_ray_output.item())
    cam = synthetic.orbit_camera(1.1, W, H)
    out = rt(cam)
    assert out.shape == (3, H, W)
    fb = rt.cuda_module.get_framebuffer()
    colour = rt.output_channels
    d = fb.ray_direction[:H, :W].moveaxis(-1, 0)
    depth = fb.output_depth[:H, :W].moveaxis(-1, 0)
    assert float(depth.abs().max()) > 0.0  # render_depth: the hit points are real
    hit = cam.origin_cuda()[:, None, None] + depth * d
    with torch.no_grad():
        ref = rt.post_mlp.network(torch.cat([colour * 2 - 1, mlp.positional_encoding(torch.cat([hit, d]), 2)])
                                  .to(torch.bfloat16)).float()
    # the same network on the same inputs (bf16; the convolution algorithm may differ between calls)
    assert torch.allclose(out.detach(), ref, rtol=2e-2, atol=2e-2)
    target = torch.rand(3, H, W, device="cuda", generator=torch.Generator(device="cuda").manual_seed(2))
    w0 = [p.detach().clone() for p in rt.post_mlp.network.parameters()]
    ch0 = g.channels.detach().clone()
    loss = torch.nn.functional.l1_loss(out, target)
    rt.backward(loss)
    torch.cuda.synchronize()
    rt.cuda_module.check_status()
    assert float(g.grad_channels.abs().sum()) > 0.0  # the MLP's gradient reached the Gaussians
    rt.step()
    torch.cuda.synchronize()
    assert any(not torch.equal(a, b.detach()) for a, b in zip(w0, rt.post_mlp.network.parameters()))
    assert not torch.equal(ch0, g.channels)  # update_channels: SH off, so the channels are optimised
