"""torch.classes.gray.Raytracer from libgray.so, driven the way the reference's gray/raytracer.py
drives it (needs a GB300).

The call sequence is gray/raytracer.py:54-197's: construct with (W, H, N, sh_max_degree,
ppll_forward_size, ppll_backward_size, inference_only), fill the config and learning-rate tensors,
write the Gaussians into the holders, rebuild_bvh, then per iteration set the camera, forward_pass,
copy the image gradient into grad_output_channels, backward_pass, step, update_bvh.  Results are
compared with gray_gb300.classes (the same C ABI from Python) and with the CPU oracle.
"""
import numpy as np
import pytest
import torch

from gray_gb300 import synthetic

pytestmark = pytest.mark.gpu

W = H = 64


@pytest.fixture(scope="module")
def gray_classes(gray_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from gray_gb300 import build as B

    torch.classes.load_library(B.build_torch_binding())
    return torch.classes.gray


def _setup(rt, sc, lr_scale=1.0):
    """gray/raytracer.py:70-98 (config and Adam knobs) and from_point_cloud's writes."""
    cfg = rt.get_config()
    cfg.alpha_threshold.fill_(0.01)
    cfg.t_threshold.fill_(0.03)
    cfg.exp_power.fill_(2.0)
    cfg.render_depth.fill_(False)
    cfg.background_channels.copy_(torch.tensor([0.0, 0.0, 0.0]))
    cfg.enable_sh.fill_(True)
    cfg.needs_ray_output.fill_(False)
    cfg.update_channels.fill_(False)
    g = rt.get_gaussians()
    for name, lr in (("lr_rotation", 1e-3), ("lr_scale", 5e-3), ("lr_mean", 1.6e-4), ("lr_opacity", 2.5e-2),
                     ("lr_channels", 2.5e-3), ("lr_sh_dc", 2.5e-3), ("lr_sh_rest", 2.5e-3)):
        getattr(g, name).fill_(lr * lr_scale)
    g.beta_1.fill_(0.9)
    g.beta_2.fill_(0.999)
    g.epsilon.fill_(1e-15)
    g.sh_update_laziness.fill_(1)
    with torch.no_grad():
        g.mean.copy_(torch.from_numpy(sc.mean))
        g.rotation.copy_(torch.from_numpy(sc.rotation))
        g.scale.copy_(torch.from_numpy(sc.scale))
        g.opacity.copy_(torch.from_numpy(sc.opacity.reshape(-1, 1)))
        g.sh_coeffs_dc.copy_(torch.from_numpy(sc.sh_dc))
        g.sh_coeffs_rest.copy_(torch.from_numpy(sc.sh_rest))
        g.current_sh_degree.fill_(3)
    rt.rebuild_bvh()


def _camera(rt, cam):
    """gray/raytracer.py:125-133"""
    c = rt.get_camera()
    c.znear.fill_(0.0)
    c.zfar.fill_(99999.9)
    rt.get_config().rays_from_python.fill_(False)
    c.vertical_fov_radians.fill_(cam.fov_y)
    c.set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())


def _iteration(rt, cam, gout):
    _camera(rt, cam)
    with torch.enable_grad():
        rt.forward_pass()
    fb = rt.get_framebuffer()
    img = fb.output_channels.detach().clone()
    with torch.no_grad():
        fb.grad_output_channels.copy_(gout)
    rt.backward_pass()
    g = rt.get_gaussians()
    grads = {k: getattr(g, k).clone() for k in ("grad_mean", "grad_rotation", "grad_scale", "grad_opacity",
                                                "grad_sh_coeffs_dc", "grad_sh_coeffs_rest")}
    rt.step()
    rt.update_bvh()
    params = {k: getattr(g, k).clone() for k in ("mean", "rotation", "scale", "opacity", "sh_coeffs_dc",
                                                 "sh_coeffs_rest")}
    return img, grads, params


def test_reference_call_sequence_matches_python_classes_and_oracle(gray_classes):
    from gray_gb300 import classes
    from oracle import oracle as O

    sc = synthetic.small_scene(seed=0)
    cam = synthetic.camera_small(W, H, 64.0)
    gout = torch.from_numpy(np.random.default_rng(0).standard_normal((H, W, 3)).astype(np.float32)).cuda()
    rt_t = gray_classes.Raytracer(W, H, sc.n, 3, 1, 4_000_000, False)
    rt_p = classes.Raytracer(W, H, sc.n, 3, 1, 4_000_000, False)
    for rt in (rt_t, rt_p):
        _setup(rt, sc)
    assert rt_t.get_num_channels() == 3 and abs(rt_t.get_max_alpha() - 0.9999) < 1e-12
    for it in range(3):
        img_t, gr_t, p_t = _iteration(rt_t, cam, gout)
        img_p, gr_p, p_p = _iteration(rt_p, cam, gout)
        torch.cuda.synchronize()
        rt_t.check_status()
        rt_p.check_status()
        assert torch.equal(img_t, img_p), it  # same kernels, same inputs: identical images
        for k in gr_t:  # float atomics in the replay: equal up to summation order
            scale = gr_p[k].abs().max().clamp(min=1e-12)
            assert ((gr_t[k] - gr_p[k]).abs().max() / scale).item() < 1e-5, (it, k)
        for k in p_t:
            assert torch.allclose(p_t[k], p_p[k], rtol=1e-6, atol=1e-7), (it, k)
        if it == 0:
            # the first forward against the oracle: colour and transmittance bit-exact
            fb = {k: getattr(rt_t.get_framebuffer(), k).reshape(-1, getattr(rt_t.get_framebuffer(), k).shape[-1])
                  .cpu().numpy() for k in ("ray_origin", "ray_direction", "transmittance")}
            geom, l2w, aabb, vis = O.snapshot(sc.mean, sc.rotation, sc.scale, sc.opacity[:, 0])
            live = O.forward_prep(sc.opacity[:, 0])
            chan = O.sh_forward(3, sc.mean, np.asarray(cam.origin, np.float32), sc.sh_dc[:, 0, :], sc.sh_rest)
            cfg = O.TraceConfig(t_threshold=0.03)
            fwd = O.trace_forward(fb["ray_origin"], fb["ray_direction"], geom, live, chan, vis, cfg)
            assert np.array_equal(img_t.reshape(-1, 3).cpu().numpy(), fwd["rgb"])
            assert np.array_equal(fb["transmittance"][:, 0], fwd["T"])
    assert int(rt_t.get_metadata().total_num_steps.item()) == 3
    assert int(rt_t.get_metadata().total_num_calls.item()) == 3


def test_holders_keep_tensor_identity_and_shrink_only(gray_classes):
    sc = synthetic.small_scene(seed=1)
    rt = gray_classes.Raytracer(W, H, sc.n, 3, 1, 1_000_000, False)
    g = rt.get_gaussians()
    assert tuple(g.mean.shape) == (sc.n, 3) and tuple(g.sh_coeffs_rest.shape) == (sc.n, 15, 3)
    assert g.mean.grad is not None and g.mean.grad.data_ptr() == g.grad_mean.data_ptr()
    m = g.mean
    m.fill_(1.5)  # the reference mutates holder tensors in place
    assert float(rt.get_gaussians().mean[0, 0]) == 1.5
    rt.resize(sc.n // 2)
    assert tuple(rt.get_gaussians().mean.shape) == (sc.n // 2, 3)
    with pytest.raises(RuntimeError, match="must not be larger"):
        rt.resize(sc.n)
    inf = gray_classes.Raytracer(W, H, sc.n, 3, 1, 1, True)
    assert inf.get_gaussians().sh_coeffs_rest.dtype == torch.float16


def test_hit_list_overflow_raises_instead_of_trapping(gray_classes):
    """The reference traps on a full hit list (cuda/core/per_pixel_linked_list.h:23-26); here the
    kernel sets a status bit and the binding raises RuntimeError, leaving the context usable."""
    sc = synthetic.small_scene(seed=0)
    cam = synthetic.camera_small(W, H, 64.0)
    rt = gray_classes.Raytracer(W, H, sc.n, 3, 1, 64, False)
    _setup(rt, sc)
    _camera(rt, cam)
    with torch.enable_grad():
        rt.forward_pass()
    with pytest.raises(RuntimeError, match="overflow"):
        rt.check_status()
    rt.check_status()  # cleared
    torch.zeros(1, device="cuda").add_(1)
    torch.cuda.synchronize()


def test_resolution_display_sh_degree_and_shrink_match_python_classes(gray_classes):
    """The rest of the surface train.py and render.py use: a smaller render rectangle
    (set_render_resolution), the SH-degree schedule (increment_sh_degree), display renders
    (forward_pass_display) and pruning (resize to fewer Gaussians, then rebuild_bvh); every image is
    identical to gray_gb300.classes on the same inputs."""
    from gray_gb300 import classes

    sc = synthetic.small_scene(seed=2, n=400)
    cam = synthetic.camera_small(W, H, 64.0)
    rts = [gray_classes.Raytracer(W, H, sc.n, 3, 1, 4_000_000, False),
           classes.Raytracer(W, H, sc.n, 3, 1, 4_000_000, False)]
    for rt in rts:
        _setup(rt, sc)
        rt.get_gaussians().current_sh_degree.fill_(0)

    def frame(rt, w, h, display):
        rt.set_render_resolution(w, h)
        _camera(rt, cam)
        if display:
            with torch.no_grad():
                rt.forward_pass_display()
        else:
            with torch.enable_grad():
                rt.forward_pass()
        return rt.get_framebuffer().output_channels[:h, :w].clone()

    for step in range(4):
        w, h = (W, H) if step % 2 == 0 else (40, 24)
        imgs = [frame(rt, w, h, display=step == 3) for rt in rts]
        torch.cuda.synchronize()
        assert torch.equal(imgs[0], imgs[1]), step
        for rt in rts:
            rt.get_gaussians().increment_sh_degree()
    assert int(rts[0].get_gaussians().current_sh_degree.item()) == 3
    keep = sc.n // 3
    for rt in rts:
        rt.set_render_resolution(W, H)
        rt.resize(keep)  # train.py prunes by compacting the holders, then shrinking them
        rt.rebuild_bvh()
    imgs = [frame(rt, W, H, display=False) for rt in rts]
    torch.cuda.synchronize()
    for rt in rts:
        rt.check_status()
    assert tuple(rts[0].get_gaussians().mean.shape) == (keep, 3)
    assert torch.equal(imgs[0], imgs[1])
