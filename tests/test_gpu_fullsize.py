"""Parity at the benchmark's full size (3M clustered Gaussians, one 1920x1080 view): the GPU's
forward outputs and hit lists on a seeded sample of pixels are bit-identical to the oracle's (own
LBVH, same rays), the backward restricted to those pixels (upstream gradient zero elsewhere)
matches the oracle's within the reduction-order tolerance, and a batched render of the view is
bit-identical to the plain forward.  The batching configuration's 16 uneven views, rendered in one
batch, match the oracle on seeded pixels of every view.  Needs a GB300 (about 5 GB of device
memory)."""
import numpy as np
import pytest
import torch

from gray_gb300 import Raytracer, RaytracerConfig, synthetic
from gray_gb300.batch import BatchRenderer
from tests import gpu_util as G

pytestmark = pytest.mark.gpu

N, W, H = 3_000_000, 1920, 1080
SAMPLE = 1500


@pytest.fixture(scope="module")
def scene(gray_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    sc = synthetic.clustered_scene(N, seed=0)
    cam = synthetic.orbit_camera(0.3, W, H)
    rt = Raytracer(RaytracerConfig(sh=True, sh_max_degree=3, ppll_backward_size=160_000_000), N, W, H)
    g = rt.cuda_module.get_gaussians()
    with torch.no_grad():
        for k, v in (("mean", sc.mean), ("rotation", sc.rotation), ("scale", sc.scale), ("opacity", sc.opacity),
                     ("sh_coeffs_dc", sc.sh_dc), ("sh_coeffs_rest", sc.sh_rest)):
            getattr(g, k).copy_(torch.from_numpy(v))
        g.current_sh_degree.fill_(3)
    rt.cuda_module.rebuild_bvh()
    yield sc, cam, rt
    del rt
    torch.cuda.empty_cache()


def test_forward_and_backward_on_sampled_pixels(scene, oracle):
    sc, cam, rt = scene
    img = rt(cam)
    torch.cuda.synchronize()
    rt.cuda_module.check_status()
    f = G.fb_numpy(rt.cuda_module)
    st = rt.cuda_module.get_stats()
    nhit = st.num_gaussians_hit.reshape(-1).cpu().numpy()
    nacc = st.num_gaussians_accumulated.reshape(-1).cpu().numpy()
    rng = np.random.default_rng(42)
    idx = np.sort(rng.choice(W * H, SAMPLE, replace=False))
    chan = rt.cuda_module.get_gaussians().channels.detach().cpu().numpy()
    geom, l2w, aabb, vis = oracle.snapshot(sc.mean, sc.rotation, sc.scale, sc.opacity[:, 0])
    live = oracle.forward_prep(sc.opacity[:, 0])
    bvh = oracle.Bvh(aabb, vis)
    cfg = oracle.TraceConfig(t_threshold=0.03)
    ro, rd = f["ray_origin"][idx], f["ray_direction"][idx]
    fwd = oracle.trace_forward(ro, rd, geom, live, chan, vis, cfg, bvh=bvh)
    assert np.array_equal(nhit[idx], fwd["nhit"])
    assert np.array_equal(nacc[idx], fwd["nacc"])
    for name, ref in (("transmittance", fwd["T"]), ("full_transmittance", fwd["fullT"])):
        assert np.array_equal(f[name][idx, 0], ref), name
    assert np.array_equal(f["remaining_channels_estimate"][idx], fwd["rem"])
    assert np.array_equal(f["output_channels"][idx], fwd["rgb"])
    ol = G.oracle_lists(fwd)
    h = rt.cuda_module.get_ppll_backward_data()
    head = h.head_per_pixel.reshape(-1).cpu().numpy().view(np.uint32)
    pool = h.pool.cpu().numpy().view(np.uint32)
    for k, i in enumerate(idx):
        segs, seg = [], head[i]
        while seg != 0xFFFFFFFF:
            cnt = int(pool[seg + 1])
            segs.append(pool[seg + 2:seg + 2 + cnt])
            seg = int(pool[seg])
        got = np.concatenate(segs[::-1]) if segs else np.zeros(0, np.uint32)
        assert np.array_equal(got, ol[k]), i
    assert fwd["nhit"].mean() > 20

    # backward of the sampled pixels only
    gout = np.zeros((W * H, 3), np.float32)
    gs = rng.standard_normal((SAMPLE, 3)).astype(np.float32)
    gout[idx] = gs
    weight = torch.from_numpy(gout).reshape(H, W, 3).permute(2, 0, 1).cuda()
    rt.backward((img * weight).sum())
    torch.cuda.synchronize()
    rt.cuda_module.check_status()
    ref = oracle.trace_backward(W, H, ro, rd, fwd, gs, geom, l2w, sc.opacity, sc.scale, sc.rotation, chan, cfg)
    g = rt.cuda_module.get_gaussians()
    touched = np.nonzero(ref[:, 15] > 0)[0]
    assert touched.size > 100
    for name, cols in (("grad_opacity", slice(7, 8)), ("grad_scale", slice(8, 11)), ("grad_rotation", slice(0, 4))):
        got = getattr(g, name).detach().cpu().numpy()[touched]
        exp = ref[touched, cols]
        scale = max(float(np.abs(exp).max()), 1e-12)
        assert float(np.abs(got - exp).max()) <= 1e-4 * scale, name
    gch = g.grad_channels.detach().cpu().numpy()[touched]
    assert float(np.abs(gch - ref[touched, 12:15]).max()) <= 1e-4 * max(float(np.abs(ref[:, 12:15]).max()), 1e-12)


def test_batched_view_equals_plain_at_full_size(scene):
    sc, cam, rt = scene
    with torch.no_grad():
        c = rt.cuda_module.get_camera()
        c.znear.fill_(0.0)
        c.zfar.fill_(99999.9)
        c.vertical_fov_radians.fill_(float(cam.fov_y))
        c.set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
        rt.cuda_module.get_config().rays_from_python.fill_(False)
        rt.cuda_module.forward_pass_display()
        plain = rt.cuda_module.get_framebuffer().output_channels.clone().permute(2, 0, 1)
        out = BatchRenderer([rt.cuda_module], use_graph=False, autotune=False).render([(0, cam)])[0]
    torch.cuda.synchronize()
    assert torch.equal(out, plain)


def test_sixteen_uneven_views_in_one_batch_match_the_oracle(scene, oracle):
    """The batching configuration: the benchmark's 16 views of uneven resolution (seed 0, as bench.py's
    batched form) of the 3M scene rendered in one persistent launch; on 200 seeded pixels of every
    view the batch's colour equals the oracle's bit for bit (the oracle traces the same rays through
    its own LBVH with the view's SH colours)."""
    sc, _, rt = scene
    tr = rt.cuda_module
    cams = synthetic.uneven_cameras(16, seed=0)
    with torch.no_grad():
        outs = BatchRenderer([tr], use_graph=False, autotune=False).render([(0, c) for c in cams])
    torch.cuda.synchronize()
    geom, l2w, aabb, vis = oracle.snapshot(sc.mean, sc.rotation, sc.scale, sc.opacity[:, 0])
    live = oracle.forward_prep(sc.opacity[:, 0])
    bvh = oracle.Bvh(aabb, vis)
    cfg = oracle.TraceConfig(t_threshold=0.03)
    rng = np.random.default_rng(11)
    ro_all, rd_all, got_all, chans = [], [], [], []
    for v, cam in enumerate(cams):
        w, h = cam.image_width, cam.image_height
        # the view's rays as the forward generates them (a training forward writes them out)
        tr.set_render_resolution(w, h)
        c = tr.get_camera()
        c.znear.fill_(0.0)
        c.zfar.fill_(99999.9)
        c.vertical_fov_radians.fill_(float(cam.fov_y))
        c.set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
        tr.get_config().rays_from_python.fill_(False)
        with torch.enable_grad():
            tr.forward_pass()
        fb = tr.get_framebuffer()
        idx = rng.choice(w * h, 200, replace=False)
        yy, xx = idx // w, idx % w
        ro_all.append(fb.ray_origin[:h, :w].reshape(-1, 3)[torch.from_numpy(idx).cuda()].cpu().numpy())
        rd_all.append(fb.ray_direction[:h, :w].reshape(-1, 3)[torch.from_numpy(idx).cuda()].cpu().numpy())
        got_all.append(outs[v][:, yy, xx].T.cpu().numpy())
        chans.append(oracle.sh_forward(3, sc.mean, np.asarray(cam.origin, np.float32), sc.sh_dc[:, 0, :],
                                       sc.sh_rest))
    tr.set_render_resolution(W, H)
    torch.cuda.synchronize()
    tr.check_status()
    for v in range(len(cams)):
        fwd = oracle.trace_forward(ro_all[v], rd_all[v], geom, live, chans[v], vis, cfg, bvh=bvh)
        assert np.array_equal(got_all[v], fwd["rgb"]), v
