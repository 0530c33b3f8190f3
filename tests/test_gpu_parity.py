"""Parity of the CUDA path (through the C ABI) with the CPU oracle.  Needs a GB300.

Bar: integer/index results bit-exact (hit counts, composited gaussian id lists, BVH codes, order and
nodes), the fp16-keyed compositing results bit-exact (transmittance T, tail estimate), values
that depend on the order hits are found in (full transmittance, hence the final colour) within
float32 rounding, and gradients (float atomics in arbitrary order) within 1e-4 relative.
"""
import ctypes
import math

import numpy as np
import pytest
import torch

from gray_gb300 import _lib, synthetic
from tests import gpu_util as G

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-4      # gradients: fp32 atomics vs the oracle's double accumulation


@pytest.fixture(scope="module", autouse=True)
def _cuda(gray_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _grad_close(gpu, ref, rtol=GRAD_RTOL):
    scale = max(float(np.abs(ref).max()), 1e-12)
    assert np.abs(gpu - ref).max() <= rtol * scale + 1e-9, (np.abs(gpu - ref).max(), scale)


def _compare_forward(rt, fwd, check_lists=True):
    f = G.fb_numpy(rt)
    st = rt.get_stats()
    nhit = st.num_gaussians_hit.reshape(-1).cpu().numpy()
    nacc = st.num_gaussians_accumulated.reshape(-1).cpu().numpy()
    alive = fwd["nhit"] >= 0

    def same(name, a, b):
        bad = np.nonzero(np.any((a != b).reshape(a.shape[0], -1), axis=1))[0]
        assert bad.size == 0, f"{name}: {bad.size} rays differ, first {bad[:5]}: gpu {a[bad[:3]]} oracle {b[bad[:3]]}"

    same("nhit", nhit[alive], fwd["nhit"][alive])
    same("nacc", nacc[alive], fwd["nacc"][alive])
    same("T", f["transmittance"][alive, 0], fwd["T"][alive])
    same("rem", f["remaining_channels_estimate"][alive], fwd["rem"][alive])
    same("fullT", f["full_transmittance"][alive, 0], fwd["fullT"][alive])
    same("rgb", f["output_channels"][alive], fwd["rgb"][alive])
    if check_lists:
        gl, ol = G.hit_lists(rt), G.oracle_lists(fwd)
        for i in np.nonzero(alive)[0]:
            assert np.array_equal(gl[i], ol[i]), i


def _oracle_scene(O, mean, rot, scale, opac, a_thr=0.01, p=2.0):
    geom, l2w, aabb, vis = O.snapshot(mean, rot, scale, np.asarray(opac).reshape(-1), a_thr, p)
    live = O.forward_prep(np.asarray(opac).reshape(-1), a_thr, p)
    return geom, l2w, aabb, vis, live


NAMES = ["single_a0.01", "single_a0.3", "multi_t0.0", "multi_t0.5"]


@pytest.mark.parametrize("name", NAMES)
def test_reference_scenes_forward_backward(oracle, golden, name):
    p = name + "_"
    a_thr, t_thr = float(golden[p + "alpha_threshold"]), float(golden[p + "t_threshold"])
    rt = G.make_tracer(32, 32, golden[p + "mean"], golden[p + "rotation"], golden[p + "log_scale"],
                       golden[p + "logit_opacity"], channels=golden[p + "color"], alpha_threshold=a_thr,
                       t_threshold=t_thr, bg=tuple(golden[p + "bg"]))
    G.trace_rays(rt, golden["rays_o"], golden["rays_d"])
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, golden[p + "mean"], golden[p + "rotation"],
                                               golden[p + "log_scale"], golden[p + "logit_opacity"], a_thr)
    cfg = oracle.TraceConfig(alpha_threshold=a_thr, t_threshold=t_thr, bg=tuple(golden[p + "bg"]))
    fwd = oracle.trace_forward(golden["rays_o"], golden["rays_d"], geom, live, golden[p + "color"], vis, cfg)
    _compare_forward(rt, fwd)
    img = G.fb_numpy(rt)["output_channels"]
    err = np.abs(img - golden[p + "ref64_rgb"]).astype(np.float64)
    assert err.max() < 3e-4  # fp16-alpha bound vs the FP64 test loop
    assert 10.0 * math.log10(1.0 / np.mean(err ** 2)) >= 60.0  # PSNR, peak 1

    gout = golden[p + "ref64_grad_out"]
    rt.get_framebuffer().grad_output_channels.copy_(torch.from_numpy(gout).reshape(32, 32, 3))
    rt.backward_pass()
    torch.cuda.synchronize()
    rt.check_status()
    ref = oracle.trace_backward(32, 32, golden["rays_o"], golden["rays_d"], fwd, gout, geom, l2w,
                                golden[p + "logit_opacity"], golden[p + "log_scale"], golden[p + "rotation"],
                                golden[p + "color"], cfg)
    g = rt.get_gaussians()
    got = {"rotation": g.grad_rotation, "mean": g.grad_mean, "logit_opacity": g.grad_opacity,
           "log_scale": g.grad_scale, "color": g.grad_channels}
    sl = {"rotation": slice(0, 4), "mean": slice(4, 7), "logit_opacity": slice(7, 8), "log_scale": slice(8, 11),
          "color": slice(12, 15)}
    for k, t in got.items():
        t = t.cpu().numpy()
        _grad_close(t, ref[:, sl[k]])
        assert np.abs(t - golden[p + "ref64_grad_" + k]).max() < 1e-4, k  # reference tests' tolerance
    assert np.allclose(g.pruning_weight.cpu().numpy()[:, 0], ref[:, 11], rtol=1e-5, atol=1e-12)
    assert np.array_equal(g.was_visible.cpu().numpy()[:, 0], ref[:, 15] > 0)


@pytest.mark.parametrize("n", [30_000, 1_500_000])
def test_snapshot_and_bvh_bit_exact(oracle, n):
    """Snapshot records, Morton codes, sorted order, nodes and root box of a rebuild, then of a refit,
    bit-exact against the oracle; 1.5M Gaussians make each digit's row of tile counts (733 tiles)
    longer than one block-wide chunk of the row scan, and the refit's blocks many."""
    sc = synthetic.clustered_scene(n, seed=3)
    rt = G.make_tracer(16, 16, sc.mean, sc.rotation, sc.scale, sc.opacity, channels=np.zeros((sc.n, 3), np.float32))
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, sc.mean, sc.rotation, sc.scale, sc.opacity)
    ws = rt.scene_workspace()
    assert np.array_equal(ws.geom.cpu().numpy(), geom)
    assert np.array_equal(ws.l2w.cpu().numpy(), l2w)
    assert np.array_equal(ws.aabb.cpu().numpy(), aabb)
    assert np.array_equal(ws.visible.cpu().numpy(), vis)
    tree = oracle.Bvh(aabb, vis)
    assert np.array_equal(ws.codes.cpu().numpy().view(np.uint32), tree.codes)
    assert np.array_equal(ws.order.cpu().numpy().view(np.uint32), tree.order)
    assert np.array_equal(ws.nodes.cpu().numpy(), tree.nodes)
    assert np.array_equal(ws.root_box.cpu().numpy(), tree.root_box)
    # refit after moving the Gaussians keeps the topology and matches the oracle's refit
    g = rt.get_gaussians()
    with torch.no_grad():
        g.mean.add_(0.01)
        g.scale.add_(0.1)
    rt.update_bvh()
    torch.cuda.synchronize()
    _, _, aabb2, vis2 = oracle.snapshot(sc.mean + np.float32(0.01), sc.rotation, sc.scale + np.float32(0.1),
                                        sc.opacity[:, 0])
    tree.refit(aabb2)
    assert np.array_equal(ws.aabb.cpu().numpy(), aabb2)
    assert np.array_equal(ws.nodes.cpu().numpy(), tree.nodes)
    assert np.array_equal(ws.root_box.cpu().numpy(), tree.root_box)
    # a refit without the sort scratch (every level through global counters) gives the same boxes
    with torch.no_grad():
        ws.nodes[:, :12].fill_(-1.0)
        ws.root_box.fill_(-1.0)
    params = rt._build_params()
    params.scene.sort_tmp = None
    _lib.call("gray_update_bvh", params, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(ws.nodes.cpu().numpy(), tree.nodes)
    assert np.array_equal(ws.root_box.cpu().numpy(), tree.root_box)


@pytest.mark.parametrize("n", [63, 64, 129, 200_003])
@pytest.mark.parametrize("fp16", [False, True])
def test_forward_prep_tiles_bit_exact(oracle, n, fp16):
    """Live values (opacity, scaling factor; -inf opacity where the snapshot is invisible), SH colours
    at degrees 0-3 and the reset visited flags of the per-forward preparation, bit-exact against the
    oracle at sizes on either side of the bulk-copy kernel's 64-Gaussian tiles (63: the tail kernel
    only; 200,003: several tiles per persistent block and a tail), with fp32 and fp16 coefficients."""
    sc = synthetic.clustered_scene(n, seed=9)
    rt = G.make_tracer(16, 16, sc.mean, sc.rotation, sc.scale, sc.opacity, sh_dc=sc.sh_dc, sh_rest=sc.sh_rest,
                       sh_degree=0, inference_only=fp16)
    g = rt.get_gaussians()
    assert (g.sh_coeffs_rest.dtype == torch.float16) == fp16
    dc = g.sh_coeffs_dc.float().cpu().numpy().reshape(n, 3)
    rest = g.sh_coeffs_rest.float().cpu().numpy()
    _, _, _, vis, live = _oracle_scene(oracle, sc.mean, sc.rotation, sc.scale, sc.opacity)
    want_live = live.copy()
    want_live[vis == 0, 0] = -np.inf
    cam = synthetic.orbit_camera(0.7, 16, 16)
    for deg in range(4):
        g.current_sh_degree.fill_(deg)
        g.was_visible.fill_(True)
        rt.get_camera().vertical_fov_radians.fill_(cam.fov_y)
        rt.get_camera().set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
        with torch.set_grad_enabled(not fp16):  # an inference tracer keeps no backward hit list
            rt.forward_pass()
        torch.cuda.synchronize()
        rt.check_status()
        chan = oracle.sh_forward(deg, sc.mean, cam.origin.astype(np.float32), dc, rest)
        assert np.array_equal(g.channels.cpu().numpy(), chan), deg
        assert np.array_equal(rt.scene_workspace().live.cpu().numpy(), want_live), deg
        assert not g.was_visible.any().item(), deg  # set again only by a backward pass


def test_forward_captured_in_a_cuda_graph_matches_eager(oracle):
    """A forward captured in a CUDA graph (the tile schedule on the library's side stream, forked from
    and joined back to the capturing stream) replays to the same image, transmittances and hit lists
    as the eager call, which match the oracle."""
    sc = synthetic.small_scene(seed=4, n=300)
    cam = synthetic.camera_small(64, 64, 64.0)
    rt = G.make_tracer(64, 64, sc.mean, sc.rotation, sc.scale, sc.opacity, sh_dc=sc.sh_dc, sh_rest=sc.sh_rest,
                       sh_degree=3)
    ro, rd = _camera_rays_gpu(rt, cam)  # eager forward (with gradients: hit lists recorded)
    eager = G.fb_numpy(rt)
    eager_lists = G.hit_lists(rt)
    chan = oracle.sh_forward(3, sc.mean, cam.origin.astype(np.float32), sc.sh_dc[:, 0, :], sc.sh_rest)
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, sc.mean, sc.rotation, sc.scale, sc.opacity)
    fwd = oracle.trace_forward(ro, rd, geom, live, chan, vis, oracle.TraceConfig(t_threshold=0.03))
    _compare_forward(rt, fwd)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side), torch.enable_grad():
        rt.forward_pass()  # warm-up on the capturing stream's thread and context
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g), torch.enable_grad():
        rt.forward_pass()
    fb = rt.get_framebuffer()
    for k in ("output_channels", "transmittance", "full_transmittance"):
        getattr(fb, k).fill_(-1.0)
    g.replay()
    torch.cuda.synchronize()
    rt.check_status()
    replayed = G.fb_numpy(rt)
    for k in ("output_channels", "transmittance", "full_transmittance", "remaining_channels_estimate"):
        assert np.array_equal(replayed[k], eager[k]), k
    assert all(np.array_equal(a, b) for a, b in zip(G.hit_lists(rt), eager_lists))


@pytest.mark.parametrize("schedule", [True, False])
def test_forward_with_and_without_a_schedule_buffer(oracle, schedule):
    """With the schedule buffer (gray_schedule_words(W, H) words: tile estimates and order, per-tile
    frontiers, super-tile frontiers seeding the tile walks) the densest tiles run first and packets
    start at their tile's frontier; without it (NULL) the tiles run in launch order from the root.
    The image, transmittances and hit lists are the same and match the oracle."""
    sc = synthetic.clustered_scene(40_000, seed=6)
    W, H = 200, 120
    cam = synthetic.orbit_camera(1.1, W, H)
    rt = G.make_tracer(W, H, sc.mean, sc.rotation, sc.scale, sc.opacity,
                       channels=np.full((sc.n, 3), 0.5, np.float32))
    if not schedule:
        rt.schedule = None
        rt._invalidate()
    ro, rd = _camera_rays_gpu(rt, cam)
    rt.check_status()
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, sc.mean, sc.rotation, sc.scale, sc.opacity)
    chan = np.full((sc.n, 3), 0.5, np.float32)
    tree = oracle.Bvh(aabb, vis)
    fwd = oracle.trace_forward(ro, rd, geom, live, chan, vis, oracle.TraceConfig(t_threshold=0.03), bvh=tree)
    _compare_forward(rt, fwd)


def test_forwards_from_two_host_threads_match_their_serial_results():
    """Each host thread gets its own side stream for the tile schedule (per thread and CUDA context):
    two threads, each with its own tracer and torch stream, running forwards at the same time give
    the images and hit lists each tracer gives alone."""
    import threading

    scenes = [synthetic.clustered_scene(20_000, seed=s) for s in (21, 22)]
    cams = [synthetic.orbit_camera(0.4 + i, 96, 64) for i in range(2)]
    rts = [G.make_tracer(96, 64, sc.mean, sc.rotation, sc.scale, sc.opacity,
                         channels=np.full((sc.n, 3), 0.5, np.float32)) for sc in scenes]
    alone = []
    for rt, cam in zip(rts, cams):
        _camera_rays_gpu(rt, cam)
        alone.append((G.fb_numpy(rt)["output_channels"], G.hit_lists(rt)))
    for rt in rts:
        rt.get_framebuffer().output_channels.zero_()
    torch.cuda.synchronize()
    errors = []

    def work(i):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for _ in range(3):
                    with torch.enable_grad():
                        rts[i].forward_pass()
            s.synchronize()
        except Exception as e:  # reported below, on the main thread
            errors.append(e)

    threads = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    torch.cuda.synchronize()
    for rt, (img, lists) in zip(rts, alone):
        rt.check_status()
        assert np.array_equal(G.fb_numpy(rt)["output_channels"], img)
        assert all(np.array_equal(a, b) for a, b in zip(G.hit_lists(rt), lists))


def _camera_rays_gpu(rt, cam):
    rt.get_camera().znear.fill_(0.0)
    rt.get_camera().zfar.fill_(99999.9)
    rt.get_camera().vertical_fov_radians.fill_(cam.fov_y)
    rt.get_camera().set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
    rt.get_config().rays_from_python.fill_(False)
    with torch.enable_grad():
        rt.forward_pass()
    torch.cuda.synchronize()
    f = G.fb_numpy(rt)
    return f["ray_origin"], f["ray_direction"]


def test_small_scene_sh_camera_and_passes(oracle):
    """64 Gaussians, SH degree 3, one 256x256 camera at distance 4; 16-slot passes are the
    reference's 32 (its BUFFER_SIZE); camera rays checked against the oracle's camera."""
    sc = synthetic.small_scene(seed=0)
    cam = synthetic.camera_small()
    rt = G.make_tracer(256, 256, sc.mean, sc.rotation, sc.scale, sc.opacity, sh_dc=sc.sh_dc, sh_rest=sc.sh_rest,
                       sh_degree=3)
    ro, rd = _camera_rays_gpu(rt, cam)
    oro, ord_ = oracle.camera_rays(256, 256, cam.fov_y, cam.origin.astype(np.float32), cam.rotation_c2w_blender())
    assert np.abs(rd - ord_).max() < 1e-6 and np.abs(ro - oro).max() == 0
    chan = oracle.sh_forward(3, sc.mean, cam.origin.astype(np.float32), sc.sh_dc[:, 0, :], sc.sh_rest)
    assert np.array_equal(rt.get_gaussians().channels.cpu().numpy(), chan)
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, sc.mean, sc.rotation, sc.scale, sc.opacity)
    cfg = oracle.TraceConfig(t_threshold=0.03)
    fwd = oracle.trace_forward(ro, rd, geom, live, chan, vis, cfg)
    _compare_forward(rt, fwd)
    assert fwd["nhit"].sum() > 1000

    rng = np.random.default_rng(5)
    gout = rng.standard_normal((256 * 256, 3)).astype(np.float32)
    rt.get_framebuffer().grad_output_channels.copy_(torch.from_numpy(gout).reshape(256, 256, 3))
    rt.backward_pass()
    torch.cuda.synchronize()
    rt.check_status()
    ref = oracle.trace_backward(256, 256, ro, rd, fwd, gout, geom, l2w, sc.opacity, sc.scale, sc.rotation, chan, cfg)
    g = rt.get_gaussians()
    _grad_close(g.grad_rotation.cpu().numpy(), ref[:, 0:4])
    _grad_close(g.grad_opacity.cpu().numpy(), ref[:, 7:8])
    _grad_close(g.grad_scale.cpu().numpy(), ref[:, 8:11])
    _grad_close(g.grad_channels.cpu().numpy(), ref[:, 12:15])
    # SH backward on the accumulated colour gradient, then mean gradient = trace + SH parts
    vis_b = (ref[:, 15] > 0).astype(np.uint8)
    gdc, grest, gmean = oracle.sh_backward(3, sc.mean, cam.origin.astype(np.float32), sc.sh_rest, chan,
                                           g.grad_channels.cpu().numpy(), vis_b, ref[:, 4:7].astype(np.float32))
    _grad_close(g.grad_sh_coeffs_dc.cpu().numpy().reshape(-1, 3), gdc)
    _grad_close(g.grad_sh_coeffs_rest.cpu().numpy(), grest)
    _grad_close(g.grad_mean.cpu().numpy(), gmean)


@pytest.mark.parametrize("exp_power, a_thr, gsf", [(1.0, 0.01, 1.0), (3.0, 0.01, 1.0), (2.5, 0.05, 1.0),
                                                   (2.0, 0.01, 1.5)])
def test_response_powers_alpha_threshold_and_scale_factor(oracle, exp_power, a_thr, gsf):
    """The reference's other Gaussian responses (exp_power 1 and 3 of its high- and low-quality
    presets, and a general power through pow), a higher alpha threshold and a global scale factor
    (applied by the snapshot, not by the backward, cuda/backward_pass.cu:101): scaling factor,
    response, hit lists and images bit-exact against the oracle, and the backward's gradients (whose
    d|x|^2 term depends on the power) within the gradient bar."""
    sc = synthetic.small_scene(seed=7, n=200)
    cam = synthetic.camera_small(96, 96, 96.0)
    rng = np.random.default_rng(8)
    chan = rng.uniform(0.0, 1.0, (sc.n, 3)).astype(np.float32)
    rt = G.make_tracer(96, 96, sc.mean, sc.rotation, sc.scale, sc.opacity, channels=chan, exp_power=exp_power,
                       alpha_threshold=a_thr)
    if gsf != 1.0:
        rt.get_config().global_scale_factor.fill_(gsf)
        rt.rebuild_bvh()
    ro, rd = _camera_rays_gpu(rt, cam)
    geom, l2w, aabb, vis = oracle.snapshot(sc.mean, sc.rotation, sc.scale, np.asarray(sc.opacity).reshape(-1), a_thr,
                                           exp_power, gsf)
    live = oracle.forward_prep(np.asarray(sc.opacity).reshape(-1), a_thr, exp_power)
    ws = rt.scene_workspace()
    assert np.array_equal(ws.geom.cpu().numpy(), geom)
    cfg = oracle.TraceConfig(exp_power=exp_power, alpha_threshold=a_thr)
    fwd = oracle.trace_forward(ro, rd, geom, live, chan, vis, cfg)
    _compare_forward(rt, fwd)
    assert fwd["nhit"].sum() > 500
    gout = rng.standard_normal((96 * 96, 3)).astype(np.float32)
    rt.get_framebuffer().grad_output_channels.copy_(torch.from_numpy(gout).reshape(96, 96, 3))
    rt.backward_pass()
    torch.cuda.synchronize()
    rt.check_status()
    ref = oracle.trace_backward(96, 96, ro, rd, fwd, gout, geom, l2w, sc.opacity, sc.scale, sc.rotation, chan, cfg)
    g = rt.get_gaussians()
    _grad_close(g.grad_rotation.cpu().numpy(), ref[:, 0:4])
    _grad_close(g.grad_mean.cpu().numpy(), ref[:, 4:7])
    _grad_close(g.grad_opacity.cpu().numpy(), ref[:, 7:8])
    _grad_close(g.grad_scale.cpu().numpy(), ref[:, 8:11])
    _grad_close(g.grad_channels.cpu().numpy(), ref[:, 12:15])


def test_jittered_primary_rays_match_the_oracle_on_the_same_rays(oracle):
    """jitter_primary_rays: each pixel's ray goes through a hashed sub-pixel offset (changing with the
    call count), so the packets fall back to per-ray traversal.  The rays the forward wrote differ from
    the pixel-centre rays by less than a pixel, change from one call to the next, and traced again by
    the oracle give the same hits, lists and images."""
    sc = synthetic.small_scene(seed=12, n=150)
    cam = synthetic.camera_small(64, 64, 64.0)
    rt = G.make_tracer(64, 64, sc.mean, sc.rotation, sc.scale, sc.opacity, sh_dc=sc.sh_dc, sh_rest=sc.sh_rest,
                       sh_degree=3)
    ro0, rd0 = _camera_rays_gpu(rt, cam)  # pixel centres
    rt.get_config().jitter_primary_rays.fill_(True)
    rt.get_stats().reset()  # the hit counters accumulate over forwards
    ro, rd = _camera_rays_gpu(rt, cam)
    rt.check_status()
    cos = np.clip((rd * rd0).sum(1) / np.linalg.norm(rd, axis=1) / np.linalg.norm(rd0, axis=1), -1.0, 1.0)
    pixel_angle = cam.fov_y / 64
    assert (np.arccos(cos) > 0).mean() > 0.9 and np.arccos(cos).max() < pixel_angle
    chan = oracle.sh_forward(3, sc.mean, cam.origin.astype(np.float32), sc.sh_dc[:, 0, :], sc.sh_rest)
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, sc.mean, sc.rotation, sc.scale, sc.opacity)
    fwd = oracle.trace_forward(ro, rd, geom, live, chan, vis, oracle.TraceConfig(t_threshold=0.03))
    _compare_forward(rt, fwd)
    assert fwd["nhit"].sum() > 300
    _, rd2 = _camera_rays_gpu(rt, cam)  # the next call's offsets differ
    assert not np.array_equal(rd2, rd)


def test_multipass_selection_and_segments(oracle):
    """Many faint Gaussians on the same rays with t_threshold = 0: rays composite hundreds of hits,
    crossing many 32-slot passes; the hit list chains one segment per traversal."""
    rng = np.random.default_rng(11)
    n = 3000
    mean = np.stack([rng.normal(0, 0.15, n), rng.normal(0, 0.15, n), rng.uniform(-3, 3, n)], 1).astype(np.float32)
    rot = rng.standard_normal((n, 4)).astype(np.float32)
    # anisotropic, so that the rotation gradient is not zero (for spheres it is rounding noise)
    scale = rng.uniform(math.log(0.15), math.log(0.45), (n, 3)).astype(np.float32)
    opac = np.full((n, 1), -2.5, np.float32)  # sigmoid ~ 0.076
    chan = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    W = H = 24
    rt = G.make_tracer(W, H, mean, rot, scale, opac, channels=chan, t_threshold=0.0, bg=(0.2, 0.3, 0.4))
    cam_o = np.array([0.0, 0.0, 6.0], np.float32)
    ys, xs = np.meshgrid(np.linspace(-0.08, 0.08, H), np.linspace(-0.08, 0.08, W), indexing="ij")
    d = np.stack([xs.ravel(), ys.ravel(), -np.ones(W * H)], 1)
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    o = np.repeat(cam_o[None], W * H, 0)
    G.trace_rays(rt, o, d)
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, mean, rot, scale, opac)
    cfg = oracle.TraceConfig(t_threshold=0.0, bg=(0.2, 0.3, 0.4))
    fwd = oracle.trace_forward(o, d, geom, live, chan, vis, cfg)
    assert fwd["nacc"].max() > 200
    _compare_forward(rt, fwd)
    gout = rng.standard_normal((W * H, 3)).astype(np.float32)
    rt.get_framebuffer().grad_output_channels.copy_(torch.from_numpy(gout).reshape(H, W, 3))
    rt.backward_pass()
    torch.cuda.synchronize()
    rt.check_status()
    ref = oracle.trace_backward(W, H, o, d, fwd, gout, geom, l2w, opac, scale, rot, chan, cfg)
    g = rt.get_gaussians()
    _grad_close(g.grad_rotation.cpu().numpy(), ref[:, 0:4], 3e-4)
    _grad_close(g.grad_mean.cpu().numpy(), ref[:, 4:7], 3e-4)
    _grad_close(g.grad_channels.cpu().numpy(), ref[:, 12:15], 3e-4)


def test_znear_zfar_and_render_rectangle(oracle):
    sc = synthetic.gradcheck_scene(seed=2, n=400)
    chan = np.random.default_rng(0).uniform(0, 1, (sc.n, 3)).astype(np.float32)
    W, H = 48, 40
    rt = G.make_tracer(W, H, sc.mean, sc.rotation, sc.scale, sc.opacity, channels=chan, render_depth=True)
    cam = synthetic.look_at((0.3, -5.0, 0.4), (0, 0, 0), (0, 0, 1), 0.9, W, H)
    rt.get_camera().znear.fill_(4.2)
    rt.get_camera().zfar.fill_(6.1)
    rt.get_camera().vertical_fov_radians.fill_(cam.fov_y)
    rt.get_camera().set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
    rt.set_render_resolution(40, 33)
    rt.get_config().rays_from_python.fill_(False)
    with torch.enable_grad():
        rt.forward_pass()
    torch.cuda.synchronize()
    f = G.fb_numpy(rt)
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, sc.mean, sc.rotation, sc.scale, sc.opacity)
    mask = np.zeros((H, W), bool)
    mask[:33, :40] = True
    idx = np.nonzero(mask.ravel())[0]
    cfg = oracle.TraceConfig(znear=4.2, zfar=6.1, render_depth=True)
    fwd = oracle.trace_forward(f["ray_origin"][idx], f["ray_direction"][idx], geom, live, chan, vis, cfg)
    assert np.array_equal(f["transmittance"][idx, 0], fwd["T"])
    assert np.array_equal(f["output_depth"][idx, 0], fwd["depth"])
    assert np.array_equal(f["output_channels"][idx], fwd["rgb"])
    lists = G.hit_lists(rt)
    ol = G.oracle_lists(fwd)
    for k, i in enumerate(idx):
        assert np.array_equal(lists[i], ol[k])
    assert all(len(lists[i]) == 0 for i in np.nonzero(~mask.ravel())[0])


def test_grazing_rays_at_the_support_sphere_match_the_oracle(oracle):
    """Camera rays that pass within 2e-4 (relative) of their Gaussian's support sphere, on both
    sides: the packets' division-free hit pretest must keep every pair the intersection program
    accepts, so hit counts, lists and images stay bit-identical to the oracle."""
    W, H = 64, 48
    n = W * H
    rot = np.tile(np.array([1.0, 0.0, 0.0, 0.0], np.float32), (n, 1))
    scale = np.full((n, 3), math.log(0.02), np.float32)
    opac = np.full((n, 1), 2.0, np.float32)
    cam = synthetic.look_at((0.0, -5.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0.9, W, H)

    def render(mean, chan):
        rt = G.make_tracer(W, H, mean, rot, scale, opac, channels=chan)
        c = rt.get_camera()
        c.vertical_fov_radians.fill_(cam.fov_y)
        c.set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
        rt.get_config().rays_from_python.fill_(False)
        with torch.enable_grad():
            rt.forward_pass()
        torch.cuda.synchronize()
        rt.check_status()
        return rt

    rng = np.random.default_rng(11)
    chan = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    f0 = G.fb_numpy(render(rng.uniform(-1.0, 1.0, (n, 3)).astype(np.float32), chan))
    ro, rd = f0["ray_origin"].astype(np.float64), f0["ray_direction"].astype(np.float64)
    radius = 1.0 / float(oracle.snapshot(np.zeros((1, 3), np.float32), rot[:1], scale[:1], opac[:, 0][:1], 0.01)[0][0, 0])
    side = rng.standard_normal((n, 3))
    side -= np.sum(side * rd, axis=1, keepdims=True) * rd / np.sum(rd * rd, axis=1, keepdims=True)
    side /= np.linalg.norm(side, axis=1, keepdims=True)
    eps = rng.uniform(-2e-4, 2e-4, n)
    mean = (ro + rng.uniform(3.5, 6.5, (n, 1)) * rd + (radius * (1.0 + eps))[:, None] * side).astype(np.float32)

    rt = render(mean, chan)
    f = G.fb_numpy(rt)
    assert np.array_equal(f["ray_direction"], f0["ray_direction"])
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, mean, rot, scale, opac)
    fwd = oracle.trace_forward(f["ray_origin"], f["ray_direction"], geom, live, chan, vis,
                               oracle.TraceConfig(t_threshold=0.03))
    _compare_forward(rt, fwd)
    # the pixels' own Gaussians: the line's distance from the centre, in support radii (float64)
    rel = ro - mean.astype(np.float64)
    cross = np.cross(rel, rd)
    dist = np.linalg.norm(cross, axis=1) / np.linalg.norm(rd, axis=1) / radius
    assert np.count_nonzero(np.abs(dist - 1.0) < 2e-5) > 150
    lists = G.hit_lists(rt)
    own = np.array([i in set(lists[i].tolist()) for i in range(n)])
    assert own[dist < 1.0 - 5e-5].all() and not own[dist > 1.0 + 5e-5].any()


def test_inactive_pixels_and_empty_scene(oracle):
    sc = synthetic.small_scene(seed=1, n=16)
    chan = np.ones((sc.n, 3), np.float32)
    rt = G.make_tracer(8, 8, sc.mean, sc.rotation, sc.scale, sc.opacity, channels=chan, bg=(0.5, 0.5, 0.5))
    o = np.zeros((64, 3), np.float32)
    o[:, 1] = -4
    d = np.zeros((64, 3), np.float32)
    d[:32, 1] = 1.0  # second half: zero direction = inactive pixel (cuda/shaders.cu:86-88)
    rt.get_framebuffer().output_channels.fill_(-7.0)
    G.trace_rays(rt, o, d)
    f = G.fb_numpy(rt)
    assert np.all(f["output_channels"][32:] == -7.0)
    assert np.all(f["output_channels"][:32] != -7.0)
    # every Gaussian pruned: the render is background only
    rt.resize(0)
    rt.rebuild_bvh()
    G.trace_rays(rt, o, d)
    f = G.fb_numpy(rt)
    assert np.allclose(f["output_channels"][:32], 0.5)


def test_hitlist_overflow_is_reported_not_trapped(oracle):
    sc = synthetic.small_scene(seed=0)
    cam = synthetic.camera_small(64, 64, 64.0)
    rt = G.make_tracer(64, 64, sc.mean, sc.rotation, sc.scale, sc.opacity, channels=np.ones((sc.n, 3), np.float32),
                       pool_words=16)
    rt.get_camera().vertical_fov_radians.fill_(cam.fov_y)
    rt.get_camera().set_pose(cam.origin_cuda(), cam.rotation_c2w_blender_cuda())
    rt.get_camera().zfar.fill_(1e5)
    with torch.enable_grad():
        rt.forward_pass()
    torch.cuda.synchronize()
    from gray_gb300 import _lib

    with pytest.raises(_lib.GrayError, match="overflow"):
        rt.check_status()
    # the context stays usable
    rt.check_status()
    assert torch.isfinite(rt.get_framebuffer().output_channels).all()


@pytest.mark.parametrize("n,laziness,update_channels", [(1037, 1, False), (40009, 2, True), (40009, 1, False)])
def test_adam_step_bit_exact(oracle, n, laziness, update_channels):
    """Fused Adam against the oracle: ragged group lengths, more work units than the persistent grid
    holds (40k Gaussians), the SH groups skipped when the step is not a multiple of the laziness, and
    the channels group either updated or only zeroed."""
    rng = np.random.default_rng(4)
    rt = G.make_tracer(8, 8, rng.normal(0, 1, (n, 3)), rng.normal(0, 1, (n, 4)), rng.normal(-3, 0.3, (n, 3)),
                       rng.normal(0, 1, (n, 1)), sh_dc=rng.normal(0.5, 0.2, (n, 1, 3)),
                       sh_rest=rng.normal(0, 0.05, (n, 15, 3)), sh_degree=3)
    g = rt.get_gaussians()
    lrs = dict(channels=0.0025, opacity=0.025, mean=1.6e-4, rotation=1e-3, scale=5e-3, sh_dc=2.5e-3, sh_rest=1.25e-4)
    st = {}
    name_map = {"sh_dc": "sh_coeffs_dc", "sh_rest": "sh_coeffs_rest"}
    with torch.no_grad():
        for name in ("channels", "opacity", "mean", "rotation", "scale", "sh_dc", "sh_rest"):
            t = name_map.get(name, name)
            p = getattr(g, t)
            for pre, scale in (("grad_", 0.1), ("first_moment_", 0.01), ("second_moment_", 0.0)):
                v = torch.from_numpy(rng.normal(0, scale, tuple(p.shape)).astype(np.float32))
                if pre == "second_moment_":
                    v = torch.from_numpy(np.abs(rng.normal(0, 1e-3, tuple(p.shape))).astype(np.float32))
                getattr(g, pre + t).copy_(v)
            getattr(g, "lr_" + name).fill_(lrs[name])
            st[name] = p.detach().cpu().numpy().reshape(-1).copy()
            st["g_" + name] = getattr(g, "grad_" + t).cpu().numpy().reshape(-1).copy()
            st["m_" + name] = getattr(g, "first_moment_" + t).cpu().numpy().reshape(-1).copy()
            st["v_" + name] = getattr(g, "second_moment_" + t).cpu().numpy().reshape(-1).copy()
    cfg = rt.get_config()
    cfg.zero_grads.fill_(True)
    cfg.update_channels.fill_(update_channels)
    g.sh_update_laziness.fill_(laziness)
    rt.get_metadata().total_num_steps.fill_(6)
    rt.step()  # step becomes 7
    torch.cuda.synchronize()
    oracle.adam_step(st, lrs, n, 15, 7, zero_grads=True, update_channels=update_channels, laziness=laziness)
    for name in ("channels", "opacity", "mean", "rotation", "scale", "sh_dc", "sh_rest"):
        t = name_map.get(name, name)
        assert np.array_equal(getattr(g, t).detach().cpu().numpy().reshape(-1), st[name]), name
        assert np.array_equal(getattr(g, "first_moment_" + t).cpu().numpy().reshape(-1), st["m_" + name]), name
        assert np.array_equal(getattr(g, "second_moment_" + t).cpu().numpy().reshape(-1), st["v_" + name]), name
        assert np.array_equal(getattr(g, "grad_" + t).cpu().numpy().reshape(-1), st["g_" + name]), name
    assert not g.grad_mean.any()  # zeroed after the update
    assert int(rt.get_metadata().total_num_steps.item()) == 7


def test_clustered_scene_with_bvh(oracle):
    """A clustered scene large enough for a deep LBVH; oracle traverses its own (bit-identical) BVH."""
    sc = synthetic.clustered_scene(60_000, seed=5)
    rng = np.random.default_rng(1)
    chan = rng.uniform(0, 1, (sc.n, 3)).astype(np.float32)
    W, H = 96, 64
    cam = synthetic.orbit_camera(0.4, W, H)
    rt = G.make_tracer(W, H, sc.mean, sc.rotation, sc.scale, sc.opacity, channels=chan)
    ro, rd = _camera_rays_gpu(rt, cam)
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, sc.mean, sc.rotation, sc.scale, sc.opacity)
    tree = oracle.Bvh(aabb, vis)
    fwd = oracle.trace_forward(ro, rd, geom, live, chan, vis, oracle.TraceConfig(), bvh=tree)
    assert fwd["nhit"].sum() > 1000
    _compare_forward(rt, fwd)


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5, 6, 7, 15, 23, 31, 8 + 3, 32 + 7, 32 + 1, 32 + 4, 32 + 31])
def test_trace_variants_are_bit_identical(oracle, variant):
    """Every forward-kernel variant (hit buffer size, register cap, packet shape, tile frontier cut
    of 64, 32 or 128 leaves or none, one tile per block or one packet per warp) gives the same bits
    as the oracle: the variant only changes
    speed."""
    sc = synthetic.clustered_scene(40_000, seed=8)
    chan = np.random.default_rng(2).uniform(0, 1, (sc.n, 3)).astype(np.float32)
    W, H = 72, 56
    rt = G.make_tracer(W, H, sc.mean, sc.rotation, sc.scale + np.float32(1.0), sc.opacity, channels=chan,
                       t_threshold=0.001)
    rt.set_trace_variant(variant)
    cam = synthetic.orbit_camera(1.1, W, H, radius=4.0)
    ro, rd = _camera_rays_gpu(rt, cam)
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, sc.mean, sc.rotation, sc.scale + np.float32(1.0), sc.opacity)
    fwd = oracle.trace_forward(ro, rd, geom, live, chan, vis, oracle.TraceConfig(t_threshold=0.001),
                               bvh=oracle.Bvh(aabb, vis))
    assert fwd["nacc"].max() > 20  # more than one 16-key buffer on some rays
    _compare_forward(rt, fwd)


def test_automatic_kernel_choice_follows_the_last_forwards_re_traversals(oracle):
    """Default variant: the scheduled kernels count the packets that need more than one traversal
    with 16 hit slots (the same count from the 16-slot and the 32-slot kernel: packets with a ray
    that composites more than 16 hits), and the next forward runs the 32-slot kernel when more than
    1/8 of the packets do; the image equals the oracle's whichever kernel ran."""
    sc = synthetic.clustered_scene(40_000, seed=8)
    chan = np.random.default_rng(2).uniform(0, 1, (sc.n, 3)).astype(np.float32)
    W, H = 72, 56
    scale = sc.scale + np.float32(1.5)
    geom, l2w, aabb, vis, live = _oracle_scene(oracle, sc.mean, sc.rotation, scale, sc.opacity)
    cam = synthetic.orbit_camera(1.1, W, H, radius=4.0)
    words = {}
    for t_thr in (0.001, 0.6):  # rays composite many hits / stop after a few
        rt = G.make_tracer(W, H, sc.mean, sc.rotation, scale, sc.opacity, channels=chan, t_threshold=t_thr)
        counts = {}
        for v in (7, 5, 0, 0):
            rt.set_trace_variant(v)
            rt.get_stats().reset()  # per-pixel hit counts accumulate over forwards
            ro, rd = _camera_rays_gpu(rt, cam)
            counts[v] = rt.schedule[48:51].cpu().tolist()
        fwd = oracle.trace_forward(ro, rd, geom, live, chan, vis, oracle.TraceConfig(t_threshold=t_thr),
                                   bvh=oracle.Bvh(aabb, vis))
        _compare_forward(rt, fwd)
        packets = 9 * 4 * 4  # 8x16-pixel tiles of four 4x8 packets
        assert counts[7][0] == counts[5][0] == counts[0][0] == packets
        assert counts[7][1] == counts[5][1] == counts[0][1]  # the same count from either kernel
        nacc = np.zeros((64, W), np.int64)
        nacc[:H] = fwd["nacc"].reshape(H, W)
        deep_rays = nacc.reshape(8, 8, W // 4, 4).transpose(0, 2, 1, 3).reshape(-1, 32).max(axis=1) > 16
        assert abs(counts[0][1] - int(deep_rays.sum())) <= 2, (counts[0][1], int(deep_rays.sum()))
        words[t_thr] = counts[0]
    deep, shallow = words[0.001], words[0.6]
    assert deep[1] * 8 > deep[0] and deep[2] == 2      # many packets need a second traversal: 32 slots
    assert shallow[1] * 8 <= shallow[0] and shallow[2] == 1


def test_copy_wait_runs_out_reports_and_leaves_the_context_usable(oracle):
    """A wait on an mbarrier phase that never completes (bytes announced, none copied) gives up after
    its limit, sets GRAY_STATUS_COPY_TIMEOUT and returns; the context then runs a traced forward
    that matches the oracle."""
    L = _lib.load()
    L.gray_selftest_copy_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    assert L.gray_selftest_copy_wait(status.data_ptr(), 20_000_000, ctypes.c_void_p(stream.cuda_stream)) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 16
    test_small_scene_sh_camera_and_passes(oracle)
