"""Training-loop pieces around the hot path on a GB300: pruning (gray/raytracer.py:296-359 with
cuda/core/gaussians.h:198-263 shrinking), the rebuild cadence (train.py:265-287) and the
safetensors scene format (gray/raytracer.py:368-438)."""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

from gray_gb300 import Raytracer, RaytracerConfig, TrainCadence, synthetic

pytestmark = pytest.mark.gpu

W, H = 160, 120
_PARAMS = ("mean", "rotation", "scale", "opacity", "channels", "sh_coeffs_dc", "sh_coeffs_rest")


@pytest.fixture(scope="module", autouse=True)
def _cuda(gray_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _cfg(**kw):
    return RaytracerConfig(sh=True, sh_max_degree=3, ppll_backward_size=20_000_000, **kw)


def _tracer(sc, cfg=None, inference_only=False):
    cfg = cfg or _cfg()
    rt = Raytracer(cfg, sc.mean.shape[0], W, H, inference_only=inference_only)
    g = rt.cuda_module.get_gaussians()
    with torch.no_grad():
        g.mean.copy_(torch.from_numpy(sc.mean))
        g.rotation.copy_(torch.from_numpy(sc.rotation))
        g.scale.copy_(torch.from_numpy(sc.scale))
        g.opacity.copy_(torch.from_numpy(sc.opacity))
        g.sh_coeffs_dc.copy_(torch.from_numpy(sc.sh_dc))
        g.sh_coeffs_rest.copy_(torch.from_numpy(sc.sh_rest))
        g.current_sh_degree.fill_(3)
    rt.cuda_module.rebuild_bvh()
    return rt


def _scene():
    sc = synthetic.clustered_scene(8_000, seed=21, clusters=20, radius=3.0)
    sc.scale[:] += np.float32(1.0)
    return sc


def _cam(i=0):
    return synthetic.orbit_camera(0.4 + 0.9 * i, W, H, radius=6.0)


def _target(i=0):
    g = torch.Generator().manual_seed(100 + i)
    return torch.rand(3, H, W, generator=g).cuda()


def _train_step(rt, i):
    img = rt(_cam(i))
    loss = F.l1_loss(img, _target(i))
    rt.backward(loss)
    rt.step()
    return img.detach()


def _grads(rt):
    g = rt.cuda_module.get_gaussians()
    return {k: getattr(g, "grad_" + k).detach().clone() for k in ("mean", "rotation", "scale", "opacity",
                                                                   "sh_coeffs_dc", "sh_coeffs_rest")}


def _close(a, b, name):
    a, b = a.double().cpu(), b.double().cpu()
    scale = max(float(b.abs().max()), 1e-30)
    assert float((a - b).abs().max()) <= 1e-4 * scale, name


def test_prune_equals_fresh_tracer_with_kept_rows():
    sc = _scene()
    a = _tracer(sc)
    for i in range(3):
        _train_step(a, i)
    torch.cuda.synchronize()
    a.cuda_module.check_status()
    g = a.cuda_module.get_gaussians()
    n = g.count
    mask = torch.from_numpy(np.random.default_rng(1).uniform(size=n) < 0.7).cuda()
    kept = {k: getattr(g, k).detach()[mask].clone() for k in _PARAMS}
    kept.update({f"{m}_{k}": getattr(g, f"{m}_{k}").detach()[mask].clone()
                 for m in ("first_moment", "second_moment") for k in _PARAMS})
    a.prune(3, mask)
    assert g.count == int(mask.sum())
    assert float(g.pruning_weight.abs().sum()) == 0.0 and int(g.pruning_counter.abs().sum()) == 0
    for k, v in kept.items():
        assert torch.equal(getattr(g, k).detach(), v), k
    a.cuda_module.rebuild_bvh()

    b = Raytracer(_cfg(), int(mask.sum()), W, H)
    gb = b.cuda_module.get_gaussians()
    with torch.no_grad():
        for k, v in kept.items():
            getattr(gb, k).copy_(v)
        gb.current_sh_degree.copy_(g.current_sh_degree)
        b.cuda_module.get_metadata().total_num_steps.copy_(a.cuda_module.get_metadata().total_num_steps)
    b.cuda_module.rebuild_bvh()

    ia, ib = a(_cam(5)), b(_cam(5))
    assert torch.equal(ia.detach(), ib.detach())
    la, lb = F.l1_loss(ia, _target(5)), F.l1_loss(ib, _target(5))
    a.backward(la)
    b.backward(lb)
    torch.cuda.synchronize()
    ga, gbb = _grads(a), _grads(b)
    for k in ga:
        _close(ga[k], gbb[k], k)
    a.step()
    b.step()
    torch.cuda.synchronize()
    a.cuda_module.check_status()
    b.cuda_module.check_status()


def test_default_prune_mask_is_average_pruning_weight():
    sc = _scene()
    rt = _tracer(sc)
    for i in range(2):
        _train_step(rt, i)
    torch.cuda.synchronize()
    g = rt.cuda_module.get_gaussians()
    avg = g.pruning_weight.squeeze(1) / g.pruning_counter.squeeze(1).clamp(min=1)
    thr = float(avg[avg > 0].median())
    rt.cfg.pruning_min_weight = thr
    expect = avg >= thr
    means = g.mean.detach()[expect].clone()
    rt.prune(2)
    assert g.count == int(expect.sum()) and 0 < g.count < sc.mean.shape[0]
    assert torch.equal(g.mean.detach(), means)


def test_cadence_rebuild_and_refit_give_the_same_images():
    """A tracer that rebuilds its BVH every iteration and one that only refits trace the same hit
    sets, so every forward image is identical while parameters agree."""
    sc = _scene()
    cfg_r = _cfg(rebuild_interval=1, pruning=False, scale_decay=0.999)
    cfg_n = _cfg(rebuild_interval=0, pruning=False, scale_decay=0.999)
    r, f = _tracer(sc, cfg_r), _tracer(sc, cfg_n)
    cr, cn = TrainCadence(cfg_r), TrainCadence(cfg_n)
    gr, gf = r.cuda_module.get_gaussians(), f.cuda_module.get_gaussians()
    for it in range(1, 4):
        # same parameters in both before each forward (backward atomics may differ in the last bits)
        with torch.no_grad():
            for k in _PARAMS:
                getattr(gf, k).copy_(getattr(gr, k))
        f.cuda_module.update_bvh()
        cr.before_iteration(r, it)
        cn.before_iteration(f, it)
        ir, i_f = _train_step(r, it), _train_step(f, it)
        assert torch.equal(ir, i_f), it
        assert cr.after_step(r, it).rebuilt and not cn.after_step(f, it).rebuilt
    torch.cuda.synchronize()
    r.cuda_module.check_status()
    f.cuda_module.check_status()


def test_safetensors_round_trip(tmp_path):
    sc = _scene()
    a = _tracer(sc)
    _train_step(a, 0)
    torch.cuda.synchronize()
    path = a.save_safetensors(str(tmp_path), 1)
    assert path.endswith("gaussians_00001.safetensors")
    b = Raytracer.from_safetensors(_cfg(), path, W, H)
    ga, gb = a.cuda_module.get_gaussians(), b.cuda_module.get_gaussians()
    for k in ("mean", "rotation", "scale", "opacity", "sh_coeffs_dc", "sh_coeffs_rest", "current_sh_degree"):
        assert torch.equal(getattr(ga, k).detach(), getattr(gb, k).detach()), k
    a.cuda_module.rebuild_bvh()
    with torch.no_grad():
        ia, ib = a(_cam(2)), b(_cam(2))
    assert torch.equal(ia, ib)
    # the reference's inference mode keeps SH in fp16
    c = Raytracer.from_safetensors(_cfg(), path, W, H, inference_only=True)
    assert c.cuda_module.get_gaussians().sh_coeffs_rest.dtype == torch.float16
    with torch.no_grad():
        ic = c(_cam(2))
    assert float((ic - ia).abs().max()) < 5e-3
