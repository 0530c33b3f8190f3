"""Generate the golden fixtures that pin the CPU oracle to the reference.

Run in a checkout where the reference source tree is available (read-only):

    python tests/golden/make_golden.py /path/to/gray-reference

It writes, next to this file:

* reference_tests.npz -- the four scenes of the reference's own tests
  (tests/test_single_gaussian.py:9-90 with alpha_threshold in {0.01, 0.3} and
  tests/test_multiple_gaussians.py:10-140 with t_threshold in {0.0, 0.5}): parameters,
  camera rays (restated from cuda/core/camera.h:17-36 in float32), the target image
  tests/data/target_1.png decoded as float32, and
    - ``ref64_*``: image and parameter gradients of the reference tests' FP64 compositing
      loops (restated here; rotation/scale matrices come from the reference's own
      tests/utils.py build_scaling_rotation, imported from the reference tree), with the
      upstream gradient of their L1 loss;
    - ``rule64_*``: the reference CUDA rule (fp16 distance/alpha keys, 32-slot passes,
      all-hit transmittance and tail estimate, cuda/forward_pass.cu:6-151) evaluated in FP64.
* sh_adam.npz -- SH colours and gradients from an FP64 restatement of the reference's
  complex recurrence (cuda/utils/sh.cu:11-287), and one Adam step restated from
  cuda/opt/adam.cu:13-83 in FP64.

Nothing in the test suite reads the reference tree; only this generator does.
"""
from __future__ import annotations

import importlib.util
import math
import os
import struct
import sys
import zlib

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
MAX_ALPHA = 0.9999
NUM_PIXELS = 32


def decode_png_rgb8(path: str) -> np.ndarray:
    """Minimal PNG reader for 8-bit RGB, non-interlaced images (the target fixture)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        ln = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + ln]
        if typ == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
            assert depth == 8 and ctype == 2 and interlace == 0
        elif typ == b"IDAT":
            idat += body
        pos += 12 + ln
    raw = zlib.decompress(idat)
    bpp, stride = 3, w * 3
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        cur = np.zeros(stride, np.int32)
        for x in range(stride):
            a = cur[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if f == 0:
                p = 0
            elif f == 1:
                p = a
            elif f == 2:
                p = b
            elif f == 3:
                p = (a + b) // 2
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            cur[x] = (line[x] + p) & 0xFF
        out[y] = cur
        prev = cur
    # [3, H, W] in [0, 1] like torchvision's to_tensor
    return (out.reshape(h, w, 3).astype(np.float32) / 255.0).transpose(2, 0, 1).copy()


def camera_rays_f32(width, height, fov_y, origin, c2w):
    """cuda/core/camera.h:17-36 in float32 (w2c rows are c2w columns)."""
    f = np.float32
    view_size = f(np.tan(f(fov_y) / f(2)))
    aspect = f(width) / f(height)
    o = np.zeros((height * width, 3), np.float32)
    d = np.zeros((height * width, 3), np.float32)
    c2w = np.asarray(c2w, np.float32)
    for j in range(height):
        for i in range(width):
            y = view_size * (f(1) - f(2) * (f(j) + f(0.5)) / f(height))
            x = aspect * view_size * (f(2) * (f(i) + f(0.5)) / f(width) - f(1))
            v = c2w[:, 0] * x + c2w[:, 1] * y - c2w[:, 2]
            inv = f(1) / np.sqrt(f(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]))
            d[j * width + i] = v * inv
            o[j * width + i] = origin
    return o, d


def load_reference_utils(ref_root):
    spec = importlib.util.spec_from_file_location("ref_test_utils", os.path.join(ref_root, "tests", "utils.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def ref64_render(utils, mu, log_scale, color, rot, logit_op, rays_o, rays_d, alpha_threshold, t_threshold, bg,
                 exp_power=2.0):
    """The FP64 compositing loop of the reference tests (single: test_single_gaussian.py:56-76,
    multiple: test_multiple_gaussians.py:78-125; the single case is the multiple rule with one
    Gaussian and a background)."""
    R, S = utils.build_scaling_rotation(log_scale.exp(), torch.nn.functional.normalize(rot, dim=-1))
    L2W = R @ S
    W2L = torch.linalg.inv(L2W)
    n = mu.shape[0]
    out = []
    for p in range(rays_o.shape[0]):
        ro, rd = rays_o[p], rays_d[p]
        ts = []
        for k in range(n):
            lo = W2L[k] @ (ro - mu[k])
            ldu = W2L[k] @ rd
            nrm = ldu.dot(ldu).sqrt()
            ld = ldu / nrm
            ts.append(-torch.dot(lo, ld) / nrm)
        order = torch.argsort(torch.stack(ts))
        T = torch.tensor(1.0, dtype=torch.float64)
        full_T = torch.tensor(1.0, dtype=torch.float64)
        pix = torch.zeros(3, dtype=torch.float64)
        rc = torch.zeros(3, dtype=torch.float64)
        ra = torch.zeros(1, dtype=torch.float64)
        for k in order:
            lo = W2L[k] @ (ro - mu[k])
            ldu = W2L[k] @ rd
            nrm = ldu.dot(ldu).sqrt()
            ld = ldu / nrm
            t = -torch.dot(lo, ld)
            hit = lo + t * ld
            gv = torch.exp(-(hit.dot(hit) ** exp_power) / (2.0 * exp_power))
            alpha = torch.sigmoid(logit_op[k, 0]) * gv * MAX_ALPHA
            if alpha < alpha_threshold:
                alpha = torch.tensor(0.0, dtype=torch.float64)
            if T > t_threshold:
                pix = pix + color[k] * T * alpha
                T = T * (1.0 - alpha)
            else:
                alpha = alpha.detach()
                rc = rc + color[k].detach() * alpha
                ra = ra + alpha
            full_T = full_T * (1.0 - alpha)
        est = rc / ra if ra > 0.0 else torch.zeros(3, dtype=torch.float64)
        pix = pix + est * (T - full_T) + bg * full_T
        out.append(pix)
    return torch.stack(out)


def rule64_render(mu, log_scale, color, rot, logit_op, rays_o, rays_d, alpha_threshold, t_threshold, bg,
                  exp_power=2.0, slots=32, max_passes=99, znear=0.0, zfar=99999.9):
    """cuda/shaders.cu:10-67 + cuda/forward_pass.cu:6-151 evaluated in FP64, with the fp16
    rounding of distances and alphas that the reference stores in its per-pixel list."""
    mu, log_scale, color, rot, logit_op = (np.asarray(a, np.float64) for a in (mu, log_scale, color, rot, logit_op))
    n = mu.shape[0]
    q = rot / np.linalg.norm(rot, axis=1, keepdims=True)
    r, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    Rm = np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)], -1),
        np.stack([2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)], -1),
        np.stack([2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)], -1)], 1)
    op = 1.0 / (1.0 + np.exp(-logit_op[:, 0]))
    L = np.log(np.maximum(op / alpha_threshold, 1e-300))
    sf = np.where(op > alpha_threshold, (2 * exp_power * L) ** (1.0 / (2 * exp_power)), 0.0)
    s = np.exp(log_scale) * sf[:, None]
    rgb = np.zeros((rays_o.shape[0], 3))
    for p in range(rays_o.shape[0]):
        ro, rd = rays_o[p].astype(np.float64), rays_d[p].astype(np.float64)
        hits = []
        full_T = 1.0
        for k in range(n):
            if op[k] <= alpha_threshold or sf[k] <= 0:
                continue
            M = (Rm[k].T) / s[k][:, None]
            lo = M @ (ro - mu[k])
            ld = M @ rd
            if lo @ ld > 0:
                continue
            nrm = np.linalg.norm(ld)
            dn = ld / nrm
            t = -(lo @ dn)
            u = lo + t * dn
            if u @ u > 1.0:
                continue
            xx = u * sf[k]
            d = xx @ xx
            a = MAX_ALPHA * op[k] * math.exp(-(d ** exp_power) / (2 * exp_power))
            full_T *= 1.0 - a
            hits.append((float(np.float16(t / nrm)), k, float(np.float16(a))))
        sa = sum(h[2] for h in hits)
        sc = sum(h[2] * color[h[1]] for h in hits) if hits else np.zeros(3)
        T, C = 1.0, np.zeros(3)
        sel = sorted([h for h in hits if h[0] > znear], key=lambda h: (h[0], h[1]))
        npass, used, tmin_sel, last_d = 0, 0, znear, znear
        for (d16, k, a16) in sel:
            if not d16 > tmin_sel:
                continue
            if used == slots:
                npass += 1
                if npass >= max_passes:
                    break
                tmin_sel = last_d
                if not tmin_sel < zfar:
                    break
                used = 0
                if not d16 > tmin_sel:
                    continue
            used += 1
            last_d = d16
            if not d16 < zfar:
                break
            sa -= a16
            sc = sc - a16 * color[k]
            C = C + color[k] * T * a16
            T = T * (1.0 - a16)
            if T < t_threshold:
                break
        est = sc / sa if sa > 1e-12 else np.zeros(3)
        rgb[p] = C + (T - full_T) * est + np.asarray(bg) * full_T
    return rgb


# ---------------------------------------------------------------------------------------------
# SH: the reference's complex recurrence (cuda/utils/sh.cu:11-78) restated in FP64 torch
# ---------------------------------------------------------------------------------------------
def sh_basis_recurrence(dirs: torch.Tensor, degree: int) -> torch.Tensor:
    """Real SH basis (without the DC term) in the reference's per-degree order:
    m = l..1 -> sqrt2 Im, m = 0 -> Re, m = 1..l -> sqrt2 Re of the complex recurrence."""
    C0 = 0.28209479177387814
    x, y, z = dirs[:, 0], dirs[:, 1], dirs[:, 2]
    idx = lambda l, m: l * (l + 1) // 2 + m
    re = {idx(0, 0): torch.full_like(x, C0)}
    im = {idx(0, 0): torch.zeros_like(x)}
    for l in range(1, degree + 1):
        pd = idx(l - 1, l - 1)
        sc = -math.sqrt((2 * l + 1) / (2 * l))
        re[idx(l, l)] = sc * (x * re[pd] - y * im[pd])
        im[idx(l, l)] = sc * (x * im[pd] + y * re[pd])
        ss = math.sqrt(2 * l + 1)
        re[idx(l, l - 1)] = re[pd] * ss * z
        im[idx(l, l - 1)] = im[pd] * ss * z
        for m in range(l - 2, -1, -1):
            den = l * l - m * m
            a = math.sqrt((4 * l * l - 1) / den)
            b = -math.sqrt(((2 * l + 1) * ((l - 1) ** 2 - m * m)) / ((2 * l - 3) * den))
            p1, p2 = idx(l - 1, m), idx(l - 2, m)
            re[idx(l, m)] = re[p1] * a * z + re[p2] * b
            im[idx(l, m)] = im[p1] * a * z + im[p2] * b
    cols = []
    s2 = math.sqrt(2.0)
    for l in range(1, degree + 1):
        for m in range(l, 0, -1):
            cols.append(s2 * im[idx(l, m)])
        cols.append(re[idx(l, 0)])
        for m in range(1, l + 1):
            cols.append(s2 * re[idx(l, m)])
    return torch.stack(cols, 1) if cols else torch.zeros(dirs.shape[0], 0, dtype=dirs.dtype)


def sh_colour64(mean, cam, dc, rest, degree):
    v = mean - cam
    dirs = v / torch.sqrt(torch.clamp((v * v).sum(1, keepdim=True), min=1e-20))
    col = 0.28209479177387814 * dc[:, 0, :]
    if degree > 0:
        b = sh_basis_recurrence(dirs, degree)
        col = col + (b[:, :, None] * rest[:, : b.shape[1], :]).sum(1)
    return torch.clamp(col + 0.5, min=0.0)


def adam64(p, m, v, g, lr, b1, b2, eps, step):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** (step + 1.0))
    vh = v / (1 - b2 ** (step + 1.0))
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def main(ref_root: str):
    torch.set_default_dtype(torch.float64)
    utils = load_reference_utils(ref_root)
    target = decode_png_rgb8(os.path.join(ref_root, "tests", "data", "target_1.png"))
    origin = np.array([0.0, 0.0, 1.0], np.float32)
    # mock camera of the reference tests: R = -I, then the pose convention of
    # gray/camera.py:109-119 (c2w = -R with column 0 negated)
    R = -np.eye(3, dtype=np.float32)
    c2w = -R
    c2w[:, 0] *= -1
    fov_y = 1.5
    rays_o, rays_d = camera_rays_f32(NUM_PIXELS, NUM_PIXELS, fov_y, origin, c2w)

    cases = {}
    single = dict(mu=[[-0.05, -0.05, 0.0]], scale=[[0.1, 0.3, 0.3]], color=[[1.0, 0.0, 0.0]],
                  rot=[[-0.5, 0.0, 0.0, 1.0]], opacity=[[0.5]], bg=[0.1, 0.1, 0.1], t_threshold=0.03)
    multi = dict(mu=[[0.05, 0.05, -0.25], [-0.05, -0.05, 0.25], [0.0, 0.0, 0.0]],
                 scale=[[1.0, 0.2, 0.1], [0.1, 0.3, 0.3], [0.4, 0.4, 0.4]],
                 color=[[0.0, 0.0, 1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]],
                 rot=[[1.0, 0.0, 0.0, 1.0]] * 3, opacity=[[0.5], [0.7], [0.7]], bg=[0.0, 0.0, 0.0])
    for a_thr in (0.01, 0.3):
        cases[f"single_a{a_thr}"] = dict(single, alpha_threshold=a_thr)
    for t_thr in (0.0, 0.5):
        cases[f"multi_t{t_thr}"] = dict(multi, alpha_threshold=0.01, t_threshold=t_thr)

    out = dict(rays_o=rays_o, rays_d=rays_d, target=target, fov_y=np.float32(fov_y), origin=origin,
               c2w=c2w.astype(np.float32), names=np.array(list(cases.keys())))
    t64 = torch.from_numpy(target.astype(np.float64))
    ro64 = torch.from_numpy(rays_o.astype(np.float64))
    rd64 = torch.from_numpy(rays_d.astype(np.float64))
    for name, c in cases.items():
        mu = torch.tensor(c["mu"]).requires_grad_()
        log_scale = torch.tensor(c["scale"]).log().requires_grad_()
        color = torch.tensor(c["color"]).requires_grad_()
        rot = torch.tensor(c["rot"]).requires_grad_()
        logit_op = torch.tensor(c["opacity"]).logit().requires_grad_()
        bg = torch.tensor(c["bg"])
        img = ref64_render(utils, mu, log_scale, color, rot, logit_op, ro64, rd64, c["alpha_threshold"],
                           c["t_threshold"], bg)
        img_chw = img.reshape(NUM_PIXELS, NUM_PIXELS, 3).permute(2, 0, 1)
        loss = torch.nn.functional.l1_loss(img_chw, t64)
        loss.backward()
        grad_out = (torch.sign(img_chw - t64) / img_chw.numel()).detach().permute(1, 2, 0).reshape(-1, 3)
        rule = rule64_render(mu.detach().numpy(), log_scale.detach().numpy(), color.detach().numpy(),
                             rot.detach().numpy(), logit_op.detach().numpy(), rays_o, rays_d, c["alpha_threshold"],
                             c["t_threshold"], c["bg"])
        p = name + "_"
        out[p + "mean"] = np.float32(mu.detach().numpy())
        out[p + "log_scale"] = np.float32(log_scale.detach().numpy())
        out[p + "color"] = np.float32(color.detach().numpy())
        out[p + "rotation"] = np.float32(rot.detach().numpy())
        out[p + "logit_opacity"] = np.float32(logit_op.detach().numpy())
        out[p + "bg"] = np.float32(c["bg"])
        out[p + "alpha_threshold"] = np.float32(c["alpha_threshold"])
        out[p + "t_threshold"] = np.float32(c["t_threshold"])
        out[p + "ref64_rgb"] = img.detach().numpy()
        out[p + "ref64_grad_out"] = grad_out.numpy().astype(np.float32)
        out[p + "ref64_grad_mean"] = mu.grad.numpy()
        out[p + "ref64_grad_log_scale"] = log_scale.grad.numpy()
        out[p + "ref64_grad_color"] = color.grad.numpy()
        out[p + "ref64_grad_rotation"] = rot.grad.numpy()
        out[p + "ref64_grad_logit_opacity"] = logit_op.grad.numpy()
        out[p + "rule64_rgb"] = rule
        print(name, "ref64 vs rule64 max |diff|", float(np.abs(img.detach().numpy() - rule).max()))
    np.savez_compressed(os.path.join(HERE, "reference_tests.npz"), **out)

    # ---- SH and Adam ----
    rng = np.random.default_rng(1234)
    n = 257
    mean = rng.uniform(-2, 2, (n, 3))
    cam = np.array([0.3, -4.0, 1.5])
    dc = rng.normal(0.5, 0.2, (n, 1, 3))
    rest = rng.normal(0.0, 0.05, (n, 15, 3))
    sh = dict(mean=np.float32(mean), cam=np.float32(cam), dc=np.float32(dc), rest=np.float32(rest))
    for deg in range(4):
        tm = torch.tensor(np.float32(mean), dtype=torch.float64, requires_grad=True)
        tdc = torch.tensor(np.float32(dc), dtype=torch.float64, requires_grad=True)
        trest = torch.tensor(np.float32(rest), dtype=torch.float64, requires_grad=True)
        col = sh_colour64(tm, torch.tensor(np.float32(cam), dtype=torch.float64), tdc, trest, deg)
        gcol = torch.tensor(rng.normal(0, 1, (n, 3)))
        (col * gcol).sum().backward()
        sh[f"deg{deg}_colour"] = col.detach().numpy()
        sh[f"deg{deg}_grad_colour"] = np.float32(gcol.numpy())
        sh[f"deg{deg}_grad_mean"] = tm.grad.numpy() if tm.grad is not None else np.zeros((n, 3))
        sh[f"deg{deg}_grad_dc"] = tdc.grad.numpy()
        sh[f"deg{deg}_grad_rest"] = trest.grad.numpy() if trest.grad is not None else np.zeros((n, 15, 3))
    m = 64
    ad = dict(p=np.float32(rng.normal(0, 1, m)), m=np.float32(rng.normal(0, 0.1, m)),
              v=np.float32(np.abs(rng.normal(0, 0.01, m))), g=np.float32(rng.normal(0, 0.1, m)))
    for step in (1, 7, 1000):
        # hyper-parameters as the float32 values the reference reads from its holder tensors
        f = lambda x: float(np.float32(x))
        p2, m2, v2 = adam64(ad["p"].astype(np.float64), ad["m"].astype(np.float64), ad["v"].astype(np.float64),
                            ad["g"].astype(np.float64), f(0.01), f(0.9), f(0.999), f(1e-15), step)
        sh[f"adam_step{step}_p"] = p2
        sh[f"adam_step{step}_m"] = m2
        sh[f"adam_step{step}_v"] = v2
    for k, v in ad.items():
        sh["adam_in_" + k] = v
    np.savez_compressed(os.path.join(HERE, "sh_adam.npz"), **sh)
    print("wrote", os.path.join(HERE, "reference_tests.npz"), os.path.join(HERE, "sh_adam.npz"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of a graphdeco-inria/gray checkout>")
    main(sys.argv[1])
