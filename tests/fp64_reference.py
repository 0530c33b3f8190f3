"""Differentiable FP64 torch restatement of the reference's compositing rule (test infrastructure).

Follows cuda/shaders.cu:10-67 and cuda/forward_pass.cu:6-151 with the hits ordered by their fp16
distance like the reference's per-pixel list but with exact (unquantised) alpha: per (ray, Gaussian) the max-density point, the hit test (in front of the origin,
inside the clipped unit sphere), alpha = 0.9999 * sigmoid(opacity) * exp(-|x|^4 / 4) (exp_power 2),
hits composited front to back until T < t_threshold, full transmittance over all hits, and the
detached tail estimate of the skipped hits.  Used as the smooth function for finite differences and
as the FP64 gradient the hand-written backward is compared with.
"""
from __future__ import annotations

import math

import torch

MAX_ALPHA = 0.9999


def quat_to_rot(q):
    q = q / q.norm(dim=-1, keepdim=True)
    r, x, y, z = q.unbind(-1)
    return torch.stack([
        torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)], -1),
        torch.stack([2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)], -1),
        torch.stack([2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)], -1)], -2)


def render(ray_o, ray_d, mean, rotation, log_scale, logit_opacity, channels, alpha_threshold=0.01, t_threshold=0.03,
           bg=(0.0, 0.0, 0.0), chunk=4096, tail_channels=None):
    """ray_o, ray_d: [R,3]; returns [R,3] colours (float64, differentiable w.r.t. the parameters).

    tail_channels: colours for the truncated-tail estimate (default: channels).  The reference's
    backward treats that estimate as a constant (it replays composited hits only), so a finite
    difference of a colour parameter matches its gradient only with the tail's colours held fixed."""
    o = torch.sigmoid(logit_opacity.reshape(-1))
    sf = torch.where(o > alpha_threshold, (4.0 * torch.log(torch.clamp(o / alpha_threshold, min=1.0))) ** 0.25,
                     torch.zeros_like(o)).detach()
    R = quat_to_rot(rotation)                         # [N,3,3]
    inv_s = torch.exp(-log_scale)                     # [N,3]
    M = R.transpose(-1, -2) * inv_s[:, :, None]        # diag(1/s) R^T (world -> standard-deviation frame)
    bgt = torch.tensor(bg, dtype=ray_o.dtype, device=ray_o.device)
    outs = []
    for c0 in range(0, ray_o.shape[0], chunk):
        ro, rd = ray_o[c0:c0 + chunk], ray_d[c0:c0 + chunk]
        rel = ro[:, None, :] - mean[None, :, :]                      # [r,N,3]
        lo = torch.einsum("nij,rnj->rni", M, rel)                     # [r,N,3]
        ld = torch.einsum("nij,rj->rni", M, rd)
        nrm2 = (ld * ld).sum(-1)
        t = -(lo * ld).sum(-1) / nrm2                                 # world distance of the max-density point
        x = lo + t[..., None] * ld                                    # closest point, std-dev frame
        d = (x * x).sum(-1)
        hit = ((lo * ld).sum(-1) <= 0) & (d <= sf[None, :] ** 2) & (o[None, :] > alpha_threshold)
        alpha = MAX_ALPHA * o[None, :] * torch.exp(-0.25 * d * d)
        alpha = torch.where(hit, alpha, torch.zeros_like(alpha))
        # the reference orders hits by their fp16-rounded distance (cuda/core/per_pixel_linked_list.h:29);
        # equal keys keep gaussian-id order (stable sort), and only keys > znear (0) are composited
        t16 = t.detach().to(torch.float16).to(t.dtype)
        key = torch.where(hit, t16, torch.full_like(t16, math.inf))
        order = torch.argsort(key, dim=-1, stable=True)
        selectable = torch.gather(hit & (t16 > 0), 1, order)
        a_s = torch.gather(alpha, 1, order)
        c_s = channels[order]                                        # [r,N,3]
        ct_s = c_s if tail_channels is None else tail_channels[order]
        one_minus = 1.0 - a_s
        T_after = torch.cumprod(torch.where(selectable, one_minus, torch.ones_like(one_minus)), dim=-1)
        T_before = torch.cat([torch.ones_like(T_after[:, :1]), T_after[:, :-1]], dim=-1)
        comp = (T_before.detach() >= t_threshold) & selectable
        w = torch.where(comp, T_before * a_s, torch.zeros_like(a_s))
        C = (w[..., None] * c_s).sum(1)
        T_fin = torch.prod(torch.where(comp, one_minus, torch.ones_like(one_minus)), dim=-1)
        full_T = torch.prod(one_minus, dim=-1)
        skipped = (~comp) & (a_s.detach() > 0)
        sa = torch.where(skipped, a_s, torch.zeros_like(a_s)).detach()
        sc = (sa[..., None] * ct_s).sum(1).detach()
        sa_sum = sa.sum(-1)
        est = torch.where(sa_sum[:, None] > 0, sc / torch.clamp(sa_sum[:, None], min=1e-300), torch.zeros_like(sc))
        outs.append(C + (T_fin - full_T)[:, None] * est + bgt[None, :] * full_T[:, None])
    return torch.cat(outs, 0)


SH_C0 = 0.28209479177387814


def sh_colour(mean, cam_origin, sh_dc, sh_rest, degree):
    """[N,3] SH colours in FP64, differentiable w.r.t. mean, sh_dc [N,1,3] and sh_rest [N,K,3].

    Restates cuda/utils/sh.cu:11-78 and :224-247: the direction is the normalised mean - origin;
    complex terms v(l, m), m = 0..l, from v(0,0) = C0, the diagonal v(l,l) = -sqrt((2l+1)/(2l)) (x+iy)
    v(l-1,l-1), the sub-diagonal v(l,l-1) = sqrt(2l+1) z v(l-1,l-1) and the three-term recurrence
    v(l,m) = a z v(l-1,m) + b v(l-2,m); per degree the basis is sqrt2 Im v(l,m) for m = l..1, Re v(l,0),
    sqrt2 Re v(l,m) for m = 1..l; colour = max(C0 dc + sum basis * rest + 0.5, 0)."""
    d = mean - cam_origin
    d = d / torch.sqrt(torch.clamp((d * d).sum(-1, keepdim=True), min=1e-20))
    x, y, z = d.unbind(-1)
    vals = {(0, 0): (torch.full_like(x, SH_C0), torch.zeros_like(x))}
    for l in range(1, degree + 1):
        pr, pi = vals[(l - 1, l - 1)]
        s = -math.sqrt((2 * l + 1) / (2 * l))
        vals[(l, l)] = (s * (x * pr - y * pi), s * (x * pi + y * pr))
        t = math.sqrt(2 * l + 1)
        vals[(l, l - 1)] = (t * z * pr, t * z * pi)
        for m in range(l - 2, -1, -1):
            den = l * l - m * m
            a = math.sqrt((4 * l * l - 1) / den)
            b = -math.sqrt(((2 * l + 1) * ((l - 1) ** 2 - m * m)) / ((2 * l - 3) * den))
            r1, i1 = vals[(l - 1, m)]
            r2, i2 = vals[(l - 2, m)]
            vals[(l, m)] = (a * z * r1 + b * r2, a * z * i1 + b * i2)
    basis = []
    for l in range(1, degree + 1):
        basis += [math.sqrt(2.0) * vals[(l, m)][1] for m in range(l, 0, -1)]
        basis.append(vals[(l, 0)][0])
        basis += [math.sqrt(2.0) * vals[(l, m)][0] for m in range(1, l + 1)]
    col = SH_C0 * sh_dc[:, 0, :] + 0.5
    for k, bk in enumerate(basis):
        col = col + bk[:, None] * sh_rest[:, k, :]
    return torch.clamp(col, min=0.0)
