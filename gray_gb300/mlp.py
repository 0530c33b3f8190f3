"""Post-processing MLP: the consumer of the ray tracer's per-pixel ray and depth outputs.

The reference's PostMLP (gray/mlp.py:143-215) maps each rendered pixel's colour, together with a
sinusoidal encoding of its view direction and hit position (gray/mlp.py:218-262), to the final
RGB with a small per-pixel network (1x1 convolutions, ReLU, bf16), trained by its own Adam step.
gray/raytracer.py:157-167 feeds it the framebuffer's ray directions and the hit points
origin + depth * direction (so it needs config.render_depth for meaningful depths, as there).
The per-pixel layers are plain matrix products over the pixels (cuBLAS through torch); the
tiny-cuda-nn variant of the reference (cfg.tcnn) is not provided.
"""
from __future__ import annotations

import torch
import torch.nn as nn


def positional_encoding_size(c: int, k: int) -> int:
    """Channels of positional_encoding for c input channels and k frequency bands (the input kept)."""
    return c if k == 0 else c + 2 * c * k


def positional_encoding(x: torch.Tensor, k: int) -> torch.Tensor:
    """[C, H, W] (or [N, C]) -> the input followed by sin and cos of each channel times 2^0 .. 2^(k-1),
    channel-major then frequency, sines before cosines."""
    if x.ndim not in (2, 3):
        raise ValueError(f"expected [N, C] or [C, H, W], got {tuple(x.shape)}")
    if k < 0:
        raise ValueError(f"k must be >= 0, got {k}")
    if k == 0:
        return x
    freqs = 2.0 ** torch.arange(k, device=x.device, dtype=x.dtype)
    if x.ndim == 3:
        c, h, w = x.shape
        scaled = (x.unsqueeze(1) * freqs.view(1, k, 1, 1)).reshape(c * k, h, w)
        return torch.cat([x, torch.sin(scaled), torch.cos(scaled)], dim=0)
    n, c = x.shape
    scaled = (x.unsqueeze(-1) * freqs).reshape(n, c * k)
    return torch.cat([x, torch.sin(scaled), torch.cos(scaled)], dim=1)


class PostMLP(nn.Module):
    def __init__(self, cfg, num_channels: int):
        super().__init__()
        if cfg.post_mlp_layers < 2:
            raise ValueError("the post-processing MLP needs at least 2 layers")
        self.cfg = cfg
        if cfg.post_mlp_freq_bands is None:
            cin = num_channels
        else:
            cin = num_channels + positional_encoding_size(6, cfg.post_mlp_freq_bands)
        width = cfg.post_mlp_width
        layers = [nn.Conv2d(cin, width, kernel_size=1), nn.ReLU()]
        for _ in range(cfg.post_mlp_layers - 2):
            layers += [nn.Conv2d(width, width, kernel_size=1), nn.ReLU(inplace=True)]
        layers.append(nn.Conv2d(width, 3, kernel_size=1))
        self.network = nn.Sequential(*layers).cuda().to(torch.bfloat16)
        for m in self.network:
            if isinstance(m, nn.Conv2d):
                nn.init.kaiming_normal_(m.weight, nonlinearity="relu")
                nn.init.zeros_(m.bias)
        self.optimizer = torch.optim.Adam(self.network.parameters(), lr=cfg.post_mlp_lr)

    def forward(self, x: torch.Tensor, view_direction: torch.Tensor, hit_position: torch.Tensor) -> torch.Tensor:
        """x: [C, H, W] rendered colour; view_direction, hit_position: [3, H, W]."""
        if self.cfg.post_mlp_freq_bands is None:
            x = x * 2 - 1
        else:
            enc = positional_encoding(torch.cat([view_direction, hit_position], dim=0), self.cfg.post_mlp_freq_bands)
            x = torch.cat([x * 2 - 1, enc], dim=0)
        return self.network(x.to(torch.bfloat16)).to(torch.float32).squeeze(-1)

    def step(self):
        self.optimizer.step()
        self.network.zero_grad()
