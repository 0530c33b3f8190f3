"""RaytracerConfig: the reference's configuration dataclass (gray/config.py:29-146), same field
names and defaults, as a plain dataclass (the reference parses it with tyro; nothing on the ray
tracing path depends on tyro)."""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional


@dataclass
class RaytracerConfig:
    render_depth: bool = False
    preview_train_image_name: Optional[str] = None
    preview_test_image_name: Optional[str] = None
    preview_iters: List[int] = field(default_factory=lambda: [1, 1_000, 2_500, 7_500, 15_000])
    test_iters: List[int] = field(default_factory=lambda: [7_500, 15_000])
    save_iters: List[int] = field(default_factory=lambda: [7_500, 15_000])
    log_loss_interval: int = 1000
    log_stats_interval: int = 1000
    viewer: bool = False
    yes: bool = False

    # memory use: the backward hit list holds ppll_backward_size 32-bit words; the forward
    # list of the reference is not materialised (ppll_forward_size is accepted and unused)
    ppll_forward_size: int = 300_000_000
    ppll_backward_size: int = 120_000_000

    bg_color: List[float] = field(default_factory=lambda: [0.0, 0.0, 0.0])

    exp_power: float = 2.0
    alpha_threshold: float = 0.01
    t_threshold: float = 0.03

    init_scale: float = 0.0005
    init_opacity: float = 0.1
    init_binning: bool = True
    init_bin_size: float = 0.0015

    half_res_iters: int = 0
    half_res_batch_size: int = 1

    lambda_ssim: float = 0.2

    iterations: int = 15_000
    lr_mean_init: float = 0.00016
    lr_mean_final: float = 0.0000016
    lr_channels: float = 0.0025
    lr_opacity_init: float = 0.02
    lr_opacity_final: float = 0.005
    lr_scale_init: float = 0.02
    lr_scale_final: float = 0.005
    lr_rotation_init: float = 0.004
    lr_rotation_final: float = 0.001
    lr_sh_dc_init: float = 0.04
    lr_sh_dc_final: float = 0.0025
    lr_sh_rest: float = 0.000625
    tiling: int = 1
    beta_1: float = 0.9
    beta_2: float = 0.999
    epsilon: float = 1e-15
    sh_update_laziness: int = 1
    lr_schedule_delay_mult: float = 0.01

    pruning: bool = True
    pruning_interval: int = 500
    pruning_from_iter: int = 500
    pruning_min_weight: float = 1e-7

    rebuild_interval: int = 500
    scale_decay: float = 0.999875

    sh: bool = True
    sh_init_degree: int = 0
    sh_max_degree: int = 3
    sh_increment_interval: int = 1000

    exposure_comp_enabled: bool = False
    exposure_comp_lr_init: float = 0.001
    exposure_comp_lr_final: float = 0.0001
    exposure_comp_lr_delay_mult: float = 0.001
    exposure_comp_lr_max_steps: int = 5000

    pre_mlp: bool = False
    pre_mlp_feature_size: int = 8
    pre_mlp_width: int = 128
    pre_mlp_layers: int = 4
    pre_mlp_lr: float = 1e-3
    pre_mlp_feature_lr: float = 3e-2
    pre_mlp_freq_bands: Optional[int] = 4
    post_mlp: bool = False
    post_mlp_width: int = 128
    post_mlp_layers: int = 5
    post_mlp_lr: float = 1e-3
    post_mlp_freq_bands: Optional[int] = 1
    tcnn: bool = False

    def __post_init__(self):
        if self.iterations not in self.save_iters:
            self.save_iters.append(self.iterations)
        if self.iterations not in self.test_iters:
            self.test_iters.append(self.iterations)
        if self.iterations not in self.preview_iters:
            self.preview_iters.append(self.iterations)
        assert self.sh_init_degree <= self.sh_max_degree
        assert 0 <= self.sh_max_degree <= 3
        if self.sh:
            assert not self.pre_mlp, "Spherical harmonics cannot be used with pre-MLP (choose either one)"
            assert not self.post_mlp, "Spherical harmonics cannot be used with post-MLP"
        if not self.sh:
            self.sh_max_degree = 0
        assert len(self.bg_color) == 3, "bg_color must contain exactly 3 channels"
