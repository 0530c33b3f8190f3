"""RaytracerConfig: the knobs of the reference's configuration dataclass (gray/config.py:29-146)
that the ray tracing path, its optimiser and its training cadence read, under the reference's
field names and defaults so that a reference config drops in.  Training-loop product features
(logging, previews, LR schedules, SSIM, half-resolution warm-up) are not on the path and have no
field here.  The post-processing MLP's knobs are kept (gray_gb300.mlp.PostMLP); the pre-MLP and
exposure-compensation switches are kept only so that a config asking for them is refused
(gray_gb300.Raytracer raises NotImplementedError)."""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional


@dataclass
class RaytracerConfig:
    render_depth: bool = False

    # memory use: the backward hit list holds ppll_backward_size 32-bit words; the forward
    # list of the reference is not materialised (ppll_forward_size is accepted and unused)
    ppll_forward_size: int = 300_000_000
    ppll_backward_size: int = 120_000_000

    bg_color: List[float] = field(default_factory=lambda: [0.0, 0.0, 0.0])

    exp_power: float = 2.0
    alpha_threshold: float = 0.01
    t_threshold: float = 0.03

    # initialisation from a point cloud (Raytracer.from_point_cloud)
    init_scale: float = 0.0005
    init_opacity: float = 0.1
    init_binning: bool = True
    init_bin_size: float = 0.0015

    # Adam: initial learning rates and moments (the reference's schedules start from these)
    lr_mean_init: float = 0.00016
    lr_channels: float = 0.0025
    lr_opacity_init: float = 0.02
    lr_scale_init: float = 0.02
    lr_rotation_init: float = 0.004
    lr_sh_dc_init: float = 0.04
    lr_sh_rest: float = 0.000625
    beta_1: float = 0.9
    beta_2: float = 0.999
    epsilon: float = 1e-15
    sh_update_laziness: int = 1

    # training cadence (gray_gb300.cadence.TrainCadence)
    pruning: bool = True
    pruning_interval: int = 500
    pruning_from_iter: int = 500
    pruning_min_weight: float = 1e-7
    rebuild_interval: int = 500
    scale_decay: float = 0.999875

    sh: bool = True
    sh_max_degree: int = 3
    sh_increment_interval: int = 1000

    # post-processing MLP on the ray / depth outputs (gray_gb300.mlp.PostMLP)
    post_mlp: bool = False
    post_mlp_width: int = 128
    post_mlp_layers: int = 5
    post_mlp_lr: float = 1e-3
    post_mlp_freq_bands: Optional[int] = 1

    # not on the path: refused when set
    exposure_comp_enabled: bool = False
    pre_mlp: bool = False

    def __post_init__(self):
        if not 0 <= self.sh_max_degree <= 3:
            raise ValueError(f"sh_max_degree must be in 0..3, got {self.sh_max_degree}")
        if self.sh and (self.pre_mlp or self.post_mlp):
            raise ValueError("spherical harmonics and the pre/post MLPs are exclusive")
        if not self.sh:
            self.sh_max_degree = 0
        if len(self.bg_color) != 3:
            raise ValueError(f"bg_color needs 3 channels, got {len(self.bg_color)}")
