"""Per-iteration training cadence around the ray tracer (reference: train.py:217-219, 262-287).

    cadence = TrainCadence(cfg)
    for iteration in range(1, iterations + 1):
        cadence.before_iteration(raytracer, iteration)     # SH degree increments
        render = raytracer(camera); raytracer.backward(loss); raytracer.step()
        cadence.after_step(raytracer, iteration)           # scale decay, pruning, full rebuilds

Order and conditions follow train.py: after Raytracer.step() (pruning statistics, Adam, BVH
refit) the log-scales decay by log(scale_decay); at pruning_from_iter and every pruning_interval
after it the Gaussians whose average pruning weight is below pruning_min_weight are removed with
their Adam moments (Raytracer.prune); a pruned tracer and every rebuild_interval-th iteration get a
full BVH rebuild instead of the per-step refit.  As in the reference, the refit inside step() runs
before the decay, so the geometry the next forward traces lags the parameters by one decay.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

from .config import RaytracerConfig


@dataclass
class CadenceEvents:
    pruned: int = 0       # Gaussians removed at this iteration
    rebuilt: bool = False  # full BVH rebuild at this iteration


class TrainCadence:
    def __init__(self, cfg: RaytracerConfig):
        self.cfg = cfg

    def before_iteration(self, raytracer, iteration: int):
        """train.py:217-219: raise the SH degree every sh_increment_interval iterations."""
        if self.cfg.sh and self.cfg.sh_increment_interval > 0 and iteration % self.cfg.sh_increment_interval == 0:
            raytracer.cuda_module.get_gaussians().increment_sh_degree()

    @torch.no_grad()
    def after_step(self, raytracer, iteration: int) -> CadenceEvents:
        """train.py:265-287, after Raytracer.step()."""
        cfg = self.cfg
        ev = CadenceEvents()
        g = raytracer.cuda_module.get_gaussians()
        if cfg.scale_decay < 1.0:
            g.scale.add_(math.log(cfg.scale_decay))
        needs_rebuild = False
        if cfg.pruning and iteration >= cfg.pruning_from_iter and cfg.pruning_interval > 0 \
                and iteration % cfg.pruning_interval == 0:
            before = g.count
            raytracer.prune(iteration)
            ev.pruned = before - g.count
            needs_rebuild = True
        if cfg.rebuild_interval > 0 and iteration % cfg.rebuild_interval == 0:
            needs_rebuild = True
        if needs_rebuild:
            raytracer.cuda_module.rebuild_bvh()
            ev.rebuilt = True
        return ev
