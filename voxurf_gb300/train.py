"""The fused training step of the Voxurf fine stage (run.py:599-659).

One step = model forward on a ray batch, the run.py loss (photometric on the
k-branch, 0.5 x photometric on rgbnet, entropy of the last ray's
transmittance), the hand-written backward, then one sweep per grid that
applies the total-variation gradient (run.py:641-658 ->
Voxurf.*_total_variation_add_grad, weight / N_rays) together with the Adam
update, and one Adam launch per MLP tensor.
"""
from __future__ import annotations

import torch
import torch.nn.functional as F

from .utils import Adam


def fine_loss(ret, target, weight_main=1.0, weight_entropy_last=0.001, weight_rgb0=0.5):
    """run.py:604-636 with the fine dtu_e2e weights (configs/dtu_e2e/fine.py:104-105
    and the surf_train default weight_entropy_last, default_fine_s.py:63)."""
    loss = weight_main * F.mse_loss(ret["rgb_marched"], target)
    if weight_entropy_last > 0:
        # run.py:608: [..., -1] of the 1-D alphainv_cum selects the last ray
        pout = ret["alphainv_cum"][..., -1].clamp(1e-6, 1 - 1e-6)
        loss = loss + weight_entropy_last * (-(pout * torch.log(pout) + (1 - pout) * torch.log(1 - pout)).mean())
    if weight_rgb0 > 0 and "rgb_marched0" in ret:
        loss = loss + F.mse_loss(ret["rgb_marched0"], target) * weight_rgb0
    return loss


def eikonal_loss(gradient: torch.Tensor) -> torch.Tensor:
    """mean((|grad| - 1)^2) over the shaded samples' finite-difference SDF
    gradient (ret['gradient'], the d = 1 probes of voxurf_fine.py:524-526)."""
    return ((gradient.float().norm(dim=-1) - 1.0) ** 2).mean()


class FineTrainer:
    """Owns the optimizer of a Voxurf model and runs fused steps (the fine
    model; the coarse model too, which has no k_rgbnet group and no
    rgb_marched0 term).

    lr_* are the per-group learning rates (utils.create_optimizer_or_freeze_model
    groups sdf / k0 / rgbnet / k_rgbnet, and lr_bg for the maskless model's
    bg_density / bg_k0 / bg_rgbnet); tv_sdf / tv_k0 are the weights
    given to *_total_variation_add_grad before the division by the batch
    size (run.py:647-655); tv_dense mirrors `global_step < tv_dense_before`.
    ori_tv=True takes the TV terms as losses instead (run.py:617-626, the
    coarse configs): weight_tv_density x density_total_variation(sdf_tv)
    and weight_tv_k0 x k0_total_variation(), with no add-grad sweeps.
    """

    def __init__(self, model, lr_sdf=1e-3, lr_k0=1e-3, lr_rgbnet=1e-3, lr_k_rgbnet=1e-3, tv_sdf=1e-4, tv_k0=1e-4,
                 tv_dense=True, n_rays=8192, loss_weights=(1.0, 0.001, 0.5), weight_tv_density=0.0,
                 smooth_grad_tv=0.0, weight_eikonal=0.0, graphed=False, lr_bg=1e-3, ori_tv=False, sdf_tv=0.0,
                 weight_tv_k0=0.0):
        self.model = model
        self.n_rays = n_rays
        # graphed=True: steps replay CUDA graphs on static buffers
        # (fused_step.GraphedFineStep); same kernels, same results
        self.graphed = graphed
        self._engine = None
        # run.py:617-622: loss += weight_tv_density * density_total_variation(smooth_grad_tv=...)
        self.weight_tv_density, self.smooth_grad_tv = weight_tv_density, smooth_grad_tv
        self.ori_tv, self.sdf_tv, self.weight_tv_k0 = bool(ori_tv), sdf_tv, weight_tv_k0
        if self.ori_tv:   # run.py:642: the add-grad sweeps run only without ori_tv
            tv_sdf = tv_k0 = 0.0
        # eikonal term mean((|grad| - 1)^2) on the shaded samples' FD gradient
        # (no counterpart in the reference loss; used by the differentiation workload)
        self.weight_eikonal = weight_eikonal
        scale = float(model.world_size.max()) / 128  # voxurf_fine.py:404, 408
        shadow = None
        if model.precision == "bf16":
            shadow = model._k0_shadow if model._k0_shadow is not None else model.refresh_k0_shadow()
        groups = [
            {"params": [model.sdf.grid], "lr": lr_sdf, "name": "sdf", "tv_weight": tv_sdf / n_rays * scale,
             "tv_dense": tv_dense},
            {"params": [model.k0.grid], "lr": lr_k0, "name": "k0", "tv_weight": tv_k0 / n_rays * scale,
             "tv_dense": tv_dense, "shadow": shadow},
            {"params": list(model.rgbnet.parameters()), "lr": lr_rgbnet, "name": "rgbnet"},
        ]
        if getattr(model, "k_rgbnet", None) is not None:   # the coarse model has no k-branch
            groups.append({"params": list(model.k_rgbnet.parameters()), "lr": lr_k_rgbnet, "name": "k_rgbnet"})
        # the maskless model's background (its own groups in
        # create_optimizer_or_freeze_model: bg_density, bg_k0, bg_rgbnet)
        for name in ("bg_density", "bg_k0"):
            g = getattr(model, name, None)
            if g is not None and g.grid.numel() > 0:
                groups.append({"params": [g.grid], "lr": lr_bg, "name": name})
        if getattr(model, "bg_rgbnet", None) is not None:
            groups.append({"params": list(model.bg_rgbnet.parameters()), "lr": lr_bg, "name": "bg_rgbnet"})
        self.optimizer = Adam(groups, betas=(0.9, 0.99))
        self.loss_weights = loss_weights
        self.global_step = 0
        self.render_kwargs = None

    def step(self, rays_o, rays_d, viewdirs, target, render_kwargs, global_step=None):
        """One training step; returns (loss, ret) -- in graphed mode ret is
        {"S2": shaded rows} and the loss tensor lives until the next step."""
        if self.graphed:
            from .fused_step import GraphedFineStep

            if self._engine is None or self._engine.rk != dict(render_kwargs):
                self._engine = GraphedFineStep(self, render_kwargs)
            loss, S2 = self._engine.step(rays_o, rays_d, viewdirs, target, global_step)
            return loss, {"S2": S2}
        if global_step is None:
            self.global_step += 1
            global_step = self.global_step
        ret = self.model(rays_o, rays_d, viewdirs, global_step=global_step, **render_kwargs)
        loss = fine_loss(ret, target, *self.loss_weights)
        if self.weight_tv_density > 0 and self.smooth_grad_tv > 0:
            loss = loss + self.weight_tv_density * self.model.density_total_variation(
                smooth_grad_tv=self.smooth_grad_tv)
        if self.weight_tv_density > 0 and self.ori_tv:
            if self.sdf_tv > 0:
                loss = loss + self.weight_tv_density * self.model.density_total_variation(sdf_tv=self.sdf_tv)
            if self.weight_tv_k0 > 0:
                loss = loss + self.weight_tv_k0 * self.model.k0_total_variation()
        if self.weight_eikonal > 0 and ret["gradient"].numel() > 0:
            loss = loss + self.weight_eikonal * eikonal_loss(ret["gradient"])
        loss.backward()
        self.optimizer.step(zero_grad=True)
        return loss.detach(), ret
