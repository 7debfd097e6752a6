"""ORACLE — test infrastructure / CPU baseline only (never imported by the
product).

Times the reference fine-stage training step on the host CPU: the oracle's
torch restatement of lib/voxurf_fine.py forward, the run.py loss, torch
autograd backward, the reference TV add-grad (C restatement of
total_variation_kernel.cu) and lib/utils.py Adam, in float32 with all host
threads.  Parameters are built with plain torch (no GPU code runs).
"""
from __future__ import annotations

import time

import numpy as np
import torch


def build_cpu_oracle(R: int, seed: int = 0, mask_voxels: float | None = 6.4, width: int = 192,
                     dtype=torch.float32):
    from voxurf_gb300 import configs, synthetic
    from voxurf_gb300.voxurf_fine import Voxurf

    from . import cref
    from .voxurf_oracle import OracleFine

    torch.manual_seed(seed)
    model = Voxurf(**configs.fine_model_kwargs(R, "fp32", width))  # parameter container, CPU only
    sdf = synthetic.make_sdf("sphere_torus", R, seed=seed)
    mask = None
    if mask_voxels is not None:
        mask = np.abs(sdf) < mask_voxels * 2.0 / R
        # _set_nonempty_mask (voxurf_fine.py:353-367): grid points are the mask
        # cells themselves, so the non-empty mask equals the mask grid
        sdf = np.where(mask, sdf, 1.0).astype(np.float32)
    with torch.no_grad():
        model.sdf.grid.data = torch.from_numpy(sdf)[None, None]
        k0 = synthetic.make_k0(R, 12, seed=seed + 1)
        model.k0.grid.data = k0.permute(3, 0, 1, 2)[None].contiguous(memory_format=torch.channels_last_3d)
    oracle = OracleFine(model, dtype=dtype)
    if mask is not None:
        scale = ((np.array(mask.shape, np.float32) - 1) / np.float32(2.0)).astype(np.float32)
        shift = (np.float32(1.0) * scale).astype(np.float32)
        oracle.mask = ("grid", torch.from_numpy(mask), torch.from_numpy(scale), torch.from_numpy(shift))
    return oracle, float(model.world_size.max())


def reference_step(oracle, opt, world_max, rays, rk, global_step, tv_weight=1e-4):
    from .voxurf_oracle import train_loss, tv_add_grad

    ro, rd, vd, tgt = rays
    ret = oracle(ro, rd, vd, global_step=global_step, **rk)
    loss = train_loss(ret, tgt)
    loss.backward()
    n = len(ro)
    tv_add_grad(oracle.sdf_grid, tv_weight / n, world_max, True)
    tv_add_grad(oracle.k0_grid, tv_weight / n, world_max, True)
    opt.step()
    for p in oracle.parameters():
        p.grad = None
    return float(loss.item())


def time_reference_steps(R: int, n_rays: int, warmup: int, steps: int, seed: int = 0):
    """Full reference training steps on the host CPU at the benchmark's own
    size (R^3 grids, n_rays rays per step, a fresh seeded batch per step):
    `warmup` untimed steps, then `steps` timed ones.  Returns the per-step
    wall times (s) and a one-line description of the sample."""
    from voxurf_gb300 import configs, synthetic

    from .voxurf_oracle import UtilsAdam

    oracle, world_max = build_cpu_oracle(R, seed=seed)
    opt = UtilsAdam([([oracle.sdf_grid], 1e-3), ([oracle.k0_grid], 1e-3), (list(oracle.rgbnet.parameters()), 1e-3),
                     (list(oracle.k_rgbnet.parameters()), 1e-3)], betas=(0.9, 0.99))
    rk = dict(configs.FINE_RENDER_KWARGS)
    total = warmup + steps
    o, d, v = synthetic.random_rays(n_rays * total, seed=seed + 1)
    t = configs.train_targets(n_rays * total, seed + 1)
    times = []
    for i in range(total):
        sl = slice(i * n_rays, (i + 1) * n_rays)
        rays = tuple(torch.from_numpy(np.ascontiguousarray(a[sl])) for a in (o, d, v, t))
        t0 = time.perf_counter()
        reference_step(oracle, opt, world_max, rays, rk, i + 1)
        if i >= warmup:
            times.append(time.perf_counter() - t0)
    sample = (f"{steps} full reference steps of {n_rays} rays (fwd+bwd+TV+Adam, FP32 torch on CPU, the {R}^3 "
              f"grids) after {warmup} warm-up: median {float(np.median(times)):.2f} s, "
              f"total {sum(times):.1f} s")
    return {"times": times, "sample": sample, "rays_per_s": n_rays * steps / sum(times)}
