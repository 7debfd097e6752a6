"""Workload definitions: model kwargs and synthetic scenes of the five
benchmark configurations (coarse 96^3, fine 256^3, gradient check 32^3,
render server 4 x 256^3, long rays 384^3).

Model hyper-parameters follow the reference's DTU configs
(configs/dtu_e2e/coarse.py:60-76 and configs/dtu_e2e/fine.py:136-165 on top
of configs/default_fine_s.py:107-138) except where the workload says
otherwise (grid size, smoothing, MLP width).
"""
from __future__ import annotations

import numpy as np
import torch

from . import synthetic

BBOX = ([-1.0, -1.0, -1.0], [1.0, 1.0, 1.0])


def fine_model_kwargs(R: int = 256, precision: str = "fp32", width: int = 192, smooth: bool = True) -> dict:
    """Fine stage (lib/voxurf_fine.py) with the dtu_e2e/fine.py settings:
    rgbnet 70 -> 192 x3 -> 3, k_rgbnet 60 -> 192 x3 -> 3, hierarchical
    displacements (0.5, 1, 1.5), center_sdf, k_res, grad norm, s_ratio 50,
    s_start 0.05; Gaussian smoothing 5^3 sigma 0.8 of the SDF each step."""
    return dict(
        xyz_min=BBOX[0], xyz_max=BBOX[1], num_voxels=R ** 3, num_voxels_base=R ** 3, alpha_init=1e-2,
        fast_color_thres=1e-4, rgbnet_dim=12, rgbnet_depth=4, rgbnet_width=width, posbase_pe=5, viewbase_pe=1,
        k_posbase_pe=5, k_viewbase_pe=1, k_res=True, k_rgbnet_depth=4, center_sdf=True,
        grad_feat=(0.5, 1.0, 1.5), sdf_feat=(0.5, 1.0, 1.5), k_grad_feat=(1.0,), use_grad_norm=True,
        s_ratio=50, s_start=0.05, smooth_ksize=5 if smooth else 0, smooth_sigma=0.8, precision=precision,
    )


FINE_RENDER_KWARGS = dict(near=0.1, far=6.0, bg=0, stepsize=0.5, inverse_y=True, flip_x=False, flip_y=False)


def build_fine_model(R: int = 256, precision: str = "fp32", device="cuda", seed: int = 0, scene: str = "sphere_torus",
                     mask_voxels: float | None = None, width: int = 192, smooth: bool = True,
                     shape: tuple | None = None):
    """Fine Voxurf model with the synthetic scene loaded.  mask_voxels: if
    given, a MaskGrid of |SDF| < mask_voxels*voxel_size (the |SDF| < 0.05
    mask of the 256^3 workload is mask_voxels = 6.4).  shape: the
    sphere_torus sizes (sphere r, torus R, torus r)."""
    from .grid import MaskGrid
    from .voxurf_fine import Voxurf

    torch.manual_seed(seed)
    sdf = torch.from_numpy(synthetic.make_sdf(scene, R, seed=seed, shape=shape))
    mask = None
    if mask_voxels is not None:
        thr = mask_voxels * 2.0 / R
        mask = MaskGrid(mask=(sdf.abs() < thr), xyz_min=BBOX[0], xyz_max=BBOX[1])
    model = Voxurf(**fine_model_kwargs(R, precision, width, smooth), mask_grid=None)
    with torch.no_grad():
        model.sdf.grid.data = sdf[None, None].clone()
        k0 = synthetic.make_k0(R, 12, seed=seed + 1)
        model.k0.grid.data = k0.permute(3, 0, 1, 2)[None].contiguous(memory_format=torch.channels_last_3d)
    model = model.to(device)
    if mask is not None:
        # as Voxurf.__init__ with a mask cache: record the non-empty mask and
        # set the SDF to 1 outside it (voxurf_fine.py:192-196, 353-367)
        model.mask_cache = mask.to(device)
        model._set_nonempty_mask()
    if precision == "bf16":
        model.refresh_k0_shadow()
    return model


def womask_model_kwargs(R: int = 64, precision: str = "fp32", width: int = 128, R_bg: int | None = None) -> dict:
    """Maskless fine stage (lib/voxurf_womask_fine.py) with the fine model's
    feature settings above, a background grid of R_bg^3 (default R^3) and
    the background MLP of the reference's defaults (bg_k0 12 + PE(xyz, 5)
    33 + PE(view, 4) 27 = 72 -> width x2 -> 3)."""
    kw = fine_model_kwargs(R, precision, width)
    kw.update(num_voxels_bg=(R_bg or R) ** 3, bg_fast_color_thres=1e-4, bg_rgbnet_dim=12, bg_posbase_pe=5,
              bg_viewbase_pe=4, bg_rgbnet_width=width, bg_rgbnet_depth=3)
    return kw


def build_womask_model(R: int = 64, precision: str = "fp32", device="cuda", seed: int = 0, width: int = 128,
                       R_bg: int | None = None):
    """Maskless fine model with a synthetic scene: the sphere r=0.5 SDF (+
    noise) inside the unit sphere, k0 and bg_k0 ~ N(0, 0.1), bg_density ~
    N(1, 2) (alphas of a few percent per background sample)."""
    from .voxurf_womask import VoxurfWomask

    torch.manual_seed(seed)
    model = VoxurfWomask(**womask_model_kwargs(R, precision, width, R_bg))
    Rb = int(model.world_size_bg[0])
    with torch.no_grad():
        model.sdf.grid.data = torch.from_numpy(synthetic.make_sdf("sphere", R, seed=seed))[None, None].clone()
        k0 = synthetic.make_k0(R, 12, seed=seed + 1)
        model.k0.grid.data = k0.permute(3, 0, 1, 2)[None].contiguous(memory_format=torch.channels_last_3d)
        bk = synthetic.make_k0(Rb, 12, seed=seed + 2)
        model.bg_k0.grid.data = bk.permute(3, 0, 1, 2)[None].contiguous(memory_format=torch.channels_last_3d)
        g = torch.Generator().manual_seed(seed + 3)
        model.bg_density.grid.data = (torch.randn((1, 1, Rb, Rb, Rb), generator=g) * 2.0 + 1.0)
    model = model.to(device)
    if precision == "bf16":
        model.refresh_k0_shadow()
    return model


def womask_coarse_model_kwargs(R: int = 96, precision: str = "fp32", width: int = 128, R_bg: int | None = None,
                               bg_k0: bool = False) -> dict:
    """Maskless coarse stage (lib/voxurf_womask_coarse.py) with the
    configs/dtu_e2e_womask/coarse.py settings on top of
    configs/default_fine_s.py: rgbnet k0 12 + PE(xyz, 5) 33 + PE(view, 4) 27
    + normal 3 = 75 -> width -> 3; bg_rgbnet PE(xyz, 5) + PE(view, 4) = 60
    (+ bg_k0 12 with bg_k0) -> width x3 -> 3; smoothing 5^3 sigma 0.8;
    s_ratio 200, s_start 0.5; both selection thresholds 1e-4."""
    return dict(
        xyz_min=BBOX[0], xyz_max=BBOX[1], num_voxels=R ** 3, num_voxels_base=R ** 3, num_voxels_bg=(R_bg or R) ** 3,
        alpha_init=1e-2, fast_color_thres=1e-4, bg_fast_color_thres=1e-4, rgbnet_dim=12, rgbnet_direct=True,
        rgbnet_full_implicit=False, rgbnet_depth=3, rgbnet_width=width, posbase_pe=5, viewbase_pe=4, geo_rgb_dim=3,
        bg_rgbnet_dim=12 if bg_k0 else 0, bg_posbase_pe=5, bg_viewbase_pe=4, bg_rgbnet_width=width,
        bg_rgbnet_depth=4, smooth_ksize=5, smooth_sigma=0.8, sdf_thr=0.5, tv_in_sphere=False, smooth_scale=True,
        s_ratio=200, s_start=0.5, precision=precision,
    )


def build_womask_coarse_model(R: int = 96, precision: str = "fp32", device="cuda", seed: int = 0, width: int = 128,
                              R_bg: int | None = None, bg_k0: bool = False):
    """Maskless coarse model with the sphere r=0.5 SDF (+ noise), k0 (and
    bg_k0) ~ N(0, 0.1) and bg_density ~ N(1, 2)."""
    from .voxurf_womask_coarse import VoxurfWomaskCoarse

    torch.manual_seed(seed)
    model = VoxurfWomaskCoarse(**womask_coarse_model_kwargs(R, precision, width, R_bg, bg_k0))
    Rb = int(model.world_size_bg[0])
    with torch.no_grad():
        model.sdf.grid.data = torch.from_numpy(synthetic.make_sdf("sphere", R, seed=seed))[None, None].clone()
        k0 = synthetic.make_k0(R, 12, seed=seed + 1)
        model.k0.grid.data = k0.permute(3, 0, 1, 2)[None].contiguous(memory_format=torch.channels_last_3d)
        if bg_k0:
            bk = synthetic.make_k0(Rb, 12, seed=seed + 2)
            model.bg_k0.grid.data = bk.permute(3, 0, 1, 2)[None].contiguous(memory_format=torch.channels_last_3d)
        g = torch.Generator().manual_seed(seed + 3)
        model.bg_density.grid.data = (torch.randn((1, 1, Rb, Rb, Rb), generator=g) * 2.0 + 1.0)
    model = model.to(device)
    if precision == "bf16":
        model.refresh_k0_shadow()
    return model


# Render-server scenes: sphere_torus with different sizes per scene
# (sphere r, torus R, torus r), each with its own seed.
SERVE_SHAPES = [(0.45, 0.6, 0.15), (0.40, 0.55, 0.12), (0.50, 0.65, 0.18), (0.35, 0.50, 0.10)]


def trained_s_val(step: int = 20000, s_ratio: float = 50.0, s_start: float = 0.05, step_start: int = 0) -> float:
    """s_val the fine stage reaches at `step` (voxurf_fine.py:466-469; the
    dtu_e2e fine schedule ends at N_iters = 20000, configs/dtu_e2e/fine.py:32)."""
    return 1.0 / (step + s_ratio / s_start - step_start) * s_ratio


def build_serve_models(R: int = 256, precision: str = "bf16", device="cuda", n: int = 4, mask_voxels: float = 6.4,
                       width: int = 192, seed: int = 100):
    """The render server's resident scenes: fine models of SERVE_SHAPES[i]
    (seed + i) with the |SDF| < mask_voxels voxel mask."""
    return [build_fine_model(R, precision, device=device, seed=seed + i, mask_voxels=mask_voxels, width=width,
                             shape=SERVE_SHAPES[i % len(SERVE_SHAPES)]) for i in range(n)]


def coarse_model_kwargs(R: int = 96, precision: str = "fp32", width: int = 128) -> dict:
    """Coarse stage (lib/voxurf_coarse.py) of the 96^3 configuration: rgbnet
    input k0 12 + PE(xyz, 5) 33 + PE(viewdir, 4) 27 + normal 3 = 75, width
    128, depth 3; smoothing 5^3 sigma 0.8; s_start 0.3 (s_ratio 50 as
    configs/dtu_e2e/coarse.py:74)."""
    return dict(
        xyz_min=BBOX[0], xyz_max=BBOX[1], num_voxels=R ** 3, num_voxels_base=R ** 3, alpha_init=1e-2,
        fast_color_thres=1e-4, rgbnet_dim=12, rgbnet_direct=True, rgbnet_full_implicit=False, rgbnet_depth=3,
        rgbnet_width=width, posbase_pe=5, viewbase_pe=4, geo_rgb_dim=3, smooth_ksize=5, smooth_sigma=0.8,
        s_ratio=50, s_start=0.3, precision=precision,
    )


def build_coarse_model(R: int = 96, precision: str = "fp32", device="cuda", seed: int = 0, width: int = 128,
                       scene: str = "sphere"):
    """Coarse Voxurf model with the sphere r=0.5 + N(0,0.01) scene loaded."""
    from .voxurf_coarse import Voxurf

    torch.manual_seed(seed)
    model = Voxurf(**coarse_model_kwargs(R, precision, width))
    with torch.no_grad():
        model.sdf.grid.data = torch.from_numpy(synthetic.make_sdf(scene, R, seed=seed))[None, None].clone()
        k0 = synthetic.make_k0(R, 12, seed=seed + 1)
        model.k0.grid.data = k0.permute(3, 0, 1, 2)[None].contiguous(memory_format=torch.channels_last_3d)
    model = model.to(device)
    if precision == "bf16":
        model.refresh_k0_shadow()
    return model


COARSE_RENDER_KWARGS = dict(near=0.1, far=6.0, bg=0, stepsize=0.5, inverse_y=True, flip_x=False, flip_y=False)


def train_targets(n: int, seed: int = 0) -> np.ndarray:
    return np.random.default_rng(seed + 7).uniform(0, 1, size=(n, 3)).astype(np.float32)
