"""Host-side mirror of the maskless coarse model (lib/voxurf_womask_coarse.py:35-780).

``VoxurfWomaskCoarse`` keeps the reference's constructor arguments,
parameter names (``sdf.grid``, ``k0.grid``, ``bg_density.grid``,
``bg_k0.grid``, ``rgbnet.*``, ``bg_rgbnet.*``) and the forward contract
(keys of voxurf_womask_coarse.py:762-779).  The foreground inside the unit
sphere is the coarse model's NeuS surface; the background outside it is a
density grid over the inverted points x/|x|^2.  Per step:

  foreground   _CoarseGeometry with the unit-sphere test in the march
               (sample_ray_cuda, then |p| < 1, :620-628), the SDF and its
               interpolated gradient grid, both from the smoothed SDF
               (:651-658), NeuS alpha, the first Alphas2Weights for the
               weight > fast_color_thres set and the second one over that set
               (:664-674), then the coarse model's MLP input rows
               [k0, PE(xyz), PE(view), normal] (:691-708) and rgbnet;
  background   the sample_ray_ori points (the background grid's step, a
               per-ray jitter in training) outside the sphere and outside
               the bbox that pass cumdist_thres at 0.95 of the foreground
               step (:630-650), _BgAlpha (bg_density + activate_density,
               :676-679), the alpha > fast_color_thres selection (:681-686),
               Alphas2Weights (:688), _BgFeatures ([bg_k0], PE(xyz of the
               un-inverted point), PE(view), :711-727) and bg_rgbnet;
  composite    rgb = clamp(sum w sigmoid(logit) + (1 - sum w) sum w_bg
               sigmoid(bg_logit)) with unclamped branch sums (:731-742).

The reference fills ``posfreq`` with bg_posbase_pe frequencies and
``bg_posfreq`` with posbase_pe ones (:135-136) while sizing the MLPs by the
other; the two only agree when posbase_pe == bg_posbase_pe, which this
build requires.  The jitter of the background samples in training
(torch.rand_like at :587) can be passed as ``bg_jitter``; otherwise it is
drawn on the device.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn as nn

from . import grid as grid_mod
from .background import background_samples, n_samples_for
from .mlp import apply_mlp, row_stride
from .voxurf_coarse import Voxurf, _CoarseGeometry
from .voxurf_womask import (SPHERE_STEPS, MasklessTV, _Alpha2Weight, _BgAlpha, _BgFeatures, _ray_offsets,
                            _WomaskComposite)
from . import _abi
from ._torch import ptr, stream_ptr


class VoxurfWomaskCoarse(MasklessTV, Voxurf):
    """lib/voxurf_womask_coarse.py:35-224 (constructor) and :611-780 (forward)."""

    def __init__(self, xyz_min, xyz_max, num_voxels=0, num_voxels_bg=0, num_voxels_base=0, alpha_init=None,
                 fast_color_thres=0, bg_fast_color_thres=0, rgbnet_dim=0, bg_rgbnet_dim=0, posbase_pe=5,
                 viewbase_pe=4, bg_posbase_pe=5, bg_viewbase_pe=4, bg_rgbnet_width=128, bg_rgbnet_depth=4,
                 sdf_thr=1.0, tv_in_sphere=True, init_ball_scale=0.5, use_layer_norm=False, bg_use_layer_norm=False,
                 set_sphere_freq=10000, smooth_scale=False, **kwargs):
        kwargs.pop("mask_cache_path", None)   # the maskless model keeps no mask cache (:215-218)
        kwargs.pop("mask_grid", None)
        if use_layer_norm or bg_use_layer_norm:
            raise NotImplementedError("the LayerNorm MLP variants are not used by the maskless configs")
        if posbase_pe != bg_posbase_pe:
            raise ValueError("posbase_pe must equal bg_posbase_pe (the reference swaps their frequency tables)")
        if bg_rgbnet_dim not in (0, 12):
            raise NotImplementedError("bg_k0 is built with 12 channels (bg_rgbnet_dim 12) or none")
        super().__init__(xyz_min, xyz_max, num_voxels=num_voxels, num_voxels_base=num_voxels_base,
                         alpha_init=alpha_init, fast_color_thres=fast_color_thres, rgbnet_dim=rgbnet_dim,
                         posbase_pe=posbase_pe, viewbase_pe=viewbase_pe, mask_cache_path=None, **kwargs)
        del self.density      # the maskless coarse model has no foreground density grid (:90)
        self.bg_fast_color_thres = bg_fast_color_thres
        self.sdf_thr, self.tv_in_sphere, self.init_ball_scale = sdf_thr, tv_in_sphere, init_ball_scale
        self.set_sphere_freq, self.smooth_scale = set_sphere_freq, smooth_scale
        # background grid resolution (:289-306)
        self.num_voxels_bg = num_voxels_bg if num_voxels_bg else num_voxels
        self.voxel_size_bg = ((self.xyz_max - self.xyz_min).prod() / self.num_voxels_bg).pow(1 / 3)
        self.world_size_bg = ((self.xyz_max - self.xyz_min) / self.voxel_size_bg).long()
        self.bg_density = grid_mod.create_grid("DenseGrid", channels=1, world_size=self.world_size_bg,
                                               xyz_min=self.xyz_min, xyz_max=self.xyz_max)
        # the ball initialisation of the SDF over the bbox (:96-103)
        ws = [int(s) for s in self.world_size]
        lo, hi = grid_mod.host_values(self.xyz_min), grid_mod.host_values(self.xyz_max)
        x, y, z = np.mgrid[lo[0]:hi[0]:ws[0] * 1j, lo[1]:hi[1]:ws[1] * 1j, lo[2]:hi[2]:ws[2] * 1j]
        self.sdf.grid.data = torch.from_numpy((x ** 2 + y ** 2 + z ** 2) ** 0.5 - init_ball_scale).float()[
            None, None, ...]
        self.bg_k0_dim = bg_rgbnet_dim
        self.bg_k0 = grid_mod.create_grid("DenseGrid", channels=self.bg_k0_dim, world_size=self.world_size_bg,
                                          xyz_min=self.xyz_min, xyz_max=self.xyz_max)
        self.bg_posbase_pe, self.bg_viewbase_pe = bg_posbase_pe, bg_viewbase_pe
        self.register_buffer("bg_posfreq", torch.FloatTensor([(2 ** i) for i in range(posbase_pe)]))
        self.register_buffer("bg_viewfreq", torch.FloatTensor([(2 ** i) for i in range(bg_viewbase_pe)]))
        self.bg_dim0 = (3 + 3 * bg_posbase_pe * 2) + (3 + 3 * bg_viewbase_pe * 2) + self.bg_k0_dim
        self.bg_rgbnet = nn.Sequential(
            nn.Linear(self.bg_dim0, bg_rgbnet_width), nn.ReLU(inplace=True),
            *[nn.Sequential(nn.Linear(bg_rgbnet_width, bg_rgbnet_width), nn.ReLU(inplace=True))
              for _ in range(bg_rgbnet_depth - 2)],
            nn.Linear(bg_rgbnet_width, 3),
        )
        nn.init.constant_(self.bg_rgbnet[-1].bias, 0)
        self.sphere_mask = None
        self._set_sphere_nonempty_mask()

    @torch.no_grad()
    def _set_sphere_nonempty_mask(self):
        """:348-359: the SDF is set to 1 at the grid points outside the unit
        sphere (grid coordinates from linspace over the bbox, float32)."""
        g = self.sdf.grid
        lo, hi = self.xyz_min.float(), self.xyz_max.float()
        axes = [torch.linspace(lo[a], hi[a], g.shape[2 + a], device=g.device) for a in range(3)]
        xs, ys, zs = torch.meshgrid(*axes, indexing="ij")
        mask = (xs ** 2 + ys ** 2 + zs ** 2) < 1.0
        self.sphere_mask = mask[None, None]
        g[~self.sphere_mask] = 1

    def get_kwargs(self):
        return {"xyz_min": self.xyz_min.cpu().numpy(), "xyz_max": self.xyz_max.cpu().numpy(),
                "num_voxels": self.num_voxels, "num_voxels_base": self.num_voxels_base,
                "alpha_init": self.alpha_init, "nearest": self.nearest, "mask_cache_path": None,
                "mask_cache_thres": self.mask_cache_thres, "fast_color_thres": self.fast_color_thres,
                "geo_rgb_dim": self.geo_rgb_dim, **self.rgbnet_kwargs}

    def forward(self, rays_o, rays_d, viewdirs, global_step=None, bg_jitter=None, **render_kwargs):
        if global_step is not None and (global_step in SPHERE_STEPS or global_step % self.set_sphere_freq == 0):
            self._set_sphere_nonempty_mask()
        N = len(rays_o)
        dev = rays_o.device
        s_val, inv_s = self.neus_s_val(global_step)
        fr = self.march_frame(rays_o, rays_d, viewdirs, inv_s, render_kwargs)
        fr.mask_cache = None
        fr.unit_sphere, fr.grad_of_smoothed = True, True
        # foreground (:620-674, 691-709)
        Xf, w, alphainv_last, normal2, alpha = _CoarseGeometry.apply(self.sdf.grid, self.k0.grid, fr)
        rgb_logit = apply_mlp(self.rgbnet, Xf)
        # background samples (:630-650)
        stepsize = render_kwargs["stepsize"]
        if global_step is not None:
            bg_jitter = torch.rand(N, device=dev) if bg_jitter is None else bg_jitter.contiguous().float()
        else:
            bg_jitter = None
        lo, hi = grid_mod.host_values(self.xyz_min), grid_mod.host_values(self.xyz_max)
        n_samp = n_samples_for(self.world_size_bg.tolist(), stepsize)
        outer, org, bray, _ = background_samples(
            fr.rays_o, fr.rays_d, lo, hi, float(render_kwargs["near"]), float(render_kwargs["far"]), stepsize,
            self.voxel_size.float(), n_samp, bg_jitter, step_voxel_size=self.voxel_size_bg.float(),
            dist_thres_factor=0.95, outbbox_only=True)
        # background density -> alpha, the alpha selection, weights (:676-688)
        bgeom = grid_mod.grid_geom(self.world_size_bg.tolist(), lo, hi)
        interval = float(stepsize * self.voxel_size_ratio.float())
        balpha = _BgAlpha.apply(self.bg_density.grid, outer, bgeom, float(self.act_shift), interval)
        if self.bg_fast_color_thres > 0:
            keep = balpha > self.fast_color_thres
            balpha, outer, org, bray = balpha[keep], outer[keep], org[keep], bray[keep]
        bw, _ = _Alpha2Weight.apply(balpha, bray, N)
        # background colours (:711-729)
        bld = row_stride(self.bg_dim0, torch.bfloat16 if fr.bf16 else torch.float32)
        XB = _BgFeatures.apply(self.bg_k0.grid if self.bg_k0_dim else None, outer.contiguous(), org.contiguous(),
                               bray, fr.viewdirs, bgeom, self.posbase_pe, self.bg_viewbase_pe, bld, fr.bf16)
        bg_logit = apply_mlp(self.bg_rgbnet, XB)
        # compositing (:731-742)
        rgb, _, _, in_m, bg_m = _WomaskComposite.apply(w, rgb_logit, None, bw, bg_logit, fr.s2_off,
                                                       _ray_offsets(bray, N), False, True)
        normal_marched = depth = disp = None
        if fr.render_extras:
            normal_marched, depth = _extras(fr, w, rgb_logit, normal2)
            disp = 1 / depth
            if not render_kwargs.get("render_grad", False):
                normal_marched = None
            if not render_kwargs.get("render_depth", False):
                depth = disp = None
        self._last_frame = fr
        return {
            "alphainv_cum": alphainv_last,
            "weights": w,
            "bg_weights": bw,
            "pts_norm": None,          # the per-sample norms are not materialised
            "rgb_marched": rgb,
            "in_marched": in_m,
            "out_marched": bg_m,
            "normal_marched": normal_marched,
            "raw_alpha": alpha,
            "raw_rgb": torch.sigmoid(rgb_logit),
            "depth": depth,
            "disp": disp,
            "mask": None,
            "mask_outbbox": None,
            "gradient": normal2,
            "s_val": s_val,
            "ray_id": fr.ray2,
            "bg_ray_id": bray,
        }


@torch.no_grad()
def _extras(fr, w, rgb_logit, normal2):
    """normal_marched = sum w g/(|g| + 1e-6) and depth = sum w step dist per
    ray (:744-758), from the coarse compositing kernel."""
    N = fr.n_rays
    dev = w.device
    f32 = torch.float32
    rgb = torch.empty((N, 3), dtype=f32, device=dev)
    raw = torch.empty((N, 3), dtype=f32, device=dev)
    nm = torch.empty((N, 3), dtype=f32, device=dev)
    depth = torch.empty(N, dtype=f32, device=dev)
    logit = rgb_logit.detach().float().contiguous()
    normal2 = normal2.detach().float().contiguous()
    a = _abi.CoarseCompositeArgs()
    a.n_rays, a.s2_off, a.w2, a.logit, a.bg = N, ptr(fr.s2_off), ptr(w.detach()), ptr(logit), 0.0
    a.rgb, a.rgb_raw = ptr(rgb), ptr(raw)
    a.normal2, a.normal_out = ptr(normal2), ptr(nm)
    a.step2, a.depth_out, a.dist = ptr(fr.step2), ptr(depth), fr.dist
    _abi.call_struct("vx_coarse_composite", a, stream_ptr())
    return nm, depth
