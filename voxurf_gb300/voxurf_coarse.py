"""Host-side mirror of the Voxurf coarse model (lib/voxurf_coarse.py:24-619).

Same constructor arguments, parameter names and forward contract as the
reference.  Per step:
  * the SDF grid is smoothed (Gaussian, when smooth_ksize > 0) and its raw
    central-difference gradient grid is built densely (neus_sdf_gradient,
    :323-332, stored [X,Y,Z,4]);
  * _CoarseGeometry: ray march (sampling, mask, SDF + interpolated gradient,
    NeuS alpha, the first Alphas2Weights for the weight > thres set and the
    second one over that set), compaction, rgbnet features;
    backward: reverse scan, alpha and normal adjoints, scatters into the
    smoothed-SDF and gradient-grid gradients, then the smoothing adjoint and
    the central-difference adjoint into sdf.grid.grad;
  * rgbnet (nn.Linear stack), then _CoarseComposite (rgb + (1 - sum w) bg,
    clamped).
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn as nn

from . import _abi, _native
from . import grid as grid_mod
from ._torch import ptr, stream_ptr
from .mlp import apply_mlp, row_stride
from .voxurf_fine import FineFrame, gaussian_taps, marching_cubes, max_steps_bound, smooth_grid, smooth_grid_adjoint
from .voxurf_fine import extract_fields as _extract_fields
from .voxurf_fine import _SmoothGradTV, query_mask, tv_mask


def sdf_gradient_grid(sdf: torch.Tensor, voxel_size: float) -> torch.Tensor:
    X, Y, Z = sdf.shape[-3:]
    G = torch.empty((X, Y, Z, 4), dtype=torch.float32, device=sdf.device)
    _abi.call("vx_sdf_gradient_grid", ptr(sdf), ptr(G), X, Y, Z, float(voxel_size), 1, stream_ptr())
    return G


def _coarse_cfg(model) -> _abi.CoarseFeatureCfg:
    c = _abi.CoarseFeatureCfg()
    c.use_k0 = int(not model.rgbnet_full_implicit)
    c.geo_rgb_dim = int(model.geo_rgb_dim)
    c.posbase_pe = model.posbase_pe
    c.viewbase_pe = model.viewbase_pe
    return c


class _CoarseGeometry(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sdf_grid, k0_grid, fr: FineFrame):
        dev = sdf_grid.device
        st = stream_ptr()
        X, Y, Z = fr.geom.X, fr.geom.Y, fr.geom.Z
        raw = sdf_grid.reshape(X, Y, Z)
        fr.sdf_s = smooth_grid(sdf_grid, fr.taps) if fr.taps is not None else raw
        # the gradient grid of the raw SDF (voxurf_coarse.py:531), or of the
        # smoothed one in the maskless model (voxurf_womask_coarse.py:657)
        grad_src = fr.sdf_s if fr.grad_of_smoothed else raw
        fr.G4 = sdf_gradient_grid(grad_src.contiguous(), fr.voxel_size)
        N, ms = fr.n_rays, fr.max_steps
        rec = torch.empty((N * ms, 4), dtype=torch.float32, device=dev)
        dw_slot = torch.empty(N * ms, dtype=torch.float32, device=dev)
        n1 = torch.empty(N, dtype=torch.int32, device=dev)
        n2 = torch.empty(N, dtype=torch.int32, device=dev)
        n2b = torch.empty(N, dtype=torch.int32, device=dev)
        alphainv_last = torch.empty(N, dtype=torch.float32, device=dev)
        a = _abi.CoarseMarchArgs()
        m = a.march
        m.rays_o, m.rays_d, m.viewdirs = ptr(fr.rays_o), ptr(fr.rays_d), ptr(fr.viewdirs)
        m.n_rays, m.near, m.stepdist, m.grid = N, fr.near, fr.stepdist, fr.geom
        m.sdf_smooth, m.voxel_size = ptr(fr.sdf_s), fr.voxel_size
        if fr.mask_cache is not None:
            fr.mask_cache.fill_march(m)
        m.unit_sphere = int(fr.unit_sphere)
        m.inv_s, m.dist, m.fast_color_thres, m.max_steps = fr.inv_s, fr.dist, fr.thres, ms
        m.rec, m.dw_slot, m.n1, m.n2, m.alphainv_last = ptr(rec), ptr(dw_slot), ptr(n1), ptr(n2), ptr(alphainv_last)
        a.grad4, a.n2b = ptr(fr.G4), ptr(n2b)
        _abi.call_struct("vx_coarse_march", a, st)

        s2_off = torch.empty(N + 1, dtype=torch.int64, device=dev)
        nb = _native.load().vx_scan_scratch_bytes(N)
        scratch = torch.empty(max(nb, 16), dtype=torch.uint8, device=dev)
        _native.call("vx_exclusive_scan_i32", ptr(n2), N, ptr(s2_off), ptr(scratch), nb, st)
        S2 = int(s2_off[-1].item())
        fr.S2 = S2
        ray2 = torch.empty(S2, dtype=torch.int32, device=dev)
        step2 = torch.empty(S2, dtype=torch.int32, device=dev)
        slot2 = torch.empty(S2, dtype=torch.int32, device=dev)
        w2 = torch.empty(S2, dtype=torch.float32, device=dev)
        alpha2 = torch.empty(S2, dtype=torch.float32, device=dev)
        pts2 = torch.empty((S2, 3), dtype=torch.float32, device=dev)
        c = _abi.FineCompactArgs()
        c.rays_o, c.rays_d, c.n_rays, c.near, c.stepdist = ptr(fr.rays_o), ptr(fr.rays_d), N, fr.near, fr.stepdist
        for i in range(3):
            c.xyz_min[i], c.xyz_max[i] = fr.geom.xyz_min[i], fr.geom.xyz_max[i]
        c.max_steps, c.rec, c.n1, c.s2_off = ms, ptr(rec), ptr(n1), ptr(s2_off)
        c.ray2, c.step2, c.slot2, c.w2, c.alpha2, c.pts2 = ptr(ray2), ptr(step2), ptr(slot2), ptr(w2), ptr(alpha2), \
            ptr(pts2)
        _abi.call_struct("vx_fine_compact", c, st)

        xdt = torch.bfloat16 if fr.bf16 else torch.float32
        Xf = torch.empty((S2, fr.ld), dtype=xdt, device=dev)
        normal2 = torch.empty((S2, 3), dtype=torch.float32, device=dev)
        f = _abi.CoarseFeaturesArgs()
        f.n_rows, f.ray2, f.pts2, f.viewdirs = S2, ptr(ray2), ptr(pts2), ptr(fr.viewdirs)
        f.grid, f.grad4 = fr.geom, ptr(fr.G4)
        if fr.k0_bf16 is not None:
            f.k0_bf16 = ptr(fr.k0_bf16)
        else:
            f.k0_f32 = ptr(k0_grid)
        f.cfg, f.ld, f.X, f.out_bf16, f.normal_out = fr.cfg, fr.ld, ptr(Xf), int(fr.bf16), ptr(normal2)
        _abi.call_struct("vx_coarse_features", f, st)
        fr.rec, fr.dw_slot, fr.n2b, fr.alphainv_last = rec, dw_slot, n2b, alphainv_last
        fr.s2_off, fr.ray2, fr.step2, fr.slot2, fr.w2, fr.alpha2, fr.pts2 = s2_off, ray2, step2, slot2, w2, alpha2, pts2
        ctx.fr, ctx.k0_like, ctx.sdf_shape = fr, k0_grid, sdf_grid.shape
        ctx.mark_non_differentiable(alpha2)
        # normal2 = the shaded samples' raw interpolated gradient (differentiable:
        # an eikonal term on it reaches the gradient grid through d_grad2)
        return Xf, w2, alphainv_last, normal2, alpha2

    @staticmethod
    def backward(ctx, dX, dw2, dlast, d_grad2, _da):
        fr = ctx.fr
        dev = fr.w2.device
        st = stream_ptr()
        X, Y, Z = fr.geom.X, fr.geom.Y, fr.geom.Z
        S2, N = fr.S2, fr.n_rays
        xdt = torch.bfloat16 if fr.bf16 else torch.float32
        dX = torch.zeros((S2, fr.ld), dtype=xdt, device=dev) if dX is None else dX.contiguous()
        dw2 = torch.zeros(S2, dtype=torch.float32, device=dev) if dw2 is None else dw2.contiguous().float()
        dlast = torch.zeros(N, dtype=torch.float32, device=dev) if dlast is None else dlast.contiguous().float()
        d_sdf_s = torch.zeros((X, Y, Z), dtype=torch.float32, device=dev)
        dG4 = torch.zeros((X, Y, Z, 4), dtype=torch.float32, device=dev)
        d_k0 = torch.zeros_like(ctx.k0_like)
        b = _abi.CoarseBackwardArgs()
        b.n_rays, b.n_rows = N, S2
        b.rays_o, b.rays_d, b.viewdirs = ptr(fr.rays_o), ptr(fr.rays_d), ptr(fr.viewdirs)
        b.near, b.stepdist, b.grid = fr.near, fr.stepdist, fr.geom
        b.sdf_smooth, b.grad4, b.voxel_size = ptr(fr.sdf_s), ptr(fr.G4), fr.voxel_size
        b.inv_s, b.dist, b.max_steps = fr.inv_s, fr.dist, fr.max_steps
        b.rec, b.dw_slot, b.n2b = ptr(fr.rec), ptr(fr.dw_slot), ptr(fr.n2b)
        b.alphainv_last, b.d_last = ptr(fr.alphainv_last), ptr(dlast)
        b.pts2, b.slot2, b.dw2 = ptr(fr.pts2), ptr(fr.slot2), ptr(dw2)
        b.cfg, b.ld, b.dX, b.in_bf16 = fr.cfg, fr.ld, ptr(dX), int(fr.bf16)
        b.d_sdf_smooth, b.d_grad4, b.d_k0 = ptr(d_sdf_s), ptr(dG4), ptr(d_k0)
        if d_grad2 is not None:
            d_grad2 = d_grad2.float().contiguous()
            b.d_grad2 = ptr(d_grad2)
        _abi.call_struct("vx_coarse_backward", b, st)
        if fr.grad_of_smoothed:
            _abi.call("vx_sdf_gradient_grid_adjoint", ptr(dG4), ptr(d_sdf_s), X, Y, Z, float(fr.voxel_size), 1, 1, st)
        d_sdf = smooth_grid_adjoint(d_sdf_s, fr.taps) if fr.taps is not None else d_sdf_s
        if not fr.grad_of_smoothed:
            _abi.call("vx_sdf_gradient_grid_adjoint", ptr(dG4), ptr(d_sdf), X, Y, Z, float(fr.voxel_size), 1, 1, st)
        return d_sdf.reshape(ctx.sdf_shape), (d_k0 if fr.use_k0 else None), None


class _CoarseComposite(torch.autograd.Function):
    @staticmethod
    def forward(ctx, w2, logit, fr: FineFrame, bg: float):
        N = fr.n_rays
        dev = w2.device
        logit = logit.float().contiguous()
        rgb = torch.empty((N, 3), dtype=torch.float32, device=dev)
        raw = torch.empty((N, 3), dtype=torch.float32, device=dev)
        a = _abi.CoarseCompositeArgs()
        a.n_rays, a.s2_off, a.w2, a.logit, a.bg = N, ptr(fr.s2_off), ptr(w2), ptr(logit), float(bg)
        a.rgb, a.rgb_raw = ptr(rgb), ptr(raw)
        if fr.render_extras:
            fr.normal_marched = torch.empty((N, 3), dtype=torch.float32, device=dev)
            fr.depth = torch.empty(N, dtype=torch.float32, device=dev)
            a.normal2, a.normal_out = ptr(fr.normal2), ptr(fr.normal_marched)
            a.step2, a.depth_out, a.dist = ptr(fr.step2), ptr(fr.depth), fr.dist
        _abi.call_struct("vx_coarse_composite", a, stream_ptr())
        ctx.save_for_backward(w2, logit, raw)
        ctx.fr, ctx.bg = fr, float(bg)
        return rgb

    @staticmethod
    def backward(ctx, g_rgb):
        w2, logit, raw = ctx.saved_tensors
        fr = ctx.fr
        dev = w2.device
        d_logit = torch.empty((fr.S2, 3), dtype=torch.float32, device=dev)
        d_w2 = torch.empty(fr.S2, dtype=torch.float32, device=dev)
        a = _abi.CoarseCompositeBwdArgs()
        a.n_rays, a.s2_off, a.w2, a.logit, a.rgb_raw = fr.n_rays, ptr(fr.s2_off), ptr(w2), ptr(logit), ptr(raw)
        g_rgb = g_rgb.contiguous()
        a.g_rgb, a.bg = ptr(g_rgb), ctx.bg
        a.d_logit, a.d_w2 = ptr(d_logit), ptr(d_w2)
        _abi.call_struct("vx_coarse_composite_backward", a, stream_ptr())
        return d_w2, d_logit, None, None


class Voxurf(nn.Module):
    """lib/voxurf_coarse.py:24-142 (constructor) and :513-619 (forward)."""

    def __init__(self, xyz_min, xyz_max, num_voxels=0, num_voxels_base=0, alpha_init=None, nearest=False,
                 mask_cache_path=None, mask_cache_thres=1e-3, fast_color_thres=0, rgbnet_dim=0,
                 rgbnet_direct=False, rgbnet_full_implicit=False, rgbnet_depth=3, rgbnet_width=128, posbase_pe=5,
                 viewbase_pe=4, geo_rgb_dim=3, grad_mode="interpolate", s_ratio=2000, s_start=0.2, s_learn=False,
                 step_start=0, smooth_ksize=0, smooth_sigma=1, precision="fp32", mask_grid=None, **kwargs):
        super().__init__()
        self.register_buffer("xyz_min", torch.as_tensor(np.asarray(xyz_min, np.float32)).clone())
        self.register_buffer("xyz_max", torch.as_tensor(np.asarray(xyz_max, np.float32)).clone())
        self.fast_color_thres = fast_color_thres
        if fast_color_thres <= 0:
            # voxurf_coarse.py:613 returns an unbound `mask` in this case
            raise ValueError("the coarse forward needs fast_color_thres > 0 (the reference fails without it)")
        self.nearest = nearest
        if nearest:
            raise NotImplementedError("nearest interpolation is not used by the Voxurf configs")
        self.s_ratio, self.s_start, self.s_learn, self.step_start = s_ratio, s_start, s_learn, step_start
        self.s_val = torch.ones(1) * s_start
        self.num_voxels_base = num_voxels_base
        self.voxel_size_base = ((self.xyz_max - self.xyz_min).prod() / self.num_voxels_base).pow(1 / 3)
        self.alpha_init = alpha_init
        self.act_shift = np.log(1 / (1 - alpha_init) - 1)
        self._set_grid_resolution(num_voxels)
        self.density = nn.Parameter(torch.zeros([1, 1, *self.world_size]))
        self.sdf = grid_mod.create_grid("DenseGrid", channels=1, world_size=self.world_size, xyz_min=self.xyz_min,
                                        xyz_max=self.xyz_max)
        ws = [int(s) for s in self.world_size]
        x, y, z = np.mgrid[-1.0:1.0:ws[0] * 1j, -1.0:1.0:ws[1] * 1j, -1.0:1.0:ws[2] * 1j]
        self.sdf.grid.data = torch.from_numpy((x ** 2 + y ** 2 + z ** 2) ** 0.5 - 1).float()[None, None, ...]
        self.init_smooth_conv(smooth_ksize, smooth_sigma)
        self.rgbnet_kwargs = {"rgbnet_dim": rgbnet_dim, "rgbnet_direct": rgbnet_direct,
                              "rgbnet_full_implicit": rgbnet_full_implicit, "rgbnet_depth": rgbnet_depth,
                              "rgbnet_width": rgbnet_width, "posbase_pe": posbase_pe, "viewbase_pe": viewbase_pe}
        self.rgbnet_full_implicit = rgbnet_full_implicit
        if rgbnet_dim <= 0:
            raise NotImplementedError("the DVGO-style colour grid (rgbnet_dim <= 0) is not part of this build")
        self.k0_dim = 0 if rgbnet_full_implicit else rgbnet_dim
        if self.k0_dim not in (0, 12):
            raise NotImplementedError("k0 must have 12 channels")
        self.k0 = grid_mod.create_grid("DenseGrid", channels=max(self.k0_dim, 12), world_size=self.world_size,
                                       xyz_min=self.xyz_min, xyz_max=self.xyz_max)
        self.rgbnet_direct = rgbnet_direct
        if not rgbnet_direct and not rgbnet_full_implicit:
            raise NotImplementedError("rgbnet_direct=False is not used by the Voxurf configs")
        self.posbase_pe, self.viewbase_pe = posbase_pe, viewbase_pe
        self.register_buffer("posfreq", torch.FloatTensor([(2 ** i) for i in range(posbase_pe)]))
        self.register_buffer("viewfreq", torch.FloatTensor([(2 ** i) for i in range(viewbase_pe)]))
        dim0 = (3 + 3 * posbase_pe * 2) + (3 + 3 * viewbase_pe * 2) + self.k0_dim
        self.geo_rgb_dim = geo_rgb_dim
        if geo_rgb_dim not in (0, 3):
            raise NotImplementedError("geo_rgb_dim must be 0 or 3")
        dim0 += geo_rgb_dim
        self.dim0 = dim0
        self.rgbnet = nn.Sequential(
            nn.Linear(dim0, rgbnet_width), nn.ReLU(inplace=True),
            *[nn.Sequential(nn.Linear(rgbnet_width, rgbnet_width), nn.ReLU(inplace=True))
              for _ in range(rgbnet_depth - 2)],
            nn.Linear(rgbnet_width, 3),
        )
        nn.init.constant_(self.rgbnet[-1].bias, 0)
        self.mask_cache_path, self.mask_cache_thres = mask_cache_path, mask_cache_thres
        self.nonempty_mask = None
        if mask_cache_path:
            # voxurf_coarse.py:128-137: known free space from an earlier checkpoint
            self.mask_cache = grid_mod.MaskCache(path=mask_cache_path, mask_cache_thres=mask_cache_thres)
            self._set_nonempty_mask()
        else:
            self.mask_cache = mask_grid
        self.grad_mode = grad_mode
        if grad_mode != "interpolate":
            raise NotImplementedError("only grad_mode='interpolate' (the configs' default) is built")
        if precision not in ("fp32", "bf16"):
            raise ValueError(precision)
        self.precision = precision
        self._k0_shadow = None

    def _set_grid_resolution(self, num_voxels):
        self.num_voxels = num_voxels
        self.voxel_size = ((self.xyz_max - self.xyz_min).prod() / num_voxels).pow(1 / 3)
        self.world_size = ((self.xyz_max - self.xyz_min) / self.voxel_size).long()
        self.voxel_size_ratio = self.voxel_size / self.voxel_size_base

    def init_smooth_conv(self, ksize=3, sigma=1):
        self.smooth_sdf = ksize > 0
        self.smooth_ksize, self.smooth_sigma = ksize, sigma
        self.smooth_taps = gaussian_taps(ksize, sigma) if self.smooth_sdf else None

    def neus_s_val(self, global_step):
        if global_step is not None:
            if not self.s_learn:
                s_val = 1.0 / (global_step + self.s_ratio / self.s_start - self.step_start) * self.s_ratio
                self.s_val = torch.ones(1) * s_val
            else:
                s_val = float(self.s_val.item())
        else:
            s_val = 0
        return s_val, float((torch.ones(1) / self.s_val.float().cpu()).item())

    def refresh_k0_shadow(self):
        g = self.k0.grid
        self._k0_shadow = g.detach().to(torch.bfloat16).contiguous(memory_format=torch.channels_last_3d)
        return self._k0_shadow

    def sdf_total_variation_add_grad(self, weight, dense_mode):
        w = weight * self.world_size.max() / 128
        self.sdf.total_variation_add_grad(w, w, w, dense_mode)

    def get_MaskCache_kwargs(self):
        return {"xyz_min": self.xyz_min.cpu().numpy(), "xyz_max": self.xyz_max.cpu().numpy(),
                "act_shift": self.act_shift, "voxel_size_ratio": self.voxel_size_ratio, "nearest": self.nearest}

    @torch.no_grad()
    def _set_nonempty_mask(self):
        # grid points inside known non-empty space (voxurf_coarse.py:255-270)
        ws = self.sdf.grid.shape[2:]
        pts = torch.stack(torch.meshgrid(
            torch.linspace(float(self.xyz_min[0]), float(self.xyz_max[0]), ws[0]),
            torch.linspace(float(self.xyz_min[1]), float(self.xyz_max[1]), ws[1]),
            torch.linspace(float(self.xyz_min[2]), float(self.xyz_max[2]), ws[2]), indexing="ij"), -1)
        nonempty = query_mask(self.mask_cache, pts)[None, None].contiguous()
        self.nonempty_mask = nonempty
        self.density.data[~nonempty.to(self.density.device)] = -100
        self.sdf.grid.data[~nonempty.to(self.sdf.grid.device)] = 1

    # -- mesh extraction (voxurf_coarse.py:652-665) ---------------------------
    @torch.no_grad()
    def mesh_sdf_grid(self) -> torch.Tensor:
        g = self.sdf.grid.detach()
        if self.smooth_sdf:
            return smooth_grid(g, self.smooth_taps)
        return g.reshape(g.shape[-3:]).float().contiguous()

    @torch.no_grad()
    def extract_fields(self, bound_min, bound_max, resolution=128) -> torch.Tensor:
        """[R, R, R] field -sdf on the lattice (device tensor)."""
        if resolution is None:
            resolution = int(self.world_size[0])
        return _extract_fields(self.mesh_sdf_grid(), self.xyz_min, self.xyz_max, bound_min, bound_max, resolution)

    def extract_geometry(self, bound_min, bound_max, resolution=128, threshold=0.0, **kwargs):
        if resolution is None:
            resolution = int(self.world_size[0])
        u = self.extract_fields(bound_min, bound_max, resolution).cpu().numpy()
        return marching_cubes(u, threshold, bound_min, bound_max, resolution)

    def k0_total_variation_add_grad(self, weight, dense_mode):
        w = weight * self.world_size.max() / 128
        self.k0.total_variation_add_grad(w, w, w, dense_mode)

    def _tv_nonempty(self):
        if self.nonempty_mask is None:
            # voxurf_coarse.py:303-306 index self.nonempty_mask, which only a
            # mask cache sets
            raise ValueError("the coarse model's TV losses need the non-empty mask of a mask cache")
        return self.nonempty_mask

    def density_total_variation(self, sdf_tv=0, smooth_grad_tv=0, sdf_thrd=0.999):
        """voxurf_coarse.py:300-308, the ori_tv loss terms of the coarse
        stage (run.py:617-626): sdf_tv x total_variation(sdf.grid,
        nonempty_mask) / 2 / voxel_size in the coarse file's sum form, and
        smooth_grad_tv on the raw SDF's gradient grid (:534)."""
        mask = self._tv_nonempty()
        tv = 0
        if sdf_tv > 0:
            tv = tv + grid_mod.total_variation(self.sdf.grid, mask, mode=0,
                                               weight=float(sdf_tv / 2 / self.voxel_size.float()))
        if smooth_grad_tv > 0:
            u8, count = tv_mask(self, mask, self.sdf.grid)
            tv = tv + _SmoothGradTV.apply(self.sdf.grid, u8, float(self.voxel_size), count) * smooth_grad_tv
        return tv

    def k0_total_variation(self, k0_tv=1., k0_grad_tv=0.):
        """voxurf_coarse.py:310-320: the sum form over the non-empty mask
        repeated on the 12 channels."""
        if k0_grad_tv > 0:
            raise NotImplementedError
        tv = 0
        if k0_tv > 0:
            tv = tv + grid_mod.total_variation(self.k0.grid, self._tv_nonempty(), mode=0)
        return tv

    def march_frame(self, rays_o, rays_d, viewdirs, inv_s: float, render_kwargs) -> FineFrame:
        """The per-forward state of _CoarseGeometry: rays, sampling, grid
        geometry, NeuS constants, feature layout."""
        N = len(rays_o)
        fr = FineFrame()
        fr.n_rays = N
        fr.rays_o = rays_o.contiguous().float()
        fr.rays_d = rays_d.contiguous().float()
        fr.viewdirs = viewdirs.contiguous().float()
        fr.near = float(render_kwargs["near"])
        vs = self.voxel_size.float()
        stepdist_t = render_kwargs["stepsize"] * vs
        fr.stepdist = fr.dist = float(stepdist_t)
        fr.voxel_size = float(vs)
        fr.inv_s = inv_s
        fr.thres = float(self.fast_color_thres)
        fr.geom = grid_mod.grid_geom(self.sdf.grid.shape[2:], grid_mod.host_values(self.xyz_min), grid_mod.host_values(self.xyz_max))
        fr.max_steps = max_steps_bound(grid_mod.host_values(self.xyz_min), grid_mod.host_values(self.xyz_max), fr.stepdist)
        fr.taps = self.smooth_taps if self.smooth_sdf else None
        fr.mask_cache = self.mask_cache  # MaskGrid (bool) or MaskCache (density), or None
        fr.unit_sphere, fr.grad_of_smoothed = False, False
        fr.cfg = _coarse_cfg(self)
        fr.use_k0 = not self.rgbnet_full_implicit
        fr.bf16 = self.precision == "bf16"
        fr.k0_bf16 = None
        if fr.bf16 and fr.use_k0:
            if self._k0_shadow is None or self._k0_shadow.shape != self.k0.grid.shape:
                self.refresh_k0_shadow()
            fr.k0_bf16 = self._k0_shadow
        fr.d1 = self.dim0
        # MLP input rows zero-padded to the stride of the MLP engine
        fr.ld = row_stride(fr.d1, torch.bfloat16 if fr.bf16 else torch.float32)
        fr.render_extras = bool(render_kwargs.get("render_depth", False) or render_kwargs.get("render_grad", False))
        return fr

    def forward(self, rays_o, rays_d, viewdirs, global_step=None, **render_kwargs):
        s_val, inv_s = self.neus_s_val(global_step)
        fr = self.march_frame(rays_o, rays_d, viewdirs, inv_s, render_kwargs)
        Xf, w2, alphainv_last, normal2, alpha2 = _CoarseGeometry.apply(self.sdf.grid, self.k0.grid, fr)
        fr.normal2 = normal2
        rgb_logit = apply_mlp(self.rgbnet, Xf)
        rgb = torch.sigmoid(rgb_logit)
        rgb_marched = _CoarseComposite.apply(w2, rgb_logit, fr, float(render_kwargs["bg"]))
        normal_marched = None
        if render_kwargs.get("render_grad", False):
            normal_marched = fr.normal_marched
        self._last_frame = fr
        return {
            "alphainv_cum": alphainv_last, "weights": w2, "rgb_marched": rgb_marched,
            "normal_marched": normal_marched, "raw_alpha": alpha2, "raw_rgb": rgb,
            # voxurf_coarse.py:594 tests getattr(render_kwargs, 'render_depth') on a
            # dict, which is always False: depth/disp are None in the reference
            "depth": None, "disp": None, "mask": None, "mask_outbbox": None, "gradient": normal2,
            "gradient_error": None, "s_val": s_val, "ray_id": fr.ray2,
        }
