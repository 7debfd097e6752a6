"""Host-side mirror of the maskless fine model (lib/voxurf_womask_fine.py:31-1071).

``VoxurfWomask`` keeps the reference's constructor arguments, parameter
names (``sdf.grid``, ``k0.grid``, ``bg_density.grid``, ``bg_k0.grid``,
``rgbnet.*``, ``k_rgbnet.*``, ``bg_rgbnet.*``) and the forward contract
(keys of voxurf_womask_fine.py:1041-1069).  The scene is a foreground inside
the unit sphere, rendered with the NeuS SDF model of the fine stage, and a
background outside it, rendered with a density grid over the inverted
points x/|x|^2.  The forward runs on the library's kernels, chained by
autograd Functions:

  foreground samples   vx_bg_samples_* (inner mode): the sample_ray_ori
                       points with |p| < 1, compacted per ray;
  _Smooth              Gaussian smoothing of the SDF grid and its adjoint;
  _FgAlpha             SDF + finite-difference gradient + NeuS alpha per
                       sample, adjoint scattered into the smoothed grid;
  _Alpha2Weight        Alphas2Weights (voxurf_womask_fine.py:882) over the
                       ray-sorted samples;
  _FgFeatures          the fine model's MLP input rows of the kept samples
                       (vx_fine_features / the feature part of
                       vx_fine_backward);
  background           vx_bg_samples_* (inverted points, cumdist_thres),
                       _BgAlpha (bg_density + activate_density), Alphas2Weights,
                       _BgFeatures (bg_k0 + encodings) and bg_rgbnet;
  _WomaskComposite     clamp(sum w sigmoid) per branch, rgb = clamp(in +
                       (1 - sum w) bg), and its backward.

The fast_color_thres selections are boolean indexing of the weights (as
the reference).  The per-ray jitter of the training samples
(torch.rand_like at voxurf_womask_fine.py:808, drawn separately for the
foreground and the background samples) can be passed as ``jitter`` /
``bg_jitter``; otherwise it is drawn on the device.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn as nn

from . import _abi, render_utils_cuda
from . import grid as grid_mod
from ._torch import ptr, stream_ptr
from .background import background_samples, n_samples_for
from .mlp import apply_mlp, row_stride
from .voxurf_fine import Voxurf, _SmoothGradTV, _feature_cfg, _mlp, smooth_grid, smooth_grid_adjoint, tv_mask

# global steps at which the forward resets the SDF outside the unit sphere
# (voxurf_womask_fine.py:836-838)
SPHERE_STEPS = (1, 100, 500, 1000, 2000, 3000, 5000, 10000, 15000, 16000, 17000, 18000, 19000, 20000)


class _Smooth(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sdf_grid, taps):
        ctx.taps, ctx.shape = taps, sdf_grid.shape
        X, Y, Z = sdf_grid.shape[-3:]
        return smooth_grid(sdf_grid, taps) if taps is not None else sdf_grid.reshape(X, Y, Z).clone()

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        d = smooth_grid_adjoint(g, ctx.taps) if ctx.taps is not None else g
        return d.reshape(ctx.shape), None


class _FgAlpha(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sdf_s, pts, ray_id, viewdirs, geom, voxel_size: float, inv_s: float, dist: float):
        n = pts.size(0)
        alpha = torch.empty(n, dtype=torch.float32, device=pts.device)
        a = _abi.WomaskFgAlphaArgs()
        a.n, a.pts, a.ray_id, a.viewdirs, a.grid, a.sdf_smooth = n, ptr(pts), ptr(ray_id), ptr(viewdirs), geom, \
            ptr(sdf_s)
        a.voxel_size, a.inv_s, a.dist, a.alpha = voxel_size, inv_s, dist, ptr(alpha)
        _abi.call_struct("vx_womask_fg_alpha", a, stream_ptr())
        ctx.save_for_backward(sdf_s, pts, ray_id, viewdirs)
        ctx.args = (geom, voxel_size, inv_s, dist)
        return alpha

    @staticmethod
    def backward(ctx, d_alpha):
        sdf_s, pts, ray_id, viewdirs = ctx.saved_tensors
        geom, voxel_size, inv_s, dist = ctx.args
        d_sdf = torch.zeros_like(sdf_s)
        a = _abi.WomaskFgAlphaArgs()
        a.n, a.pts, a.ray_id, a.viewdirs, a.grid, a.sdf_smooth = pts.size(0), ptr(pts), ptr(ray_id), ptr(viewdirs), \
            geom, ptr(sdf_s)
        a.voxel_size, a.inv_s, a.dist = voxel_size, inv_s, dist
        a.d_alpha, a.d_sdf_smooth = ptr(d_alpha.contiguous()), ptr(d_sdf)
        _abi.call_struct("vx_womask_fg_alpha", a, stream_ptr())
        return d_sdf, None, None, None, None, None, None, None


class _Alpha2Weight(torch.autograd.Function):
    """Alphas2Weights (lib/voxurf_fine.py:980-998) on the library's scan."""

    @staticmethod
    def forward(ctx, alpha, ray_id, n_rays: int):
        w, T, last, i_start, i_end = render_utils_cuda.alpha2weight(alpha, ray_id, n_rays)
        ctx.save_for_backward(alpha, w, T, last, i_start, i_end)
        ctx.n_rays = n_rays
        return w, last

    @staticmethod
    def backward(ctx, g_w, g_last):
        alpha, w, T, last, i_start, i_end = ctx.saved_tensors
        g_w = torch.zeros_like(w) if g_w is None else g_w.contiguous()
        g_last = torch.zeros_like(last) if g_last is None else g_last.contiguous()
        g = render_utils_cuda.alpha2weight_backward(alpha, w, T, last, i_start, i_end, ctx.n_rays, g_w, g_last)
        return g, None, None


class _FgFeatures(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sdf_s, k0_grid, pts, ray2, viewdirs, fr):
        n = pts.size(0)
        dev = pts.device
        xdt = torch.bfloat16 if fr.bf16 else torch.float32
        X1 = torch.empty((n, fr.ld1), dtype=xdt, device=dev)
        X2 = torch.empty((n, fr.ld2), dtype=xdt, device=dev)
        if n:
            f = _abi.FineFeaturesArgs()
            f.n_rows, f.ray2, f.pts2, f.viewdirs = n, ptr(ray2), ptr(pts), ptr(viewdirs)
            f.grid, f.sdf_smooth, f.voxel_size = fr.geom, ptr(sdf_s), fr.voxel_size
            if fr.k0_bf16 is not None:
                f.k0_bf16 = ptr(fr.k0_bf16)
            else:
                f.k0_f32 = ptr(k0_grid)
            f.cfg, f.ld1, f.ld2 = fr.cfg, fr.ld1, fr.ld2
            f.X1, f.X2, f.out_bf16 = ptr(X1), ptr(X2), int(fr.bf16)
            _abi.call_struct("vx_fine_features", f, stream_ptr())
        ctx.save_for_backward(sdf_s, pts)
        ctx.fr, ctx.k0_like = fr, k0_grid
        return X1, X2

    @staticmethod
    def backward(ctx, dX1, dX2):
        sdf_s, pts = ctx.saved_tensors
        fr = ctx.fr
        n = pts.size(0)
        xdt = torch.bfloat16 if fr.bf16 else torch.float32
        d_sdf = torch.zeros_like(sdf_s)
        d_k0 = torch.zeros_like(ctx.k0_like)
        if n:
            dX1 = torch.zeros((n, fr.ld1), dtype=xdt, device=pts.device) if dX1 is None else dX1.contiguous()
            dX2 = torch.zeros((n, fr.ld2), dtype=xdt, device=pts.device) if dX2 is None else dX2.contiguous()
            b = _abi.FineBackwardArgs()
            b.n_rays, b.n_rows = 0, n
            b.grid, b.sdf_smooth, b.voxel_size = fr.geom, ptr(sdf_s), fr.voxel_size
            b.pts2, b.cfg, b.ld1, b.ld2 = ptr(pts), fr.cfg, fr.ld1, fr.ld2
            b.dX1, b.dX2, b.in_bf16 = ptr(dX1), ptr(dX2), int(fr.bf16)
            b.d_sdf_smooth, b.d_k0 = ptr(d_sdf), ptr(d_k0)
            _abi.call_struct("vx_fine_backward", b, stream_ptr())
        return d_sdf, d_k0, None, None, None, None


class _BgAlpha(torch.autograd.Function):
    @staticmethod
    def forward(ctx, dens_grid, pts, geom, act_shift: float, interval: float):
        n = pts.size(0)
        alpha = torch.empty(n, dtype=torch.float32, device=pts.device)
        a = _abi.WomaskBgAlphaArgs()
        a.n, a.pts, a.grid, a.density = n, ptr(pts), geom, ptr(dens_grid)
        a.act_shift, a.interval, a.alpha = act_shift, interval, ptr(alpha)
        _abi.call_struct("vx_womask_bg_alpha", a, stream_ptr())
        ctx.save_for_backward(dens_grid, pts)
        ctx.args = (geom, act_shift, interval)
        return alpha

    @staticmethod
    def backward(ctx, d_alpha):
        dens_grid, pts = ctx.saved_tensors
        geom, act_shift, interval = ctx.args
        d = torch.zeros_like(dens_grid)
        a = _abi.WomaskBgAlphaArgs()
        a.n, a.pts, a.grid, a.density = pts.size(0), ptr(pts), geom, ptr(dens_grid)
        a.act_shift, a.interval = act_shift, interval
        a.d_alpha, a.d_density = ptr(d_alpha.contiguous()), ptr(d)
        _abi.call_struct("vx_womask_bg_alpha", a, stream_ptr())
        return d, None, None, None, None


class _BgFeatures(torch.autograd.Function):
    @staticmethod
    def forward(ctx, bg_k0_grid, outer, org, ray_id, viewdirs, geom, pos_pe: int, view_pe: int, ld: int, bf16: bool):
        n = outer.size(0)
        X = torch.empty((n, ld), dtype=torch.bfloat16 if bf16 else torch.float32, device=outer.device)
        a = _abi.WomaskBgFeaturesArgs()
        a.n, a.outer_pts, a.pts_org, a.ray_id, a.viewdirs, a.grid = n, ptr(outer), ptr(org), ptr(ray_id), \
            ptr(viewdirs), geom
        a.bg_k0, a.posbase_pe, a.viewbase_pe, a.ld, a.X, a.bf16 = ptr(bg_k0_grid), pos_pe, view_pe, ld, ptr(X), \
            int(bf16)
        _abi.call_struct("vx_womask_bg_features", a, stream_ptr())
        ctx.save_for_backward(outer)
        ctx.args, ctx.k0_like = (geom, pos_pe, view_pe, ld, bf16), bg_k0_grid
        return X

    @staticmethod
    def backward(ctx, dX):
        (outer,) = ctx.saved_tensors
        geom, pos_pe, view_pe, ld, bf16 = ctx.args
        if ctx.k0_like is None:
            return (None,) * 10
        d = torch.zeros_like(ctx.k0_like)
        if dX is not None and outer.size(0):
            a = _abi.WomaskBgFeaturesArgs()
            a.n, a.outer_pts, a.grid, a.bg_k0 = outer.size(0), ptr(outer), geom, ptr(ctx.k0_like)
            a.posbase_pe, a.viewbase_pe, a.ld, a.bf16 = pos_pe, view_pe, ld, int(bf16)
            a.dX, a.d_bg_k0 = ptr(dX.contiguous()), ptr(d)
            _abi.call_struct("vx_womask_bg_features", a, stream_ptr())
        return d, None, None, None, None, None, None, None, None, None


class _WomaskComposite(torch.autograd.Function):
    @staticmethod
    def forward(ctx, w, logit, kout, bw, blogit, fg_off, bg_off, k_into_logit: bool, unclamped_parts: bool = False):
        N = fg_off.numel() - 1
        dev = w.device
        f32 = torch.float32
        logit, blogit = logit.float().contiguous(), blogit.float().contiguous()
        kout = None if kout is None else kout.float().contiguous()
        stats = torch.empty((N, 10), dtype=f32, device=dev)
        rgb0 = torch.empty((N, 3), dtype=f32, device=dev)
        rgbk = torch.empty((N, 3), dtype=f32, device=dev) if kout is not None else None
        ainv = torch.empty(N, dtype=f32, device=dev)
        in_m = torch.empty((N, 3), dtype=f32, device=dev)
        bg_m = torch.empty((N, 3), dtype=f32, device=dev)
        a = _abi.WomaskCompositeArgs()
        a.n_rays, a.fg_off, a.w, a.logit, a.kout = N, ptr(fg_off), ptr(w), ptr(logit), ptr(kout)
        a.bg_off, a.bw, a.blogit, a.stats = ptr(bg_off), ptr(bw), ptr(blogit), ptr(stats)
        a.rgb0, a.rgbk, a.ainv, a.in_marched, a.bg_marched = ptr(rgb0), ptr(rgbk), ptr(ainv), ptr(in_m), ptr(bg_m)
        a.unclamped_parts = int(bool(unclamped_parts))
        _abi.call_struct("vx_womask_composite", a, stream_ptr())
        ctx.save_for_backward(w, logit, kout, bw, blogit, fg_off, bg_off, stats)
        ctx.k_into_logit, ctx.unclamped_parts = bool(k_into_logit), bool(unclamped_parts)
        ctx.mark_non_differentiable(in_m, bg_m)
        return (rgbk if rgbk is not None else rgb0), rgb0, ainv, in_m, bg_m

    @staticmethod
    def backward(ctx, g_rgbk, g_rgb0, g_ainv, _gi, _gb):
        w, logit, kout, bw, blogit, fg_off, bg_off, stats = ctx.saved_tensors
        has_k = kout is not None
        if not has_k:   # rgb_marched is rgb0 itself: both gradients land there
            g_rgb0 = g_rgbk if g_rgb0 is None else (g_rgb0 if g_rgbk is None else g_rgb0 + g_rgbk)
            g_rgbk = None
        N = fg_off.numel() - 1
        d_logit = torch.empty_like(logit)
        d_kout = torch.empty_like(kout) if has_k else None
        d_w = torch.empty_like(w)
        d_blogit = torch.empty_like(blogit)
        d_bw = torch.empty_like(bw)
        c = lambda t: None if t is None else t.contiguous()
        a = _abi.WomaskCompositeArgs()
        a.n_rays, a.fg_off, a.w, a.logit, a.kout = N, ptr(fg_off), ptr(w), ptr(logit), ptr(kout)
        a.bg_off, a.bw, a.blogit, a.stats = ptr(bg_off), ptr(bw), ptr(blogit), ptr(stats)
        g_rgb0, g_rgbk, g_ainv = c(g_rgb0), c(g_rgbk), c(g_ainv)
        a.g_rgb0, a.g_rgbk, a.g_ainv = ptr(g_rgb0), ptr(g_rgbk), ptr(g_ainv)
        a.d_logit, a.d_kout, a.d_w, a.d_blogit, a.d_bw = ptr(d_logit), ptr(d_kout), ptr(d_w), ptr(d_blogit), \
            ptr(d_bw)
        a.k_into_logit, a.unclamped_parts = int(ctx.k_into_logit), int(ctx.unclamped_parts)
        _abi.call_struct("vx_womask_composite", a, stream_ptr())
        return d_w, d_logit, d_kout, d_bw, d_blogit, None, None, None, None


def _ray_offsets(ray_id: torch.Tensor, n_rays: int) -> torch.Tensor:
    off = torch.zeros(n_rays + 1, dtype=torch.int64, device=ray_id.device)
    if ray_id.numel():
        off[1:] = torch.cumsum(torch.bincount(ray_id, minlength=n_rays), 0)
    return off


class MasklessTV:
    """The regularisers of the maskless models (voxurf_womask_fine.py:484-548,
    voxurf_womask_coarse.py:398-440), mixed into both.  The TV mask is the
    non-empty mask, else the unit-sphere mask; with tv_in_sphere False the
    reference sets that mask to all ones in place (every voxel counts).  The
    smooth_grad_tv term takes the gradient grid of the smoothed SDF, as the
    forward does (self.gradient at voxurf_womask_fine.py:878,
    voxurf_womask_coarse.py:657); the smoothing is recomputed here, inside
    the same autograd graph as the loss."""

    def _sphere_mask_now(self):
        if self.sphere_mask is None:
            g = self.sdf.grid
            lo, hi = self.xyz_min.float(), self.xyz_max.float()
            axes = [torch.linspace(lo[a], hi[a], g.shape[2 + a], device=g.device) for a in range(3)]
            xs, ys, zs = torch.meshgrid(*axes, indexing="ij")
            return ((xs ** 2 + ys ** 2 + zs ** 2) < 1.0)[None, None]
        return self.sphere_mask

    def _tv_region(self):
        if not self.tv_in_sphere:
            return None
        return self.nonempty_mask if self.nonempty_mask is not None else self._sphere_mask_now()

    def density_total_variation(self, sdf_tv=0, smooth_grad_tv=0, bg_density_tv=0.):
        mask = self._tv_region()
        inv2vs = 1.0 / 2.0 / float(self.voxel_size.float())
        tv = 0
        if sdf_tv > 0:
            tv = tv + grid_mod.total_variation(self.sdf.grid, mask, mode=1, weight=inv2vs * sdf_tv)
        if smooth_grad_tv > 0:
            taps = self.smooth_taps if self.smooth_sdf else None
            u8, count = tv_mask(self, mask, self.sdf.grid)
            sdf_s = _Smooth.apply(self.sdf.grid, taps)
            tv = tv + _SmoothGradTV.apply(sdf_s, u8, float(self.voxel_size), count) * smooth_grad_tv
        if bg_density_tv > 0:
            # voxurf_womask_coarse.py:414 passes the DenseGrid module itself;
            # its grid is meant (as voxurf_womask_fine.py:514)
            tv = tv + grid_mod.total_variation(self.bg_density.grid, None, mode=1, weight=inv2vs * bg_density_tv)
        return tv

    def k0_total_variation(self, k0_tv=1., k0_grad_tv=0.):
        if k0_grad_tv > 0:
            raise NotImplementedError
        tv = 0
        if k0_tv > 0:
            tv = tv + grid_mod.total_variation(self.k0.grid, self._tv_region(), mode=1)
        return tv

    def bg_k0_total_variation(self, bg_k0_tv=1., bg_k0_grad_tv=0.):
        if bg_k0_grad_tv > 0:
            raise NotImplementedError
        tv = 0
        if bg_k0_tv > 0 and self.bg_k0 is not None and self.bg_k0_dim > 0:
            tv = tv + grid_mod.total_variation(self.bg_k0.grid, self._tv_region(), mode=1)
        return tv

    def bg_density_total_variation_add_grad(self, weight, dense_mode):
        w = weight * self.world_size.max() / 128
        self.bg_density.total_variation_add_grad(w, w, w, dense_mode)

    def bg_k0_total_variation_add_grad(self, weight, dense_mode):
        w = weight * self.world_size.max() / 128
        self.bg_k0.total_variation_add_grad(w, w, w, dense_mode)


class VoxurfWomask(MasklessTV, Voxurf):
    """lib/voxurf_womask_fine.py:31-303 (constructor) and :833-1071 (forward)."""

    def __init__(self, xyz_min, xyz_max, num_voxels=0, num_voxels_bg=0, num_voxels_base=0, alpha_init=None,
                 fast_color_thres=0, bg_fast_color_thres=0, bg_rgbnet_dim=12, bg_posbase_pe=5, bg_viewbase_pe=4,
                 bg_rgbnet_width=128, bg_rgbnet_depth=3, tv_in_sphere=False, init_ball_scale=0.5,
                 init_bg_density_fix=False, set_sphere_freq=20000, **kwargs):
        kwargs.pop("mask_cache_path", None)   # the maskless model ignores it (:245-247)
        kwargs.pop("mask_grid", None)
        super().__init__(xyz_min, xyz_max, num_voxels=num_voxels, num_voxels_base=num_voxels_base,
                         alpha_init=alpha_init, fast_color_thres=fast_color_thres, mask_cache_path=None, **kwargs)
        if bg_rgbnet_dim not in (0, 12):
            raise NotImplementedError("bg_k0 is built with 12 channels (bg_rgbnet_dim 12) or none")
        self.bg_fast_color_thres = bg_fast_color_thres
        self.tv_in_sphere, self.init_ball_scale = tv_in_sphere, init_ball_scale
        self.init_bg_density_fix, self.set_sphere_freq = init_bg_density_fix, set_sphere_freq
        # background grid resolution (voxurf_womask_fine.py:371-388)
        self.num_voxels_bg = num_voxels_bg if num_voxels_bg else num_voxels
        self.voxel_size_bg = ((self.xyz_max - self.xyz_min).prod() / self.num_voxels_bg).pow(1 / 3)
        self.world_size_bg = ((self.xyz_max - self.xyz_min) / self.voxel_size_bg).long()
        self.bg_density = grid_mod.create_grid("DenseGrid", channels=1, world_size=self.world_size_bg,
                                               xyz_min=self.xyz_min, xyz_max=self.xyz_max)
        # the ball initialisation of the SDF (:101-108)
        ws = [int(s) for s in self.world_size]
        lo, hi = grid_mod.host_values(self.xyz_min), grid_mod.host_values(self.xyz_max)
        x, y, z = np.mgrid[lo[0]:hi[0]:ws[0] * 1j, lo[1]:hi[1]:ws[1] * 1j, lo[2]:hi[2]:ws[2] * 1j]
        self.sdf.grid.data = torch.from_numpy((x ** 2 + y ** 2 + z ** 2) ** 0.5 - init_ball_scale).float()[
            None, None, ...]
        self.bg_k0_dim = bg_rgbnet_dim
        self.bg_k0 = grid_mod.create_grid("DenseGrid", channels=self.bg_k0_dim, world_size=self.world_size_bg,
                                          xyz_min=self.xyz_min, xyz_max=self.xyz_max) if self.bg_k0_dim else None
        self.bg_posbase_pe, self.bg_viewbase_pe = bg_posbase_pe, bg_viewbase_pe
        self.register_buffer("bg_posfreq", torch.FloatTensor([(2 ** i) for i in range(bg_posbase_pe)]))
        self.register_buffer("bg_viewfreq", torch.FloatTensor([(2 ** i) for i in range(bg_viewbase_pe)]))
        bg_dim0 = (3 + 3 * bg_posbase_pe * 2) + (3 + 3 * bg_viewbase_pe * 2) + self.bg_k0_dim
        self.bg_dim0 = bg_dim0
        self.bg_rgbnet = _mlp(bg_dim0, bg_rgbnet_width, bg_rgbnet_depth, self.use_layer_norm)
        nn.init.constant_(self.bg_rgbnet[-1].bias, 0)
        self.sphere_mask = None
        if self.k_center_sdf:
            raise NotImplementedError("k_center_sdf is not used by the maskless configs (its column sits before "
                                      "the gradient there, after it in the masked model)")
        # rgbnet input order (voxurf_womask_fine.py:913-951): [k0], all_feat,
        # all_grad, xyz_emb, view_emb, [sdf]; the feature kernel writes the
        # masked model's [k0], xyz_emb, view_emb, [sdf], all_feat, all_grad
        # (voxurf_fine.py:694-716), so the rows are permuted before the MLP
        K = len(self.hier_disps)
        blocks, col = {}, 0
        for name, n in (("k0", 12 if self.use_rgbnet_k0 else 0), ("xyz", 3 + 6 * self.posbase_pe),
                        ("view", 3 + 6 * self.viewbase_pe), ("sdf", 1 if self.center_sdf else 0),
                        ("feat", 6 * K), ("grad", 3 * K)):
            blocks[name] = list(range(col, col + n))
            col += n
        perm = [c for name in ("k0", "feat", "grad", "xyz", "view", "sdf") for c in blocks[name]]
        self.register_buffer("rgb_perm", torch.tensor(perm, dtype=torch.int64), persistent=False)

    @torch.no_grad()
    def _set_sphere_nonempty_mask(self):
        """voxurf_womask_fine.py:435-444: the SDF is set to 1 at the grid
        points outside the unit sphere (grid coordinates from linspace over
        the bbox, float32 as the reference)."""
        g = self.sdf.grid
        lo, hi = self.xyz_min.float(), self.xyz_max.float()
        axes = [torch.linspace(lo[a], hi[a], g.shape[2 + a], device=g.device) for a in range(3)]
        xs, ys, zs = torch.meshgrid(*axes, indexing="ij")
        mask = (xs ** 2 + ys ** 2 + zs ** 2) < 1.0
        self.sphere_mask = mask[None, None]
        g[~self.sphere_mask] = 1

    def get_kwargs(self):
        kw = super().get_kwargs()
        kw.update({"num_voxels_bg": self.num_voxels_bg, "bg_fast_color_thres": self.bg_fast_color_thres,
                   "bg_rgbnet_dim": self.bg_k0_dim, "bg_posbase_pe": self.bg_posbase_pe,
                   "bg_viewbase_pe": self.bg_viewbase_pe, "tv_in_sphere": self.tv_in_sphere,
                   "init_ball_scale": self.init_ball_scale, "set_sphere_freq": self.set_sphere_freq})
        return kw

    def forward(self, rays_o, rays_d, viewdirs, global_step=None, jitter=None, bg_jitter=None, **render_kwargs):
        if global_step is not None and (global_step in SPHERE_STEPS or global_step % self.set_sphere_freq == 0):
            self._set_sphere_nonempty_mask()
        N = len(rays_o)
        dev = rays_o.device
        is_train = global_step is not None
        s_val, inv_s = self.neus_s_val(global_step)
        rays_o = rays_o.contiguous().float()
        rays_d = rays_d.contiguous().float()
        viewdirs = viewdirs.contiguous().float()
        near, far, stepsize = float(render_kwargs["near"]), float(render_kwargs["far"]), render_kwargs["stepsize"]
        if is_train:
            jitter = torch.rand(N, device=dev) if jitter is None else jitter.contiguous().float()
            bg_jitter = torch.rand(N, device=dev) if bg_jitter is None else bg_jitter.contiguous().float()
        else:
            jitter = bg_jitter = None
        lo, hi = grid_mod.host_values(self.xyz_min), grid_mod.host_values(self.xyz_max)
        vs = self.voxel_size.float()
        n_samp = n_samples_for(self.sdf.grid.shape[2:], stepsize)
        # foreground: the samples inside the unit sphere (:843-849)
        pts, _, ray_id, _ = background_samples(rays_o, rays_d, lo, hi, near, far, stepsize, vs, n_samp, jitter,
                                               inner=True)
        # background: inverted samples outside the sphere (:852-870)
        outer, org, bray, _ = background_samples(rays_o, rays_d, lo, hi, near, far, stepsize, vs, n_samp, bg_jitter)

        fr = _frame(self, stepsize)
        sdf_s = _Smooth.apply(self.sdf.grid, fr.taps)
        dist = float(stepsize * vs)
        alpha = _FgAlpha.apply(sdf_s, pts, ray_id, viewdirs, fr.geom, fr.voxel_size, inv_s, dist)
        w, _ = _Alpha2Weight.apply(alpha, ray_id, N)
        if self.fast_color_thres > 0:
            keep = w > self.fast_color_thres
            w, pts, ray_id, alpha = w[keep], pts[keep], ray_id[keep], alpha[keep]
        # background density -> weights (:896-911; the selection compares with
        # fast_color_thres, as the reference does)
        bgeom = grid_mod.grid_geom(self.world_size_bg.tolist(), lo, hi)
        interval = float(stepsize * self.voxel_size_ratio.float())
        balpha = _BgAlpha.apply(self.bg_density.grid, outer, bgeom, float(self.act_shift), interval)
        bw, _ = _Alpha2Weight.apply(balpha, bray, N)
        if self.bg_fast_color_thres > 0:
            bkeep = bw > self.fast_color_thres
            bw, outer, org, bray = bw[bkeep], outer[bkeep], org[bkeep], bray[bkeep]
        # foreground colours (the fine model's rows and MLPs, :913-1009)
        ray2 = ray_id.to(torch.int32)
        X1, X2a = _FgFeatures.apply(sdf_s, self.k0.grid, pts.contiguous(), ray2, viewdirs, fr)
        direct_k = self.use_rgb_k and (not self.k_res or self.k_detach_1)
        logit_cols = X2a[:, fr.d2a:fr.d2a + 3] if (direct_k and self.k_res) else None
        X1 = nn.functional.pad(X1.index_select(1, self.rgb_perm), (0, fr.ld1 - fr.d1))
        rgb_logit = apply_mlp(self.rgbnet, X1, logit_cols)
        kout = None
        if self.use_rgb_k:
            k_in = X2a if direct_k else torch.cat([X2a[:, :fr.d2a], rgb_logit.to(X2a.dtype)], -1)
            kout = apply_mlp(self.k_rgbnet, k_in)
        # background colours (:955-970)
        xdt = torch.bfloat16 if fr.bf16 else torch.float32
        bld = row_stride(self.bg_dim0, xdt)
        XB = _BgFeatures.apply(self.bg_k0.grid if self.bg_k0 is not None else None, outer.contiguous(),
                               org.contiguous(), bray, viewdirs, bgeom, self.bg_posbase_pe, self.bg_viewbase_pe, bld,
                               fr.bf16)
        bg_logit = apply_mlp(self.bg_rgbnet, XB)
        fg_off, bg_off = _ray_offsets(ray_id, N), _ray_offsets(bray, N)
        rgb, rgb0, ainv, in_m, bg_m = _WomaskComposite.apply(w, rgb_logit, kout, bw, bg_logit, fg_off, bg_off,
                                                             not self.k_detach_2)
        ret = {
            "alphainv_cum": ainv,
            "weights": w,
            "bg_weights": bw,
            "pts_norm": None,          # the dense [N, S] norms are never materialised
            "rgb_marched": rgb,
            "in_marched": in_m,
            "out_marched": bg_m,
            "normal_marched": None,
            "raw_alpha": alpha,
            "raw_rgb": torch.sigmoid(rgb_logit),
            "depth": None,
            "disp": 0,
            "mask": None,
            "mask_outbbox": None,
            "gradient": X2a[:, self._grad_col:self._grad_col + 3].float(),
            "gradient_error": None,
            "s_val": s_val,
            "ray_id": ray_id,
            "bg_ray_id": bray,
        }
        if self.use_rgb_k:
            ret["rgb_marched0"] = rgb0
        return ret


class _Frame:
    pass


def _frame(model: VoxurfWomask, stepsize: float) -> _Frame:
    fr = _Frame()
    vs = model.voxel_size.float()
    fr.voxel_size = float(vs)
    fr.geom = grid_mod.grid_geom(model.sdf.grid.shape[2:], grid_mod.host_values(model.xyz_min),
                                 grid_mod.host_values(model.xyz_max))
    fr.taps = model.smooth_taps if model.smooth_sdf else None
    fr.cfg = _feature_cfg(model)
    fr.bf16 = model.precision == "bf16"
    fr.k0_bf16 = None
    if fr.bf16:
        if model._k0_shadow is None or model._k0_shadow.shape != model.k0.grid.shape:
            model.refresh_k0_shadow()
        fr.k0_bf16 = model._k0_shadow
    fr.d1 = model.dim0
    fr.d2a = model.k_dim0 - (3 if model.k_res else 0)
    xdt = torch.bfloat16 if fr.bf16 else torch.float32
    fr.ld1 = row_stride(fr.d1, xdt)
    fr.ld2 = row_stride(model.k_dim0 if model.use_rgb_k else fr.d2a, xdt)
    return fr
