"""ORACLE — test infrastructure only (never imported by the product).

CPU restatement, in torch, of the reference Voxurf training/rendering step
(lib/voxurf_fine.py:440-802 and lib/voxurf_coarse.py:323-619, the loss of
run.py:600-659, the TV add-grad of grid.py:67-78 and lib/utils.py:Adam),
runnable in float64 (the correctness oracle) or float32 (the timed CPU
baseline).  The reference's CUDA ops come from oracle/ops.py.  Ray sampling
and the mask lookup always run in float32 with the kernels' operation order
so that sample sets are bit-identical to the GPU's.  Threshold decisions
downstream (fast_color_thres on FP64 weights) can meet ties at FP32
precision; OracleCoarse.forward(device_keep=...) resolves those (weights
within 1e-5 relative of the threshold) with the device's decision.

The module takes its parameters from a voxurf_gb300 model's state (converted
to channel-first layout and the oracle dtype), so both sides start from the
same weights.  tests/golden/ pins this restatement against the reference's
own Python model code.
"""
from __future__ import annotations

import copy
import math

import numpy as np
import torch
import torch.nn as nn
import torch.nn.functional as F

from .ops import Alphas2WeightsOracle, RenderUtilsOracle, tv_add_grad_torch, TotalVariationOracle, trace


def gaussian_kernel3d(ksize: int, sigma: float) -> np.ndarray:
    """Voxurf._gaussian_3dconv weights (voxurf_fine.py:246-258): the
    exponentials are cast to the (float32) grid dtype first and normalised
    by their float32 sum, as the reference does."""
    x = np.arange(-(ksize // 2), ksize // 2 + 1, 1)
    xx, yy, zz = np.meshgrid(x, x, x)
    k = torch.from_numpy(np.exp(-(xx ** 2 + yy ** 2 + zz ** 2) / (2 * sigma ** 2))).float()
    return (k / k.sum()).numpy()


def smooth3d(grid: torch.Tensor, kernel: torch.Tensor) -> torch.Tensor:
    """nn.Conv3d(1,1,k,padding=k//2,padding_mode='replicate') with no bias."""
    p = kernel.shape[-1] // 2
    return F.conv3d(F.pad(grid, (p, p, p, p, p, p), mode="replicate"), kernel[None, None])


def grid_sample_pts(grid, xyz, xyz_min, xyz_max):
    """DenseGrid.forward / grid_sampler (grid.py:47-58, voxurf_fine.py:507-520)."""
    C = grid.shape[1]
    ind_norm = ((xyz - xyz_min) / (xyz_max - xyz_min)).flip((-1,)) * 2 - 1
    out = F.grid_sample(grid, ind_norm.reshape(1, 1, 1, -1, 3), mode="bilinear", align_corners=True)
    return out.reshape(C, -1).T


def maskcache_query(density, xyz_min, xyz_max, act_shift, voxel_size_ratio, thres, xyz):
    """MaskCache.forward (voxurf_fine.py:930-942, bilinear mode) in FP32 on
    the already max-pooled density [1,1,X,Y,Z]: alpha >= thres."""
    d = grid_sample_pts(density.float(), xyz.float(), xyz_min.float(), xyz_max.float())[:, 0]
    alpha = 1 - torch.exp(-F.softplus(d + act_shift) * voxel_size_ratio)
    return alpha >= thres


def _mask_state(model):
    """The oracle's copy of a model's mask cache: ('grid', mask, scale,
    shift) for a MaskGrid, ('density', density, xyz_min, xyz_max, act_shift,
    voxel_size_ratio, thres) for a MaskCache, or None."""
    mc = model.mask_cache
    if mc is None:
        return None
    if hasattr(mc, "density"):
        return ("density", mc.density.detach().cpu().float(), mc.xyz_min.cpu().float(), mc.xyz_max.cpu().float(),
                float(mc.act_shift), float(mc.voxel_size_ratio), float(mc.mask_cache_thres))
    return ("grid", mc.mask.cpu(), mc.xyz2ijk_scale.cpu().float(), mc.xyz2ijk_shift.cpu().float())


def _apply_mask(mask, pts32, ops=RenderUtilsOracle):
    if mask[0] == "grid":
        dev = pts32.device
        return ops.maskcache_lookup(mask[1].to(dev), pts32, mask[2].to(dev), mask[3].to(dev))
    return maskcache_query(*[m.to(pts32.device) if torch.is_tensor(m) else m for m in mask[1:]], pts32)


class _Alphas2WeightsOps(torch.autograd.Function):
    """lib/voxurf_fine.py:981-997 over a given render_utils op set (the
    oracle's restatement or a drop-in module)."""

    @staticmethod
    def forward(ctx, alpha, ray_id, N, ops):
        w, T, last, i_s, i_e = ops.alpha2weight(alpha, ray_id, N)
        ctx.save_for_backward(alpha, w, T, last, i_s, i_e)
        ctx.n_rays, ctx.ops = N, ops
        return w, last

    @staticmethod
    def backward(ctx, grad_w, grad_last):
        alpha, w, T, last, i_s, i_e = ctx.saved_tensors
        g = ctx.ops.alpha2weight_backward(alpha, w, T, last, i_s, i_e, ctx.n_rays, grad_w.contiguous(),
                                          grad_last.contiguous())
        return g, None, None, None


def extract_fields(grid, xyz_min, xyz_max, bound_min, bound_max, resolution, sign=-1.0):
    """extract_fields (dvgo_ori.py:679-693) with the mesh query of
    Voxurf.extract_geometry (voxurf_fine.py:903, voxurf_coarse.py:658):
    grid_sampler(pts, sign * grid) on the lattice linspace(bound_min,
    bound_max, R) per axis (meshgrid 'ij'), all chunks at once."""
    axes = [torch.linspace(float(bound_min[a]), float(bound_max[a]), int(resolution)) for a in range(3)]
    xx, yy, zz = torch.meshgrid(*axes, indexing="ij")
    pts = torch.stack([xx.reshape(-1), yy.reshape(-1), zz.reshape(-1)], -1).to(grid.dtype)
    val = grid_sample_pts(sign * grid, pts, xyz_min.to(grid.dtype), xyz_max.to(grid.dtype))
    return val.reshape(int(resolution), int(resolution), int(resolution))


def sample_sdfs(xyz, grid, displace_list, xyz_min, xyz_max, voxel_size, use_grad_norm):
    """voxurf_fine.py:537-577."""
    n = xyz.shape[0]
    xyz = xyz.reshape(1, 1, 1, -1, 3)
    ind_norm = ((xyz - xyz_min) / (xyz_max - xyz_min)).flip((-1,)) * 2 - 1
    gs = grid.size()[-3:]
    dev = xyz.device
    size_zyx = torch.tensor([gs[2], gs[1], gs[0]], device=dev)
    ind = ((ind_norm + 1) / 2) * (size_zyx - 1)
    offset = torch.tensor([[-1, 0, 0], [1, 0, 0], [0, -1, 0], [0, 1, 0], [0, 0, -1], [0, 0, 1]], device=dev)
    displace = torch.tensor(displace_list, device=dev)
    offset = offset[:, None, :] * displace[None, :, None]
    all_ind = ind.unsqueeze(-2) + offset.view(-1, 3)
    all_ind = all_ind.view(1, 1, 1, -1, 3)
    for a in range(3):
        all_ind[..., a] = all_ind[..., a].clamp(min=0, max=int(size_zyx[a]) - 1)
    all_ind_norm = (all_ind / (size_zyx - 1)) * 2 - 1
    feat = F.grid_sample(grid, all_ind_norm, mode="bilinear", align_corners=True)
    K = len(displace_list)
    all_ind = all_ind.view(1, 1, 1, -1, 6, K, 3)
    diff = all_ind[:, :, :, :, 1::2, :, :] - all_ind[:, :, :, :, 0::2, :, :]
    diff, _ = diff.max(dim=-1)
    feat_ = feat.view(1, 1, 1, -1, 6, K)
    feat_diff = feat_[:, :, :, :, 1::2, :] - feat_[:, :, :, :, 0::2, :]
    grad = feat_diff / diff / voxel_size
    feat = feat.view(n, 6, K)
    grad = grad.view(n, 3, K)
    if use_grad_norm:
        grad = grad / (grad.norm(dim=1, keepdim=True) + 1e-5)
    return feat.view(n, 6 * K), grad.view(n, 3 * K)


def neus_alpha(viewdirs, ray_id, dist, sdf, gradients, inv_s):
    """voxurf_fine.py:475-499 (use_mid, cos_anneal_ratio = 1)."""
    dirs = viewdirs[ray_id]
    true_cos = (dirs * gradients).sum(-1, keepdim=True)
    trace("cos<0", true_cos < 0)
    iter_cos = -(F.relu(-true_cos * 0.5 + 0.5) * 0.0 + F.relu(-true_cos) * 1.0)
    sdf = sdf.unsqueeze(-1)
    est_next = sdf + iter_cos * dist * 0.5
    est_prev = sdf - iter_cos * dist * 0.5
    prev_cdf = torch.sigmoid(est_prev * inv_s)
    next_cdf = torch.sigmoid(est_next * inv_s)
    p = prev_cdf - next_cdf
    c = prev_cdf
    raw = (p + 1e-5) / (c + 1e-5)
    trace("alpha in [0,1]", (raw >= 0) & (raw <= 1))
    return raw.clip(0.0, 1.0).squeeze(-1)


def mlp_relu_ties(net, x, device_masks=None, tie=1e-6):
    """net(x) for a Linear/ReLU stack (voxurf_fine.py:132-151), returning
    (output, ties).  With device_masks (one [S, W] bool per hidden layer: the
    device's ReLU decisions, rows in the same order), a pre-activation within
    tie * (the layer's RMS) of zero takes the device's decision instead of its
    own sign: there FP32 and FP64 legitimately disagree on the ReLU, like a
    fast_color_thres tie; `ties` counts them (mlp_relu_ties.examined counts
    the pre-activations looked at, for bounds proportional to the batch)."""
    if device_masks is None:
        return net(x), 0          # the module itself (its ReLU modules' hooks fire)
    lin = [m for m in net.modules() if isinstance(m, nn.Linear)]
    h, ties = x, 0
    mlp_relu_ties.examined = 0
    for i, m in enumerate(lin):
        h = F.linear(h, m.weight, m.bias)
        if i == len(lin) - 1:
            break
        hd = h.detach()
        near = hd.abs() <= tie * hd.pow(2).mean().sqrt()
        keep = torch.where(near, device_masks[i].to(hd.device), hd > 0)
        ties += int(near.sum())
        mlp_relu_ties.examined += hd.numel()
        h = h * keep.to(h.dtype)
    return h, ties


def pe(x, freq):
    emb = (x.unsqueeze(-1) * freq).flatten(-2)
    return torch.cat([x, emb.sin(), emb.cos()], -1)


def f32(v) -> float:
    return float(np.float32(v))


class OracleFine(nn.Module):
    """Reference fine-stage step (voxurf_fine.py:620-802) with parameters
    copied from a voxurf_gb300 fine model.

    ops / device: the render_utils op set the step calls (sample_pts_on_rays,
    maskcache_lookup, alpha2weight and its backward, with the reference
    extension's signatures) and the device of every tensor.  The default is
    the oracle's own restatement on the CPU; a drop-in module with float32
    on a GPU runs the reference's step on that module's kernels, as the
    reference itself would after its extension is swapped."""

    def __init__(self, model, dtype=torch.float64, ops=None, device="cpu"):
        super().__init__()
        self.dtype = dtype
        self.ops = RenderUtilsOracle if ops is None else ops
        self.device = torch.device(device)
        sd = {k: v.detach().cpu() for k, v in model.state_dict().items()}
        self.sdf_grid = nn.Parameter(sd["sdf.grid"].contiguous().to(dtype))
        self.k0_grid = nn.Parameter(sd["k0.grid"].contiguous().to(dtype))
        self.rgbnet = copy.deepcopy(model.rgbnet).cpu().to(dtype)
        self.k_rgbnet = copy.deepcopy(model.k_rgbnet).cpu().to(dtype)
        self.xyz_min = sd["xyz_min"].to(dtype)
        self.xyz_max = sd["xyz_max"].to(dtype)
        self.xyz_min32 = sd["xyz_min"].float()
        self.xyz_max32 = sd["xyz_max"].float()
        self.voxel_size = f32(model.voxel_size)
        self.fast_color_thres = model.fast_color_thres
        self.smooth_sdf = model.smooth_sdf
        if self.smooth_sdf:
            self.kernel = torch.from_numpy(gaussian_kernel3d(model.smooth_ksize, model.smooth_sigma)).to(dtype)
        self.posfreq = sd["posfreq"].to(dtype)
        self.viewfreq = sd["viewfreq"].to(dtype)
        self.k_posfreq = sd["k_posfreq"].to(dtype)
        self.k_viewfreq = sd["k_viewfreq"].to(dtype)
        for k in ("s_ratio", "s_start", "s_learn", "step_start", "center_sdf", "use_rgbnet_k0", "k_center_sdf",
                  "k_res", "k_detach_1", "k_detach_2", "use_rgb_k", "use_grad_norm", "grad_feat", "k_grad_feat",
                  "sdf_feat", "k_sdf_feat"):
            setattr(self, k, getattr(model, k))
        self.s_val = model.s_val.clone().float().cpu()
        self.mask = _mask_state(model)
        # None, or a dict holding the detached rgbnet logits of a base
        # forward (recorded on first use, then reused): see forward()
        self.frozen = None
        if self.device.type != "cpu":
            self.to(self.device)
            for k in ("xyz_min", "xyz_max", "xyz_min32", "xyz_max32", "posfreq", "viewfreq", "k_posfreq",
                      "k_viewfreq"):
                setattr(self, k, getattr(self, k).to(self.device))
            if self.smooth_sdf:
                self.kernel = self.kernel.to(self.device)

    def smoothed(self):
        return smooth3d(self.sdf_grid, self.kernel) if self.smooth_sdf else self.sdf_grid

    def smooth_grad_tv(self, nonempty_mask, weight):
        """density_total_variation(smooth_grad_tv=weight), voxurf_fine.py:417-420,
        with tv_smooth_conv = the normalised [1,2,1]^3 kernel (:237-242, sigma 0)
        and replicate padding."""
        grad = neus_sdf_gradient(self.sdf_grid, self.voxel_size).permute(1, 0, 2, 3, 4)
        k1 = torch.tensor([1.0, 2.0, 1.0], dtype=self.dtype)
        k = (k1[:, None, None] * k1[None, :, None] * k1[None, None, :]) / 64.0
        sm = F.conv3d(F.pad(grad, (1, 1, 1, 1, 1, 1), mode="replicate"), k[None, None])
        err = (sm.detach() - grad)
        if nonempty_mask is not None:
            err = err[nonempty_mask.cpu().repeat(3, 1, 1, 1, 1)]
        return (err ** 2).mean() * weight

    def forward(self, rays_o, rays_d, viewdirs, global_step=None, relu_device=None, relu_tie=1e-6, **rk):
        """relu_device: optional {"rgbnet": masks, "k_rgbnet": masks}, the
        device's ReLU decisions of the same shaded rows (see mlp_relu_ties);
        the tie count lands in self.relu_ties."""
        dt = self.dtype
        N = len(rays_o)
        rd = relu_device or {}
        self.relu_ties = 0
        stepdist = f32(rk["stepsize"] * np.float32(self.voxel_size))
        ru = self.ops
        dev = self.device
        ray_pts, mask_outbbox, ray_id, step_id, _, _, _ = ru.sample_pts_on_rays(
            rays_o.float().to(dev).contiguous(), rays_d.float().to(dev).contiguous(), self.xyz_min32,
            self.xyz_max32, rk["near"], 1e9, stepdist)
        inb = ~mask_outbbox
        ray_pts32, ray_id, step_id = ray_pts[inb], ray_id[inb], step_id[inb]
        if self.mask is not None:
            m = _apply_mask(self.mask, ray_pts32.contiguous(), ru)
            ray_pts32, ray_id, step_id = ray_pts32[m], ray_id[m], step_id[m]
        ray_pts = ray_pts32.to(dt)
        viewdirs = viewdirs.to(dev).to(dt)
        sdf_grid = self.smoothed()
        sdf = grid_sample_pts(sdf_grid, ray_pts, self.xyz_min, self.xyz_max)[:, 0]
        _, g = sample_sdfs(ray_pts, sdf_grid, [1.0], self.xyz_min, self.xyz_max, self.voxel_size, False)
        gradient = torch.cat([g[:, [2]], g[:, [1]], g[:, [0]]], dim=-1)
        dist = f32(rk["stepsize"] * np.float32(self.voxel_size))
        if global_step is not None:
            if not self.s_learn:
                s_val = 1.0 / (global_step + self.s_ratio / self.s_start - self.step_start) * self.s_ratio
                self.s_val = torch.ones(1) * s_val
            else:
                s_val = float(self.s_val.item())
        else:
            s_val = 0
        inv_s = float((torch.ones(1) / self.s_val.float()).item())
        alpha = neus_alpha(viewdirs, ray_id, dist, sdf, gradient, inv_s)
        thr = self.fast_color_thres
        if thr > 0:
            m = alpha > thr
            trace("alpha > thres", m)
            alpha, ray_id, ray_pts, step_id, gradient, sdf = alpha[m], ray_id[m], ray_pts[m], step_id[m], \
                gradient[m], sdf[m]
        weights, alphainv_last = _Alphas2WeightsOps.apply(alpha.contiguous(), ray_id.contiguous(), N, ru)
        if thr > 0:
            m = weights > thr
            trace("weights > thres", m)
            weights, alpha, ray_pts, ray_id, step_id, gradient, sdf = weights[m], alpha[m], ray_pts[m], ray_id[m], \
                step_id[m], gradient[m], sdf[m]
        k0 = grid_sample_pts(self.k0_grid, ray_pts, self.xyz_min, self.xyz_max)
        disps = sorted(set(tuple(self.grad_feat) + tuple(self.k_grad_feat)))
        all_feat, all_grad = sample_sdfs(ray_pts, sdf_grid, disps, self.xyz_min, self.xyz_max, self.voxel_size,
                                         self.use_grad_norm)
        rays_xyz = (ray_pts - self.xyz_min) / (self.xyz_max - self.xyz_min)
        xyz_emb = pe(rays_xyz, self.posfreq)
        view_emb = pe(viewdirs, self.viewfreq)
        parts = ([k0] if self.use_rgbnet_k0 else []) + [xyz_emb, view_emb[ray_id]]
        if self.center_sdf:
            parts.append(sdf[:, None])
        parts += [all_feat, all_grad]
        rgb_feat = torch.cat(parts, -1)
        rgb_logit, t1 = mlp_relu_ties(self.rgbnet, rgb_feat, rd.get("rgbnet"), relu_tie)
        self.relu_ties += t1
        self.relu_examined = getattr(mlp_relu_ties, "examined", 0) if rd else 0
        rgb = torch.sigmoid(rgb_logit)
        out = {"alphainv_cum": alphainv_last, "weights": weights, "raw_rgb": rgb, "raw_alpha": alpha,
               "gradient": gradient, "ray_id": ray_id, "step_id": step_id, "s_val": s_val, "rgb_feat": rgb_feat}
        bg = rk["bg"]
        if self.use_rgb_k:
            k_feat = torch.cat([k0, pe(rays_xyz, self.k_posfreq), pe(viewdirs, self.k_viewfreq)[ray_id], gradient]
                               + ([sdf[:, None]] if self.k_center_sdf else []), -1)
            # the detached rgbnet logits; a finite-difference check of the
            # detached graph holds them at their unperturbed values (frozen)
            detached = rgb_logit.detach()
            if self.frozen is not None:
                if "rgb_logit" in self.frozen:
                    detached = self.frozen["rgb_logit"]
                else:
                    self.frozen["rgb_logit"] = detached
            if self.k_res:
                k_feat = torch.cat([k_feat, detached if self.k_detach_1 else rgb_logit], -1)
            base = detached if self.k_detach_2 else rgb_logit
            k_out, t2 = mlp_relu_ties(self.k_rgbnet, k_feat, rd.get("k_rgbnet"), relu_tie)
            self.relu_ties += t2
            self.relu_examined += getattr(mlp_relu_ties, "examined", 0) if rd else 0
            k_rgb = torch.sigmoid(base + k_out)
            k_marched = torch.zeros([N, 3], dtype=dt, device=dev).index_add(0, ray_id, weights.unsqueeze(-1) * k_rgb) \
                + alphainv_last[..., None] * bg
            trace("k_rgb in [0,1]", (k_marched >= 0) & (k_marched <= 1))
            out["rgb_marched"] = k_marched.clamp(0, 1)
            out["k_rgb_feat"] = k_feat
        rgb_marched = torch.zeros([N, 3], dtype=dt, device=dev).index_add(0, ray_id, weights.unsqueeze(-1) * rgb) \
            + alphainv_last[..., None] * bg
        if self.use_rgb_k:
            out["rgb_marched0"] = rgb_marched
        else:
            out["rgb_marched"] = rgb_marched
        if rk.get("render_depth", False):
            with torch.no_grad():
                out["depth"] = torch.zeros([N], dtype=dt, device=dev).index_add(0, ray_id, weights * step_id * dist)
        if rk.get("render_grad", False):
            normal = gradient / (gradient.norm(2, -1, keepdim=True) + 1e-6)
            out["normal_marched"] = torch.zeros([N, 3], dtype=dt, device=dev).index_add(0, ray_id, weights.unsqueeze(-1) * normal)
        return out


def camera_rays_f32(c2w, fx, fy, cx, cy, H, W, inverse_y=True):
    """get_rays + viewdirs (voxurf_fine.py:1001-1029, 1064) in float32 with
    one rounding per operation: pixel centres i+0.5, j+0.5; dir =
    [(i-cx)/fx, +-(j-cy)/fy, +-1]; rays_d[a] = (dir0*R[a,0] + dir1*R[a,1]) +
    dir2*R[a,2]; viewdir = rays_d / |rays_d|.  Row-major over (j, i)."""
    f = np.float32
    c = np.asarray(c2w, np.float32)
    jj, ii = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    i = ii.reshape(-1).astype(np.float32) + f(0.5)
    j = jj.reshape(-1).astype(np.float32) + f(0.5)
    d0 = (i - f(cx)) / f(fx)
    d1 = (j - f(cy)) / f(fy)
    if inverse_y:
        d2 = np.ones_like(d0)
    else:
        d1 = -d1
        d2 = -np.ones_like(d0)
    d = np.stack([(d0 * c[a, 0] + d1 * c[a, 1]) + d2 * c[a, 2] for a in range(3)], -1).astype(np.float32)
    n = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
    v = (d / n[:, None]).astype(np.float32)
    o = np.broadcast_to(c[:3, 3], d.shape).astype(np.float32).copy()
    return o, d, v


def neus_sdf_gradient(sdf, voxel_size):
    """voxurf_coarse.py:323-332, 'interpolate' mode."""
    g = torch.zeros([1, 3] + list(sdf.shape[-3:]), dtype=sdf.dtype)
    g[:, 0, 1:-1, :, :] = (sdf[:, 0, 2:, :, :] - sdf[:, 0, :-2, :, :]) / 2 / voxel_size
    g[:, 1, :, 1:-1, :] = (sdf[:, 0, :, 2:, :] - sdf[:, 0, :, :-2, :]) / 2 / voxel_size
    g[:, 2, :, :, 1:-1] = (sdf[:, 0, :, :, 2:] - sdf[:, 0, :, :, :-2]) / 2 / voxel_size
    return g


class OracleCoarse(nn.Module):
    """Reference coarse-stage step (voxurf_coarse.py:513-619) with parameters
    copied from a voxurf_gb300 coarse model."""

    def __init__(self, model, dtype=torch.float64):
        super().__init__()
        self.dtype = dtype
        sd = {k: v.detach().cpu() for k, v in model.state_dict().items()}
        self.sdf_grid = nn.Parameter(sd["sdf.grid"].contiguous().to(dtype))
        self.full_implicit = model.rgbnet_full_implicit
        self.k0_grid = nn.Parameter(sd["k0.grid"].contiguous().to(dtype))
        self.rgbnet = copy.deepcopy(model.rgbnet).cpu().to(dtype)
        self.xyz_min, self.xyz_max = sd["xyz_min"].to(dtype), sd["xyz_max"].to(dtype)
        self.xyz_min32, self.xyz_max32 = sd["xyz_min"].float(), sd["xyz_max"].float()
        self.voxel_size = f32(model.voxel_size)
        self.fast_color_thres = model.fast_color_thres
        self.smooth_sdf = model.smooth_sdf
        if self.smooth_sdf:
            self.kernel = torch.from_numpy(gaussian_kernel3d(model.smooth_ksize, model.smooth_sigma)).to(dtype)
        self.posfreq, self.viewfreq = sd["posfreq"].to(dtype), sd["viewfreq"].to(dtype)
        self.geo_rgb_dim = model.geo_rgb_dim
        for k in ("s_ratio", "s_start", "s_learn", "step_start"):
            setattr(self, k, getattr(model, k))
        self.s_val = model.s_val.clone().float().cpu()
        self.mask = _mask_state(model)

    def forward(self, rays_o, rays_d, viewdirs, global_step=None, device_keep=None, tie_rel=1e-5, relu_device=None,
                relu_tie=1e-6, **rk):
        """device_keep: optional set of (ray_id, step_id) pairs that a device
        run kept after the fast_color_thres test.  A sample whose weight is
        within tie_rel (relative) of the threshold (a tie at FP32 precision)
        then takes the device's decision, so that both sides shade the same
        set.  relu_device: the device's ReLU decisions of the rgbnet hidden
        layers for the same shaded rows (see mlp_relu_ties)."""
        dt = self.dtype
        N = len(rays_o)
        stepdist = f32(rk["stepsize"] * np.float32(self.voxel_size))
        ru = RenderUtilsOracle
        ray_pts, mask_outbbox, ray_id, step_id, _, _, _ = ru.sample_pts_on_rays(
            rays_o.float().cpu(), rays_d.float().cpu(), self.xyz_min32, self.xyz_max32, rk["near"], 1e9, stepdist)
        inb = ~mask_outbbox
        ray_pts32, ray_id, step_id = ray_pts[inb], ray_id[inb], step_id[inb]
        if self.mask is not None:
            m = _apply_mask(self.mask, ray_pts32)
            ray_pts32, ray_id, step_id = ray_pts32[m], ray_id[m], step_id[m]
        ray_pts = ray_pts32.to(dt)
        viewdirs = viewdirs.cpu().to(dt)
        sdf_grid = smooth3d(self.sdf_grid, self.kernel) if self.smooth_sdf else self.sdf_grid
        sdf = grid_sample_pts(sdf_grid, ray_pts, self.xyz_min, self.xyz_max)[:, 0]
        gradient_grid = neus_sdf_gradient(self.sdf_grid, self.voxel_size)
        gradient = grid_sample_pts(gradient_grid, ray_pts, self.xyz_min, self.xyz_max)
        dist = f32(rk["stepsize"] * np.float32(self.voxel_size))
        if global_step is not None:
            if not self.s_learn:
                s_val = 1.0 / (global_step + self.s_ratio / self.s_start - self.step_start) * self.s_ratio
                self.s_val = torch.ones(1) * s_val
            else:
                s_val = float(self.s_val.item())
        else:
            s_val = 0
        inv_s = float((torch.ones(1) / self.s_val.float()).item())
        alpha = neus_alpha(viewdirs, ray_id, dist, sdf, gradient, inv_s)
        weights, _ = Alphas2WeightsOracle.apply(alpha, ray_id, N)
        m = weights > self.fast_color_thres
        if device_keep is not None:
            near = ((weights.detach() - self.fast_color_thres).abs() <= tie_rel * self.fast_color_thres).nonzero()
            for i in near.reshape(-1).tolist():
                m[i] = (int(ray_id[i]), int(step_id[i])) in device_keep
            self.ties = int(near.numel())
        trace("weights > thres", m)
        ray_pts, ray_id, step_id, alpha, gradient = ray_pts[m], ray_id[m], step_id[m], alpha[m], gradient[m]
        weights, alphainv_last = Alphas2WeightsOracle.apply(alpha, ray_id, N)
        feats = []
        if not self.full_implicit:
            feats.append(grid_sample_pts(self.k0_grid, ray_pts, self.xyz_min, self.xyz_max))
        rays_xyz = (ray_pts - self.xyz_min) / (self.xyz_max - self.xyz_min)
        feats += [pe(rays_xyz, self.posfreq), pe(viewdirs, self.viewfreq)[ray_id]]
        rgb_feat = torch.cat(feats, -1)
        if self.geo_rgb_dim == 3:
            normal = gradient / (gradient.norm(dim=-1, keepdim=True) + 1e-5)
            rgb_feat = torch.cat([rgb_feat, normal], -1)
        logit, self.relu_ties = mlp_relu_ties(self.rgbnet, rgb_feat, relu_device, relu_tie)
        self.relu_examined = getattr(mlp_relu_ties, "examined", 0) if relu_device is not None else 0
        rgb = torch.sigmoid(logit)
        rgb_marched = torch.zeros([N, 3], dtype=dt).index_add(0, ray_id, weights.unsqueeze(-1) * rgb)
        cum_w = torch.zeros([N, 1], dtype=dt).index_add(0, ray_id, weights.unsqueeze(-1))
        rgb_marched = rgb_marched + (1 - cum_w) * rk["bg"]
        trace("rgb in [0,1]", (rgb_marched >= 0) & (rgb_marched <= 1))
        rgb_marched = rgb_marched.clamp(0, 1)
        out = {"alphainv_cum": alphainv_last, "weights": weights, "rgb_marched": rgb_marched, "raw_rgb": rgb,
               "raw_alpha": alpha, "gradient": gradient, "ray_id": ray_id, "step_id": step_id, "s_val": s_val,
               "rgb_feat": rgb_feat}
        if rk.get("render_grad", False):
            nrm = gradient / (gradient.norm(2, -1, keepdim=True) + 1e-6)
            out["normal_marched"] = torch.zeros([N, 3], dtype=dt).index_add(0, ray_id, weights.unsqueeze(-1) * nrm)
        return out


def train_loss(ret, target, weight_main=1.0, weight_entropy_last=0.001, weight_rgb0=0.5):
    """run.py:604-636 (the loss terms of the fine dtu_e2e stage)."""
    target = target.to(ret["rgb_marched"].dtype)
    loss = weight_main * F.mse_loss(ret["rgb_marched"], target)
    if weight_entropy_last > 0:
        # run.py:608 indexes [..., -1] of a 1-D tensor: the LAST RAY only
        last = ret["alphainv_cum"][..., -1]
        trace("pout in range", (last >= 1e-6) & (last <= 1 - 1e-6))
        pout = last.clamp(1e-6, 1 - 1e-6)
        loss = loss + weight_entropy_last * (-(pout * torch.log(pout) + (1 - pout) * torch.log(1 - pout)).mean())
    if weight_rgb0 > 0 and "rgb_marched0" in ret:
        loss = loss + F.mse_loss(ret["rgb_marched0"], target) * weight_rgb0
    return loss


class UtilsAdam:
    """lib/utils.py:54-199 (Adam with per-voxel lr) in plain torch."""

    def __init__(self, groups, betas=(0.9, 0.99), eps=1e-8):
        self.groups = groups  # list of (params, lr)
        self.betas, self.eps = betas, eps
        self.state = {}
        self.per_lr = None

    @torch.no_grad()
    def step(self):
        b1, b2 = self.betas
        for params, lr in self.groups:
            for p in params:
                if p.grad is None:
                    continue
                st = self.state.setdefault(id(p), {"step": 0, "m": torch.zeros_like(p), "v": torch.zeros_like(p)})
                st["step"] += 1
                t = st["step"]
                bc1, bc2 = 1 - b1 ** t, 1 - b2 ** t
                st["m"].mul_(b1).add_(p.grad, alpha=1 - b1)
                st["v"].mul_(b2).addcmul_(p.grad, p.grad, value=1 - b2)
                denom = (st["v"].sqrt() / math.sqrt(bc2)).add_(self.eps)
                per_lr = self.per_lr if (self.per_lr is not None and p.shape == self.per_lr.shape) else None
                if per_lr is not None:
                    p.addcdiv_(st["m"] * per_lr, denom, value=-lr / bc1)
                else:
                    p.addcdiv_(st["m"], denom, value=-lr / bc1)


def tv_add_grad(grid_param, weight, world_size_max, dense_mode, mask=None):
    """Voxurf.*_total_variation_add_grad (voxurf_fine.py:403-409) -> grid.py:67-78."""
    w = weight * world_size_max / 128
    if grid_param.grad is None:
        grid_param.grad = torch.zeros_like(grid_param)
    if grid_param.dtype == torch.float32:
        if mask is None:
            TotalVariationOracle.total_variation_add_grad(grid_param.data, grid_param.grad, w, w, w, dense_mode)
        else:
            TotalVariationOracle.total_variation_add_grad_new(grid_param.data, grid_param.grad, mask, w, w, w,
                                                              dense_mode)
    else:
        tv_add_grad_torch(grid_param.data, grid_param.grad, w, w, w, dense_mode, mask)


def total_variation_loss(v: torch.Tensor, mask=None, mode: int = 1) -> torch.Tensor:
    """total_variation(v, mask) of the model files: the absolute forward
    differences along X, Y and Z, restricted to the pairs whose two voxels
    are in the mask (the mask holds v's channels, or one channel that is
    repeated).  mode 0, lib/voxurf_coarse.py:702-715: the three sums over 3
    x the mask's entries; mode 1, lib/voxurf_fine.py:956-969 (the maskless
    models hold copies): the mean of each axis's selection, averaged."""
    C = v.shape[1]
    if mask is not None and mask.shape[1] != C:
        mask = mask.expand(-1, C, -1, -1, -1)
    sums, means = [], []
    for dim in (2, 3, 4):
        n = v.shape[dim]
        d = (v.narrow(dim, 1, n - 1) - v.narrow(dim, 0, n - 1)).abs()
        if mask is not None:
            d = d[mask.narrow(dim, 0, n - 1) & mask.narrow(dim, 1, n - 1)]
        sums.append(d.sum())
        means.append(d.mean())
    if mode == 0:
        return (sums[0] + sums[1] + sums[2]) / 3 / mask.sum()
    return (means[0] + means[1] + means[2]) / 3
