"""Generates the golden vectors of tests/golden/ by running the REFERENCE
Voxurf Python code (lib/voxurf_fine.py, lib/voxurf_coarse.py, lib/grid.py,
lib/utils.py) on the CPU in float64.

Run in a container that has the reference sources, with their path in
$VOXURF_REFERENCE; the GPU machine never runs this.  The reference imports
several packages that are absent here and JIT-builds CUDA extensions; this
script stubs them:
  * cv2, mcubes, matplotlib, plyfile, imageio, skimage, trimesh, lpips ->
    empty modules (imported, never used on this path);
  * torch_scatter.segment_coo(src, index, out, reduce='sum') ->
    out.index_add(0, index, src) (same sum);
  * torch.utils.cpp_extension.load -> the oracle's restatement of the CUDA
    ops (oracle/ops.py), since no GPU exists here;
  * Tensor.cuda / Module.cuda -> no-ops;
  * torch.load -> weights_only=False (the torch 1.10 behaviour the
    reference's checkpoint loading relies on).
PYTHONDONTWRITEBYTECODE keeps the read-only reference tree clean.

    VOXURF_REFERENCE=<reference checkout> python tests/golden/make_golden.py [ops] [fine] [coarse] [mesh] [ckpt] [bg] [womask] [womask_coarse] [tv]
    (default: all)
"""
from __future__ import annotations

import importlib.abc
import importlib.machinery
import os
import sys
import types

os.environ["PYTHONDONTWRITEBYTECODE"] = "1"
sys.dont_write_bytecode = True

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("VOXURF_REFERENCE")
sys.path.insert(0, REPO)

from oracle import cref  # noqa: E402
from oracle.ops import RenderUtilsOracle, TotalVariationOracle  # noqa: E402

STUBS = ("cv2", "mcubes", "matplotlib", "matplotlib.pyplot", "matplotlib.cm", "plyfile", "imageio", "skimage",
         "skimage.measure", "trimesh", "lpips", "mmcv")


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, name, path, target=None):
        if name in STUBS:
            return importlib.machinery.ModuleSpec(name, self, is_package=True)
        return None

    def create_module(self, spec):
        m = types.ModuleType(spec.name)
        m.__path__ = []

        def _attr(attr):
            if attr.startswith("__"):
                raise AttributeError(attr)
            return type(attr, (), {})

        m.__getattr__ = _attr
        return m

    def exec_module(self, module):
        pass


def install_stubs():
    sys.meta_path.insert(0, _StubFinder())
    ts = types.ModuleType("torch_scatter")

    def segment_coo(src, index, out=None, reduce="sum"):
        assert reduce == "sum"
        return out.to(src.dtype).index_add(0, index, src)

    ts.segment_coo = segment_coo
    sys.modules["torch_scatter"] = ts
    import torch.utils.cpp_extension as cpp

    def fake_load(name, sources=None, verbose=False, **kw):
        if name == "render_utils_cuda":
            return RenderUtilsOracle
        if name == "total_variation_cuda":
            return TotalVariationOracle
        if name == "ub360_utils_cuda":
            return types.SimpleNamespace(
                cumdist_thres=lambda dist, thres: torch.from_numpy(cref.cumdist_thres(dist.numpy(), float(thres))))
        return types.SimpleNamespace()

    cpp.load = fake_load
    # like a real .cuda(), a Parameter comes back as a plain tensor (so the
    # reference's `self.s_val = nn.Parameter(...).cuda()` stays unregistered
    # and float32 under model.double(), voxurf_fine.py:61)
    torch.Tensor.cuda = lambda self, *a, **k: self.data if isinstance(self, torch.nn.Parameter) else self
    torch.nn.Module.cuda = lambda self, *a, **k: self
    # the reference targets torch 1.10, whose torch.load unpickles the numpy
    # arrays run.py stores in checkpoints (MaskCache_kwargs['xyz_min'], ...)
    _load = torch.load
    torch.load = lambda *a, **k: _load(*a, **{"weights_only": False, **k})
    if not REF or not os.path.isdir(os.path.join(REF, "lib")):
        raise SystemExit("set VOXURF_REFERENCE to a checkout of the reference (the directory holding lib/)")
    sys.path.insert(0, REF)


def _state_from_ours(model):
    sd = {k: v.detach().cpu().contiguous() for k, v in model.state_dict().items()}
    return sd


def fine_step_fixture(path, R=16, n_rays=128, width=64, mask_voxels=3.0, bg=1, seed=3):
    """One fine-stage training step of the reference model in float64."""
    import lib.grid as rgrid
    import lib.voxurf_fine as rf
    from voxurf_gb300 import configs, synthetic
    from voxurf_gb300.grid import MaskGrid

    ours = configs.build_fine_model(R, "fp32", device="cpu", seed=seed, width=width, mask_voxels=None)
    kw = configs.fine_model_kwargs(R, "fp32", width)
    kw.pop("precision")
    ref = rf.Voxurf(**kw)
    sd = _state_from_ours(ours)
    missing, unexpected = ref.load_state_dict(sd, strict=False)
    assert not unexpected, unexpected
    # mask |SDF| < mask_voxels voxels through the reference's MaskGrid, then the
    # reference's own non-empty-mask initialisation (voxurf_fine.py:353-367)
    mask_bool = ref.sdf.grid.detach()[0, 0].abs() < mask_voxels * 2.0 / R
    ref.mask_cache = rgrid.MaskGrid(mask=mask_bool, xyz_min=kw["xyz_min"], xyz_max=kw["xyz_max"])
    ref._set_nonempty_mask()
    sd = {k: v for k, v in ref.state_dict().items()}
    sd["mask_cache.mask"] = mask_bool
    ref = ref.double()
    ro, rd, vd = synthetic.random_rays(n_rays, seed=seed + 11)
    tgt = configs.train_targets(n_rays, seed)
    rk = dict(configs.FINE_RENDER_KWARGS, bg=bg)
    T = lambda a: torch.from_numpy(a).double()
    ret = ref(T(ro), T(rd), T(vd), global_step=1, **rk)
    # run.py:604-636 with the fine dtu_e2e weights (main 1, entropy_last 1e-3, rgb0 0.5)
    target = T(tgt)
    loss = 1.0 * torch.nn.functional.mse_loss(ret["rgb_marched"], target)
    pout = ret["alphainv_cum"][..., -1].clamp(1e-6, 1 - 1e-6)
    loss = loss + 0.001 * (-(pout * torch.log(pout) + (1 - pout) * torch.log(1 - pout)).mean())
    loss = loss + torch.nn.functional.mse_loss(ret["rgb_marched0"], target) * 0.5
    loss.backward()
    out = {
        "R": R, "n_rays": n_rays, "width": width, "mask_voxels": mask_voxels, "bg": bg, "seed": seed,
        "rays_o": ro, "rays_d": rd, "viewdirs": vd, "target": tgt,
        "rgb_marched": ret["rgb_marched"].detach().numpy(), "rgb_marched0": ret["rgb_marched0"].detach().numpy(),
        "alphainv_cum": ret["alphainv_cum"].detach().numpy(), "weights": ret["weights"].detach().numpy(),
        "loss": np.array(loss.item()),
        "grad_sdf": ref.sdf.grid.grad.numpy(), "grad_k0": ref.k0.grid.grad.numpy(),
    }
    for name, p in list(ref.rgbnet.named_parameters()) + [("k." + n, p) for n, p in ref.k_rgbnet.named_parameters()]:
        out["grad_mlp." + name] = p.grad.numpy()
    for k, v in sd.items():
        if v.dtype.is_floating_point:
            out["state." + k] = v.float().numpy()
        elif v.dtype == torch.bool:
            out["state." + k] = v.numpy()
    np.savez_compressed(path, **out)
    print("wrote", path, "shaded samples", ret["weights"].numel())


def coarse_step_fixture(path, R=16, n_rays=128, width=32, bg=1, seed=4):
    """One coarse-stage training step of the reference model in float64
    (lib/voxurf_coarse.py:513-619, loss of run.py:604-610)."""
    import lib.voxurf_coarse as rc
    from voxurf_gb300 import configs, synthetic

    ours = configs.build_coarse_model(R, "fp32", device="cpu", seed=seed, width=width)
    kw = configs.coarse_model_kwargs(R, "fp32", width)
    kw.pop("precision")
    ref = rc.Voxurf(**kw)
    sd = _state_from_ours(ours)
    missing, unexpected = ref.load_state_dict(sd, strict=False)
    assert not unexpected, unexpected
    sd = {k: v for k, v in ref.state_dict().items()}
    ref = ref.double()
    ro, rd, vd = synthetic.random_rays(n_rays, seed=seed + 11)
    tgt = configs.train_targets(n_rays, seed)
    rk = dict(configs.COARSE_RENDER_KWARGS, bg=bg)
    T = lambda a: torch.from_numpy(a).double()
    # voxurf_coarse.py:329 allocates the gradient grid with the default dtype,
    # so the float64 run needs float64 as the default (which also makes the
    # reference's inv_s = ones(1)/s_val float64 here, voxurf_coarse.py:360)
    torch.set_default_dtype(torch.float64)
    try:
        ret = ref(T(ro), T(rd), T(vd), global_step=1, **rk)
    finally:
        torch.set_default_dtype(torch.float32)
    target = T(tgt)
    loss = torch.nn.functional.mse_loss(ret["rgb_marched"], target)
    pout = ret["alphainv_cum"][..., -1].clamp(1e-6, 1 - 1e-6)
    loss = loss + 0.001 * (-(pout * torch.log(pout) + (1 - pout) * torch.log(1 - pout)).mean())
    loss.backward()
    out = {"R": R, "n_rays": n_rays, "width": width, "bg": bg, "seed": seed, "rays_o": ro, "rays_d": rd,
           "viewdirs": vd, "target": tgt, "rgb_marched": ret["rgb_marched"].detach().numpy(),
           "alphainv_cum": ret["alphainv_cum"].detach().numpy(), "weights": ret["weights"].detach().numpy(),
           "loss": np.array(loss.item()), "grad_sdf": ref.sdf.grid.grad.numpy(), "grad_k0": ref.k0.grid.grad.numpy()}
    for name, p in ref.rgbnet.named_parameters():
        out["grad_mlp." + name] = p.grad.numpy()
    for k, v in sd.items():
        if v.dtype.is_floating_point:
            out["state." + k] = v.float().numpy()
    np.savez_compressed(path, **out)
    print("wrote", path, "shaded samples", ret["weights"].numel())


def ops_fixture(path, seed=5):
    """Reference torch code for individual pieces of the path."""
    import lib.grid as rgrid
    import lib.utils as rutils
    import lib.voxurf_fine as rf

    g = torch.Generator().manual_seed(seed)
    out = {}
    # (1) cumprod_exclusive / get_ray_marching_ray (voxurf_fine.py:947-954):
    # weights of rays that never reach T < 1e-3
    alpha = torch.rand((64, 100), generator=g, dtype=torch.float64) * 0.02
    w, alphainv_cum = rf.get_ray_marching_ray(alpha)
    out.update({"march_alpha": alpha.numpy(), "march_weights": w.numpy(), "march_alphainv": alphainv_cum.numpy()})
    # (2) utils.Adam (utils.py:54-199) incl. per-voxel lr on the first param
    p0 = torch.randn((4, 5, 6), generator=g)
    p1 = torch.randn((33,), generator=g)
    params = [torch.nn.Parameter(p0.clone()), torch.nn.Parameter(p1.clone())]
    opt = rutils.Adam([{"params": [params[0]], "lr": 1e-2}, {"params": [params[1]], "lr": 3e-3}], betas=(0.9, 0.99))
    count = torch.randint(1, 9, (4, 5, 6), generator=g)
    opt.set_pervoxel_lr(count)
    grads = []
    for it in range(3):
        gs = [torch.randn(p.shape, generator=g) * 1e-2 for p in params]
        grads.append(gs)
        for p, gg in zip(params, gs):
            p.grad = gg.clone()
        opt.step()
    out.update({"adam_p0": p0.numpy(), "adam_p1": p1.numpy(), "adam_count": count.numpy(),
                "adam_grads0": np.stack([gs[0].numpy() for gs in grads]),
                "adam_grads1": np.stack([gs[1].numpy() for gs in grads]),
                "adam_out0": params[0].detach().numpy(), "adam_out1": params[1].detach().numpy()})
    # (3) DenseGrid.forward (grid.py:47-58)
    dg = rgrid.DenseGrid(channels=5, world_size=torch.tensor([7, 9, 11]), xyz_min=[-1.0, -0.5, -2.0],
                         xyz_max=[1.0, 1.5, 0.5])
    dg.grid.data = torch.randn((1, 5, 7, 9, 11), generator=g)
    xyz = torch.rand((500, 3), generator=g) * torch.tensor([2.4, 2.4, 2.9]) + torch.tensor([-1.2, -0.7, -2.2])
    out.update({"dg_grid": dg.grid.data.numpy(), "dg_xyz": xyz.numpy(), "dg_out": dg(xyz).detach().numpy()})
    # (4) Gaussian smoothing (voxurf_fine.py:246-258) and the central-difference
    #     gradient grid (voxurf_fine.py:440-450)
    sdf = torch.randn((1, 1, 12, 10, 14), generator=g)
    holder = types.SimpleNamespace(sdf=types.SimpleNamespace(grid=sdf), voxel_size=torch.tensor(0.0625))
    conv = rf.Voxurf._gaussian_3dconv(holder, ksize=5, sigma=0.8)
    out.update({"smooth_in": sdf.numpy(), "smooth_out": conv(sdf).detach().numpy()})
    holder.grad_mode = "interpolate"
    gradient = rf.Voxurf.neus_sdf_gradient(holder, mode="interpolate", sdf=sdf)
    out.update({"sdfgrad_out": gradient.numpy(), "sdfgrad_voxel": np.array(0.0625)})
    np.savez_compressed(path, **out)
    print("wrote", path)


def mesh_fixture(path, seed=6):
    """extract_fields (lib/dvgo_ori.py:679-693) with the fine model's mesh
    query (voxurf_fine.py:894-910: grid_sampler(pts, -sdf_grid) on the grid
    smoothed by init_smooth_conv_test_k3, sigma 0.5), in FP32 as the
    reference runs it, with 8^3 chunks so that chunk borders are covered."""
    import lib.dvgo_ori as rdvgo
    import lib.voxurf_fine as rf

    g = torch.Generator().manual_seed(seed)
    sdf = torch.randn((1, 1, 11, 13, 9), generator=g)
    holder = types.SimpleNamespace(sdf=types.SimpleNamespace(grid=sdf), nearest=False,
                                   xyz_min=torch.tensor([-1.0, -0.8, -1.2]), xyz_max=torch.tensor([1.1, 0.9, 0.7]))
    conv = rf.Voxurf._gaussian_3dconv(holder, ksize=3, sigma=0.5)
    with torch.no_grad():
        grid_s = conv(sdf)
    bmin, bmax = torch.tensor([-0.9, -0.7, -1.0]), torch.tensor([1.0, 0.85, 0.6])
    u = rdvgo.extract_fields(bmin, bmax, 21, lambda pts: rf.Voxurf.grid_sampler(holder, pts, -grid_s), N=8)
    np.savez_compressed(path, sdf=sdf.numpy(), xyz_min=holder.xyz_min.numpy(), xyz_max=holder.xyz_max.numpy(),
                        bound_min=bmin.numpy(), bound_max=bmax.numpy(), resolution=np.array(21), sigma=np.array(0.5),
                        field=u)
    print("wrote", path)


def ckpt_fixture(dirpath, R=16, seed=7):
    """Checkpoints in run.py's format (run.py:786-793) written by the
    reference models, and the reference's answers on them:
      coarse_last.tar  a coarse model (lib/voxurf_coarse.py) whose density
                       is high within |sdf| < 0.3 (the mask cache source);
      fine_last.tar    a fine model (lib/voxurf_fine.py) built with
                       mask_cache_path = coarse_last.tar (MaskCache,
                       _set_nonempty_mask applied to its SDF);
      ckpt_golden.npz  MaskCache point queries (and the alphas, for ties),
                       hit_coarse_geo of 256 rays, and a FP32 forward of
                       the fine model (rgb, shaded-sample count)."""
    import lib.voxurf_coarse as rc
    import lib.voxurf_fine as rf
    from voxurf_gb300 import configs, synthetic

    torch.manual_seed(seed)
    kw = configs.coarse_model_kwargs(R, "fp32", 32)
    kw.pop("precision")
    coarse = rc.Voxurf(**kw)
    ours = configs.build_coarse_model(R, "fp32", device="cpu", seed=seed, width=32)
    coarse.load_state_dict(_state_from_ours(ours), strict=False)
    with torch.no_grad():
        coarse.density.data = (10.0 * (0.3 - coarse.sdf.grid.detach().abs())).clone()
    ckpt_c = os.path.join(dirpath, "coarse_last.tar")
    torch.save({"global_step": 1000, "model_kwargs": coarse.get_kwargs(),
                "MaskCache_kwargs": coarse.get_MaskCache_kwargs(), "model_state_dict": coarse.state_dict(),
                "optimizer_state_dict": {}}, ckpt_c)
    fkw = configs.fine_model_kwargs(R, "fp32", 32)
    fkw.pop("precision")
    fkw.update(mask_cache_path=ckpt_c, mask_cache_thres=1e-3)
    fine = rf.Voxurf(**fkw)
    fours = configs.build_fine_model(R, "fp32", device="cpu", seed=seed, width=32)
    sd = _state_from_ours(fours)
    fine.load_state_dict({k: v for k, v in sd.items() if not k.startswith("mask_cache")}, strict=False)
    fine._set_nonempty_mask()
    ckpt_f = os.path.join(dirpath, "fine_last.tar")
    torch.save({"global_step": 1000, "model_kwargs": fine.get_kwargs(),
                "MaskCache_kwargs": fine.get_MaskCache_kwargs(), "model_state_dict": fine.state_dict(),
                "optimizer_state_dict": {}}, ckpt_f)
    g = torch.Generator().manual_seed(seed)
    pts = torch.rand((4000, 3), generator=g) * 2.2 - 1.1
    mc = fine.mask_cache
    with torch.no_grad():
        inside = mc(pts)
        xyz = pts.reshape(1, 1, 1, -1, 3)
        ind_norm = ((xyz - mc.xyz_min) / (mc.xyz_max - mc.xyz_min)).flip((-1,)) * 2 - 1
        dens = torch.nn.functional.grid_sample(mc.density, ind_norm, align_corners=True)
        alpha = (1 - torch.exp(-torch.nn.functional.softplus(dens + mc.act_shift) * mc.voxel_size_ratio)).reshape(-1)
    ro, rd, vd = synthetic.random_rays(256, seed=seed + 1)
    T = lambda a: torch.from_numpy(a)
    rk = dict(configs.FINE_RENDER_KWARGS)
    with torch.no_grad():
        hit = fine.hit_coarse_geo(T(ro), T(rd), **rk)
        ret = fine(T(ro), T(rd), T(vd), global_step=1, **rk)
    np.savez_compressed(os.path.join(dirpath, "ckpt_golden.npz"), pts=pts.numpy(), inside=inside.numpy(),
                        alpha=alpha.numpy(), rays_o=ro, rays_d=rd, viewdirs=vd, hit=hit.numpy(),
                        rgb_marched=ret["rgb_marched"].numpy(), n_shaded=np.array(ret["weights"].numel()),
                        mask_cache_thres=np.array(1e-3))
    print("wrote", ckpt_c, ckpt_f, "shaded samples", ret["weights"].numel(), "hits", int(hit.sum()))


def tv_fixture(path, seed=21):
    """The loss-form total variation of the model files, called directly:
    lib/voxurf_coarse.py:702-715 (sum over 3 x the mask's entries) and
    lib/voxurf_fine.py:956-969 (per-axis means; the maskless models'
    copies, voxurf_womask_fine.py:1242-1255 and voxurf_womask_coarse.py:
    858-871, are the same statements), in float64 with their gradients by
    autograd.  Grids of 1 and 12 channels with quantised values (so that
    some neighbour differences are exactly zero), with a random voxel mask
    and, for the mean form, without one."""
    import lib.voxurf_coarse as rc
    import lib.voxurf_fine as rf

    g = torch.Generator().manual_seed(seed)
    out = {}
    for C, shape in ((1, (9, 10, 11)), (12, (7, 8, 9))):
        v = torch.randint(0, 5, (1, C, *shape), generator=g).double() / 4.0
        v = v + (torch.rand((1, C, *shape), generator=g, dtype=torch.float64) < 0.5) * torch.randn(
            (1, C, *shape), generator=g, dtype=torch.float64) * 0.1
        mask = torch.rand((1, 1, *shape), generator=g) < 0.7
        out[f"c{C}_v"] = v.numpy()
        out[f"c{C}_mask"] = mask.numpy()
        for name, fn, m in (("sum", rc.total_variation, mask), ("mean", rf.total_variation, mask),
                            ("mean_nomask", rf.total_variation, None)):
            x = v.clone().requires_grad_(True)
            mm = None if m is None else m.repeat(1, C, 1, 1, 1)
            loss = fn(x, mm)
            loss.backward()
            out[f"c{C}_{name}_loss"] = np.array(loss.item())
            out[f"c{C}_{name}_grad"] = x.grad.numpy()
    np.savez_compressed(path, **out)
    print("wrote", path)


def bg_fixture(path, seed=8):
    """Background samples of the models without an object mask: the
    reference's sample_ray_ori and outside_sphere_trans (womask fine
    :789-825, womask coarse :568-604) called on a holder object, then the
    mask and compaction statements of voxurf_womask_fine.py:860-870 and
    voxurf_womask_coarse.py:637-650 as written there, with cumdist_thres from
    the oracle (its CUDA source cannot run on the host).  The per-ray
    training jitter (torch.rand_like at :808) is fixed by the fixture."""
    import lib.voxurf_womask_coarse as wc
    import lib.voxurf_womask_fine as wf

    from oracle import cref

    g = torch.Generator().manual_seed(seed)
    n = 96
    o = torch.rand((n, 3), generator=g) * 3.2 - 1.6
    d = torch.randn((n, 3), generator=g)
    d[:6, 0] = 0.0   # zero direction components (the 1e-6 substitution)
    d[6:10, 1:] = 0.0
    d[10:14] = -o[10:14] + 0.05 * torch.randn((4, 3), generator=g)   # towards the centre
    jit = torch.rand((n,), generator=g)
    xyz_min, xyz_max = torch.tensor([-1.0, -1.0, -1.0]), torch.tensor([1.0, 1.0, 1.0])
    R, Rb, stepsize, near, far = 24, 20, 0.5, 0.2, 6.0
    vs = ((xyz_max - xyz_min).prod() / R ** 3).pow(1 / 3)
    vs_bg = ((xyz_max - xyz_min).prod() / Rb ** 3).pow(1 / 3)
    holder = types.SimpleNamespace(xyz_min=xyz_min, xyz_max=xyz_max, voxel_size=vs, voxel_size_bg=vs_bg,
                                   sdf=types.SimpleNamespace(grid=torch.zeros((1, 1, R, R, R))),
                                   bg_density=types.SimpleNamespace(grid=torch.zeros((1, 1, Rb, Rb, Rb))))
    ub = types.SimpleNamespace(cumdist_thres=lambda dist, thres: torch.from_numpy(
        cref.cumdist_thres(dist.numpy(), float(thres))))
    out = {"rays_o": o.numpy(), "rays_d": d.numpy(), "jitter": jit.numpy(), "xyz_min": xyz_min.numpy(),
           "xyz_max": xyz_max.numpy(), "near": np.float32(near), "far": np.float32(far),
           "stepsize": np.float32(stepsize), "voxel_size": vs.numpy(), "voxel_size_bg": vs_bg.numpy()}
    rand_like = torch.rand_like
    try:
        torch.rand_like = lambda x: jit[:, None].clone()
        for tag, mod, train in (("fine", wf, False), ("fine_train", wf, True), ("coarse", wc, True)):
            cls = mod.Voxurf
            use_bg = tag == "coarse"
            pts_org, mask_outbbox, _ = cls.sample_ray_ori(holder, o, d, near, far, stepsize, is_train=train,
                                                          use_bg=use_bg)
            # womask fine :860-868 / womask coarse :637-646
            pn = torch.linalg.norm(pts_org, ord=2, dim=-1, keepdim=True)
            inside = (pn < 1.0)[..., 0]
            inv = cls.outside_sphere_trans(holder, pts_org, pn, filtered=True)
            if use_bg:
                bg_mask = ~inside & mask_outbbox
                dist_thres = vs * stepsize * 0.95
            else:
                bg_mask = ~inside
                dist_thres = vs * stepsize * 0.5
            dist = (inv[:, 1:] - inv[:, :-1]).norm(dim=-1)
            bg_mask[:, 1:] &= ub.cumdist_thres(dist, dist_thres)
            out.update({f"{tag}_pts": pts_org.numpy(), f"{tag}_inv": inv.numpy(), f"{tag}_keep": bg_mask.numpy(),
                        f"{tag}_dist": dist.numpy(), f"{tag}_thres": np.float32(dist_thres)})
    finally:
        torch.rand_like = rand_like
    np.savez_compressed(path, **out)
    print("wrote", path)


def womask_step_fixture(path, R=16, R_bg=12, n_rays=96, width=32, seed=9):
    """One training step of the reference's maskless fine model
    (lib/voxurf_womask_fine.py:833-1071) in float64, loss of run.py:604-610
    and 627 (rgb_marched, entropy of alphainv_cum[-1], rgb_marched0 x 0.5).
    The two per-ray jitters of sample_ray_ori (torch.rand_like at :808, once
    for the foreground samples, once for the background samples) are fixed
    by the fixture; global_step 1 also runs _set_sphere_nonempty_mask."""
    import lib.voxurf_womask_fine as rw
    from voxurf_gb300 import configs, synthetic

    ours = configs.build_womask_model(R, "fp32", device="cpu", seed=seed, width=width, R_bg=R_bg)
    kw = configs.womask_model_kwargs(R, "fp32", width, R_bg)
    kw.pop("precision")
    ref = rw.Voxurf(**kw)
    sd = _state_from_ours(ours)
    missing, unexpected = ref.load_state_dict(sd, strict=False)
    assert not unexpected, unexpected
    sd = {k: v for k, v in ref.state_dict().items()}
    ref = ref.double()
    ro, rd, vd = synthetic.random_rays(n_rays, seed=seed + 11)
    tgt = configs.train_targets(n_rays, seed)
    g = torch.Generator().manual_seed(seed + 5)
    jit = torch.rand((2, n_rays), generator=g)
    rk = dict(configs.FINE_RENDER_KWARGS, bg=1)
    T = lambda a: torch.from_numpy(a).double()
    calls = []
    rand_like = torch.rand_like

    def fixed_rand_like(x):
        calls.append(x.shape)
        return jit[len(calls) - 1][:, None].to(x.dtype).clone()

    torch.rand_like = fixed_rand_like
    try:
        ret = ref(T(ro), T(rd), T(vd), global_step=1, **rk)
    finally:
        torch.rand_like = rand_like
    assert len(calls) == 2, calls
    target = T(tgt)
    loss = torch.nn.functional.mse_loss(ret["rgb_marched"], target)
    pout = ret["alphainv_cum"][..., -1].clamp(1e-6, 1 - 1e-6)
    loss = loss + 0.001 * (-(pout * torch.log(pout) + (1 - pout) * torch.log(1 - pout)).mean())
    loss = loss + torch.nn.functional.mse_loss(ret["rgb_marched0"], target) * 0.5
    loss.backward()
    out = {"R": R, "R_bg": R_bg, "n_rays": n_rays, "width": width, "seed": seed, "rays_o": ro, "rays_d": rd,
           "viewdirs": vd, "target": tgt, "jitter": jit.numpy(),
           "rgb_marched": ret["rgb_marched"].detach().numpy(), "rgb_marched0": ret["rgb_marched0"].detach().numpy(),
           "alphainv_cum": ret["alphainv_cum"].detach().numpy(), "in_marched": ret["in_marched"].detach().numpy(),
           "out_marched": ret["out_marched"].detach().numpy(), "n_weights": np.array(ret["weights"].numel()),
           "n_bg_weights": np.array(ret["bg_weights"].numel()), "loss": np.array(loss.item())}
    for name in ("sdf", "k0", "bg_density", "bg_k0"):
        out["grad_" + name] = getattr(ref, name).grid.grad.numpy()
    for net in ("rgbnet", "k_rgbnet", "bg_rgbnet"):
        for n, p in getattr(ref, net).named_parameters():
            out[f"grad_{net}.{n}"] = p.grad.numpy()
    for k, v in sd.items():
        if v.dtype.is_floating_point:
            out["state." + k] = v.float().numpy()
    np.savez_compressed(path, **out)
    print("wrote", path, "fg samples", ret["weights"].numel(), "bg samples", ret["bg_weights"].numel())


def womask_coarse_step_fixture(path, R=16, R_bg=12, n_rays=96, width=32, seed=13):
    """One training step of the reference's maskless coarse model
    (lib/voxurf_womask_coarse.py:611-780) in float64 with the
    dtu_e2e_womask coarse settings (no bg_k0), loss of run.py:604-610
    (rgb_marched and the entropy of alphainv_cum[-1]).  The per-ray jitter
    of the background samples (torch.rand_like at :587, the one draw of the
    step: the foreground samples come from sample_ray_cuda) is fixed by the
    fixture; global_step 1 also runs _set_sphere_nonempty_mask."""
    import lib.voxurf_womask_coarse as rw
    from voxurf_gb300 import configs, synthetic

    ours = configs.build_womask_coarse_model(R, "fp32", device="cpu", seed=seed, width=width, R_bg=R_bg)
    kw = configs.womask_coarse_model_kwargs(R, "fp32", width, R_bg)
    kw.pop("precision")
    ref = rw.Voxurf(**kw)
    sd = _state_from_ours(ours)
    missing, unexpected = ref.load_state_dict(sd, strict=False)
    assert not unexpected, unexpected
    sd = {k: v for k, v in ref.state_dict().items()}
    ref = ref.double()
    ro, rd, vd = synthetic.random_rays(n_rays, seed=seed + 11)
    tgt = configs.train_targets(n_rays, seed)
    g = torch.Generator().manual_seed(seed + 5)
    jit = torch.rand((n_rays,), generator=g)
    rk = dict(configs.COARSE_RENDER_KWARGS, bg=1)
    T = lambda a: torch.from_numpy(a).double()
    calls = []
    rand_like = torch.rand_like

    def fixed_rand_like(x):
        calls.append(x.shape)
        return jit[:, None].to(x.dtype).clone()

    torch.rand_like = fixed_rand_like
    # the gradient grid and inv_s take the default dtype (voxurf_womask_coarse.py:457, 490)
    torch.set_default_dtype(torch.float64)
    try:
        ret = ref(T(ro), T(rd), T(vd), global_step=1, **rk)
    finally:
        torch.rand_like = rand_like
        torch.set_default_dtype(torch.float32)
    assert len(calls) == 1, calls
    target = T(tgt)
    loss = torch.nn.functional.mse_loss(ret["rgb_marched"], target)
    pout = ret["alphainv_cum"][..., -1].clamp(1e-6, 1 - 1e-6)
    loss = loss + 0.001 * (-(pout * torch.log(pout) + (1 - pout) * torch.log(1 - pout)).mean())
    loss.backward()
    out = {"R": R, "R_bg": R_bg, "n_rays": n_rays, "width": width, "seed": seed, "rays_o": ro, "rays_d": rd,
           "viewdirs": vd, "target": tgt, "jitter": jit.numpy(),
           "rgb_marched": ret["rgb_marched"].detach().numpy(), "alphainv_cum": ret["alphainv_cum"].detach().numpy(),
           "in_marched": ret["in_marched"].detach().numpy(), "out_marched": ret["out_marched"].detach().numpy(),
           "weights": ret["weights"].detach().numpy(), "bg_weights": ret["bg_weights"].detach().numpy(),
           "loss": np.array(loss.item())}
    for name in ("sdf", "k0", "bg_density"):
        out["grad_" + name] = getattr(ref, name).grid.grad.numpy()
    for net in ("rgbnet", "bg_rgbnet"):
        for n, p in getattr(ref, net).named_parameters():
            out[f"grad_{net}.{n}"] = p.grad.numpy()
    # the ori_tv regularisers of the coarse stage (run.py:617-626) on the
    # state of the same step: density_total_variation(sdf_tv=0.1,
    # smooth_grad_tv=0.05) + 0.01 k0_total_variation(), with tv_in_sphere
    # True (the unit-sphere voxel mask; the dtu_e2e_womask setting False
    # makes the mask all ones).  self.gradient comes from a second, identical
    # forward (the first one's graph is spent).
    for p in ref.parameters():
        p.grad = None
    ref.tv_in_sphere = True
    calls.clear()
    torch.rand_like = fixed_rand_like
    torch.set_default_dtype(torch.float64)
    try:
        ref(T(ro), T(rd), T(vd), global_step=1, **rk)
        tv = ref.density_total_variation(sdf_tv=0.1, smooth_grad_tv=0.05) + 0.01 * ref.k0_total_variation()
    finally:
        torch.rand_like = rand_like
        torch.set_default_dtype(torch.float32)
    tv.backward()
    out["tv_loss"] = np.array(tv.item())
    out["tv_grad_sdf"] = ref.sdf.grid.grad.numpy()
    out["tv_grad_k0"] = ref.k0.grid.grad.numpy()
    for k, v in sd.items():
        if v.dtype.is_floating_point:
            out["state." + k] = v.float().numpy()
    np.savez_compressed(path, **out)
    print("wrote", path, "fg samples", ret["weights"].numel(), "bg samples", ret["bg_weights"].numel(),
          "tv", tv.item())


def main():
    install_stubs()
    torch.set_default_dtype(torch.float32)
    which = sys.argv[1:] or ["ops", "fine", "coarse", "mesh", "ckpt", "bg", "womask", "womask_coarse", "tv"]
    # VOXURF_GOLDEN_OUT: write elsewhere (tests/test_golden_reproducible.py
    # regenerates into a temporary directory and compares)
    out = os.environ.get("VOXURF_GOLDEN_OUT", HERE)
    os.makedirs(out, exist_ok=True)
    if "ops" in which:
        ops_fixture(os.path.join(out, "ops_golden.npz"))
    if "fine" in which:
        fine_step_fixture(os.path.join(out, "fine_step_golden.npz"))
    if "coarse" in which:
        coarse_step_fixture(os.path.join(out, "coarse_step_golden.npz"))
    if "mesh" in which:
        mesh_fixture(os.path.join(out, "mesh_golden.npz"))
    if "ckpt" in which:
        ckpt_fixture(out)
    if "bg" in which:
        bg_fixture(os.path.join(out, "bg_golden.npz"))
    if "womask" in which:
        womask_step_fixture(os.path.join(out, "womask_step_golden.npz"))
    if "womask_coarse" in which:
        womask_coarse_step_fixture(os.path.join(out, "womask_coarse_step_golden.npz"))
    if "tv" in which:
        tv_fixture(os.path.join(out, "tv_golden.npz"))


if __name__ == "__main__":
    main()
