"""Checkpoints written by the reference models in run.py's format
(tests/golden/make_golden.py `ckpt`): utils.load_model / load_checkpoint,
the MaskCache of a coarse checkpoint (trilinear max-pooled density as the
fine stage's known-free-space test, voxurf_fine.py:917-942) in the march
kernels, hit_coarse_geo and the maskcache training-ray sampler, and the
loaded scene in the render server.  Against the reference's own answers
(FP32, CPU) and the FP64 oracle."""
import os

import numpy as np
import pytest
import torch

from oracle.voxurf_oracle import OracleFine, maskcache_query, train_loss
from voxurf_gb300 import configs, grid as vgrid, serve, utils
from voxurf_gb300 import voxurf_coarse, voxurf_fine

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
COARSE = os.path.join(HERE, "coarse_last.tar")
FINE = os.path.join(HERE, "fine_last.tar")
GOLD = np.load(os.path.join(HERE, "ckpt_golden.npz"))
THRES = float(GOLD["mask_cache_thres"])


def _rel_l2(a, b):
    a = a.detach().double().cpu().reshape(-1)
    b = b.detach().double().cpu().reshape(-1)
    return float((a - b).norm() / (b.norm() + 1e-30))


def _fine(cuda):
    # run.py:1013 reloads with the config's model kwargs (get_kwargs stores
    # only part of them); the mask cache path is this machine's copy
    kw = configs.fine_model_kwargs(16, "fp32", 32)
    kw.pop("precision")
    kw.update(mask_cache_path=COARSE, mask_cache_thres=THRES)
    model = utils.load_model(voxurf_fine.Voxurf, FINE, new_kwargs=kw)
    return model.to(cuda)


def test_maskcache_points_vs_reference(cuda):
    mc = vgrid.MaskCache(path=COARSE, mask_cache_thres=THRES).to(cuda)
    got = mc(torch.from_numpy(GOLD["pts"]).to(cuda)).cpu().numpy()
    tie = np.abs(GOLD["alpha"] - THRES) <= 1e-6 * THRES
    assert np.array_equal(got[~tie], GOLD["inside"][~tie])
    assert tie.sum() <= 2


def test_load_model_state_and_nonempty_mask(cuda):
    model = _fine(cuda)
    st = torch.load(FINE, map_location="cpu", weights_only=False)["model_state_dict"]
    assert isinstance(model.mask_cache, vgrid.MaskCache)
    assert torch.equal(model.sdf.grid.detach().cpu(), st["sdf.grid"])
    assert torch.equal(model.k0.grid.detach().cpu().contiguous(), st["k0.grid"])
    assert model.k0.grid.is_contiguous(memory_format=torch.channels_last_3d)
    for n, p in model.rgbnet.named_parameters():
        assert torch.equal(p.detach().cpu(), st["rgbnet." + n])
    # the nonempty mask recomputed from the MaskCache equals the reference's
    # (up to threshold ties at FP32 rounding)
    assert int((model.nonempty_mask.cpu() != st["nonempty_mask"]).sum()) <= 2
    assert 0 < int(st["nonempty_mask"].sum()) < st["nonempty_mask"].numel()


def test_hit_coarse_geo_and_ray_sampling(cuda):
    model = _fine(cuda)
    rk = dict(configs.FINE_RENDER_KWARGS)
    hit = model.hit_coarse_geo(torch.from_numpy(GOLD["rays_o"]), torch.from_numpy(GOLD["rays_d"]), **rk)
    assert int((hit.cpu().numpy() != GOLD["hit"]).sum()) == 0
    # maskcache sampling over two small views: the kept rays are the hits
    from voxurf_gb300 import synthetic

    poses = synthetic.fibonacci_poses(2, 3.0)
    H, W = 24, 32
    K = synthetic.intrinsics(H, W)
    imgs = [torch.rand((H, W, 3), device=cuda) for _ in poses]
    rgb, o, d, v, imsz = voxurf_fine.get_training_rays_in_maskcache_sampling(
        imgs, [torch.as_tensor(p) for p in poses], [(H, W)] * 2, [K] * 2, False, True, False, False, model, rk)
    assert len(imsz) == 2 and rgb.shape[0] == o.shape[0] == sum(imsz) > 0
    assert bool(model.hit_coarse_geo(o, d, **rk).all())


def test_loaded_fine_forward_vs_reference_and_oracle(cuda):
    model = _fine(cuda)
    rk = dict(configs.FINE_RENDER_KWARGS)
    T = lambda a: torch.from_numpy(a).to(cuda)
    ret = model(T(GOLD["rays_o"]), T(GOLD["rays_d"]), T(GOLD["viewdirs"]), global_step=1, **rk)
    assert ret["weights"].numel() == int(GOLD["n_shaded"])
    np.testing.assert_allclose(ret["rgb_marched"].detach().cpu().numpy(), GOLD["rgb_marched"], atol=2e-5)
    # training step with the density mask in the march: gradients vs FP64
    tgt = configs.train_targets(len(GOLD["rays_o"]), 5)
    model.zero_grad(set_to_none=True)
    oracle = OracleFine(model)
    gl = train_loss(ret, T(tgt))
    gl.backward()
    o = oracle(*(torch.from_numpy(GOLD[k]) for k in ("rays_o", "rays_d", "viewdirs")), global_step=1, **rk)
    ol = train_loss(o, torch.from_numpy(tgt).double())
    ol.backward()
    assert o["weights"].numel() == ret["weights"].numel()
    assert (ret["rgb_marched"].double().detach().cpu() - o["rgb_marched"].detach()).abs().max().item() <= 1e-5
    assert _rel_l2(model.sdf.grid.grad, oracle.sdf_grid.grad) <= 1e-5
    assert _rel_l2(model.k0.grid.grad, oracle.k0_grid.grad) <= 1e-5


def test_loaded_scene_in_render_server(cuda):
    model = _fine(cuda)
    scene = serve.ResidentScene(model, s_val=0.01, precision="fp32")
    srv = serve.RenderServer([scene], tick_rays=1 << 14, arena_pixels=1 << 16)
    from voxurf_gb300 import synthetic

    c2w = np.asarray(synthetic.fibonacci_poses(3, 3.0)[1])
    rgb, depth = srv.render(0, c2w, 30, 40)
    model.s_val = torch.ones(1) * 0.01
    prgb, pdepth = serve.plain_render(model, c2w, 30, 40)
    assert np.abs(rgb - prgb.cpu().numpy()).max() <= 1e-5


def test_coarse_checkpoint_loads_and_renders(cuda):
    model = utils.load_model(voxurf_coarse.Voxurf, COARSE).to(cuda)
    st = torch.load(COARSE, map_location="cpu", weights_only=False)["model_state_dict"]
    assert torch.equal(model.density.detach().cpu(), st["density"])
    ro, rd, vd = (torch.from_numpy(GOLD[k]).to(cuda) for k in ("rays_o", "rays_d", "viewdirs"))
    ret = model(ro, rd, vd, global_step=1, **configs.COARSE_RENDER_KWARGS)
    assert torch.isfinite(ret["rgb_marched"]).all()
    # the same checkpoint as a mask cache answers like the oracle restatement
    mc = vgrid.MaskCache(path=COARSE, mask_cache_thres=THRES).to(cuda)
    pts = torch.from_numpy(GOLD["pts"])
    ref = maskcache_query(mc.density.cpu(), mc.xyz_min.cpu(), mc.xyz_max.cpu(), mc.act_shift, mc.voxel_size_ratio,
                          THRES, pts)
    tie = np.abs(GOLD["alpha"] - THRES) <= 1e-6 * THRES
    assert np.array_equal(mc(pts.to(cuda)).cpu().numpy()[~tie], ref.numpy()[~tie])
