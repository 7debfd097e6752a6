"""Fused fine-model step (forward + hand-written backward) against the FP64
oracle restatement of the reference step on the same seeded inputs.

Tolerances (plain FP32 path): rendered RGB max abs error <= 1e-5, gradients
of the SDF grid, the k0 grid and every MLP weight rel-L2 <= 1e-5.  The set
of shaded samples (count and ray order) must match exactly.  Mixed BF16 path:
RGB max abs error <= 1e-3.
"""
import numpy as np
import pytest
import torch

from oracle.voxurf_oracle import OracleFine, train_loss
from voxurf_gb300 import configs, synthetic

pytestmark = pytest.mark.gpu

RK = dict(configs.FINE_RENDER_KWARGS)


def _rel_l2(a, b):
    a = a.detach().double().cpu().reshape(-1)
    b = b.detach().double().cpu().reshape(-1)
    return float((a - b).norm() / (b.norm() + 1e-30))


def _setup(cuda, R=32, n_rays=256, precision="fp32", mask_voxels=None, seed=0, bg=0, scene="sphere_torus"):
    model = configs.build_fine_model(R, precision, device=cuda, seed=seed, mask_voxels=mask_voxels, scene=scene)
    oracle = OracleFine(model, dtype=torch.float64)
    ro, rd, vd = synthetic.random_rays(n_rays, seed=seed + 11)
    tgt = configs.train_targets(n_rays, seed)
    rk = dict(RK, bg=bg)
    return model, oracle, (ro, rd, vd, tgt), rk


def _run_gpu(model, rays, rk, step=1):
    ro, rd, vd, tgt = (torch.from_numpy(a).cuda() for a in rays)
    ret = model(ro, rd, vd, global_step=step, **rk)
    loss = train_loss(ret, tgt)
    loss.backward()
    torch.cuda.synchronize()
    return ret, loss


def _run_oracle(oracle, rays, rk, step=1):
    ro, rd, vd, tgt = (torch.from_numpy(a) for a in rays)
    ret = oracle(ro, rd, vd, global_step=step, **rk)
    loss = train_loss(ret, tgt.double())
    loss.backward()
    return ret, loss


@pytest.mark.parametrize("mask_voxels,bg", [(None, 0), (3.0, 1), (None, 1)])
def test_fine_step_fp32_matches_fp64_oracle(cuda, mask_voxels, bg):
    model, oracle, rays, rk = _setup(cuda, mask_voxels=mask_voxels, bg=bg)
    g, gl = _run_gpu(model, rays, rk)
    o, ol = _run_oracle(oracle, rays, rk)
    # identical shaded sample set, ray-major
    assert g["weights"].numel() == o["weights"].numel() > 100
    assert torch.equal(g["ray_id"].long().cpu(), o["ray_id"])
    np.testing.assert_allclose(g["weights"].detach().cpu().numpy(), o["weights"].detach().numpy(), rtol=0, atol=2e-6)
    np.testing.assert_allclose(g["alphainv_cum"].detach().cpu().numpy(), o["alphainv_cum"].detach().numpy(), rtol=0,
                               atol=2e-6)
    for key in ("rgb_marched", "rgb_marched0"):
        err = (g[key].double().cpu() - o[key]).abs().max().item()
        assert err <= 1e-5, (key, err)
    assert abs(gl.item() - ol.item()) <= 1e-6 * max(1.0, abs(ol.item()))
    # gradients
    assert _rel_l2(model.sdf.grid.grad, oracle.sdf_grid.grad) <= 1e-5
    assert _rel_l2(model.k0.grid.grad, oracle.k0_grid.grad) <= 1e-5
    for (n, p), (_, q) in zip(model.rgbnet.named_parameters(), oracle.rgbnet.named_parameters()):
        assert _rel_l2(p.grad, q.grad) <= 1e-5, ("rgbnet", n)
    for (n, p), (_, q) in zip(model.k_rgbnet.named_parameters(), oracle.k_rgbnet.named_parameters()):
        assert _rel_l2(p.grad, q.grad) <= 1e-5, ("k_rgbnet", n)


def test_fine_render_extras(cuda):
    model, oracle, rays, rk = _setup(cuda)
    rk = dict(rk, render_depth=True, render_grad=True)
    ro, rd, vd, _ = (torch.from_numpy(a).cuda() for a in rays)
    with torch.no_grad():
        g = model(ro, rd, vd, global_step=None, **rk)
    o = oracle(*(torch.from_numpy(a) for a in rays[:3]), global_step=None, **rk)
    assert (g["depth"].double().cpu() - o["depth"]).abs().max().item() <= 1e-5
    assert (g["normal_marched"].double().cpu() - o["normal_marched"]).abs().max().item() <= 1e-5
    assert (g["rgb_marched"].double().cpu() - o["rgb_marched"].detach()).abs().max().item() <= 1e-5


def test_fine_step_bf16_rgb_error(cuda):
    model, oracle, rays, rk = _setup(cuda, precision="bf16")
    g, _ = _run_gpu(model, rays, rk)
    o, _ = _run_oracle(oracle, rays, rk)
    err = (g["rgb_marched"].double().detach().cpu() - o["rgb_marched"].detach()).abs().max().item()
    assert err <= 1e-3, err
    # BF16 GEMMs bound the gradient agreement with FP64 at the percent level
    assert _rel_l2(model.sdf.grid.grad, oracle.sdf_grid.grad) <= 1e-1
    assert _rel_l2(model.k0.grid.grad, oracle.k0_grid.grad) <= 1e-1


def test_fine_forward_no_rays_hit(cuda):
    model = configs.build_fine_model(32, device=cuda)
    o = torch.tensor([[5.0, 5.0, 5.0]] * 4, device=cuda)
    d = torch.tensor([[1.0, 1.0, 1.0]] * 4, device=cuda)
    ret = model(o, d, d / d.norm(dim=-1, keepdim=True), global_step=1, **RK)
    assert ret["weights"].numel() == 0
    assert torch.all(ret["alphainv_cum"] == 1)
    assert torch.all(ret["rgb_marched"] == 0)


@pytest.mark.parametrize("masked", [True, False])
def test_smooth_grad_tv_matches_oracle(cuda, masked):
    """density_total_variation(smooth_grad_tv) (voxurf_fine.py:417-420): value
    and SDF-grid gradient against the FP64 restatement."""
    model = configs.build_fine_model(24, device=cuda, seed=5, mask_voxels=4.0 if masked else None)
    oracle = OracleFine(model, dtype=torch.float64)
    loss = model.density_total_variation(smooth_grad_tv=0.05)
    loss.backward()
    ol = oracle.smooth_grad_tv(model.nonempty_mask, 0.05)
    ol.backward()
    assert abs(loss.item() - ol.item()) <= 1e-5 * abs(ol.item())
    assert _rel_l2(model.sdf.grid.grad, oracle.sdf_grid.grad) <= 1e-5


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("bf16", 1e-3)])
def test_long_rays_match_fp64_oracle(cuda, precision, tol):
    """Long-ray workload at a size the oracle finishes quickly: 64 random
    spheres on a 128^3 grid, stepsize 0.25 voxel (up to 700 samples per ray,
    74 of the 192 rays beyond 512), s-density 0.05 (global_step 0).  Same
    shaded-sample set, RGB within tol; FP32 gradients rel-L2 <= 1e-5."""
    R = 128
    model = configs.build_fine_model(R, precision, device=cuda, seed=7, scene="spheres64", width=32)
    oracle = OracleFine(model, dtype=torch.float64)
    ro, rd, vd = synthetic.random_rays(192, seed=31)
    rays = (ro, rd, vd, configs.train_targets(192, 31))
    rk = dict(RK, stepsize=0.25)
    g, gl = _run_gpu(model, rays, rk, step=0)
    o, ol = _run_oracle(oracle, rays, rk, step=0)
    from oracle.ops import RenderUtilsOracle

    stepdist = float(np.float32(0.25) * np.float32(model.voxel_size.item()))
    n_steps = RenderUtilsOracle.sample_pts_on_rays(torch.from_numpy(ro), torch.from_numpy(rd), oracle.xyz_min32,
                                                   oracle.xyz_max32, rk["near"], 1e9, stepdist)[4]
    assert int(n_steps.max()) > 512, int(n_steps.max())   # rays marched beyond 512 samples
    if precision == "fp32":
        assert torch.equal(g["ray_id"].long().cpu(), o["ray_id"])
    err = (g["rgb_marched"].detach().double().cpu() - o["rgb_marched"].detach()).abs().max().item()
    assert err <= tol, err
    if precision == "fp32":
        assert _rel_l2(model.sdf.grid.grad, oracle.sdf_grid.grad) <= 1e-5
        assert _rel_l2(model.k0.grid.grad, oracle.k0_grid.grad) <= 1e-5
