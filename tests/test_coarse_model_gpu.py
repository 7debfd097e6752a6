"""Fused coarse-model step (lib/voxurf_coarse.py:513-619) against the FP64
oracle restatement: identical shaded-sample set, RGB max abs error <= 1e-5,
gradients rel-L2 <= 1e-5 (plain FP32)."""
import numpy as np
import pytest
import torch

from oracle.voxurf_oracle import OracleCoarse, train_loss
from voxurf_gb300 import configs, synthetic

pytestmark = pytest.mark.gpu


def _rel_l2(a, b):
    a = a.detach().double().cpu().reshape(-1)
    b = b.detach().double().cpu().reshape(-1)
    return float((a - b).norm() / (b.norm() + 1e-30))


@pytest.mark.parametrize("bg,R", [(0, 32), (1, 24)])
def test_coarse_step_fp32_matches_fp64_oracle(cuda, bg, R):
    model = configs.build_coarse_model(R, "fp32", device=cuda, seed=R)
    oracle = OracleCoarse(model)
    ro, rd, vd = synthetic.random_rays(256, seed=R + 3)
    tgt = configs.train_targets(256, R)
    rk = dict(configs.COARSE_RENDER_KWARGS, bg=bg)
    T = lambda a: torch.from_numpy(a).to(cuda)
    g = model(T(ro), T(rd), T(vd), global_step=1, **rk)
    gl = train_loss(g, T(tgt), weight_rgb0=0)
    gl.backward()
    o = oracle(*(torch.from_numpy(a) for a in (ro, rd, vd)), global_step=1, **rk)
    ol = train_loss(o, torch.from_numpy(tgt).double(), weight_rgb0=0)
    ol.backward()
    assert g["weights"].numel() == o["weights"].numel() > 100
    assert torch.equal(g["ray_id"].long().cpu(), o["ray_id"])
    np.testing.assert_allclose(g["weights"].detach().cpu().numpy(), o["weights"].detach().numpy(), atol=2e-6)
    assert (g["rgb_marched"].double().detach().cpu() - o["rgb_marched"].detach()).abs().max().item() <= 1e-5
    assert abs(gl.item() - ol.item()) <= 1e-6 * max(1.0, abs(ol.item()))
    assert _rel_l2(model.sdf.grid.grad, oracle.sdf_grid.grad) <= 1e-5
    assert _rel_l2(model.k0.grid.grad, oracle.k0_grid.grad) <= 1e-5
    for (n, p), (_, q) in zip(model.rgbnet.named_parameters(), oracle.rgbnet.named_parameters()):
        assert _rel_l2(p.grad, q.grad) <= 1e-5, n


def test_sdf_gradient_grid_vs_reference(cuda):
    from test_oracle_golden import OPS
    from voxurf_gb300.voxurf_coarse import sdf_gradient_grid

    sdf = torch.from_numpy(OPS["smooth_in"]).to(cuda)
    G = sdf_gradient_grid(sdf[0, 0], float(OPS["sdfgrad_voxel"]))
    ref = OPS["sdfgrad_out"][0]  # [3, X, Y, Z]
    np.testing.assert_allclose(G[..., :3].permute(3, 0, 1, 2).cpu().numpy(), ref, rtol=1e-6, atol=1e-6)
