"""Edge cases of the model-level path: empty ray batches, batches in which no
ray reaches the surface (no shaded samples), and render requests of one
pixel or with every ray outside the scene box."""
import numpy as np
import pytest
import torch

from voxurf_gb300 import configs, serve, synthetic
from voxurf_gb300.train import FineTrainer

pytestmark = pytest.mark.gpu

RK = dict(configs.FINE_RENDER_KWARGS)


def _away_rays(n, cuda):
    """Rays that start outside the [-1,1]^3 box and point away from it."""
    o = torch.full((n, 3), 3.0, device=cuda)
    d = torch.ones((n, 3), device=cuda)
    d[:, 1] += torch.linspace(0, 1, n, device=cuda)
    v = d / d.norm(dim=-1, keepdim=True)
    return o, d, v


@pytest.mark.parametrize("kind", ["fine", "coarse"])
def test_empty_batch_forward_backward(cuda, kind):
    if kind == "fine":
        model = configs.build_fine_model(16, "fp32", device=cuda, seed=1, width=32)
        rk = RK
    else:
        model = configs.build_coarse_model(16, "fp32", device=cuda, seed=1, width=32)
        rk = dict(configs.COARSE_RENDER_KWARGS)
    e = torch.empty((0, 3), device=cuda)
    ret = model(e, e, e, global_step=1, **rk)
    assert ret["rgb_marched"].shape == (0, 3) and ret["weights"].numel() == 0
    ret["rgb_marched"].sum().backward()


@pytest.mark.parametrize("graphed", [False, True])
def test_step_with_no_shaded_sample(cuda, graphed):
    """Every ray misses the box: the loss is the background's, the grid
    gradients come from TV alone, the step runs (graph capture included)."""
    model = configs.build_fine_model(16, "bf16" if graphed else "fp32", device=cuda, seed=2, width=32)
    tr = FineTrainer(model, n_rays=64, graphed=graphed)
    o, d, v = _away_rays(64, cuda)
    tgt = torch.rand((64, 3), device=cuda, generator=torch.Generator(cuda).manual_seed(0))
    k0_before = model.k0.grid.detach().clone()
    for _ in range(2):
        loss, ret = tr.step(o, d, v, tgt, RK)
        torch.cuda.synchronize()
        assert np.isfinite(float(loss))
    # bg = 0: rgb 0 everywhere, so the loss is mse(0, target) (+ the entropy term)
    assert abs(float(loss) - float((tgt ** 2).mean()) * 1.5) < 5e-3
    # TV still moves k0 (dense TV mode), and nothing blew up
    assert torch.isfinite(model.k0.grid).all() and not torch.equal(model.k0.grid.detach(), k0_before)


def test_render_requests_one_pixel_and_all_background(cuda):
    model = configs.build_fine_model(32, "fp32", device=cuda, seed=3, width=32, mask_voxels=3.0)
    scene = serve.ResidentScene(model, s_val=0.01, precision="fp32", bg=0.25)
    srv = serve.RenderServer([scene], tick_rays=4096, arena_pixels=1 << 16)
    pose = np.asarray(synthetic.fibonacci_poses(5, 3.0)[2])
    rgb, depth = srv.render(0, pose, 1, 1)
    assert rgb.shape == (1, 1, 3) and np.isfinite(rgb).all()
    away = pose.copy()
    away[:3, 2] *= -1.0   # look away from the origin
    away[:3, 0] *= -1.0   # keep the frame right-handed
    rgb, depth = srv.render(0, away, 12, 16)
    assert np.allclose(rgb, 0.25) and np.all(depth == 0)
