"""The loss-form total variation (vx_tv_loss / vx_tv_loss_backward behind
grid.total_variation) and the model TV methods built on it.

* against the reference functions' own float64 outputs
  (tests/golden/tv_golden.npz): both forms (sum over 3 x the mask's entries,
  voxurf_coarse.py:702-715; per-axis means, voxurf_fine.py:956-969), 1 and
  12 channels in both memory layouts, with and without a voxel mask; values
  quantised so that neighbour differences of exactly zero occur (their
  gradient is 0, as torch's abs).  Bars: loss within 1e-6 relative,
  gradients within 1e-6 of the largest entry (the inputs are float32
  roundings of the golden float64 values);
* against the oracle's restatement on a 40x50x60x12 grid: the same bars;
* deterministic: two runs give bit-identical loss and gradient;
* an empty selection gives NaN, as the reference's mean of nothing;
* the maskless coarse model's density_total_variation(sdf_tv,
  smooth_grad_tv) + 0.01 k0_total_variation() with the unit-sphere mask
  against the reference model's own float64 run
  (tests/golden/womask_coarse_step_golden.npz): loss within 1e-5 relative,
  gradients rel-L2 within 1e-5; and the coarse model's terms against the
  oracle with a non-empty mask.
"""
import os

import numpy as np
import pytest
import torch

from oracle.voxurf_oracle import total_variation_loss
from voxurf_gb300 import configs
from voxurf_gb300.grid import total_variation

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TV = np.load(os.path.join(HERE, "tv_golden.npz"))


def _dev_grid(v64: np.ndarray, cuda, channel_last: bool) -> torch.Tensor:
    v = torch.from_numpy(v64).float().to(cuda)
    if channel_last:
        v = v.contiguous(memory_format=torch.channels_last_3d)
    return v.requires_grad_(True)


@pytest.mark.parametrize("C,channel_last", [(1, False), (12, False), (12, True)])
@pytest.mark.parametrize("form", ["sum", "mean", "mean_nomask"])
def test_tv_loss_matches_reference_golden(cuda, C, channel_last, form):
    v = _dev_grid(TV[f"c{C}_v"], cuda, channel_last)
    mask = None if form == "mean_nomask" else torch.from_numpy(TV[f"c{C}_mask"]).to(cuda)
    loss = total_variation(v, mask, mode=0 if form == "sum" else 1)
    loss.backward()
    torch.cuda.synchronize()
    ref_loss = float(TV[f"c{C}_{form}_loss"])
    assert abs(loss.item() - ref_loss) <= 1e-6 * abs(ref_loss)
    g = v.grad.detach().cpu().numpy()
    ref_g = TV[f"c{C}_{form}_grad"]
    assert np.abs(g - ref_g).max() <= 1e-6 * np.abs(ref_g).max()
    if channel_last:
        assert v.grad.is_contiguous(memory_format=torch.channels_last_3d)


@pytest.mark.parametrize("mode", [0, 1])
def test_tv_loss_matches_oracle_large(cuda, mode):
    g = torch.Generator().manual_seed(3)
    shape = (40, 50, 60)
    v64 = (torch.randint(0, 6, (1, 12, *shape), generator=g).double() / 5.0
           + torch.randn((1, 12, *shape), generator=g, dtype=torch.float64) * 0.05)
    v64 = v64.float().double()  # the device sees the float32 values
    mask = torch.rand((1, 1, *shape), generator=g) < 0.8
    x = v64.clone().requires_grad_(True)
    ref = total_variation_loss(x, mask, mode) * 0.37
    ref.backward()
    v = _dev_grid(v64.numpy(), cuda, True)
    loss = total_variation(v, mask.to(cuda), mode=mode, weight=0.37)
    loss.backward()
    torch.cuda.synchronize()
    assert abs(loss.item() - ref.item()) <= 1e-6 * abs(ref.item())
    gr = x.grad.numpy()
    assert np.abs(v.grad.cpu().numpy() - gr).max() <= 1e-6 * np.abs(gr).max()


def test_tv_loss_is_deterministic(cuda):
    g = torch.Generator().manual_seed(4)
    v = torch.randn((1, 12, 64, 64, 64), generator=g).to(cuda).contiguous(memory_format=torch.channels_last_3d)
    mask = (torch.rand((1, 1, 64, 64, 64), generator=g) < 0.5).to(cuda)
    out = []
    for _ in range(2):
        x = v.clone().requires_grad_(True)
        loss = total_variation(x, mask, mode=1)
        loss.backward()
        out.append((loss.detach().cpu(), x.grad.cpu()))
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])


def test_tv_loss_empty_selection_is_nan(cuda):
    v = torch.randn((1, 1, 5, 6, 7), device=cuda)
    mask = torch.zeros((1, 1, 5, 6, 7), dtype=torch.bool, device=cuda)
    mask[0, 0, 2, 3, 4] = True   # one voxel: no pair has both ends in the mask
    for mode in (0, 1):
        loss = total_variation(v, mask, mode=mode)
        assert torch.isnan(loss).item() == (mode == 1)
    mask[...] = False
    assert torch.isnan(total_variation(v, mask, mode=0)).item()


def _rel(a, b):
    a, b = np.asarray(a, np.float64).reshape(-1), np.asarray(b, np.float64).reshape(-1)
    return float(np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30))


def test_womask_coarse_tv_terms_match_reference_golden(cuda):
    from voxurf_gb300.voxurf_womask_coarse import VoxurfWomaskCoarse

    WC = np.load(os.path.join(HERE, "womask_coarse_step_golden.npz"))
    R, Rb, width = int(WC["R"]), int(WC["R_bg"]), int(WC["width"])
    model = VoxurfWomaskCoarse(**configs.womask_coarse_model_kwargs(R, "fp32", width, Rb))
    sd = {k[len("state."):]: torch.from_numpy(WC[k]) for k in WC.files if k.startswith("state.")}
    sd = {k: v for k, v in sd.items() if not k.split(".")[0] in ("smooth_conv", "grad_conv", "tv_smooth_conv")}
    model.load_state_dict(sd, strict=False)
    model = model.to(cuda)
    model.tv_in_sphere = True
    T = lambda a: torch.from_numpy(np.asarray(a)).to(cuda)
    with torch.no_grad():   # the step's sphere reset of the SDF, as in the reference run
        model(T(WC["rays_o"]), T(WC["rays_d"]), T(WC["viewdirs"]), global_step=1, bg_jitter=T(WC["jitter"]),
              **dict(configs.COARSE_RENDER_KWARGS, bg=1))
    tv = model.density_total_variation(sdf_tv=0.1, smooth_grad_tv=0.05) + 0.01 * model.k0_total_variation()
    tv.backward()
    torch.cuda.synchronize()
    ref = float(WC["tv_loss"])
    assert abs(tv.item() - ref) <= 1e-5 * abs(ref)
    assert _rel(model.sdf.grid.grad.cpu().numpy(), WC["tv_grad_sdf"]) <= 1e-5
    assert _rel(model.k0.grid.grad.contiguous().cpu().numpy(), WC["tv_grad_k0"]) <= 1e-5


def test_coarse_tv_terms_need_and_use_the_nonempty_mask(cuda):
    from oracle.voxurf_oracle import neus_sdf_gradient

    model = configs.build_coarse_model(24, "fp32", device=cuda, seed=2, width=32)
    with pytest.raises(ValueError, match="non-empty mask"):
        model.density_total_variation(sdf_tv=0.1)
    sdf = model.sdf.grid.detach()
    mask = (sdf.abs() < 0.3)
    model.nonempty_mask = mask
    tv = model.density_total_variation(sdf_tv=0.1, smooth_grad_tv=0.05) + 0.01 * model.k0_total_variation()
    tv.backward()
    torch.cuda.synchronize()
    # oracle: the coarse sum form on sdf and k0, smooth_grad_tv on the raw
    # SDF's gradient grid (voxurf_coarse.py:300-320, 534)
    s = sdf.double().cpu().requires_grad_(True)
    k = model.k0.grid.detach().double().cpu().contiguous().requires_grad_(True)
    m = mask.cpu()
    vs = float(model.voxel_size)
    G = neus_sdf_gradient(s, vs)
    kern = torch.tensor([1.0, 2.0, 1.0], dtype=torch.float64)
    k3 = (kern[:, None, None] * kern[None, :, None] * kern[None, None, :]) / 64.0
    Gp = G.permute(1, 0, 2, 3, 4)
    Sm = torch.nn.functional.conv3d(torch.nn.functional.pad(Gp, (1,) * 6, mode="replicate"), k3[None, None])
    err = (Sm.detach() - Gp)[m.repeat(3, 1, 1, 1, 1)] ** 2
    ref = (total_variation_loss(s, m, 0) / 2 / vs * 0.1 + err.mean() * 0.05
           + 0.01 * total_variation_loss(k, m, 0))
    ref.backward()
    assert abs(tv.item() - ref.item()) <= 1e-5 * abs(ref.item())
    assert _rel(model.sdf.grid.grad.cpu().numpy(), s.grad.numpy()) <= 1e-5
    assert _rel(model.k0.grid.grad.contiguous().cpu().numpy(), k.grad.numpy()) <= 1e-5
