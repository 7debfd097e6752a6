"""The maskless fine model (lib/voxurf_womask_fine.py:833-1071): the
foreground sample generator against the reference's sample_ray_ori points
(bit for bit), and one training step (forward, loss, backward) against the
reference model's own float64 run (tests/golden/womask_step_golden.npz,
made by tests/golden/make_golden.py with the reference's jitters fixed).

FP32 bars as the fine model's golden test: rgb_marched, rgb_marched0,
alphainv_cum, in_marched and out_marched within 1e-5 absolute; every
parameter gradient (sdf, k0, bg_density, bg_k0, rgbnet, k_rgbnet,
bg_rgbnet) within rel-L2 1e-5 (the FP32 sums against the reference's FP64;
gradient sums of order 1e3 terms).  The kept foreground and background
sample counts equal the reference's.  BF16 (k0 from its BF16 copy, the
three MLPs on the tensor cores): colours within 2e-3, gradients rel-L2
within 5e-2.
"""
import os

import numpy as np
import pytest
import torch

from voxurf_gb300 import background, configs
from voxurf_gb300.train import fine_loss

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
WM = np.load(os.path.join(HERE, "womask_step_golden.npz"))
BG = np.load(os.path.join(HERE, "bg_golden.npz"))


def _model(device, precision):
    from voxurf_gb300.voxurf_womask import VoxurfWomask

    R, Rb, width = int(WM["R"]), int(WM["R_bg"]), int(WM["width"])
    model = VoxurfWomask(**configs.womask_model_kwargs(R, precision, width, Rb))
    sd = {k[len("state."):]: torch.from_numpy(WM[k]) for k in WM.files if k.startswith("state.")}
    # the reference's smoothing / gradient convolutions are buffers of fixed
    # kernels there; here the smoothing is a kernel parameterised by its taps
    sd = {k: v for k, v in sd.items() if not k.split(".")[0] in ("smooth_conv", "grad_conv", "tv_smooth_conv")}
    missing, unexpected = model.load_state_dict(sd, strict=False)
    assert not unexpected, unexpected
    assert not [k for k in missing if k.endswith(("grid", "weight", "bias"))], missing
    model = model.to(device)
    if precision == "bf16":
        model.refresh_k0_shadow()
    return model


def _rel(a, b):
    a, b = np.asarray(a, np.float64).reshape(-1), np.asarray(b, np.float64).reshape(-1)
    return float(np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30))


@pytest.mark.parametrize("tag", ["fine", "fine_train"])
def test_foreground_samples_match_reference(cuda, tag):
    """inner mode of the sample generator = the reference's sample_ray_ori
    points with |p| < 1 (voxurf_womask_fine.py:843-849), in ray order."""
    z = BG
    pts = z[f"{tag}_pts"]
    norm = torch.linalg.norm(torch.from_numpy(pts), ord=2, dim=-1).numpy()
    ray_id, step_id = np.nonzero(norm < 1.0)
    o = torch.from_numpy(z["rays_o"]).to(cuda)
    d = torch.from_numpy(z["rays_d"]).to(cuda)
    jit = None if tag == "fine" else torch.from_numpy(z["jitter"]).to(cuda)
    S = background.n_samples_for([24] * 3, float(z["stepsize"]))
    got, org, rid, sid = background.background_samples(o, d, z["xyz_min"], z["xyz_max"], float(z["near"]),
                                                        float(z["far"]), float(z["stepsize"]), z["voxel_size"], S,
                                                        jit, inner=True)
    torch.cuda.synchronize()
    assert org is None
    assert np.array_equal(rid.cpu().numpy(), ray_id) and np.array_equal(sid.cpu().numpy(), step_id)
    assert np.array_equal(got.cpu().numpy(), pts[ray_id, step_id])


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_womask_step_vs_reference_golden(cuda, precision):
    model = _model(cuda, precision)
    T = lambda a: torch.from_numpy(np.asarray(a)).to(cuda)
    rk = dict(configs.FINE_RENDER_KWARGS, bg=1)
    ret = model(T(WM["rays_o"]), T(WM["rays_d"]), T(WM["viewdirs"]), global_step=1, jitter=T(WM["jitter"][0]),
                bg_jitter=T(WM["jitter"][1]), **rk)
    loss = fine_loss(ret, T(WM["target"]))
    loss.backward()
    torch.cuda.synchronize()
    assert ret["weights"].numel() == int(WM["n_weights"])
    assert ret["bg_weights"].numel() == int(WM["n_bg_weights"])
    col_tol = 1e-5 if precision == "fp32" else 2e-3
    for k in ("rgb_marched", "rgb_marched0", "alphainv_cum", "in_marched", "out_marched"):
        err = np.abs(ret[k].detach().cpu().numpy() - WM[k]).max()
        assert err <= col_tol, (k, err)
    g_tol = 1e-5 if precision == "fp32" else 5e-2
    errs = {}
    for name in ("sdf", "k0", "bg_density", "bg_k0"):
        g = getattr(model, name).grid.grad.contiguous().cpu().numpy()
        errs[name] = _rel(g, WM["grad_" + name])
    for net in ("rgbnet", "k_rgbnet", "bg_rgbnet"):
        for n, p in getattr(model, net).named_parameters():
            errs[f"{net}.{n}"] = _rel(p.grad.cpu().numpy(), WM[f"grad_{net}.{n}"])
    print(precision, {k: f"{v:.2e}" for k, v in errs.items()})
    bad = {k: v for k, v in errs.items() if not v <= g_tol}
    assert not bad, bad
    assert abs(float(loss.detach()) - float(WM["loss"])) <= (1e-5 if precision == "fp32" else 2e-3) * max(1.0, float(WM["loss"]))


def test_womask_render_without_training(cuda):
    """global_step None: no jitter, no sphere reset; runs and keeps shapes."""
    model = _model(cuda, "fp32")
    T = lambda a: torch.from_numpy(np.asarray(a)).to(cuda)
    rk = dict(configs.FINE_RENDER_KWARGS, bg=1)
    before = model.sdf.grid.detach().clone()
    with torch.no_grad():
        ret = model(T(WM["rays_o"]), T(WM["rays_d"]), T(WM["viewdirs"]), **rk)
    n = WM["rays_o"].shape[0]
    assert ret["rgb_marched"].shape == (n, 3) and ret["alphainv_cum"].shape == (n,)
    assert torch.equal(before, model.sdf.grid.detach())
    assert torch.isfinite(ret["rgb_marched"]).all()
