"""Pins the oracle against golden vectors produced by the reference's own
Python code (tests/golden/make_golden.py runs lib/voxurf_fine.py, lib/grid.py
and lib/utils.py in float64 on the CPU).  CPU only."""
import os

import numpy as np
import pytest
import torch

from oracle import cref
from oracle.voxurf_oracle import OracleFine, UtilsAdam, gaussian_kernel3d, grid_sample_pts, smooth3d, train_loss

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
OPS = np.load(os.path.join(HERE, "ops_golden.npz"))
FINE = np.load(os.path.join(HERE, "fine_step_golden.npz"))
COARSE = np.load(os.path.join(HERE, "coarse_step_golden.npz"))


def test_alpha2weight_matches_reference_cumprod():
    """get_ray_marching_ray (voxurf_fine.py:951-954) == alpha2weight on rays
    that never reach T < 1e-3."""
    alpha = OPS["march_alpha"]
    n_rays, n = alpha.shape
    ray_id = np.repeat(np.arange(n_rays), n)
    w, T, last, i_s, i_e = cref.alpha2weight(alpha.reshape(-1), ray_id, n_rays)
    np.testing.assert_allclose(w.reshape(n_rays, n), OPS["march_weights"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(last, OPS["march_alphainv"][:, -1], rtol=1e-13, atol=0)
    # float32 (reference-kernel arithmetic) agrees to float32 precision
    w32, *_ = cref.alpha2weight(alpha.reshape(-1).astype(np.float32), ray_id, n_rays)
    np.testing.assert_allclose(w32.reshape(n_rays, n), OPS["march_weights"], rtol=2e-6, atol=0)


def test_utils_adam_restatement():
    p0, p1 = torch.from_numpy(OPS["adam_p0"]).clone(), torch.from_numpy(OPS["adam_p1"]).clone()
    params = [torch.nn.Parameter(p0), torch.nn.Parameter(p1)]
    opt = UtilsAdam([([params[0]], 1e-2), ([params[1]], 3e-3)], betas=(0.9, 0.99))
    count = torch.from_numpy(OPS["adam_count"])
    opt.per_lr = count.float() / count.max()
    for it in range(3):
        params[0].grad = torch.from_numpy(OPS["adam_grads0"][it]).clone()
        params[1].grad = torch.from_numpy(OPS["adam_grads1"][it]).clone()
        opt.step()
    np.testing.assert_array_equal(params[0].detach().numpy(), OPS["adam_out0"])
    np.testing.assert_array_equal(params[1].detach().numpy(), OPS["adam_out1"])


def test_dense_grid_restatement():
    grid = torch.from_numpy(OPS["dg_grid"])
    xyz = torch.from_numpy(OPS["dg_xyz"])
    out = grid_sample_pts(grid, xyz, torch.tensor([-1.0, -0.5, -2.0]), torch.tensor([1.0, 1.5, 0.5]))
    np.testing.assert_array_equal(out.numpy(), OPS["dg_out"])


def test_extract_fields_restatement():
    """The oracle's extract_fields + mesh query against the reference's own
    dvgo_ori.extract_fields with Voxurf.grid_sampler (FP32, 8^3 chunks)."""
    from oracle.voxurf_oracle import extract_fields

    M = np.load(os.path.join(HERE, "mesh_golden.npz"))
    k = torch.from_numpy(gaussian_kernel3d(3, float(M["sigma"])))
    grid = smooth3d(torch.from_numpy(M["sdf"]), k)
    u = extract_fields(grid, torch.from_numpy(M["xyz_min"]), torch.from_numpy(M["xyz_max"]), M["bound_min"],
                       M["bound_max"], int(M["resolution"]))
    np.testing.assert_allclose(u.numpy(), M["field"], rtol=1e-6, atol=1e-7)


def test_maskcache_restatement():
    """MaskCache (voxurf_fine.py:917-942) restated: max-pool 3^3 of the
    coarse checkpoint's density at load, then the FP32 alpha test, against
    the reference MaskCache's own answers on 4,000 points."""
    import torch.nn.functional as F

    from oracle.voxurf_oracle import maskcache_query

    C = np.load(os.path.join(HERE, "ckpt_golden.npz"))
    st = torch.load(os.path.join(HERE, "coarse_last.tar"), map_location="cpu", weights_only=False)
    kw = st["MaskCache_kwargs"]
    dens = F.max_pool3d(st["model_state_dict"]["density"], kernel_size=3, padding=1, stride=1)
    inside = maskcache_query(dens, torch.as_tensor(kw["xyz_min"]), torch.as_tensor(kw["xyz_max"]),
                             float(kw["act_shift"]), float(kw["voxel_size_ratio"]), float(C["mask_cache_thres"]),
                             torch.from_numpy(C["pts"]))
    np.testing.assert_array_equal(inside.numpy(), C["inside"])
    assert 0 < C["inside"].sum() < len(C["inside"])


def test_smoothing_restatement():
    k = torch.from_numpy(gaussian_kernel3d(5, 0.8))
    out = smooth3d(torch.from_numpy(OPS["smooth_in"]), k)
    np.testing.assert_allclose(out.numpy(), OPS["smooth_out"], rtol=1e-6, atol=1e-7)


def _model_from_fixture(device="cpu", precision="fp32"):
    from voxurf_gb300 import configs
    from voxurf_gb300.grid import MaskGrid

    R, width = int(FINE["R"]), int(FINE["width"])
    model = configs.build_fine_model(R, precision, device="cpu", seed=int(FINE["seed"]), width=width)
    sd = {k[len("state."):]: torch.from_numpy(FINE[k]) for k in FINE.files if k.startswith("state.")}
    model.load_state_dict(sd, strict=False)
    model = model.to(device)
    mask = sd["mask_cache.mask"]
    model.mask_cache = MaskGrid(mask=mask, xyz_min=[-1, -1, -1], xyz_max=[1, 1, 1]).to(device)
    model.nonempty_mask = mask[None, None].to(device)
    if precision == "bf16":
        model.refresh_k0_shadow()
    return model


def fine_fixture_inputs():
    rk = dict(near=0.1, far=6.0, bg=float(FINE["bg"]), stepsize=0.5)
    return FINE["rays_o"], FINE["rays_d"], FINE["viewdirs"], FINE["target"], rk


def test_fine_step_oracle_matches_reference():
    model = _model_from_fixture()
    oracle = OracleFine(model, dtype=torch.float64)
    ro, rd, vd, tgt, rk = fine_fixture_inputs()
    ret = oracle(torch.from_numpy(ro), torch.from_numpy(rd), torch.from_numpy(vd), global_step=1, **rk)
    loss = train_loss(ret, torch.from_numpy(tgt).double())
    loss.backward()
    assert ret["weights"].numel() == FINE["weights"].size
    np.testing.assert_allclose(ret["weights"].detach().numpy(), FINE["weights"], rtol=1e-12, atol=1e-15)
    for k in ("rgb_marched", "rgb_marched0", "alphainv_cum"):
        np.testing.assert_allclose(ret[k].detach().numpy(), FINE[k], rtol=1e-12, atol=1e-15)
    assert abs(loss.item() - float(FINE["loss"])) < 1e-13
    np.testing.assert_allclose(oracle.sdf_grid.grad.numpy(), FINE["grad_sdf"], rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(oracle.k0_grid.grad.numpy(), FINE["grad_k0"], rtol=1e-9, atol=1e-15)
    for n, p in oracle.rgbnet.named_parameters():
        np.testing.assert_allclose(p.grad.numpy(), FINE["grad_mlp." + n], rtol=1e-9, atol=1e-15)
    for n, p in oracle.k_rgbnet.named_parameters():
        np.testing.assert_allclose(p.grad.numpy(), FINE["grad_mlp.k." + n], rtol=1e-9, atol=1e-15)


def coarse_model_from_fixture(device="cpu"):
    from voxurf_gb300 import configs

    R, width = int(COARSE["R"]), int(COARSE["width"])
    model = configs.build_coarse_model(R, "fp32", device="cpu", seed=int(COARSE["seed"]), width=width)
    sd = {k[len("state."):]: torch.from_numpy(COARSE[k]) for k in COARSE.files if k.startswith("state.")}
    model.load_state_dict(sd, strict=False)
    return model.to(device)


def coarse_fixture_inputs():
    rk = dict(near=0.1, far=6.0, bg=float(COARSE["bg"]), stepsize=0.5)
    return COARSE["rays_o"], COARSE["rays_d"], COARSE["viewdirs"], COARSE["target"], rk


def test_coarse_step_oracle_matches_reference():
    """The reference coarse run used float64 as torch's default dtype, which
    makes its inv_s float64 (the oracle keeps float32 inv_s as the FP32
    reference computes it): agreement to ~1e-7 relative."""
    from oracle.voxurf_oracle import OracleCoarse

    oracle = OracleCoarse(coarse_model_from_fixture())
    ro, rd, vd, tgt, rk = coarse_fixture_inputs()
    ret = oracle(torch.from_numpy(ro), torch.from_numpy(rd), torch.from_numpy(vd), global_step=1, **rk)
    loss = train_loss(ret, torch.from_numpy(tgt).double(), weight_rgb0=0)
    loss.backward()
    assert ret["weights"].numel() == COARSE["weights"].size
    np.testing.assert_allclose(ret["weights"].detach().numpy(), COARSE["weights"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(ret["rgb_marched"].detach().numpy(), COARSE["rgb_marched"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(ret["alphainv_cum"].detach().numpy(), COARSE["alphainv_cum"], rtol=1e-6)
    rel = lambda a, b: np.linalg.norm((a - b).reshape(-1)) / np.linalg.norm(b.reshape(-1))
    assert rel(oracle.sdf_grid.grad.numpy(), COARSE["grad_sdf"]) < 1e-6
    assert rel(oracle.k0_grid.grad.numpy(), COARSE["grad_k0"]) < 1e-6
    for n, p in oracle.rgbnet.named_parameters():
        assert rel(p.grad.numpy(), COARSE["grad_mlp." + n]) < 1e-6, n


def _bg_case(z, tag):
    coarse = tag == "coarse"
    vs = np.float32(z["voxel_size_bg"] if coarse else z["voxel_size"])
    return dict(near=float(z["near"]), far=float(z["far"]), stepdist=float(np.float32(z["stepsize"]) * vs),
                dist_thres=float(z[f"{tag}_thres"]), n_samples=z[f"{tag}_pts"].shape[1],
                jitter=None if tag == "fine" else z["jitter"], outbbox_only=coarse)


@pytest.mark.parametrize("tag", ["fine", "fine_train", "coarse"])
def test_background_samples_restatement(tag):
    """The oracle's background candidates (points, inverted points, kept
    mask) equal the reference's sample_ray_ori / outside_sphere_trans /
    cumdist_thres composition bit for bit (womask fine and coarse)."""
    z = np.load(os.path.join(HERE, "bg_golden.npz"))
    pts, inv, keep = cref.bg_samples_dense(z["rays_o"], z["rays_d"], z["xyz_min"], z["xyz_max"], **_bg_case(z, tag))
    assert np.array_equal(pts, z[f"{tag}_pts"])
    assert np.array_equal(inv, z[f"{tag}_inv"])
    assert np.array_equal(keep, z[f"{tag}_keep"])
    assert 0 < keep.sum() < keep.size


def test_cumdist_thres_restatement():
    """cumdist_thres on the reference's own distances: marks where the
    running sum since the last mark first exceeds the threshold."""
    z = np.load(os.path.join(HERE, "bg_golden.npz"))
    dist, thres = z["fine_dist"], float(z["fine_thres"])
    m = cref.cumdist_thres(dist, thres)
    # the same recurrence written out in float32 numpy
    want = np.zeros_like(m)
    for r in range(dist.shape[0]):
        cum = np.float32(0)
        for i in range(dist.shape[1]):
            cum = np.float32(cum + dist[r, i])
            want[r, i] = cum > np.float32(thres)
            if want[r, i]:
                cum = np.float32(0)
    assert np.array_equal(m, want)


@pytest.mark.parametrize("C", [1, 12])
@pytest.mark.parametrize("form", ["sum", "mean", "mean_nomask"])
def test_total_variation_loss_restatement(C, form):
    """The loss-form total_variation (sum and per-axis mean forms) and its
    gradient against the reference functions' own float64 outputs."""
    from oracle.voxurf_oracle import total_variation_loss

    z = np.load(os.path.join(HERE, "tv_golden.npz"))
    v = torch.from_numpy(z[f"c{C}_v"]).requires_grad_(True)
    mask = None if form == "mean_nomask" else torch.from_numpy(z[f"c{C}_mask"])
    loss = total_variation_loss(v, mask, mode=0 if form == "sum" else 1)
    loss.backward()
    assert abs(loss.item() - float(z[f"c{C}_{form}_loss"])) <= 1e-12
    assert np.abs(v.grad.numpy() - z[f"c{C}_{form}_grad"]).max() <= 1e-12
