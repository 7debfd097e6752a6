"""Background branch of the models without an object mask
(lib/voxurf_womask_fine.py:857-870, lib/voxurf_womask_coarse.py:633-650):
the cumdist_thres drop-in and the fused background sample generator against
the oracle and the reference's golden vectors, bit for bit."""
import os

import numpy as np
import pytest
import torch

from oracle import cref
from voxurf_gb300 import background, ub360_utils_cuda

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bg_golden.npz")


@pytest.mark.parametrize("shape", [(1, 1), (5, 31), (33, 64), (70, 100), (257, 891), (0, 7), (3, 0)])
def test_cumdist_thres_matches_oracle(cuda, shape):
    g = np.random.default_rng(shape[0] * 1000 + shape[1])
    dist = (g.random(shape) * 0.05).astype(np.float32)
    dist[:, ::7] = 0.0
    thres = 0.06
    got = ub360_utils_cuda.cumdist_thres(torch.from_numpy(dist).to(cuda), thres).cpu().numpy()
    assert got.dtype == np.bool_ and got.shape == shape
    assert np.array_equal(got, cref.cumdist_thres(dist, thres))


def test_cumdist_thres_on_reference_distances(cuda):
    z = np.load(GOLDEN)
    for tag in ("fine", "fine_train", "coarse"):
        dist, thres = z[f"{tag}_dist"], float(z[f"{tag}_thres"])
        got = ub360_utils_cuda.cumdist_thres(torch.from_numpy(dist).to(cuda), thres).cpu().numpy()
        assert np.array_equal(got, cref.cumdist_thres(dist, thres)), tag


def _reference_compacted(z, tag):
    keep = z[f"{tag}_keep"]
    ray_id, step_id = np.nonzero(keep)
    return z[f"{tag}_inv"][keep], z[f"{tag}_pts"][keep], ray_id, step_id


@pytest.mark.parametrize("tag", ["fine", "fine_train", "coarse"])
def test_background_samples_match_reference_golden(cuda, tag):
    """The compacted samples equal the reference's outer_pts, outer_pts_org,
    outer_ray_id, outer_step_id (voxurf_womask_fine.py:868-870)."""
    z = np.load(GOLDEN)
    coarse = tag == "coarse"
    o = torch.from_numpy(z["rays_o"]).to(cuda)
    d = torch.from_numpy(z["rays_d"]).to(cuda)
    jit = None if tag == "fine" else torch.from_numpy(z["jitter"]).to(cuda)
    grid_r = 20 if coarse else 24
    S = background.n_samples_for([grid_r] * 3, float(z["stepsize"]))
    assert S == z[f"{tag}_pts"].shape[1]
    out = background.background_samples(
        o, d, z["xyz_min"], z["xyz_max"], float(z["near"]), float(z["far"]), float(z["stepsize"]),
        z["voxel_size"], S, jit, step_voxel_size=z["voxel_size_bg"] if coarse else None,
        dist_thres_factor=0.95 if coarse else 0.5, outbbox_only=coarse)
    torch.cuda.synchronize()
    want = _reference_compacted(z, tag)
    for got, w in zip(out, want):
        assert np.array_equal(got.cpu().numpy(), w)


@pytest.mark.parametrize("outbbox_only", [False, True])
def test_background_samples_match_oracle_large(cuda, outbbox_only):
    """2048 rays from all around the box on a 96^3 grid's sample count, with
    training jitter: bit-exact against the oracle."""
    g = np.random.default_rng(11 + outbbox_only)
    n = 2048
    o = (g.random((n, 3)) * 4.0 - 2.0).astype(np.float32)
    d = g.standard_normal((n, 3)).astype(np.float32)
    d[:64, 2] = 0.0
    jit = g.random(n).astype(np.float32)
    mn, mx = np.array([-1.0, -0.9, -1.1], np.float32), np.array([1.0, 1.2, 0.8], np.float32)
    vs = np.float32(2.0 / 96)
    S = background.n_samples_for([96, 96, 96], 0.5)
    out = background.background_samples(
        torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda), mn, mx, 0.1, 8.0, 0.5, vs, S,
        torch.from_numpy(jit).to(cuda), dist_thres_factor=0.95 if outbbox_only else 0.5, outbbox_only=outbbox_only)
    torch.cuda.synchronize()
    stepdist = float(np.float32(np.float32(0.5) * vs))
    thres = float(np.float32(np.float32(vs * np.float32(0.5)) * np.float32(0.95 if outbbox_only else 0.5)))
    want = cref.bg_samples(o, d, mn, mx, 0.1, 8.0, stepdist, thres, S, jit, outbbox_only)
    assert want[0].shape[0] > 10000
    for got, w in zip(out, want):
        assert np.array_equal(got.cpu().numpy(), w)


def test_background_samples_empty_batch(cuda):
    e = torch.empty((0, 3), device=cuda)
    out = background.background_samples(e, e, [-1, -1, -1], [1, 1, 1], 0.2, 6.0, 0.5, 2.0 / 24, 87)
    assert all(t.shape[0] == 0 for t in out)
