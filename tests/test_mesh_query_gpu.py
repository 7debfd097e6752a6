"""Dense SDF field for mesh extraction (vx_sdf_field; extract_fields of
lib/dvgo_ori.py:679-693 with the query of Voxurf.extract_geometry,
voxurf_fine.py:894-910 / voxurf_coarse.py:652-665) against the reference's
own FP32 output (tests/golden/mesh_golden.npz) and the FP64 oracle."""
import os

import numpy as np
import pytest
import torch

from oracle.voxurf_oracle import extract_fields as oracle_fields
from oracle.voxurf_oracle import gaussian_kernel3d, smooth3d
from voxurf_gb300 import configs
from voxurf_gb300.voxurf_fine import extract_fields, gaussian_taps, smooth_grid

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_field_vs_reference_fixture(cuda):
    M = np.load(os.path.join(HERE, "mesh_golden.npz"))
    sdf = torch.from_numpy(M["sdf"]).to(cuda)
    grid = smooth_grid(sdf, gaussian_taps(3, float(M["sigma"])))
    u = extract_fields(grid, torch.from_numpy(M["xyz_min"]), torch.from_numpy(M["xyz_max"]), M["bound_min"],
                       M["bound_max"], int(M["resolution"]))
    np.testing.assert_allclose(u.cpu().numpy(), M["field"], rtol=1e-5, atol=2e-6)


@pytest.mark.parametrize("kind,smooth_model", [("fine", True), ("fine", False), ("coarse", True)])
def test_model_fields_vs_fp64_oracle(cuda, kind, smooth_model):
    """Model-level extract_fields over the whole bbox and over an off-centre
    sub-box (lattice points between and on voxel centres, outside-grid
    samples at the box border), for the three grids extract_geometry picks:
    smooth_conv(sdf), the 3^3 sigma-0.5 test kernel, the raw grid."""
    if kind == "fine":
        model = configs.build_fine_model(24, "fp32", device=cuda, seed=2, width=32)
    else:
        model = configs.build_coarse_model(24, "fp32", device=cuda, seed=2, width=32)
    if not smooth_model:
        model.init_smooth_conv(0)
    sdf64 = model.sdf.grid.detach().double().cpu()
    xyz_min, xyz_max = model.xyz_min.cpu().double(), model.xyz_max.cpu().double()
    cases = [(False, None), (True, 0.5)] if (kind == "fine" and not smooth_model) else [(True, 0.5)]
    for smooth, sigma in cases:
        if model.smooth_sdf:
            grid64 = smooth3d(sdf64, torch.from_numpy(gaussian_kernel3d(model.smooth_ksize, model.smooth_sigma)).double())
        elif smooth and kind == "fine":
            grid64 = smooth3d(sdf64, torch.from_numpy(gaussian_kernel3d(3, sigma)).double())
        else:
            grid64 = sdf64
        for bmin, bmax, R in [((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), 47), ((-0.83, -0.2, -1.1), (0.61, 0.9, 0.35), 30)]:
            if kind == "fine":
                u = model.extract_fields(bmin, bmax, R, smooth=smooth, sigma=sigma if sigma else 0.5)
            else:
                u = model.extract_fields(bmin, bmax, R)
            ref = oracle_fields(grid64, xyz_min, xyz_max, bmin, bmax, R)
            assert u.shape == (R, R, R)
            np.testing.assert_allclose(u.cpu().double().numpy(), ref.numpy(), rtol=1e-5, atol=2e-6,
                                       err_msg=str((kind, smooth_model, smooth, bmin, R)))


def test_extract_geometry_needs_a_host_mesher(cuda):
    model = configs.build_fine_model(16, "fp32", device=cuda, seed=1, width=32)
    try:
        import mcubes  # noqa: F401
    except ImportError:
        with pytest.raises(RuntimeError, match="PyMCubes"):
            model.extract_geometry(model.xyz_min, model.xyz_max, resolution=20)
        return
    v, t = model.extract_geometry(model.xyz_min, model.xyz_max, resolution=20)
    assert len(t) > 0 and np.all(v >= model.xyz_min.cpu().numpy() - 1e-6)
