"""Host-side logic of the background branch (no GPU): the candidate count
of sample_ray_ori (voxurf_womask_fine.py:792-795) against the reference's
own arrays in the golden fixture, and the drop-in modules' input checks
(CHECK_INPUT of the reference: CUDA, contiguous, float32)."""
import os

import numpy as np
import pytest
import torch

from voxurf_gb300 import background, ub360_utils_cuda

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bg_golden.npz")


def test_candidate_count_matches_reference_arrays():
    z = np.load(GOLDEN)
    st = float(z["stepsize"])
    assert background.n_samples_for([24, 24, 24], st) == z["fine_pts"].shape[1]
    assert background.n_samples_for([20, 20, 20], st) == z["coarse_pts"].shape[1]
    # the 256^3 workload of the benchmark
    assert background.n_samples_for([256, 256, 256], 0.5) == 891


def test_inputs_must_be_cuda_float32():
    o = torch.zeros((4, 3))
    with pytest.raises(RuntimeError, match="CUDA"):
        background.background_samples(o, o, [-1] * 3, [1] * 3, 0.2, 6.0, 0.5, 2.0 / 24, 87)
    with pytest.raises(RuntimeError, match="CUDA"):
        ub360_utils_cuda.cumdist_thres(torch.zeros((2, 5)), 0.1)


def test_womask_coarse_model_parameters_match_reference_state():
    """The maskless coarse model's parameters and buffers carry the
    reference's names and shapes (the state of its float64 golden run)."""
    from voxurf_gb300 import configs

    z = np.load(os.path.join(os.path.dirname(GOLDEN), "womask_coarse_step_golden.npz"))
    R, Rb, width = int(z["R"]), int(z["R_bg"]), int(z["width"])
    model = configs.build_womask_coarse_model(R, "fp32", device="cpu", seed=int(z["seed"]), width=width, R_bg=Rb)
    ours = {k: tuple(v.shape) for k, v in model.state_dict().items()}
    ref = {k[len("state."):]: z[k].shape for k in z.files if k.startswith("state.")}
    ref = {k: v for k, v in ref.items() if k.split(".")[0] not in ("smooth_conv", "grad_conv", "tv_smooth_conv")}
    assert ours == ref
    # same initial state as the fixture (both are built by the same builder)
    for k, v in model.state_dict().items():
        assert np.array_equal(v.float().numpy(), z["state." + k]), k


def test_womask_coarse_model_rejects_swapped_frequencies():
    from voxurf_gb300 import configs
    from voxurf_gb300.voxurf_womask_coarse import VoxurfWomaskCoarse

    kw = configs.womask_coarse_model_kwargs(8, "fp32", 16)
    kw["bg_posbase_pe"] = 4
    with pytest.raises(ValueError, match="bg_posbase_pe"):
        VoxurfWomaskCoarse(**kw)
