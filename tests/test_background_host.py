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
