"""Host logic of oracle/ref_cuda.py on the CPU: which of a module's
(Itanium-mangled) kernels a name and template-argument list select,
argument checks that run before any driver call, and the float Adam step
size of the reference's launchers."""
import numpy as np
import pytest
import torch

from oracle import ref_cuda

NAMES = [
    "_Z26infer_t_minmax_cuda_kernelIfEvPT_S1_S1_S1_ffiS1_S1_",
    "_Z26infer_t_minmax_cuda_kernelIdEvPT_S1_S1_S1_ffiS1_S1_",
    "_Z24__set_1_at_ray_seg_startPlS_i",
    "_Z13__set_step_idPlS_S_i",
    "_Z36total_variation_add_grad_cuda_kernelIfLb1EEvPKT_PS0_fffmmmm",
    "_Z36total_variation_add_grad_cuda_kernelIfLb0EEvPKT_PS0_fffmmmm",
    "_Z36total_variation_add_grad_cuda_kernelIdLb1EEvPKT_PS0_fffmmmm",
    "_Z40total_variation_add_grad_cuda_kernel_newIfLb1EEvPKT_PS0_S3_fffmmmm",
    "_Z40total_variation_add_grad_cuda_kernel_newIfLb0EEvPKT_PS0_S3_fffmmmm",
]


def _module():
    m = object.__new__(ref_cuda._Module)
    m.funcs = {n: i for i, n in enumerate(NAMES)}
    return m


def test_kernel_selection_by_name_and_template_arguments():
    m = _module()
    assert m.kernel("infer_t_minmax_cuda_kernel", "IfE") == 0
    assert m.kernel("infer_t_minmax_cuda_kernel", "IdE") == 1
    assert m.kernel("__set_1_at_ray_seg_start", None) == 2
    assert m.kernel("__set_step_id", None) == 3
    assert m.kernel("total_variation_add_grad_cuda_kernel", "IfLb1EE") == 4
    assert m.kernel("total_variation_add_grad_cuda_kernel", "IfLb0EE") == 5
    # the _new variant is a different name, not a prefix match
    assert m.kernel("total_variation_add_grad_cuda_kernel_new", "IfLb0EE") == 8
    with pytest.raises(RuntimeError):
        m.kernel("infer_t_minmax_cuda_kernel", None)  # a template needs its arguments
    with pytest.raises(RuntimeError):
        m.kernel("alpha2weight_cuda_kernel", "IfE")  # absent


def test_launch_checks_arguments_before_the_driver():
    t = torch.zeros(4)
    # nothing to launch: returns without loading a module
    ref_cuda._launch("render_utils", "x", None, 0, (ref_cuda.P,), t)
    with pytest.raises(ValueError):
        ref_cuda._launch("render_utils", "x", None, 4, (ref_cuda.P, ref_cuda.I), t)  # argument count
    with pytest.raises(ValueError):
        ref_cuda._launch("render_utils", "x", None, 4, (ref_cuda.P,), t)  # host tensor
    with pytest.raises(ValueError):
        ref_cuda._launch("render_utils", "x", None, 4, (ref_cuda.I,), 2 ** 31)  # int range
    assert not ref_cuda._modules


@pytest.mark.parametrize("step", [1, 2, 10, 1000])
def test_adam_step_size_is_the_float_expression(step):
    ss = ref_cuda.adam_step_size(step, 0.9, 0.99, 1e-3)
    assert isinstance(ss, np.float32)
    # the exact value of the expression from the float32 inputs; each float
    # rounding adds at most 2^-24 relative, and 1 - beta^t cancels (its error
    # relative to itself grows as 1 / (1 - beta^t))
    b1, b2, lr = (float(np.float32(x)) for x in (0.9, 0.99, 1e-3))
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    exact = lr * np.sqrt(c2) / c1
    bound = 2.0 ** -24 * exact * (4 + 1 / c2 + 1 / c1)
    assert abs(float(ss) - exact) <= bound
