"""Colour-MLP forward/backward through apply_mlp (the FP32 CUDA-core engine
for FP32 rows, the tcgen05 engine for BF16 rows) against plain torch autograd
of the reference nn.Sequential (FP64) and torch's BF16 autocast."""
import pytest
import torch
import torch.nn as nn

from voxurf_gb300.mlp import apply_mlp

pytestmark = pytest.mark.gpu


def _net(d_in, width, depth, seed):
    torch.manual_seed(seed)
    return nn.Sequential(nn.Linear(d_in, width), nn.ReLU(inplace=True),
                         *[nn.Sequential(nn.Linear(width, width), nn.ReLU(inplace=True)) for _ in range(depth - 2)],
                         nn.Linear(width, 3))


@pytest.mark.parametrize("M,d_in,width,depth", [(3000, 70, 192, 4), (1037, 60, 192, 4), (513, 75, 128, 3), (0, 70, 64, 3)])
def test_mlp_fp32_matches_autograd(cuda, M, d_in, width, depth):
    net = _net(d_in, width, depth, M).to(cuda).double()
    x = torch.randn(M, d_in, device=cuda, dtype=torch.float64, requires_grad=True)
    gy = torch.randn(M, 3, device=cuda, dtype=torch.float64)
    y_ref = net(x)
    (y_ref * gy).sum().backward()
    ref = [x.grad.clone()] + [p.grad.clone() for p in net.parameters()]
    net32 = net.float()
    for p in net32.parameters():
        p.grad = None
    x32 = x.detach().float().requires_grad_(True)
    y = apply_mlp(net32, x32)
    (y * gy.float()).sum().backward()
    got = [x32.grad] + [p.grad for p in net32.parameters()]
    assert torch.allclose(y.double(), y_ref.detach(), rtol=1e-5, atol=1e-5)
    for g, r in zip(got, ref):
        assert g.dtype == torch.float32
        if r.numel():
            assert float((g.double() - r).norm() / (r.norm() + 1e-30)) < 1e-5


def test_mlp_bf16_matches_torch_autocast(cuda):
    """BF16 path (tcgen05 engine) against the FP64 result: each gradient within
    3e-2, or within 1.5x of torch's own BF16 autocast of the same
    nn.Sequential, whichever is larger (both round operands to BF16 and
    accumulate in FP32)."""
    net = _net(70, 192, 4, 0).to(cuda)
    x = torch.randn(4096, 70, device=cuda)
    gy = torch.randn(4096, 3, device=cuda)
    net64 = _net(70, 192, 4, 0).to(cuda).double()
    net64.load_state_dict({k: v.double() for k, v in net.state_dict().items()})
    y64 = net64(x.bfloat16().double())
    (y64 * gy.double()).sum().backward()
    g64 = [p.grad.clone() for p in net64.parameters()]
    with torch.autocast("cuda", dtype=torch.bfloat16):
        y_ref = net(x.bfloat16())
    (y_ref.float() * gy).sum().backward()
    g_ref = [p.grad.clone() for p in net.parameters()]
    for p in net.parameters():
        p.grad = None
    y16 = apply_mlp(net, x.bfloat16()).float()
    (y16 * gy).sum().backward()
    assert float((y16 - y_ref.float()).abs().max().detach()) < 2e-2
    for p, r, t in zip(net.parameters(), g64, g_ref):
        assert p.grad.dtype == torch.float32
        e = float((p.grad.double() - r).norm() / r.norm())
        et = float((t.double() - r).norm() / r.norm())
        assert e <= max(3e-2, 1.5 * et), (e, et)
