"""Fused tcgen05 colour-MLP forward (vx_mlp_tc_forward) against a torch
reference of the same arithmetic: BF16 inputs and weights, FP32
accumulation, hidden activations rounded to BF16 after bias + ReLU, FP32
output layer.  Tolerance: max abs logit error <= 2e-3 (a hidden unit that
rounds to the neighbouring BF16 value moves a logit by ~1e-4; tensor-core
and torch accumulation orders differ)."""
import pytest
import torch
import torch.nn as nn

from voxurf_gb300.mlp import TensorCoreMLP

pytestmark = pytest.mark.gpu


def _net(k_in, seed, cuda):
    torch.manual_seed(seed)
    net = nn.Sequential(nn.Linear(k_in, 192), nn.ReLU(inplace=True),
                        *[nn.Sequential(nn.Linear(192, 192), nn.ReLU(inplace=True)) for _ in range(2)],
                        nn.Linear(192, 3)).to(cuda)
    for m in net.modules():   # biases away from zero so that the bias path is exercised
        if isinstance(m, nn.Linear):
            nn.init.uniform_(m.bias, -0.2, 0.2)
    return net


def _reference(net, X, k_in):
    lin = [m for m in net.modules() if isinstance(m, nn.Linear)]
    h = X[:, :k_in].float()
    for m in lin[:3]:
        W = m.weight.detach().to(torch.bfloat16).float()
        b = m.bias.detach().to(torch.bfloat16).float()
        h = torch.relu(h @ W.t() + b).to(torch.bfloat16).float()
    return h @ lin[3].weight.detach().float().t() + lin[3].bias.detach().float()


@pytest.mark.parametrize("k_in,K0,ld", [(70, 80, 80), (63, 64, 64), (60, 64, 72)])
@pytest.mark.parametrize("n", [1, 127, 128, 129, 5000, 70001])
def test_tc_mlp_matches_reference(cuda, k_in, K0, ld, n):
    net = _net(k_in, n + k_in, cuda)
    X = torch.zeros((n, ld), dtype=torch.bfloat16, device=cuda)
    X[:, :k_in] = (torch.randn((n, k_in), device=cuda) * 0.7).to(torch.bfloat16)
    mlp = TensorCoreMLP(net, K0)
    out = torch.full((n, 3), float("nan"), device=cuda)
    mlp.forward(X, out)
    torch.cuda.synchronize()
    ref = _reference(net, X, k_in)
    err = (out - ref).abs().max().item()
    assert err <= 2e-3, err


def test_tc_mlp_residual_and_columns(cuda):
    """add = residual logits; cols = the logits written back as BF16 into a
    row-major buffer (the k_rgbnet input's last columns)."""
    n, k_in = 3000, 70
    net = _net(k_in, 3, cuda)
    X = torch.zeros((n, 80), dtype=torch.bfloat16, device=cuda)
    X[:, :k_in] = torch.randn((n, k_in), device=cuda).to(torch.bfloat16)
    add = torch.randn((n, 3), device=cuda)
    out = torch.empty((n, 3), device=cuda)
    cols = torch.zeros((n, 64), dtype=torch.bfloat16, device=cuda)
    TensorCoreMLP(net, 80).forward(X, out, add=add, cols=cols[:, 60:], ld_cols=64)
    torch.cuda.synchronize()
    ref = _reference(net, X, k_in) + add
    assert (out - ref).abs().max().item() <= 2e-3
    assert torch.equal(cols[:, 60:63], out.to(torch.bfloat16))
    assert torch.count_nonzero(cols[:, :60]) == 0 and torch.count_nonzero(cols[:, 63]) == 0


def test_tc_mlp_rejects_unsupported(cuda):
    net = _net(100, 0, cuda)
    assert not TensorCoreMLP.supports(net, 112)
    with pytest.raises(ValueError):
        TensorCoreMLP(net, 112)


@pytest.mark.parametrize("K0,ld", [(80, 80), (64, 72)])
@pytest.mark.parametrize("n", [1, 128, 129, 383, 5000, 152 * 128 * 2 + 77, 152 * 128 * 5 + 1])
def test_two_tiles_in_flight_is_bit_identical(cuda, K0, ld, n):
    """pipeline 1 (two tiles in flight per CTA, a shared A operand) issues the
    same MMAs and epilogue arithmetic as pipeline 0: identical logits,
    residual sums and BF16 columns, for tile counts that leave a CTA's last
    pair half empty and for every row past the end untouched."""
    k_in = K0 - 10
    net = _net(k_in, n + K0, cuda)
    X = torch.zeros((n, ld), dtype=torch.bfloat16, device=cuda)
    X[:, :k_in] = (torch.randn((n, k_in), device=cuda) * 0.7).to(torch.bfloat16)
    add = torch.randn((n, 3), device=cuda)
    mlp = TensorCoreMLP(net, K0)
    res = []
    for pipeline in (0, 1):
        out = torch.full((n + 5, 3), float("nan"), device=cuda)
        cols = torch.full((n, 8), -7.0, dtype=torch.bfloat16, device=cuda)
        mlp.forward(X, out[:n], add=add, cols=cols, ld_cols=8, pipeline=pipeline)
        torch.cuda.synchronize()
        res.append((out, cols))
    assert torch.equal(res[0][0][:n], res[1][0][:n])
    assert torch.isnan(res[1][0][n:]).all()
    assert torch.equal(res[0][1], res[1][1])
    assert bool((res[1][1][:, 3:] == -7.0).all())
