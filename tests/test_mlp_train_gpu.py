"""Colour-MLP training on the tensor cores (vx_mlp_train_*: forward, the
input-gradient chain, the weight-gradient passes and their ordered sums)
against torch.

Two references on the same seeded inputs:
* an FP64 emulation of the kernels' rounding points (BF16 input rows, BF16
  weights, BF16 hidden activations and hidden-layer gradients, the output
  layer's weights and dy as BF16 hi + lo pairs): logits, dX and every
  weight/bias gradient within rel-L2 3e-3 (the FP32 tensor-core sums differ
  from FP64 in order, which moves a few BF16 roundings by one unit);
* torch autograd of the unrounded FP32 MLP (what the reference runs): each
  output's rel-L2 error within 3e-2 or within 1.5x the error of torch's own
  BF16 autocast of the same MLP against the same FP32 result, whichever is
  larger (the input gradient is a sum of products of either sign, which
  magnifies the BF16 rounding of its operands to several percent in any
  BF16 implementation).
Shapes: the fine rgbnet / k_rgbnet (192 wide, 3 hidden layers, K0 80 / 64),
the coarse rgbnet (128 wide, 2 hidden layers), the test widths 64 and 32;
row counts of one partial tile, one tile per CTA, and several tiles per CTA
(the persistent loops and the two-stage weight-gradient pipeline).
"""
import numpy as np
import pytest
import torch
import torch.nn as nn

from voxurf_gb300.mlp import TcTrainMLP

pytestmark = pytest.mark.gpu


def _net(d_in, W, L, seed):
    g = torch.Generator().manual_seed(seed)
    layers = [nn.Linear(d_in, W), nn.ReLU()]
    for _ in range(L - 1):
        layers += [nn.Linear(W, W), nn.ReLU()]
    layers += [nn.Linear(W, 3)]
    net = nn.Sequential(*layers)
    for m in net.modules():
        if isinstance(m, nn.Linear):
            m.weight.data = torch.randn(m.weight.shape, generator=g) * (1.5 / np.sqrt(m.in_features))
            m.bias.data = torch.randn(m.bias.shape, generator=g) * 0.1
    return net


def _bf(t):
    return t.to(torch.bfloat16).to(torch.float64)


def _emulate(net, X, dY):
    """FP64 with the kernels' rounding points."""
    lin = [m for m in net.modules() if isinstance(m, nn.Linear)]
    L = len(lin) - 1
    Ws = [_bf(m.weight.detach().cpu().double()) for m in lin[:L]]
    bs = [m.bias.detach().cpu().double() for m in lin[:L]]
    Wh = lin[L].weight.detach().cpu().float()
    hi = Wh.to(torch.bfloat16).float()
    Wh_eff = (hi.double() + (Wh - hi).to(torch.bfloat16).double())
    x = X.double()
    hs = []
    h = x
    for l in range(L):
        h = _bf(torch.relu(h @ Ws[l].T + bs[l]))
        hs.append(h)
    logits = h @ Wh_eff.T + lin[L].bias.detach().cpu().double()
    dy = dY.double()
    dz = _bf((dy @ lin[L].weight.detach().cpu().double()) * (hs[-1] > 0))
    grads = {"Wh": (_bf(dY.float()) + _bf(dY.float() - _bf(dY.float()).float())).T @ hs[-1], "bh": dy.sum(0)}
    for l in range(L - 1, 0, -1):
        grads[f"W{l}"] = dz.T @ hs[l - 1]
        grads[f"b{l}"] = dz.sum(0)
        dz = _bf((dz @ Ws[l]) * (hs[l - 1] > 0))
    grads["W0"] = dz.T @ x
    grads["b0"] = dz.sum(0)
    dX = dz @ Ws[0]
    return logits, dX, grads


def _autograd32(net, X, dY, autocast=False):
    """torch autograd of net on X (FP32, or torch's BF16 autocast on the GPU)."""
    net32 = [m for m in net.modules() if isinstance(m, nn.Linear)]
    for m in net32:
        m.weight.grad = m.bias.grad = None
    x = X.float().clone().requires_grad_(True)
    if autocast:
        with torch.autocast("cuda", dtype=torch.bfloat16):
            y = net(x)
        y = y.float()
    else:
        y = net.float()(x)
    y.backward(dY.float().to(y.device))
    L = len(net32) - 1
    grads = {"Wh": net32[L].weight.grad.clone(), "bh": net32[L].bias.grad.clone()}
    for l in range(L):
        grads[f"W{l}"] = net32[l].weight.grad.clone()
        grads[f"b{l}"] = net32[l].bias.grad.clone()
    return y.detach(), x.grad.detach(), grads


def _rel(a, b):
    a = a.detach().double().cpu().reshape(-1)
    b = b.detach().double().cpu().reshape(-1)
    return float((a - b).norm() / (b.norm() + 1e-30))


def _names(L):
    out = []
    for l in range(L):
        out += [f"W{l}", f"b{l}"]
    return out + ["Wh", "bh"]


@pytest.mark.parametrize("W,L,d_in,K0", [(192, 3, 70, 80), (192, 3, 60, 64), (128, 2, 75, 80), (64, 3, 70, 80),
                                         (32, 3, 70, 80), (32, 2, 16, 16)])
@pytest.mark.parametrize("n", [77, 5000, 152 * 128 * 3 + 77])
def test_mlp_train_matches_torch(cuda, W, L, d_in, K0, n):
    net = _net(d_in, W, L, seed=W + L + d_in).to(cuda)
    g = torch.Generator().manual_seed(n + W)
    Xf = torch.randn((n, d_in), generator=g)
    X = torch.zeros((n, K0), dtype=torch.bfloat16)
    X[:, :d_in] = Xf.to(torch.bfloat16)
    dY = torch.randn((n, 3), generator=g) / n
    tc = TcTrainMLP(net, K0)
    tc.pack()
    Xd = X.to(cuda)
    logits, st = tc.forward(Xd)
    dX, grads = tc.backward(st, dY.to(cuda), dx_dtype=torch.float32)
    torch.cuda.synchronize()
    e_logits, e_dX, e_grads = _emulate(net.cpu(), X[:, :d_in].double(), dY)
    assert _rel(logits, e_logits) <= 3e-3
    assert _rel(dX[:, :d_in], e_dX) <= 3e-3
    names = _names(L)
    got = dict(zip(names, grads))
    for k in names:
        assert _rel(got[k], e_grads[k]) <= 3e-3, (k, _rel(got[k], e_grads[k]))
    a_logits, a_dX, a_grads = _autograd32(net.cpu(), X[:, :d_in].float(), dY)
    net.to(cuda)
    t_logits, t_dX, t_grads = _autograd32(net, X[:, :d_in].float().to(cuda), dY, autocast=True)

    def bound(ours, torch_bf16, truth, what):
        e, et = _rel(ours, truth), _rel(torch_bf16, truth)
        assert e <= max(3e-2, 1.5 * et), (what, e, et)

    bound(logits, t_logits, a_logits, "logits")
    bound(dX[:, :d_in], t_dX, a_dX, "dX")
    for k in names:
        bound(got[k], t_grads[k], a_grads[k], k)


def test_mlp_train_device_row_count_and_bf16_dx(cuda):
    """Rows beyond a device-side row count (graph replay over a capacity) are
    neither computed nor counted; dX in BF16; two forwards in a row keep
    separate saved state."""
    W, L, d_in, K0, cap, n = 192, 3, 70, 80, 3000, 2345
    net = _net(d_in, W, L, seed=5).to(cuda)
    g = torch.Generator().manual_seed(9)
    X = torch.zeros((cap, K0), dtype=torch.bfloat16)
    X[:, :d_in] = torch.randn((cap, d_in), generator=g).to(torch.bfloat16)
    dY = torch.randn((cap, 3), generator=g) / n
    tc = TcTrainMLP(net, K0)
    tc.pack()
    n_dev = torch.tensor([n], dtype=torch.int64, device=cuda)
    Xd = X.to(cuda)
    out = torch.full((cap, 3), 7.0, device=cuda)
    logits, st = tc.forward(Xd, out=out, n_rows_dev=n_dev)
    dX = torch.full((cap, K0), 5.0, dtype=torch.bfloat16, device=cuda)
    dX, grads = tc.backward(st, dY.to(cuda), dX=dX)
    torch.cuda.synchronize()
    assert torch.all(logits[n:] == 7.0) and torch.all(dX[n:].float() == 5.0)
    e_logits, e_dX, e_grads = _emulate(net.cpu(), X[:n, :d_in].double(), dY[:n])
    assert _rel(logits[:n], e_logits) <= 3e-3
    assert _rel(dX[:n, :d_in].float(), e_dX) <= 5e-3
    for k, v in zip(_names(L), grads):
        assert _rel(v, e_grads[k]) <= 3e-3, k


def test_weight_gradients_of_two_mlps_in_one_launch(cuda):
    """The weight-gradient passes of two MLPs in one launch (the SMs split
    over eight passes) give the gradients of two separate launches up to
    the grouping of the FP32 partial sums (rel-L2 1e-5), and the same
    launch twice gives bit-identical gradients (fixed summation order)."""
    from voxurf_gb300._torch import stream_ptr

    n = 152 * 128 * 2 + 33
    nets = [_net(70, 192, 3, seed=21).to(cuda), _net(60, 192, 3, seed=22).to(cuda)]
    K0s = [80, 64]
    g = torch.Generator().manual_seed(4)
    engs, states, dYs = [], [], []
    for net, K0 in zip(nets, K0s):
        d_in = net[0].in_features
        X = torch.zeros((n, K0), dtype=torch.bfloat16)
        X[:, :d_in] = torch.randn((n, d_in), generator=g).to(torch.bfloat16)
        tc = TcTrainMLP(net, K0)
        tc.pack()
        _, st = tc.forward(X.to(cuda))
        engs.append(tc)
        states.append(st)
        dYs.append((torch.randn((n, 3), generator=g) / n).to(cuda))
    sep = [tc.backward(st, dY, dx_dtype=torch.float32)[1] for tc, st, dY in zip(engs, states, dYs)]
    runs = []
    for _ in range(2):
        pend, grads = [], []
        for tc, st, dY in zip(engs, states, dYs):
            _, gr, p = tc.backward_chain(st, dY, dx_dtype=torch.float32)
            pend.append(p)
            grads.append(gr)
        TcTrainMLP.weight_gradients(pend, stream_ptr(cuda))
        torch.cuda.synchronize()
        runs.append([[t.clone() for t in gr] for gr in grads])
    for a_list, b_list in zip(runs[0], sep):
        for a, b in zip(a_list, b_list):
            assert _rel(a, b) <= 1e-5
    for a_list, b_list in zip(runs[0], runs[1]):
        for a, b in zip(a_list, b_list):
            assert torch.equal(a, b)
