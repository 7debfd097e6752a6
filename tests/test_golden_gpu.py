"""The CUDA path against golden vectors of the reference's own Python code
(tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest
import torch

from oracle.voxurf_oracle import train_loss
from voxurf_gb300 import grid as vgrid
from voxurf_gb300 import _native
from voxurf_gb300._torch import ptr, stream_ptr
from voxurf_gb300.voxurf_fine import gaussian_taps, smooth_grid

from test_oracle_golden import FINE, OPS, _model_from_fixture, fine_fixture_inputs

pytestmark = pytest.mark.gpu


def test_dense_grid_forward_vs_reference(cuda):
    g = vgrid.DenseGrid(5, [7, 9, 11], [-1.0, -0.5, -2.0], [1.0, 1.5, 0.5]).to(cuda)
    with torch.no_grad():
        g.grid.copy_(torch.from_numpy(OPS["dg_grid"]))
    assert not g.grid.is_contiguous()  # channel-last storage
    out = g(torch.from_numpy(OPS["dg_xyz"]).to(cuda))
    np.testing.assert_allclose(out.detach().cpu().numpy(), OPS["dg_out"], rtol=1e-5, atol=2e-6)
    # backward = scatter adjoint: <d out, out> == <d grid, grid> for a linear map
    w = torch.randn_like(out)
    (out * w).sum().backward()
    lhs = float((out.detach() * w).double().sum())
    rhs = float((g.grid.grad * g.grid.detach()).double().sum())
    assert abs(lhs - rhs) <= 1e-4 * max(1.0, abs(lhs))


def test_smoothing_vs_reference(cuda):
    src = torch.from_numpy(OPS["smooth_in"]).to(cuda)
    out = smooth_grid(src, gaussian_taps(5, 0.8))
    np.testing.assert_allclose(out.cpu().numpy(), OPS["smooth_out"][0, 0], rtol=1e-5, atol=1e-6)


def test_smoothing_adjoint_identity(cuda):
    from voxurf_gb300.voxurf_fine import smooth_grid_adjoint

    torch.manual_seed(0)
    for shape in [(12, 10, 14), (3, 1, 7), (33, 2, 5)]:
        a = torch.randn(shape, device=cuda)
        b = torch.randn(shape, device=cuda)
        taps = gaussian_taps(5, 0.8)
        lhs = float((smooth_grid(a, taps).double() * b.double()).sum())
        rhs = float((a.double() * smooth_grid_adjoint(b, taps).double()).sum())
        assert abs(lhs - rhs) <= 1e-5 * max(1.0, abs(lhs)), shape


@pytest.mark.parametrize("ksize", [1, 3, 5, 7, 9])
def test_smoothing_and_adjoint_vs_oracle_conv(cuda, ksize):
    """Forward against the oracle's replicate-padded conv3d in FP64 and the
    adjoint against its autograd, on grids with ragged tiles (sizes that are
    not multiples of the 16 x 32 column tile or the x chunk), degenerate axes
    and the accumulate mode."""
    from oracle.voxurf_oracle import gaussian_kernel3d, smooth3d
    from voxurf_gb300.voxurf_fine import smooth_grid_adjoint

    sigma = 0.8
    taps = gaussian_taps(ksize, sigma)
    k3 = torch.from_numpy(np.einsum("i,j,k->ijk", *(taps.astype(np.float64),) * 3))
    gen = torch.Generator().manual_seed(ksize)
    for shape in [(40, 20, 37), (9, 33, 65), (1, 1, 1), (2, 3, 1), (17, 5, 2), (70, 17, 33)]:
        a = torch.randn(shape, generator=gen, dtype=torch.float64)
        g = torch.randn(shape, generator=gen, dtype=torch.float64)
        ad = a.clone().requires_grad_(True)
        ref = smooth3d(ad[None, None], k3)[0, 0]
        (ref * g).sum().backward()
        out = smooth_grid(a.float().to(cuda), taps)
        np.testing.assert_allclose(out.cpu().double().numpy(), ref.detach().numpy(), rtol=1e-5, atol=1e-6,
                                   err_msg=str(shape))
        adj = smooth_grid_adjoint(g.float().to(cuda), taps)
        np.testing.assert_allclose(adj.cpu().double().numpy(), ad.grad.numpy(), rtol=1e-5, atol=2e-6,
                                   err_msg=str(shape))
        base = torch.randn(shape, generator=gen).to(cuda)
        acc = smooth_grid_adjoint(g.float().to(cuda), taps, out=base.clone(), accumulate=True)
        np.testing.assert_allclose(acc.cpu().numpy(), (base + adj).cpu().numpy(), rtol=1e-6, atol=1e-6)
    # the 3-D kernel the oracle builds (float32 exponentials, normalised) is the taps' cube
    np.testing.assert_allclose(gaussian_kernel3d(ksize, sigma), k3.numpy(), rtol=1e-6, atol=1e-8)


def test_utils_adam_vs_reference(cuda):
    p0 = torch.from_numpy(OPS["adam_p0"]).to(cuda).contiguous()
    p1 = torch.from_numpy(OPS["adam_p1"]).to(cuda).contiguous()
    count = torch.from_numpy(OPS["adam_count"]).to(cuda)
    per_lr = (count.float() / count.max()).contiguous()
    ms = [torch.zeros_like(p0), torch.zeros_like(p1)]
    vs = [torch.zeros_like(p0), torch.zeros_like(p1)]
    for it in range(3):
        for p, m, v, gkey, lr, pl in ((p0, ms[0], vs[0], "adam_grads0", 1e-2, per_lr),
                                      (p1, ms[1], vs[1], "adam_grads1", 3e-3, None)):
            g = torch.from_numpy(OPS[gkey][it]).to(cuda).contiguous()
            _native.call("vx_adam_step", ptr(p), ptr(g), ptr(m), ptr(v), ptr(pl), p.numel(), lr, 0.9, 0.99, 1e-8,
                         it + 1, 0, stream_ptr())
    np.testing.assert_allclose(p0.cpu().numpy(), OPS["adam_out0"], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(p1.cpu().numpy(), OPS["adam_out1"], rtol=1e-6, atol=1e-7)


def test_fine_step_vs_reference_golden(cuda):
    model = _model_from_fixture(device=cuda)
    ro, rd, vd, tgt, rk = fine_fixture_inputs()
    T = lambda a: torch.from_numpy(a).to(cuda)
    ret = model(T(ro), T(rd), T(vd), global_step=1, **rk)
    loss = train_loss(ret, T(tgt))
    loss.backward()
    assert ret["weights"].numel() == FINE["weights"].size
    for k in ("rgb_marched", "rgb_marched0"):
        assert np.abs(ret[k].detach().cpu().numpy() - FINE[k]).max() <= 1e-5, k
    rel = lambda a, b: np.linalg.norm(a.reshape(-1) - b.reshape(-1)) / np.linalg.norm(b.reshape(-1))
    assert rel(model.sdf.grid.grad.cpu().numpy(), FINE["grad_sdf"]) <= 1e-5
    k0g = model.k0.grid.grad.contiguous().cpu().numpy()
    assert rel(k0g, FINE["grad_k0"]) <= 1e-5
    for n, p in model.rgbnet.named_parameters():
        assert rel(p.grad.cpu().numpy(), FINE["grad_mlp." + n]) <= 1e-5, n
    for n, p in model.k_rgbnet.named_parameters():
        assert rel(p.grad.cpu().numpy(), FINE["grad_mlp.k." + n]) <= 1e-5, n


def test_coarse_step_vs_reference_golden(cuda):
    from test_oracle_golden import COARSE, coarse_fixture_inputs, coarse_model_from_fixture

    model = coarse_model_from_fixture(device=cuda)
    ro, rd, vd, tgt, rk = coarse_fixture_inputs()
    T = lambda a: torch.from_numpy(a).to(cuda)
    ret = model(T(ro), T(rd), T(vd), global_step=1, **rk)
    loss = train_loss(ret, T(tgt), weight_rgb0=0)
    loss.backward()
    assert ret["weights"].numel() == COARSE["weights"].size
    assert np.abs(ret["rgb_marched"].detach().cpu().numpy() - COARSE["rgb_marched"]).max() <= 1e-5
    rel = lambda a, b: np.linalg.norm(a.reshape(-1) - b.reshape(-1)) / np.linalg.norm(b.reshape(-1))
    assert rel(model.sdf.grid.grad.cpu().numpy(), COARSE["grad_sdf"]) <= 1e-5
    assert rel(model.k0.grid.grad.contiguous().cpu().numpy(), COARSE["grad_k0"]) <= 1e-5
    for n, p in model.rgbnet.named_parameters():
        assert rel(p.grad.cpu().numpy(), COARSE["grad_mlp." + n]) <= 1e-5, n
