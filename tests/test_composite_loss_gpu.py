"""vx_fine_composite_loss (compositing + photometric loss + compositing
backward in one pass) against vx_fine_composite, torch's loss with autograd
and vx_fine_composite_backward on the same inputs.

Cases: rays without shaded rows, rays whose k-branch colour leaves [0, 1]
(clamp backward), the last ray's alphainv_last inside and outside the
entropy clamp, both k_into_logit settings.  FP32 throughout: outputs equal
the unfused path's to 1e-6 relative (the forward sums are the same per-lane
sums; the loss gradient's scale factor is formed in another order, the loss
sums are added in another order).
"""
import numpy as np
import pytest
import torch

from voxurf_gb300 import _abi, _native
from voxurf_gb300._torch import ptr, stream_ptr

pytestmark = pytest.mark.gpu


def _case(cuda, N, seed, last_value):
    g = torch.Generator().manual_seed(seed)
    n_rows = torch.randint(0, 70, (N,), generator=g)
    n_rows[::7] = 0
    off = torch.zeros(N + 1, dtype=torch.int64)
    off[1:] = torch.cumsum(n_rows, 0)
    S2 = int(off[-1])
    w2 = torch.rand(S2, generator=g) * 0.08
    logit = torch.randn((S2, 3), generator=g) * 2
    kout = torch.randn((S2, 3), generator=g) * 3       # pushes some k colours past 0 / 1
    alast = torch.rand(N, generator=g)
    alast[-1] = last_value
    target = torch.rand((N, 3), generator=g)
    return [t.to(cuda) for t in (off, w2, logit, kout, alast, target)], S2


def _unfused(cuda, off, w2, logit, kout, alast, target, bg, wm, w0, we, k_into):
    N, S2 = target.shape[0], w2.shape[0]
    klogit = logit + kout
    rgb0 = torch.empty((N, 3), device=cuda)
    rgbk = torch.empty((N, 3), device=cuda)
    raw = torch.empty((N, 3), device=cuda)
    a = _abi.FineCompositeArgs()
    a.n_rays, a.s2_off, a.w2, a.logit, a.klogit, a.alphainv_last, a.bg = N, ptr(off), ptr(w2), ptr(logit), \
        ptr(klogit), ptr(alast), bg
    a.rgb0, a.rgbk, a.rgbk_raw, a.has_k = ptr(rgb0), ptr(rgbk), ptr(raw), 1
    _abi.call_struct("vx_fine_composite", a, stream_ptr())
    r0 = rgb0.clone().requires_grad_(True)
    rk = rgbk.clone().requires_grad_(True)
    al = alast.clone().requires_grad_(True)
    loss = wm * torch.nn.functional.mse_loss(rk, target) + w0 * torch.nn.functional.mse_loss(r0, target)
    if we > 0:
        p = al[..., -1].clamp(1e-6, 1 - 1e-6)
        loss = loss + we * (-(p * torch.log(p) + (1 - p) * torch.log(1 - p))).mean()
    loss.backward()
    g_last = al.grad if we > 0 else torch.zeros_like(alast)
    d_logit = torch.zeros((S2, 3), device=cuda)
    d_klogit = torch.zeros((S2, 3), device=cuda)
    d_w2 = torch.empty(S2, device=cuda)
    d_last = torch.empty(N, device=cuda)
    b = _abi.FineCompositeBwdArgs()
    b.n_rays, b.s2_off, b.w2, b.logit, b.klogit, b.rgbk_raw = N, ptr(off), ptr(w2), ptr(logit), ptr(klogit), ptr(raw)
    b.g_rgb0, b.g_rgbk, b.bg, b.g_last_in = ptr(r0.grad), ptr(rk.grad), bg, ptr(g_last)
    b.d_logit, b.d_klogit, b.d_w2, b.d_last, b.has_k = ptr(d_logit), ptr(d_klogit), ptr(d_w2), ptr(d_last), 1
    _abi.call_struct("vx_fine_composite_backward", b, stream_ptr())
    if k_into:
        d_logit = d_logit + d_klogit
    return dict(rgb0=rgb0, rgbk=rgbk, d_logit=d_logit, d_kout=d_klogit, d_w2=d_w2, d_last=d_last,
                loss=loss.detach().reshape(1))


def _fused(cuda, off, w2, logit, kout, alast, target, bg, wm, w0, we, k_into):
    N, S2 = target.shape[0], w2.shape[0]
    lib = _native.load()
    _abi._declare()
    nb = int(lib.vx_fine_composite_loss_scratch_bytes(N))
    out = dict(rgb0=torch.empty((N, 3), device=cuda), rgbk=torch.empty((N, 3), device=cuda),
               d_logit=torch.full((S2, 3), 7.0, device=cuda), d_kout=torch.full((S2, 3), 7.0, device=cuda),
               d_w2=torch.empty(S2, device=cuda), d_last=torch.empty(N, device=cuda),
               loss=torch.empty(1, device=cuda))
    scratch = torch.empty(nb, dtype=torch.uint8, device=cuda)
    a = _abi.FineCompositeLossArgs()
    a.n_rays, a.s2_off, a.w2, a.logit, a.kout, a.alphainv_last, a.target, a.bg = N, ptr(off), ptr(w2), \
        ptr(logit), ptr(kout), ptr(alast), ptr(target), bg
    a.w_main, a.w_rgb0, a.w_entropy_last = wm, w0, we
    a.rgb0, a.rgbk, a.d_logit, a.d_kout = ptr(out["rgb0"]), ptr(out["rgbk"]), ptr(out["d_logit"]), \
        ptr(out["d_kout"])
    a.d_w2, a.d_last, a.loss = ptr(out["d_w2"]), ptr(out["d_last"]), ptr(out["loss"])
    a.scratch, a.scratch_bytes, a.k_into_logit = ptr(scratch), nb, int(k_into)
    _abi.call_struct("vx_fine_composite_loss", a, stream_ptr())
    return out


@pytest.mark.parametrize("N,last_value,k_into", [(1, 0.3, 1), (37, 0.0, 0), (8192, 0.7, 1), (3000, 1.0, 0),
                                                 (257, 0.5e-6, 1)])
@pytest.mark.parametrize("weights", [(1.0, 0.5, 0.001), (1.0, 0.5, 0.0)])
def test_fused_composite_loss_matches_unfused(cuda, N, last_value, k_into, weights):
    wm, w0, we = weights
    (off, w2, logit, kout, alast, target), S2 = _case(cuda, N, N + 11, last_value)
    bg = 1.0
    ref = _unfused(cuda, off, w2, logit, kout, alast, target, bg, wm, w0, we, k_into)
    got = _fused(cuda, off, w2, logit, kout, alast, target, bg, wm, w0, we, k_into)
    torch.cuda.synchronize()
    for k in ("rgb0", "rgbk", "d_w2", "d_last", "d_logit", "d_kout"):
        a, b = got[k].double().cpu(), ref[k].double().cpu()
        # rtol per element, atol 1e-6 of the largest entry (sums of terms of
        # either sign can cancel, and a one-ulp difference of a loss gradient
        # then shows up relative to the terms, not to their sum)
        scale = float(b.abs().max()) if b.numel() else 0.0
        assert torch.allclose(a, b, rtol=1e-6, atol=1e-6 * scale), (k, float((a - b).abs().max()), scale)
    np.testing.assert_allclose(float(got["loss"]), float(ref["loss"]), rtol=1e-6)


def test_fused_composite_loss_rejects_bad_arguments(cuda):
    lib = _native.load()
    _abi._declare()
    a = _abi.FineCompositeLossArgs()
    a.n_rays = 0
    assert lib.vx_fine_composite_loss(a, stream_ptr()) != 0
    a.n_rays = 4
    assert lib.vx_fine_composite_loss(a, stream_ptr()) != 0       # null pointers
