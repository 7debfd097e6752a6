"""Parity of the TV and Adam drop-ins (and the fused grid sweep) with the
oracle.  The float pipelines round the same operations on both sides (once
per operation, and the Adam moments with the fused multiply-adds of the
reference's compiled kernel), so the restatements must match bit for bit."""
import numpy as np
import pytest
import torch

from oracle import cref
from voxurf_gb300 import adam_upd_cuda, total_variation_cuda
from voxurf_gb300._torch import ptr, stream_ptr
from voxurf_gb300 import _native

pytestmark = pytest.mark.gpu


def _grid(C, X, Y, Z, seed, sparse=False):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.7, size=(1, C, X, Y, Z)).astype(np.float32)
    g = rng.normal(0, 1e-3, size=p.shape).astype(np.float32)
    if sparse:
        g[rng.uniform(size=g.shape) < 0.7] = 0
    m = (rng.uniform(size=p.shape) < 0.8).astype(np.float32)
    return p, g, m


@pytest.mark.parametrize("C,X,Y,Z", [(1, 32, 32, 32), (12, 16, 20, 24), (1, 7, 1, 5)])
@pytest.mark.parametrize("dense", [True, False])
def test_tv_add_grad_bit_exact(cuda, C, X, Y, Z, dense):
    p, g, m = _grid(C, X, Y, Z, seed=C + X, sparse=not dense)
    wx, wy, wz = 0.3, 0.7, 1.1
    ref = cref.tv_add_grad(p, g.copy(), wx, wy, wz, dense)
    tp, tg = torch.from_numpy(p).to(cuda), torch.from_numpy(g).to(cuda)
    total_variation_cuda.total_variation_add_grad(tp, tg, wx, wy, wz, dense)
    assert np.array_equal(tg.cpu().numpy(), ref)
    ref_m = cref.tv_add_grad(p, g.copy(), wx, wy, wz, dense, mask=m)
    tg = torch.from_numpy(g).to(cuda)
    total_variation_cuda.total_variation_add_grad_new(tp, tg, torch.from_numpy(m).to(cuda), wx, wy, wz, dense)
    assert np.array_equal(tg.cpu().numpy(), ref_m)


def test_tv_channel_last_matches_channel_first(cuda):
    C, X, Y, Z = 12, 9, 10, 11
    p, g, _ = _grid(C, X, Y, Z, seed=5)
    pcl = np.ascontiguousarray(p[0].transpose(1, 2, 3, 0))
    gcl = np.ascontiguousarray(g[0].transpose(1, 2, 3, 0))
    tp, tg = torch.from_numpy(pcl).to(cuda), torch.from_numpy(gcl).to(cuda)
    _native.call("vx_total_variation_add_grad", ptr(tp), ptr(tg), 1.0, 0.5, 0.25, 1, C, X, Y, Z, 1, stream_ptr())
    ref = cref.tv_add_grad(p, g.copy(), 1.0, 0.5, 0.25, True)
    assert np.array_equal(tg.cpu().numpy(), ref[0].transpose(1, 2, 3, 0))


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_adam_upd_bit_exact(cuda, mode):
    rng = np.random.default_rng(mode)
    n = 100003
    p = rng.normal(size=n).astype(np.float32)
    g = rng.normal(size=n).astype(np.float32)
    g[rng.uniform(size=n) < 0.3] = 0
    m = rng.normal(size=n).astype(np.float32) * 0.1
    v = rng.uniform(size=n).astype(np.float32) * 0.01
    pl = rng.uniform(size=n).astype(np.float32)
    rp, rm, rv = p.copy(), m.copy(), v.copy()
    cref.adam_upd(mode, rp, g, rm, rv, 7, 0.9, 0.99, 1e-2, 1e-8, perlr=pl if mode == 2 else None)
    T = lambda a: torch.from_numpy(a.copy()).to(cuda)
    tp, tg, tm, tv = T(p), T(g), T(m), T(v)
    if mode == 0:
        adam_upd_cuda.adam_upd(tp, tg, tm, tv, 7, 0.9, 0.99, 1e-2, 1e-8)
    elif mode == 1:
        adam_upd_cuda.masked_adam_upd(tp, tg, tm, tv, 7, 0.9, 0.99, 1e-2, 1e-8)
    else:
        adam_upd_cuda.adam_upd_with_perlr(tp, tg, tm, tv, T(pl), 7, 0.9, 0.99, 1e-2, 1e-8)
    assert np.array_equal(tp.cpu().numpy(), rp)
    assert np.array_equal(tm.cpu().numpy(), rm)
    assert np.array_equal(tv.cpu().numpy(), rv)


def _torch_utils_adam(p, g, m, v, step, lr, betas, eps, per_lr=None):
    """lib/utils.py:177-199 on CPU float32 torch (the reference optimizer)."""
    b1, b2 = betas
    bc1 = 1 - b1 ** step
    bc2 = 1 - b2 ** step
    m.mul_(b1).add_(g, alpha=1 - b1)
    v.mul_(b2).addcmul_(g, g, value=1 - b2)
    denom = (v.sqrt() / (bc2 ** 0.5)).add_(eps)
    step_size = lr / bc1
    if per_lr is not None:
        p.addcdiv_(m * per_lr, denom, value=-step_size)
    else:
        p.addcdiv_(m, denom, value=-step_size)


@pytest.mark.parametrize("per_lr", [False, True])
def test_adam_step_matches_utils_adam(cuda, per_lr):
    torch.manual_seed(0)
    n = 4099
    p, g = torch.randn(n), torch.randn(n) * 1e-2
    m, v = torch.zeros(n), torch.zeros(n)
    pl = torch.rand(n) if per_lr else None
    gp, gg, gm, gv = p.to(cuda), g.to(cuda), m.to(cuda), v.to(cuda)
    gpl = pl.to(cuda) if per_lr else None
    for step in range(1, 4):
        _torch_utils_adam(p, g, m, v, step, 1e-3, (0.9, 0.99), 1e-8, pl)
        _native.call("vx_adam_step", ptr(gp), ptr(gg), ptr(gm), ptr(gv), ptr(gpl), n, 1e-3, 0.9, 0.99, 1e-8, step, 0,
                     stream_ptr())
    torch.testing.assert_close(gp.cpu(), p, rtol=1e-6, atol=1e-7)
    torch.testing.assert_close(gm.cpu(), m, rtol=1e-6, atol=1e-9)
    torch.testing.assert_close(gv.cpu(), v, rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("C,R,dense", [(1, 24, True), (12, 20, True), (12, 20, False)])
def test_fused_grid_tv_adam(cuda, C, R, dense):
    """TV(old p) -> utils.Adam -> new p, bf16 shadow, grad reset; against the
    oracle TV (channel-last) followed by the torch utils.Adam."""
    rng = np.random.default_rng(C * R)
    p = rng.normal(size=(R, R, R, C)).astype(np.float32)
    g = rng.normal(scale=1e-3, size=p.shape).astype(np.float32)
    if not dense:
        g[rng.uniform(size=g.shape) < 0.5] = 0
    m = rng.normal(scale=1e-3, size=p.shape).astype(np.float32)
    v = rng.uniform(size=p.shape).astype(np.float32) * 1e-5
    w = 0.05
    g_tv = cref.tv_add_grad(p, g.copy(), w, w, w, dense, channel_last=True)
    tp, tg, tm, tv = (torch.from_numpy(a.copy()) for a in (p, g_tv, m, v))
    _torch_utils_adam(tp, tg, tm, tv, 3, 1e-2, (0.9, 0.99), 1e-8)
    T = lambda a: torch.from_numpy(a.copy()).to(cuda)
    gin, gg, gm, gv = T(p), T(g), T(m), T(v)
    gout = torch.empty_like(gin)
    shadow = torch.empty(gin.shape, dtype=torch.bfloat16, device=cuda)
    _native.call("vx_grid_tv_adam_step", ptr(gin), ptr(gout), ptr(gg), ptr(gm), ptr(gv), None, ptr(shadow), C, R, R,
                 R, 1, 1, w, int(dense), 1e-2, 0.9, 0.99, 1e-8, 3, 1, stream_ptr())
    torch.testing.assert_close(gout.cpu(), tp, rtol=1e-6, atol=1e-7)
    torch.testing.assert_close(gm.cpu(), tm, rtol=1e-6, atol=1e-10)
    # the shadow is the round-to-nearest BF16 copy of the kernel's own FP32 result
    torch.testing.assert_close(shadow.float(), gout.bfloat16().float(), rtol=0, atol=0)
    assert torch.count_nonzero(gg) == 0


@pytest.mark.parametrize("dense", [True, False])
def test_row_sweep_bit_identical_to_generic_sweep(cuda, dense):
    """The row-structured sweep (channel-last, 12 channels) and the generic
    sweep (channel-first) apply the same operations in the same order."""
    C, X, Y, Z = 12, 9, 14, 20
    rng = np.random.default_rng(int(dense))
    p = rng.normal(size=(C, X, Y, Z)).astype(np.float32)
    g = rng.normal(scale=1e-3, size=p.shape).astype(np.float32)
    g[rng.uniform(size=g.shape) < 0.4] = 0
    m = rng.normal(scale=1e-3, size=p.shape).astype(np.float32)
    v = rng.uniform(size=p.shape).astype(np.float32) * 1e-5
    outs = []
    for cl in (0, 1):
        conv = (lambda a: np.ascontiguousarray(a.transpose(1, 2, 3, 0))) if cl else (lambda a: a.copy())
        T = lambda a: torch.from_numpy(conv(a)).to(cuda)
        pin, gg, gm, gv = T(p), T(g), T(m), T(v)
        pout = torch.empty_like(pin)
        _native.call("vx_grid_tv_adam_step", ptr(pin), ptr(pout), ptr(gg), ptr(gm), ptr(gv), None, None, C, X, Y, Z,
                     cl, 1, 0.07, int(dense), 1e-2, 0.9, 0.99, 1e-8, 2, 0, stream_ptr())
        res = [pout, gm, gv]
        if cl:
            res = [r.permute(3, 0, 1, 2) for r in res]
        outs.append([r.cpu() for r in res])
    for a, b in zip(*outs):
        assert torch.equal(a, b)


@pytest.mark.parametrize("C,dense,shadow", [(12, True, True), (12, False, False), (1, True, False),
                                            (1, False, False)])
@pytest.mark.parametrize("Z", [36, 48])
def test_touched_sweep_bit_identical_to_dense_sweep(cuda, C, dense, shadow, Z):
    """A gradient that is zero outside marked voxels: the sweep that reads it
    only at the marks gives bit-identical parameters, moments and shadow to
    the dense sweep; zero_grad resets exactly the marked voxels; the clear
    kernel then zeroes marked rows and the marks (incl. a ragged tail)."""
    X, Y = 7, 11
    rng = np.random.default_rng(C + 2 * int(dense))
    p = rng.normal(size=(X, Y, Z, C)).astype(np.float32)
    marks = rng.uniform(size=(X, Y, Z)) < 0.15
    g = rng.normal(scale=1e-3, size=p.shape).astype(np.float32) * marks[..., None]
    g[rng.uniform(size=g.shape) < 0.1] = 0           # marked voxels may hold exact zeros
    m = rng.normal(scale=1e-3, size=p.shape).astype(np.float32)
    v = rng.uniform(size=p.shape).astype(np.float32) * 1e-5
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    touched = torch.zeros(_round16(X * Y * Z), dtype=torch.uint8, device=cuda)
    touched[:X * Y * Z] = T(marks.reshape(-1).astype(np.uint8))
    outs = []
    for fn in ("vx_grid_tv_adam_step", "vx_grid_tv_adam_step_touched"):
        pin, gg, gm, gv = T(p), T(g), T(m), T(v)
        pout = torch.empty_like(pin)
        sh = torch.empty(pin.shape, dtype=torch.bfloat16, device=cuda) if shadow else None
        extra = (ptr(touched),) if fn.endswith("touched") else ()
        _native.call(fn, ptr(pin), ptr(pout), ptr(gg), ptr(gm), ptr(gv), None, ptr(sh), C, X, Y, Z, int(C > 1), 1,
                     0.07, int(dense), 1e-2, 0.9, 0.99, 1e-8, 2, 1, *extra, stream_ptr())
        outs.append([pout.cpu(), gm.cpu(), gv.cpu(), gg.cpu()] + ([sh.float().cpu()] if shadow else []))
    for a, b in zip(*outs):
        assert torch.equal(a, b)
    assert torch.count_nonzero(outs[1][3]) == 0
    # clear kernel
    gg = T(g)
    n_vox = X * Y * Z
    _native.call("vx_grid_clear_touched", ptr(gg), ptr(touched), n_vox, C, stream_ptr())
    assert torch.count_nonzero(gg) == 0 and torch.count_nonzero(touched) == 0
    with pytest.raises(RuntimeError):
        _native.call("vx_grid_clear_touched", ptr(gg), ptr(touched[1:]), n_vox - 1, C, stream_ptr())


def _round16(n):
    return (n + 15) // 16 * 16


def test_adam_multi_matches_single(cuda):
    """One multi-tensor launch == one vx_adam_step launch per tensor."""
    import ctypes

    torch.manual_seed(1)
    sizes = [70 * 192, 192, 192 * 192, 192, 3 * 192, 3, 5000, 1]
    lrs = [1e-3, 1e-3, 3e-3, 3e-3, 1e-2, 1e-2, 1e-3, 1e-3]
    steps = [1, 1, 5, 5, 2, 2, 9, 9]
    a = [[torch.randn(n, device=cuda) for n in sizes] for _ in range(4)]
    b = [[t.clone() for t in grp] for grp in a]
    b[2] = [t.abs() * 1e-3 for t in b[2]]
    a[2] = [t.clone() for t in b[2]]
    a[3] = [t.abs() * 1e-4 for t in a[3]]
    b[3] = [t.clone() for t in a[3]]
    for (p, g, m, v), n, lr, s in zip(zip(*a), sizes, lrs, steps):
        _native.call("vx_adam_step", ptr(p), ptr(g), ptr(m), ptr(v), None, n, lr, 0.9, 0.99, 1e-8, s, 0, stream_ptr())
    k = len(sizes)
    P = ctypes.c_void_p * k
    _native.call("vx_adam_step_multi", k, *[P(*[t.data_ptr() for t in grp]) for grp in b],
                 (ctypes.c_int64 * k)(*sizes), (ctypes.c_double * k)(*lrs), (ctypes.c_int64 * k)(*steps), 0.9, 0.99,
                 1e-8, stream_ptr())
    for grp_a, grp_b in zip(a, b):
        for x, y in zip(grp_a, grp_b):
            assert torch.equal(x, y)
