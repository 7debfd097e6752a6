"""Render server against the FP64 oracle of the reference forward
(global_step=None) and the plain per-request FP32 render; each result must
be the same alone and in a mix of requests.

Tolerances: FP32 server RGB max abs <= 1e-5 (oracle and plain render);
BF16 server (k0 + MLP in BF16) RGB max abs <= 1e-3 against the oracle; a
request's result alone vs in a mix <= 1e-3 max abs (BF16 bound; cuBLAS may
pick other GEMM kernels for other row counts), depth relative to its scale.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle.voxurf_oracle import OracleFine, camera_rays_f32
from voxurf_gb300 import _native, configs, serve
from voxurf_gb300._torch import ptr, stream_ptr

pytestmark = pytest.mark.gpu

RK = dict(configs.FINE_RENDER_KWARGS)
S_VAL = 0.02


def _models(cuda, precision, n=2, R=32):
    ms = configs.build_serve_models(R, precision, device=cuda, n=n, mask_voxels=3.0, width=64)
    for m in ms:
        m.s_val = torch.ones(1) * S_VAL
    return ms


def _server(cuda, models, precision, **kw):
    scenes = [serve.ResidentScene(m, s_val=S_VAL, precision=precision) for m in models]
    kw.setdefault("arena_pixels", 1 << 20)
    return serve.RenderServer(scenes, **kw)


def _oracle_view(model, c2w, H, W):
    f = 1.2 * W
    o, d, v = camera_rays_f32(c2w, f, f, W / 2.0, H / 2.0, H, W)
    orc = OracleFine(model, dtype=torch.float64)
    with torch.no_grad():
        ret = orc(torch.from_numpy(o), torch.from_numpy(d), torch.from_numpy(v), global_step=None,
                  **dict(RK, render_depth=True))
    return ret["rgb_marched"].numpy().reshape(H, W, 3), ret["depth"].numpy().reshape(H, W)


def _pose(i):
    return serve.random_pose(np.random.default_rng(1000 + i))


def test_camera_rays_bit_exact(cuda):
    H, W = 30, 41
    c2w = _pose(0)
    f = 1.2 * W
    out = [torch.empty(H * W, 3, device=cuda) for _ in range(3)]
    m = (ctypes.c_float * 12)(*np.asarray(c2w, np.float32)[:3, :4].reshape(-1))
    _native.call("vx_camera_rays", m, f, f, W / 2.0, H / 2.0, H, W, 1, *[ptr(t) for t in out], stream_ptr())
    for got, want in zip(out, camera_rays_f32(c2w, f, f, W / 2.0, H / 2.0, H, W)):
        assert np.array_equal(got.cpu().numpy(), want)


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("bf16", 1e-3)])
def test_server_matches_fp64_oracle(cuda, precision, tol):
    models = _models(cuda, precision)
    srv = _server(cuda, models, precision, tick_rays=700)
    views = [(0, _pose(1), 24, 32), (1, _pose(2), 30, 20), (0, _pose(3), 16, 16)]
    reqs = [srv.submit(s, c2w, H, W) for s, c2w, H, W in views]
    srv.run_until_idle()
    assert srv.ticks >= 3 and srv.rows_shaded > 200
    for r, (s, c2w, H, W) in zip(reqs, views):
        rgb, depth = _oracle_view(models[s], c2w, H, W)
        err = np.abs(r.rgb - rgb).max()
        assert err <= tol, (precision, s, err)
        derr = np.abs(r.depth - depth).max() / max(1.0, np.abs(depth).max())
        assert derr <= 10 * tol, (precision, s, derr)


def test_server_fp32_matches_plain_render(cuda):
    models = _models(cuda, "fp32")
    srv = _server(cuda, models, "fp32", tick_rays=1000)
    for i, s in enumerate([1, 0]):
        c2w = _pose(10 + i)
        rgb, depth = srv.render(s, c2w, 40, 48)
        prgb, pdepth = serve.plain_render(models[s], c2w, 40, 48, chunk=512)
        assert np.abs(rgb - prgb.cpu().numpy()).max() <= 1e-5
        assert np.abs(depth - pdepth.cpu().numpy()).max() <= 1e-5 * max(1.0, float(pdepth.abs().max()))


def test_same_alone_and_in_mix(cuda):
    """Requests admitted while others are on the GPU share ticks with them;
    each result equals the one rendered alone."""
    models = _models(cuda, "bf16", n=3)
    views = [(0, _pose(20), 60, 80), (2, _pose(21), 30, 40), (1, _pose(22), 50, 50), (0, _pose(23), 12, 16)]
    alone = []
    for s, c2w, H, W in views:
        srv = _server(cuda, models, "bf16", tick_rays=2048)
        alone.append(srv.render(s, c2w, H, W))
    srv = _server(cuda, models, "bf16", tick_rays=2048)
    reqs = [srv.submit(*views[0])]
    srv.tick()                      # the first request is on the GPU ...
    reqs += [srv.submit(*v) for v in views[1:]]   # ... when the others arrive
    srv.run_until_idle()
    assert srv.ticks < sum(-(-H * W // 2048) for _, _, H, W in views)  # ticks were shared
    for r, (rgb, depth) in zip(reqs, alone):
        assert np.abs(r.rgb - rgb).max() <= 1e-3
        assert np.abs(r.depth - depth).max() <= 1e-3 * max(1.0, np.abs(depth).max())


def test_tensor_core_mlp_path_matches_oracle(cuda):
    """192-wide BF16 scenes shade through the fused tcgen05 MLP: same result
    as the per-layer MLP engines and within the BF16 bound of the oracle."""
    models = configs.build_serve_models(32, "bf16", device=cuda, n=2, mask_voxels=3.0, width=192)
    for m in models:
        m.s_val = torch.ones(1) * S_VAL
    scenes = [serve.ResidentScene(m, s_val=S_VAL, precision="bf16") for m in models]
    assert all(s.tc is not None for s in scenes)
    views = [(0, _pose(50), 24, 32), (1, _pose(51), 20, 20)]
    res = {}
    for mlp in ("tc", "layers"):
        srv = serve.RenderServer(scenes, tick_rays=600, arena_pixels=1 << 16, mlp=mlp)
        reqs = [srv.submit(*v) for v in views]
        srv.run_until_idle()
        res[mlp] = [r.rgb for r in reqs]
    for (s, c2w, H, W), a, b in zip(views, res["tc"], res["layers"]):
        assert np.abs(a - b).max() <= 1e-3
        rgb, _ = _oracle_view(models[s], c2w, H, W)
        assert np.abs(a - rgb).max() <= 1e-3


def test_empty_space_skipping_is_exact(cuda):
    """Skipping the samples that lie in empty blocks of the mask leaves every
    result unchanged (same shaded rows; RGB equal up to the grouping of the
    FP64 transmittance products)."""
    models = _models(cuda, "fp32", n=2)
    views = [(0, _pose(40), 48, 64), (1, _pose(41), 40, 40), (0, _pose(42), 33, 17)]
    out = []
    for block in (0, 4, 8):
        scenes = [serve.ResidentScene(m, s_val=S_VAL, precision="fp32", skip_block=block) for m in models]
        srv = serve.RenderServer(scenes, tick_rays=1500, arena_pixels=1 << 16)
        reqs = [srv.submit(*v) for v in views]
        srv.run_until_idle()
        out.append((srv.rows_shaded, [r.rgb for r in reqs], [r.depth for r in reqs]))
    for rows, rgbs, depths in out[1:]:
        assert rows == out[0][0]
        for a, b in zip(rgbs, out[0][1]):
            assert np.abs(a - b).max() <= 1e-6
        for a, b in zip(depths, out[0][2]):
            assert np.abs(a - b).max() <= 1e-6


def test_admission_waits_for_arena(cuda):
    """With an arena of 2 x 40x40 pixels the third request waits for a free
    range; every request still completes with the result it has alone."""
    models = _models(cuda, "fp32", n=1)
    srv = _server(cuda, models, "fp32", tick_rays=512, arena_pixels=3200)
    reqs = [srv.submit(0, _pose(30 + i), 40, 40) for i in range(4)]
    srv.tick()
    assert len(srv.queue) == 2 and len(srv.active) == 2
    srv.run_until_idle()
    assert all(r.t_done is not None for r in reqs)
    ref = _server(cuda, models, "fp32", tick_rays=512)
    for i, r in enumerate(reqs):
        rgb, _ = ref.render(0, _pose(30 + i), 40, 40)
        assert np.abs(r.rgb - rgb).max() <= 1e-6


@pytest.mark.parametrize("staging", [0, 1])
def test_row_capacity_growth_and_feature_staging(cuda, staging):
    """A tick with more shaded rows than its slot holds grows the slot and
    redoes the tick's rows and features (the row count is read on the
    device, so the first pass skipped the rows beyond the capacity); both
    row assemblies of the features kernel give the same images as a server
    whose slots never overflow."""
    models = _models(cuda, "bf16", n=2)   # BF16 rows: both assemblies apply
    views = [(0, _pose(60), 40, 48), (1, _pose(61), 36, 36), (0, _pose(62), 20, 30)]
    out = []
    for rpr, stg in ((0.05, staging), (6.0, -1)):
        srv = _server(cuda, models, "bf16", tick_rays=1500, staging=stg, rows_per_ray=rpr)
        cap0 = [sl.rows_cap for sl in srv.slots]
        reqs = [srv.submit(*v) for v in views]
        srv.run_until_idle()
        caps = [sl.rows_cap for sl in srv.slots]
        out.append((srv.rows_shaded, [r.rgb for r in reqs], [r.depth for r in reqs], cap0, caps))
    rows, rgbs, depths, cap0, caps = out[0]
    assert rows == out[1][0] and rows > 0
    assert any(c > c0 for c, c0 in zip(caps, cap0))   # the small slots grew
    for a, b in zip(rgbs, out[1][1]):
        assert np.abs(a - b).max() <= 1e-6
    for a, b in zip(depths, out[1][2]):
        assert np.abs(a - b).max() <= 1e-6
