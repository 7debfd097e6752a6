"""The reference's own CUDA kernels, run on the same GPU, as the pin of the
C restatement and of this library's kernels.

oracle/ref_build.py compiles the reference's lib/cuda/*_kernel.cu, unmodified,
into PTX; oracle/ref_cuda.py launches those kernels with the reference
launchers' shapes and host steps.  On the same inputs:

* the reference kernels' outputs must equal, bit for bit, the form of
  oracle/fma_forms.py recorded in fma_forms.REFERENCE: for each float
  expression, whether nvcc (default --fmad=true) fused an a*b+c into one
  multiply-add.  The test also reports every form that matches;
* the C restatement (oracle/cref.c) and this library's drop-in ops must equal
  the reference bit for bit: sampling (points included), the mask lookup
  (rounding ties included), TV, the three Adam updates and cumdist_thres;
  alpha2weight, whose scan this library carries in parallel, within the
  bars of the C-restatement tests.

Skips when the PTX was not built (the reference checkout was absent where
the build ran).  With VX_REF_KERNEL_REPORT=<path> the findings are written
there as JSON.
"""
import json
import os

import numpy as np
import pytest
import torch

from oracle import cref
from oracle import fma_forms as ff
from oracle import ref_cuda

pytestmark = pytest.mark.gpu

BMIN = np.array([-1.0, -1.0, -1.0], np.float32)
BMAX = np.array([1.0, 1.0, 1.0], np.float32)
REPORT: dict = {}


@pytest.fixture(scope="module")
def ref(cuda):
    if not ref_cuda.available():
        pytest.skip("the reference kernels' PTX was not built (no reference checkout where build() ran)")
    yield ref_cuda
    path = os.environ.get("VX_REF_KERNEL_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(REPORT, f, indent=1, sort_keys=True)


def _to(dev):
    return lambda a: torch.from_numpy(np.array(a, copy=True, order="C")).to(dev)


def _np(t):
    return t.detach().cpu().numpy()


def _forms_equal(forms: dict, got) -> list:
    return [k for k, v in forms.items() if np.array_equal(v, got)]


def _ulps(a, b) -> int:
    a = np.asarray(a, np.float32).ravel()
    b = np.asarray(b, np.float32).ravel()
    if a.size == 0:
        return 0
    ia, ib = a.view(np.int32).astype(np.int64), b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return int(np.max(np.abs(ia - ib)))


def _rays(n, seed):
    """Camera rays plus axis-aligned ones (zero components), rays that miss
    the box, rays starting inside it and tiny/huge directions."""
    from voxurf_gb300 import synthetic

    o, d, _ = synthetic.random_rays(n, seed=seed)
    rng = np.random.default_rng(seed + 7)
    eo = rng.uniform(-3, 3, size=(48, 3)).astype(np.float32)
    ed = rng.normal(size=(48, 3)).astype(np.float32)
    ed[:8, 1:] = 0
    ed[8:16, 0] = 0
    eo[16:24] = rng.uniform(-0.5, 0.5, size=(8, 3))
    ed[24:32] *= 1e-3
    ed[32:40] *= 1e3
    eo[40:48] = 5.0
    ed[40:48] = np.abs(ed[40:48])
    return np.concatenate([o, eo]), np.concatenate([d, ed])


@pytest.mark.parametrize("R,stepsize,n", [(96, 0.5, 2048), (256, 0.5, 8192), (384, 0.25, 512)])
def test_sampling_matches_reference_kernels(cuda, ref, R, stepsize, n):
    from voxurf_gb300 import render_utils_cuda as ru

    to = _to(cuda)
    o, d = _rays(n, seed=R + n)
    sd = np.float32(stepsize * 2.0 / R)
    args = (to(o), to(d), to(BMIN), to(BMAX), 0.1, 1e9, float(sd))
    got_ref = [_np(t) for t in ref.sample_pts_on_rays(*args)]
    got_ours = [_np(t) for t in ru.sample_pts_on_rays(*args)]
    restated = cref.sample_pts_on_rays(o, d, BMIN, BMAX, 0.1, 1e9, sd)
    names = ["rays_pts", "mask_outbbox", "ray_id", "step_id", "N_steps", "t_min", "t_max"]

    # which form of |d| and of the ray start the reference computes
    t_min = to(restated[5])
    st, di = (_np(t) for t in ref.infer_ray_start_dir(to(o), to(d), t_min))
    norms = ff.ray_norm(d)
    dir_forms = {k: d / v[:, None] for k, v in norms.items()}
    norm_hit = _forms_equal(dir_forms, di)
    start_hit = _forms_equal(ff.ray_start(o, d, restated[5]), st)
    rec = {"n_rays": len(o), "n_samples": int(restated[4].sum()), "norm_forms": norm_hit, "start_forms": start_hit}
    assert ff.REFERENCE["ray_norm"] in norm_hit and ff.REFERENCE["ray_start"] in start_hit, rec
    pts_hit = []
    for pf in ("plain", "fma"):
        cand = ff.sample_pts_on_rays(o, d, BMIN, BMAX, 0.1, 1e9, sd, ff.REFERENCE["ray_norm"],
                                     ff.REFERENCE["ray_start"], pf)
        if all(np.array_equal(a, b) for a, b in zip(cand, got_ref)):
            pts_hit.append(pf)
    rec["pts_forms"] = pts_hit
    rec["ours_vs_ref_pts_max_ulps"] = _ulps(got_ours[0], got_ref[0])
    rec["ours_vs_ref_pts_max_abs"] = float(np.max(np.abs(got_ours[0] - got_ref[0]))) if got_ref[0].size else 0.0
    rec["ours_vs_ref_pts_differing"] = int(np.sum(got_ours[0] != got_ref[0]))
    REPORT[f"sample_pts_on_rays R={R} stepsize={stepsize} n={n}"] = rec
    assert ff.REFERENCE["sample_point"] in pts_hit, rec
    for name, a, b, c in zip(names, got_ours, got_ref, restated):
        assert a.shape == b.shape, name
        assert np.array_equal(b, c), (name, "C restatement", np.argwhere(b != c)[:5])
        assert np.array_equal(a, b), (name, np.argwhere(a != b)[:5])


@pytest.mark.parametrize("shape", [(32, 32, 32), (17, 40, 9), (96, 96, 96)])
def test_maskcache_lookup_matches_reference_kernel(cuda, ref, shape):
    from voxurf_gb300 import render_utils_cuda as ru

    to = _to(cuda)
    rng = np.random.default_rng(sum(shape))
    world = rng.uniform(size=shape) < 0.3
    xyz = rng.uniform(-1.2, 1.2, size=(50000, 3)).astype(np.float32)
    scale = ((np.array(shape, np.float32) - 1) / (BMAX - BMIN)).astype(np.float32)
    shift = (-BMIN * scale).astype(np.float32)
    # points whose index lands on a half-way value: the rounding tie
    half = np.floor(rng.uniform(0, 1, size=(1000, 3)) * (np.array(shape) - 1)) + 0.5
    xyz[:1000] = ((half - shift) / scale).astype(np.float32)
    got_ref = _np(ref.maskcache_lookup(to(world), to(xyz), to(scale), to(shift)))
    got_ours = _np(ru.maskcache_lookup(to(world), to(xyz), to(scale), to(shift)))
    forms = ff.maskcache_lookup(world, xyz, scale, shift)
    hit = _forms_equal(forms, got_ref)
    agree = forms["plain"] == forms["fma"]
    rec = {"forms": hit, "points": len(xyz), "points_where_forms_differ": int((~agree).sum()),
           "ours_vs_ref_differing": int(np.sum(got_ours != got_ref))}
    REPORT[f"maskcache_lookup {shape}"] = rec
    assert ff.REFERENCE["maskcache_lookup"] in hit, rec
    assert np.array_equal(got_ref, cref.maskcache_lookup(world, xyz, scale, shift))
    assert np.array_equal(got_ours, got_ref), rec


def _segments(n_rays, seed, max_len=700):
    rng = np.random.default_rng(seed)
    lens = rng.integers(1, max_len, size=n_rays)
    lens[rng.uniform(size=n_rays) < 0.1] = 0
    ray_id = np.repeat(np.arange(n_rays), lens).astype(np.int64)
    alpha = rng.uniform(0, 0.05, size=ray_id.size).astype(np.float32)
    alpha[rng.uniform(size=alpha.size) < 0.002] = 0.9  # early termination
    return ray_id, alpha


def _near_stop_rays(alpha, ray_id, n_rays, rel=1e-4):
    """Rays whose running transmittance passes within `rel` of the 1e-3 stop:
    there the stop index is a threshold decision that a float loop and an
    FP64 scan may take one sample apart."""
    starts = np.searchsorted(ray_id, np.arange(n_rays))
    ends = np.searchsorted(ray_id, np.arange(n_rays), side="right")
    near = np.zeros(n_rays, bool)
    for r in range(n_rays):
        if ends[r] > starts[r]:
            Tc = np.cumprod(1.0 - alpha[starts[r]:ends[r]].astype(np.float64))
            near[r] = bool(np.any(np.abs(Tc / 1e-3 - 1.0) < rel))
    return near


def test_alpha2weight_matches_reference_kernels(cuda, ref):
    from voxurf_gb300 import render_utils_cuda as ru

    to = _to(cuda)
    n_rays = 1500
    ray_id, alpha = _segments(n_rays, seed=5)
    got_ref = [_np(t) for t in ref.alpha2weight(to(alpha), to(ray_id), n_rays)]
    restated = cref.alpha2weight(alpha, ray_id, n_rays)
    rec = {"forward_equals_restatement": [bool(np.array_equal(a, b)) for a, b in zip(got_ref, restated)]}
    got_ours = [_np(t) for t in ru.alpha2weight(to(alpha), to(ray_id), n_rays)]
    keep = ~_near_stop_rays(alpha, ray_id, n_rays)
    ks = keep[ray_id]
    rec["rays_near_stop"] = int((~keep).sum())
    rec["ours_vs_ref_weight_max_rel"] = float(np.max(np.abs(got_ours[0][ks] - got_ref[0][ks])
                                                     / (np.abs(got_ref[0][ks]) + 1e-9), initial=0.0))
    w, T, last, i_s, i_e = restated
    rng = np.random.default_rng(6)
    gw = rng.normal(size=alpha.size).astype(np.float32)
    gl = rng.normal(size=n_rays).astype(np.float32)
    state = [to(a) for a in (alpha, w, T, last, i_s, i_e)]
    g_ref = _np(ref.alpha2weight_backward(*state, n_rays, to(gw), to(gl)))
    rec["backward_forms"] = _forms_equal(ff.alpha2weight_backward(alpha, w, T, last, i_s, i_e, gw, gl), g_ref)
    g_ours = _np(ru.alpha2weight_backward(*state, n_rays, to(gw), to(gl)))
    rec["ours_vs_ref_grad_max_rel"] = float(np.max(np.abs(g_ours - g_ref)) / (np.max(np.abs(g_ref)) + 1e-12))
    REPORT["alpha2weight"] = rec
    assert all(rec["forward_equals_restatement"]), rec
    assert ff.REFERENCE["alpha2weight_backward"] in rec["backward_forms"], rec
    assert np.array_equal(g_ref, cref.alpha2weight_backward(alpha, w, T, last, i_s, i_e, n_rays, gw, gl))
    # this library carries the transmittance in a parallel scan, the reference
    # in a serial float loop: the bars of the C-restatement tests
    for a, b in zip(got_ours[3:], got_ref[3:]):
        assert np.array_equal(a[keep], b[keep])
    for a, b, sel in ((got_ours[0], got_ref[0], ks), (got_ours[1], got_ref[1], ks), (got_ours[2], got_ref[2], keep)):
        np.testing.assert_allclose(a[sel], b[sel], rtol=4e-6, atol=1e-9)
    assert rec["ours_vs_ref_grad_max_rel"] < 2e-5, rec


@pytest.mark.parametrize("dense", [True, False])
@pytest.mark.parametrize("masked", [False, True])
def test_total_variation_matches_reference_kernels(cuda, ref, dense, masked):
    from voxurf_gb300 import total_variation_cuda as tv

    to = _to(cuda)
    rng = np.random.default_rng(11 + 2 * dense + masked)
    p = (rng.normal(size=(1, 4, 19, 23, 17)) * 0.7).astype(np.float32)
    g = rng.normal(size=p.shape).astype(np.float32)
    g[rng.uniform(size=p.shape) < 0.5] = 0
    mk = (rng.uniform(size=p.shape) < 0.7).astype(np.float32) if masked else None
    w = (1e-2, 3e-3, 5e-2)
    gr, go = to(g.copy()), to(g.copy())
    if masked:
        ref.total_variation_add_grad_new(to(p), gr, to(mk), *w, dense)
        tv.total_variation_add_grad_new(to(p), go, to(mk), *w, dense)
    else:
        ref.total_variation_add_grad(to(p), gr, *w, dense)
        tv.total_variation_add_grad(to(p), go, *w, dense)
    forms = ff.tv_add_grad(p[0], g[0], *w, dense, mask=None if mk is None else mk[0])
    got_ref, got_ours = _np(gr)[0], _np(go)[0]
    rec = {"forms": _forms_equal(forms, got_ref), "ours_vs_ref_max_ulps": _ulps(got_ours, got_ref),
           "ours_vs_ref_differing": int(np.sum(got_ours != got_ref))}
    REPORT[f"total_variation dense={dense} masked={masked}"] = rec
    assert ff.REFERENCE["total_variation"] in rec["forms"], rec
    assert np.array_equal(got_ours, got_ref), rec


@pytest.mark.parametrize("mode", ["adam_upd", "masked_adam_upd", "adam_upd_with_perlr"])
def test_adam_matches_reference_kernels(cuda, ref, mode):
    from voxurf_gb300 import adam_upd_cuda as au

    to = _to(cuda)
    rng = np.random.default_rng(21)
    N = 200003
    p = rng.normal(size=N).astype(np.float32)
    g = (rng.normal(size=N) * 0.01).astype(np.float32)
    g[::7] = 0
    m = (rng.normal(size=N) * 0.01).astype(np.float32)
    v = (np.abs(rng.normal(size=N)) * 1e-4).astype(np.float32)
    pl = rng.uniform(0.5, 1.5, size=N).astype(np.float32)
    hp = (5, 0.9, 0.99, 1e-3, 1e-8)
    bufs = {}
    for side, mod in (("ref", ref), ("ours", au)):
        P, M, V = to(p), to(m), to(v)
        extra = (to(pl),) if mode == "adam_upd_with_perlr" else ()
        getattr(mod, mode)(P, to(g), M, V, *extra, *hp)
        bufs[side] = [_np(P), _np(M), _np(V)]
    ms, vs = ff.adam_moments(m, v, g, hp[1], hp[2])
    sel = (g != 0) if mode == "masked_adam_upd" else np.ones(N, bool)
    ms = {k: np.where(sel, x, m) for k, x in ms.items()}
    vs = {k: np.where(sel, x, v) for k, x in vs.items()}
    P, M, V = bufs["ref"]
    rec = {"exp_avg_forms": _forms_equal(ms, M), "exp_avg_sq_forms": _forms_equal(vs, V)}
    ss = ref_cuda.adam_step_size(hp[0], hp[1], hp[2], hp[3])
    pn = ff.adam_param(p, ms[ff.REFERENCE["exp_avg"]], vs[ff.REFERENCE["exp_avg_sq"]], ss, hp[4],
                       pl if mode == "adam_upd_with_perlr" else None)
    rec["param_equals_form"] = bool(np.array_equal(np.where(sel, pn, p), P))
    for i, nm in enumerate(("param", "exp_avg", "exp_avg_sq")):
        rec[f"ours_vs_ref_{nm}_max_ulps"] = _ulps(bufs["ours"][i], bufs["ref"][i])
        rec[f"ours_vs_ref_{nm}_differing"] = int(np.sum(bufs["ours"][i] != bufs["ref"][i]))
    REPORT[mode] = rec
    assert ff.REFERENCE["exp_avg"] in rec["exp_avg_forms"], rec
    assert ff.REFERENCE["exp_avg_sq"] in rec["exp_avg_sq_forms"] and rec["param_equals_form"], rec
    for i in range(3):
        assert np.array_equal(bufs["ours"][i], bufs["ref"][i]), rec


def test_cumdist_thres_matches_reference_kernel(cuda, ref):
    from voxurf_gb300 import ub360_utils_cuda as ub

    to = _to(cuda)
    rng = np.random.default_rng(31)
    dist = rng.uniform(0, 0.02, size=(3000, 257)).astype(np.float32)
    got_ref = _np(ref.cumdist_thres(to(dist), 0.05))
    got_ours = _np(ub.cumdist_thres(to(dist), 0.05))
    restated = cref.cumdist_thres(dist, 0.05)
    REPORT["cumdist_thres"] = {"ref_equals_restatement": bool(np.array_equal(got_ref, restated)),
                               "ours_vs_ref_differing": int(np.sum(got_ours != got_ref))}
    assert np.array_equal(got_ref, restated)
    assert np.array_equal(got_ours, got_ref)
