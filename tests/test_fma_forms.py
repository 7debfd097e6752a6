"""The forms of the reference's float expressions (oracle/fma_forms.py) on
the CPU: the C restatement (oracle/cref.c) computes, bit for bit, the form
that the reference's compiled kernels were measured to compute
(fma_forms.REFERENCE), the other forms differ from it only by rounding, and
the index outputs of the sampling cases that the GPU pin uses do not depend
on the form.  Also the recipe that compiles the reference's own kernels.
"""
import itertools
import os

import numpy as np
import pytest

from oracle import cref
from oracle import fma_forms as ff
from oracle import ref_build

BMIN = np.array([-1.0, -1.0, -1.0], np.float32)
BMAX = np.array([1.0, 1.0, 1.0], np.float32)


def _rays(n, seed):
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


def test_fmaf_rounds_once():
    a = np.float32(1 + 2.0 ** -12)
    assert cref.fmaf(a, a, np.float32(-1))[()] == np.float32(2.0 ** -11 + 2.0 ** -24)
    assert a * a - np.float32(1) == np.float32(2.0 ** -11)


@pytest.mark.parametrize("R,stepsize,n", [(96, 0.5, 2048), (384, 0.25, 512)])
def test_sampling_forms(R, stepsize, n):
    o, d = _rays(n, seed=R + n)
    sd = np.float32(stepsize * 2.0 / R)
    ours = cref.sample_pts_on_rays(o, d, BMIN, BMAX, 0.1, 1e9, sd)
    ref = (ff.REFERENCE["ray_norm"], ff.REFERENCE["ray_start"], ff.REFERENCE["sample_point"])
    for nf, sf, pf in itertools.product(ff.ray_norm(d[:1]).keys(), ("plain", "fma"), ("plain", "fma")):
        got = ff.sample_pts_on_rays(o, d, BMIN, BMAX, 0.1, 1e9, sd, nf, sf, pf)
        if (nf, sf, pf) == ref:
            assert all(np.array_equal(a, b) for a, b in zip(got, ours))
        # every form gives the same index outputs on these rays
        for i in (1, 2, 3, 4, 5, 6):
            assert np.array_equal(got[i], ours[i]), (nf, sf, pf, i)
        assert np.all(np.abs(got[0] - ours[0]) <= 1e-5 * np.maximum(1.0, np.abs(ours[0])))
    # the infer_* ops use the same forms
    t_min, t_max = cref.infer_t_minmax(o, d, BMIN, BMAX, 0.1, 1e9)
    rn = ff.ray_norm(d)[ref[0]]
    assert np.array_equal(cref.infer_n_samples(d, t_min, t_max, sd), ff.n_samples(t_min, t_max, rn, sd))
    st, di = cref.infer_ray_start_dir(o, d, t_min)
    assert np.array_equal(st, ff.ray_start(o, d, t_min)[ref[1]]) and np.array_equal(di, d / rn[:, None])


def test_maskcache_forms():
    rng = np.random.default_rng(3)
    shape = (17, 40, 9)
    world = rng.uniform(size=shape) < 0.3
    xyz = rng.uniform(-1.2, 1.2, size=(20000, 3)).astype(np.float32)
    scale = ((np.array(shape, np.float32) - 1) / (BMAX - BMIN)).astype(np.float32)
    shift = (-BMIN * scale).astype(np.float32)
    ref = ff.REFERENCE["maskcache_lookup"]
    forms = ff.maskcache_lookup(world, xyz, scale, shift)
    assert np.array_equal(forms[ref], cref.maskcache_lookup(world, xyz, scale, shift))
    # half-way points: the two forms round differently at some of them
    half = np.floor(rng.uniform(0, 1, size=(2000, 3)) * (np.array(shape) - 1)) + 0.5
    xh = ((half - shift) / scale).astype(np.float32)
    fh = ff.maskcache_lookup(world, xh, scale, shift)
    assert np.array_equal(fh[ref], cref.maskcache_lookup(world, xh, scale, shift))
    assert 0 < np.sum(fh["plain"] != fh["fma"]) < 0.2 * len(xh)


def test_alpha2weight_backward_forms():
    rng = np.random.default_rng(4)
    n_rays = 300
    lens = rng.integers(0, 200, size=n_rays)
    ray_id = np.repeat(np.arange(n_rays), lens).astype(np.int64)
    alpha = rng.uniform(0, 0.05, size=ray_id.size).astype(np.float32)
    w, T, last, i_s, i_e = cref.alpha2weight(alpha, ray_id, n_rays)
    gw = rng.normal(size=alpha.size).astype(np.float32)
    gl = rng.normal(size=n_rays).astype(np.float32)
    ours = cref.alpha2weight_backward(alpha, w, T, last, i_s, i_e, n_rays, gw, gl)
    forms = ff.alpha2weight_backward(alpha, w, T, last, i_s, i_e, gw, gl)
    assert np.array_equal(forms[ff.REFERENCE["alpha2weight_backward"]], ours)
    scale = np.abs(ours).max()
    for k, v in forms.items():
        assert np.abs(v - ours).max() <= 1e-6 * scale, k


@pytest.mark.parametrize("dense,masked", [(True, False), (False, False), (True, True), (False, True)])
def test_tv_forms(dense, masked):
    rng = np.random.default_rng(5 + 2 * dense + masked)
    p = (rng.normal(size=(3, 9, 11, 13)) * 0.7).astype(np.float32)
    g = rng.normal(size=p.shape).astype(np.float32)
    g[rng.uniform(size=p.shape) < 0.5] = 0
    mk = (rng.uniform(size=p.shape) < 0.7).astype(np.float32) if masked else None
    G = g.copy()[None]
    cref.tv_add_grad(p[None], G, 1e-2, 3e-3, 5e-2, dense, mask=None if mk is None else mk[None])
    forms = ff.tv_add_grad(p, g, 1e-2, 3e-3, 5e-2, dense, mask=mk)
    assert np.array_equal(forms[ff.REFERENCE["total_variation"]], G[0])
    assert np.all(np.abs(forms["fma"] - forms["plain"]) <= 2.0 ** -21 * (np.abs(g) + 6e-2))


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_adam_forms(mode):
    from oracle import ref_cuda

    rng = np.random.default_rng(6)
    N = 50000
    p = rng.normal(size=N).astype(np.float32)
    g = (rng.normal(size=N) * 0.01).astype(np.float32)
    g[::7] = 0
    m = (rng.normal(size=N) * 0.01).astype(np.float32)
    v = (np.abs(rng.normal(size=N)) * 1e-4).astype(np.float32)
    pl = rng.uniform(0.5, 1.5, size=N).astype(np.float32)
    P, M, V = p.copy(), m.copy(), v.copy()
    cref.adam_upd(mode, P, g, M, V, 5, 0.9, 0.99, 1e-3, 1e-8, perlr=pl if mode == 2 else None)
    ms, vs = ff.adam_moments(m, v, g, 0.9, 0.99)
    m_ref, v_ref = ms[ff.REFERENCE["exp_avg"]], vs[ff.REFERENCE["exp_avg_sq"]]
    sel = (g != 0) if mode == 1 else np.ones(N, bool)
    ss = ref_cuda.adam_step_size(5, 0.9, 0.99, 1e-3)
    pn = ff.adam_param(p, m_ref, v_ref, ss, 1e-8, pl if mode == 2 else None)
    assert np.array_equal(np.where(sel, m_ref, m), M)
    assert np.array_equal(np.where(sel, v_ref, v), V)
    assert np.array_equal(np.where(sel, pn, p), P)
    for k, x in ms.items():
        assert np.all(np.abs(x - m_ref) <= 2.0 ** -20 * (np.abs(0.9 * m) + np.abs(0.1 * g))), k


@pytest.mark.skipif(ref_build.reference_root() is None, reason="the reference checkout is not present here")
def test_reference_kernels_compile_to_ptx():
    paths = ref_build.build()
    assert [os.path.basename(p) for p in paths] == [u + ".ptx" for u in ref_build.UNITS]
    assert all(os.path.getsize(p) > 1000 for p in paths)
