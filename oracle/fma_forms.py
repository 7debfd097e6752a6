"""ORACLE — test infrastructure only (never imported by the product).

The float expressions of the reference's CUDA kernels, in each form that
nvcc may give them.  The reference is built with nvcc's default
``--fmad=true``, under which an ``a*b + c`` of the source may be computed as
one fused multiply-add (one rounding instead of two), and where two products
meet in one sum either of them may be the fused one.  "plain" is the source
with one rounding per operation; the other forms fuse, built from C99
``fmaf`` (``cref.fmaf``).  Running the reference's own kernels on the GPU
(``oracle/ref_cuda.py``) against every form tells which one the reference
binary computes; ``REFERENCE`` records the answer, and ``oracle/cref.c``
restates exactly those forms.

Every function returns a dict {form name: array}.
"""
from __future__ import annotations

import numpy as np

from . import cref

f32 = np.float32

# The form of each expression in the reference's compiled kernels (nvcc 13.0,
# compute_103a, run on a GB300 by tests/test_zy_reference_kernels_gpu.py,
# which asserts these on every run).
REFERENCE = {
    "ray_norm": "fma(x;y)",               # sqrt(fma(z, z, fma(x, x, y*y)))
    "ray_start": "fma",                   # fma(d, t_min, o)
    "sample_point": "fma",                # fma(dir, stepdist*k, start)
    "maskcache_lookup": "fma",            # round(fma(xyz, scale, shift))
    "alpha2weight_backward": "cum=fma,sub=plain",  # back_cum = fma(gw, w, back_cum)
    "exp_avg": "fma(b1*m)",               # fma(beta1, m, (1-beta1)*g)
    "exp_avg_sq": "fma(b2*v)",            # fma(beta2, v, (1-beta2)*g*g)
    "total_variation": "plain",
}


def _fma(a, b, c):
    return cref.fmaf(a, b, c)


# ---- render_utils_kernel.cu:46-51, 67-70: |d| = sqrt(dx*dx + dy*dy + dz*dz) ----

def ray_norm(d) -> dict:
    d = np.ascontiguousarray(d, f32)
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    return {
        "plain": np.sqrt((x * x + y * y) + z * z),
        "fma(y;x)": np.sqrt(_fma(z, z, _fma(y, y, x * x))),
        "fma(x;y)": np.sqrt(_fma(z, z, _fma(x, x, y * y))),
    }


def n_samples(t_min, t_max, rnorm, stepdist) -> np.ndarray:
    """render_utils_kernel.cu:53: max(ceil((t_max-t_min)*|d|/stepdist), 1.)."""
    c = np.ceil(((t_max - t_min) * rnorm) / f32(stepdist)).astype(np.float64)
    return np.maximum(c, 1.0).astype(np.int64)


def ray_start(o, d, t_min) -> dict:
    """render_utils_kernel.cu:71-73: o + d*t_min."""
    o, d = np.ascontiguousarray(o, f32), np.ascontiguousarray(d, f32)
    t = np.asarray(t_min, f32)[:, None]
    return {"plain": o + d * t, "fma": _fma(d, t, o)}


def sample_pts_on_rays(o, d, xyz_min, xyz_max, near, far, stepdist, norm_form: str, start_form: str,
                       pts_form: str) -> list:
    """render_utils_kernel.cu:196-242 with the given forms of |d|, the ray
    start and the point (start + dir*dist): [rays_pts, mask_outbbox, ray_id,
    step_id, N_steps, t_min, t_max]."""
    o, d = np.ascontiguousarray(o, f32), np.ascontiguousarray(d, f32)
    mn, mx = np.asarray(xyz_min, f32), np.asarray(xyz_max, f32)
    t_min, t_max = cref.infer_t_minmax(o, d, mn, mx, near, far)
    rn = ray_norm(d)[norm_form]
    ns = n_samples(t_min, t_max, rn, stepdist)
    start = ray_start(o, d, t_min)[start_form]
    direc = d / rn[:, None]
    ray_id = np.repeat(np.arange(len(ns), dtype=np.int64), ns)
    first = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
    step_id = np.arange(ray_id.size, dtype=np.int64) - first[ray_id]
    dist = (f32(stepdist) * step_id.astype(f32))[:, None]
    if pts_form == "plain":
        pts = start[ray_id] + direc[ray_id] * dist
    else:
        pts = _fma(direc[ray_id], dist, start[ray_id])
    out = np.any(mn[None, :] > pts, axis=1) | np.any(mx[None, :] < pts, axis=1)
    return [pts.astype(f32), out, ray_id, step_id, ns, t_min, t_max]


# ---- render_utils_kernel.cu:384-390: round(xyz*scale + shift) -----------------

def maskcache_lookup(world, xyz, scale, shift) -> dict:
    world = np.asarray(world, bool)
    xyz = np.ascontiguousarray(xyz, f32)
    scale, shift = np.asarray(scale, f32), np.asarray(shift, f32)
    forms = {"plain": xyz * scale[None, :] + shift[None, :], "fma": _fma(xyz, scale[None, :], shift[None, :])}
    res = {}
    for k, v in forms.items():
        v64 = v.astype(np.float64)
        ijk = (np.sign(v64) * np.floor(np.abs(v64) + 0.5)).astype(np.int64)  # C round: half away from zero
        ok = np.all((ijk >= 0) & (ijk < np.array(world.shape)[None, :]), axis=1)
        out = np.zeros(len(xyz), bool)
        out[ok] = world[ijk[ok, 0], ijk[ok, 1], ijk[ok, 2]]
        res[k] = out
    return res


# ---- render_utils_kernel.cu:668-690: the reverse scan of alpha2weight's backward --

def alpha2weight_backward(alpha, weight, T, alphainv_last, i_start, i_end, grad_weights, grad_last) -> dict:
    """grad[i] = gw[i]*T[i] - back_cum / (1-alpha[i] + 1e-10) (a float
    product promoted to double, or the product fused into the double
    subtraction), back_cum += gw[i]*weight[i] (plain or fused).  Rays run in
    lockstep from their ends."""
    a, w, T, gw = (np.asarray(x, f32) for x in (alpha, weight, T, grad_weights))
    last, gl = np.asarray(alphainv_last, f32), np.asarray(grad_last, f32)
    i_s, i_e = np.asarray(i_start, np.int64), np.asarray(i_end, np.int64)
    res = {}
    for cum_form in ("plain", "fma"):
        for sub_form in ("plain", "fused"):
            grad = np.zeros(a.shape, f32)
            back = gl * last
            n_max = int((i_e - i_s).max()) if len(i_s) else 0
            for j in range(n_max):
                live = (i_e - 1 - j) >= i_s
                idx = (i_e - 1 - j)[live]
                b = back[live]
                q = b.astype(np.float64) / ((f32(1) - a[idx]).astype(np.float64) + 1e-10)
                if sub_form == "plain":
                    g = (gw[idx] * T[idx]).astype(np.float64) - q
                else:
                    g = gw[idx].astype(np.float64) * T[idx].astype(np.float64) - q
                grad[idx] = g.astype(f32)
                if cum_form == "plain":
                    back[live] = b + gw[idx] * w[idx]
                else:
                    back[live] = _fma(gw[idx], w[idx], b)
            res[f"cum={cum_form},sub={sub_form}"] = grad
    return res


# ---- adam_upd_kernel.cu:18-22: the two moment updates --------------------------

def adam_moments(exp_avg, exp_avg_sq, grad, beta1, beta2) -> tuple[dict, dict]:
    """exp_avg' = beta1*m + (1-beta1)*g and exp_avg_sq' = beta2*v +
    (1-beta2)*g*g, each plain or with either product fused."""
    m, v, g = (np.asarray(x, f32) for x in (exp_avg, exp_avg_sq, grad))
    b1, b2 = f32(beta1), f32(beta2)
    c1, c2 = f32(1) - b1, f32(1) - b2
    gg = (c2 * g) * g
    ms = {"plain": b1 * m + c1 * g, "fma(b1*m)": _fma(b1, m, c1 * g), "fma(c1*g)": _fma(c1, g, b1 * m)}
    vs = {"plain": b2 * v + gg, "fma(b2*v)": _fma(b2, v, gg), "fma(c2g*g)": _fma(c2 * g, g, b2 * v)}
    return ms, vs


def adam_param(param, exp_avg_new, exp_avg_sq_new, step_size, eps, perlr=None) -> np.ndarray:
    """adam_upd_kernel.cu:21, 56: param - step_size[*perlr]*m / (sqrt(v) + eps)."""
    p, m, v = (np.asarray(x, f32) for x in (param, exp_avg_new, exp_avg_sq_new))
    num = f32(step_size) * m if perlr is None else (f32(step_size) * np.asarray(perlr, f32)) * m
    return p - num / (np.sqrt(v) + f32(eps))


# ---- total_variation_kernel.cu:14-66: grad_to_add += w * clamp(param - neighbour) --

def tv_add_grad(param, grad, wx, wy, wz, dense_mode: bool, mask=None) -> dict:
    """New grad ([C, X, Y, Z] float32) for the plain form and for the form
    with every neighbour term fused into the running sum.  The weights are
    divided by 6 as the launcher does; the variant without a mask weighs the
    k and i neighbours by wz and the j neighbours by wy (as the reference
    source does), the masked variant uses wx, wy, wz for k, j, i."""
    p = np.asarray(param, f32)
    g0 = np.asarray(grad, f32)
    m = None if mask is None else np.asarray(mask, f32)
    wx, wy, wz = (f32(w) / f32(6) for w in (wx, wy, wz))
    axes = [(3, -1, wz if m is None else wx), (3, 1, wz if m is None else wx), (2, -1, wy), (2, 1, wy),
            (1, -1, wz), (1, 1, wz)]
    res = {}
    for form in ("plain", "fma"):
        acc = np.zeros_like(p)
        for ax, off, w in axes:
            nb = np.roll(p, -off, axis=ax)  # nb[..., x] = p[..., x + off]
            valid = np.ones(p.shape, bool)
            sl = [slice(None)] * 4
            sl[ax] = slice(p.shape[ax] - 1, None) if off == 1 else slice(0, 1)
            valid[tuple(sl)] = False
            c = np.clip(p - nb, f32(-1), f32(1))
            if m is None:
                a, b = np.broadcast_to(w, p.shape), c
            else:
                a, b = (w * c) * m, np.roll(m, -off, axis=ax)
            new = (acc + a * b) if form == "plain" else _fma(a, b, acc)
            acc = np.where(valid, new, acc)
        sel = np.ones(p.shape, bool) if dense_mode else (g0 != 0)
        res[form] = np.where(sel, g0 + acc, g0).astype(f32)
    return res
