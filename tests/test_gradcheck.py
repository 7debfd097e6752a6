"""Gradient check of the hand-written backward against FP64 central finite
differences of the reference step (the oracle restatement in FP64) on a
32^3 grid with 256 rays: 64 randomly chosen voxels (SDF and k0) and 64
randomly chosen MLP weights, step h = 1e-4.

A coordinate whose +-h perturbation takes any non-smooth operation of the
step to its other branch (the shaded-sample set, i.e. a fast_color_thres or
T < 1e-3 decision; relu of the cosine; the alpha clip; output clamps; an MLP
ReLU) has no central difference of its derivative and is replaced by the
next random candidate.

CPU tests pin the oracle's autograd against the finite differences; GPU
tests check the sm_103a gradients (FP32 and the BF16 k0/MLP variant) against
the same finite differences.  Tolerances are stated per test.
"""
import numpy as np
import pytest
import torch

import oracle.ops as vo
from oracle.voxurf_oracle import OracleCoarse, OracleFine, train_loss
from voxurf_gb300 import configs, synthetic

RK = dict(configs.FINE_RENDER_KWARGS)
H = 1e-4
N_RAYS = 256
EIKONAL = 0.1


def _loss_fine(ret, tgt):
    return train_loss(ret, tgt)


def _loss_coarse(ret, tgt):
    loss = ((ret["rgb_marched"] - tgt) ** 2).mean()
    g = ret["gradient"]
    if g.numel():
        loss = loss + EIKONAL * ((g.norm(dim=-1) - 1.0) ** 2).mean()
    return loss


def _setup(kind, device="cpu", precision="fp32", seed=0):
    if kind == "fine":
        model = configs.build_fine_model(32, precision, device=device, seed=seed, width=32)
        oracle = OracleFine(model, dtype=torch.float64)
        lossf = _loss_fine
    else:
        model = configs.build_coarse_model(32, precision, device=device, seed=seed, width=32)
        oracle = OracleCoarse(model, dtype=torch.float64)
        lossf = _loss_coarse
    ro, rd, vd = synthetic.random_rays(N_RAYS, seed=seed + 21)
    tgt = configs.train_targets(N_RAYS, seed + 3)
    return model, oracle, (ro, rd, vd, tgt), lossf


def _oracle_loss(oracle, rays, lossf, signature=False):
    """Loss of the FP64 reference step; with signature=True also the branch
    pattern of every non-smooth operation (sample set, relu of the cosine,
    alpha clip, output clamps, the MLP ReLUs)."""
    ro, rd, vd, tgt = (torch.from_numpy(a) for a in rays)
    vo.TRACE = [] if signature else None
    hooks = []
    if signature:
        for m in oracle.modules():
            if isinstance(m, torch.nn.ReLU):
                hooks.append(m.register_forward_hook(lambda mod, i, o: vo.TRACE.append(("relu", o > 0))))
    try:
        ret = oracle(ro, rd, vd, global_step=1, **RK)
        loss = lossf(ret, tgt.double())
        sig = None
        if signature:
            sig = [("ray_id", ret["ray_id"].clone())] + vo.TRACE
    finally:
        vo.TRACE = None
        for h in hooks:
            h.remove()
    return loss, sig


def _params(oracle):
    """(name, tensor) of the coordinates under test: SDF grid, k0 grid, MLP."""
    return [("sdf", oracle.sdf_grid), ("k0", oracle.k0_grid)] + \
        [("rgbnet." + n, p) for n, p in oracle.rgbnet.named_parameters()] + \
        ([("k_rgbnet." + n, p) for n, p in oracle.k_rgbnet.named_parameters()] if hasattr(oracle, "k_rgbnet") else [])


def _candidates(oracle, rays, lossf, seed=0):
    """Voxels (SDF and k0, alternating) with a nonzero autograd gradient and
    MLP weights, each list in random order; also the oracle's autograd
    gradient."""
    oracle.zero_grad()
    loss, _ = _oracle_loss(oracle, rays, lossf)
    loss.backward()
    rng = np.random.default_rng(seed)
    grads = {n: p.grad.detach().clone() for n, p in _params(oracle)}
    per = []
    for name in ("sdf", "k0"):
        nz = torch.nonzero(grads[name].reshape(-1)).reshape(-1).numpy()
        per.append([(name, int(i)) for i in rng.permutation(nz)[:96]])
    voxels = [c for pair in zip(*per) for c in pair]
    mlp = [(n, p.numel()) for n, p in _params(oracle) if "." in n]
    total = sum(c for _, c in mlp)
    weights = []
    for j in rng.permutation(total)[:192]:
        for n, c in mlp:
            if j < c:
                weights.append((n, int(j)))
                break
            j -= c
    return voxels, weights, grads


def _same(a, b):
    return len(a) == len(b) and all(na == nb and x.shape == y.shape and torch.equal(x, y)
                                    for (na, x), (nb, y) in zip(a, b))


def _finite_differences(oracle, rays, lossf, candidates, want=64):
    """Central differences of the first `want` candidates whose +-h
    perturbations keep every branch of the step (the rest are skipped).

    The reference step differentiates a graph with stop-gradients (the
    k-branch uses rgb_logit.detach(), voxurf_fine.py:733-738): the
    perturbed forwards hold the detached logits at their base values, so
    the differences measure the derivative that the backward computes."""
    params = dict(_params(oracle))
    if hasattr(oracle, "frozen"):
        oracle.frozen = {}
    with torch.no_grad():
        _, s0 = _oracle_loss(oracle, rays, lossf, signature=True)
    fd, skipped = {}, []
    with torch.no_grad():
        for name, i in candidates:
            if len(fd) == want:
                break
            flat = params[name].data.view(-1)
            v = flat[i].item()
            flat[i] = v + H
            lp, sp = _oracle_loss(oracle, rays, lossf, signature=True)
            flat[i] = v - H
            lm, sm = _oracle_loss(oracle, rays, lossf, signature=True)
            flat[i] = v
            if not (_same(sp, s0) and _same(sm, s0)):
                skipped.append((name, i))
                continue
            fd[(name, i)] = (lp.item() - lm.item()) / (2 * H)
    if hasattr(oracle, "frozen"):
        oracle.frozen = None
    return fd, skipped


_CACHE = {}


def _reference(kind):
    """FD gradients and oracle autograd of one setup (computed once)."""
    if kind not in _CACHE:
        model, oracle, rays, lossf = _setup(kind)
        voxels, weights, grads = _candidates(oracle, rays, lossf)
        fd_v, sk_v = _finite_differences(oracle, rays, lossf, voxels)
        fd_w, sk_w = _finite_differences(oracle, rays, lossf, weights)
        _CACHE[kind] = (grads, {**fd_v, **fd_w}, (len(fd_v), len(sk_v), len(fd_w), len(sk_w)))
    return _CACHE[kind]


def _compare(fd, getter, rtol, atol_frac):
    """|g - fd| <= atol_frac * max|fd| + rtol * |fd| for every coordinate."""
    scale = max(abs(v) for v in fd.values())
    bad = []
    for key, v in fd.items():
        g = getter(*key)
        if abs(g - v) > atol_frac * scale + rtol * abs(v):
            bad.append((key, g, v))
    return bad, scale


@pytest.mark.parametrize("kind", ["fine", "coarse"])
def test_oracle_autograd_matches_central_differences(kind):
    grads, fd, (n_v, sk_v, n_w, sk_w) = _reference(kind)
    assert n_v == 64 and n_w == 64, (n_v, sk_v, n_w, sk_w)
    bad, scale = _compare(fd, lambda n, i: grads[n].reshape(-1)[i].item(), 1e-5, 1e-7)
    assert not bad, (scale, bad[:5])


def _gpu_grads(kind, precision, cuda):
    model, _, rays, _ = _setup(kind, device=cuda, precision=precision)
    ro, rd, vd, tgt = (torch.from_numpy(a).to(cuda) for a in rays)
    ret = model(ro, rd, vd, global_step=1, **RK)
    if kind == "fine":
        loss = train_loss(ret, tgt)
    else:
        loss = _loss_coarse(ret, tgt)
    loss.backward()
    torch.cuda.synchronize()
    g = {"sdf": model.sdf.grid.grad, "k0": model.k0.grid.grad.contiguous()}
    for n, p in model.rgbnet.named_parameters():
        g["rgbnet." + n] = p.grad
    if kind == "fine":
        for n, p in model.k_rgbnet.named_parameters():
            g["k_rgbnet." + n] = p.grad
    return {k: v.detach().double().cpu() for k, v in g.items()}


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["fine", "coarse"])
@pytest.mark.parametrize("precision,rtol,atol_frac", [("fp32", 1e-4, 1e-6), ("bf16", 5e-2, 2e-2)])
def test_gpu_gradients_match_central_differences(cuda, kind, precision, rtol, atol_frac):
    """FP32: |g - fd| <= 1e-6 max|fd| + 1e-4 |fd|.  BF16 (k0 and MLP inputs
    rounded to 8 mantissa bits): <= 2e-2 max|fd| + 5e-2 |fd|."""
    _, fd, _ = _reference(kind)
    g = _gpu_grads(kind, precision, cuda)
    bad, scale = _compare(fd, lambda n, i: g[n].reshape(-1)[i].item(), rtol, atol_frac)
    assert not bad, (precision, scale, bad[:5])
