"""Parity at the benchmark's own configurations, against the FP64 oracle.

bench.py times three training workloads on full-size grids; the other model
tests use small grids.  Here the GPU runs the bench's exact scenes, masks,
model sizes and ray batches, and the FP64 oracle (the reference step
restated, lib/voxurf_fine.py:620-802, run.py:599-659) runs the same step on
a sub-batch it finishes in seconds:

* 256^3 fine workload (sphere + torus, |SDF| < 0.05 mask, MLPs 192 x 4):
  the first 384 rays of the bench's first 8192-ray batch.  Plain FP32
  (eager step, the bench's `value` arm): identical shaded-sample set, RGB
  max abs <= 1e-5, loss <= 1e-6 relative, every gradient rel-L2 <= 1e-5,
  and the parameter update of the whole step (TV + Adam on both grids, Adam
  on the MLPs) rel-L2 <= 1e-5.  Mixed BF16 (graph-replayed step, the
  bench's `fused_bf16` arm): RGB max abs <= 1e-3 and per-output gradient
  bounds set from the measured errors (printed).  The full 8192-ray forward
  is also checked on those 384 rays (rays are independent until the loss).
* 384^3 long-ray workload (64 spheres, stepsize 0.25, s-density 0.05): 64
  rays of the bench's first batch that march more than 512 samples plus 32
  shorter ones; FP32 at the 1e-5 bars, BF16 RGB <= 1e-3.
* 96^3 coarse differentiation workload with eikonal 0.1 at the bench's
  32768-ray batch (the whole batch).
"""
import numpy as np
import pytest
import torch

from oracle.voxurf_oracle import OracleCoarse, OracleFine, UtilsAdam, train_loss, tv_add_grad
from voxurf_gb300 import configs, synthetic
from voxurf_gb300.train import FineTrainer

pytestmark = pytest.mark.gpu

RK = dict(configs.FINE_RENDER_KWARGS)
BENCH_RAYS = 8192
BENCH_BATCHES = 25          # bench.py default: 5 warm-up + 20 timed batches from one seeded draw
SUB = 384


def _rel_l2(a, b):
    a = a.detach().double().cpu().reshape(-1)
    b = b.detach().double().cpu().reshape(-1)
    return float((a - b).norm() / (b.norm() + 1e-30))


def _bench_batch(n_rays, n_batches, seed):
    """The first batch of bench.make_batches / run_long_rays / run_eikonal."""
    o, d, v = synthetic.random_rays(n_rays * n_batches, seed=seed)
    t = configs.train_targets(n_rays * n_batches, seed)
    return tuple(np.ascontiguousarray(a[:n_rays]) for a in (o, d, v, t))


def _grab_grads(tr, store):
    model = tr.model
    named = [("sdf", model.sdf.grid), ("k0", model.k0.grid)] + \
        [("rgbnet." + n, p) for n, p in model.rgbnet.named_parameters()] + \
        [("k_rgbnet." + n, p) for n, p in model.k_rgbnet.named_parameters()]
    orig = tr.optimizer.step

    def step(*a, **k):
        store.update({n: p.grad.detach().cpu().clone() for n, p in named})
        return orig(*a, **k)

    tr.optimizer.step = step


def _oracle_grads(orc):
    g = {"sdf": orc.sdf_grid.grad.clone(), "k0": orc.k0_grid.grad.clone()}
    for n, q in orc.rgbnet.named_parameters():
        g["rgbnet." + n] = q.grad.clone()
    for n, q in orc.k_rgbnet.named_parameters():
        g["k_rgbnet." + n] = q.grad.clone()
    return g


def _params(obj_sdf, obj_k0, rgbnet, k_rgbnet):
    p = {"sdf": obj_sdf.detach().double().cpu().clone(), "k0": obj_k0.detach().double().cpu().clone()}
    for n, q in rgbnet.named_parameters():
        p["rgbnet." + n] = q.detach().double().cpu().clone()
    for n, q in k_rgbnet.named_parameters():
        p["k_rgbnet." + n] = q.detach().double().cpu().clone()
    return p


class _Lazy:
    """A module fixture's oracle result, computed on first use: the first
    caller (the FP32 test) passes the device's ReLU decisions for the
    oracle's near-tie pre-activations; later callers reuse the result."""

    def __init__(self, fn):
        self.fn, self.val = fn, None

    def get(self, relu_device=None):
        if self.val is None:
            self.val = self.fn(relu_device)
        return self.val


def _device_relu(model):
    from voxurf_gb300.mlp import last_relu_masks

    return {"rgbnet": [m.cpu() for m in last_relu_masks(model.rgbnet)],
            "k_rgbnet": [m.cpu() for m in last_relu_masks(model.k_rgbnet)]}


def _relu_ties_ok(orc):
    """ReLU ties (pre-activations within 1e-6 of their layer's RMS from zero)
    are as rare as a smooth density at zero makes them: about 1e-6 of the
    pre-activations examined, bounded here at 4e-6 of them plus 64."""
    return orc.relu_ties <= 64 + 4e-6 * getattr(orc, "relu_examined", 0)


@pytest.fixture(scope="module")
def fine256(cuda):
    """The FP64 oracle's step on the 384-ray sub-batch of the 256^3 bench
    workload: outputs, gradients and the parameter update of one full
    training step (TV add-grad weight / N_rays, utils.Adam lr 1e-3)."""
    full = _bench_batch(BENCH_RAYS, BENCH_BATCHES, 0)
    rays = tuple(a[:SUB] for a in full)

    def run(relu_device):
        model = configs.build_fine_model(256, "fp32", device=cuda, seed=0, mask_voxels=6.4)
        orc = OracleFine(model, dtype=torch.float64)
        world_max = float(model.world_size.max())
        model32 = model
        del model
        before = _params(orc.sdf_grid, orc.k0_grid, orc.rgbnet, orc.k_rgbnet)
        ro, rd, vd, tgt = (torch.from_numpy(a) for a in rays)
        ret = orc(ro, rd, vd, global_step=1, relu_device=relu_device, **RK)
        ties = orc.relu_ties
        assert _relu_ties_ok(orc), (orc.relu_ties, orc.relu_examined)
        loss = train_loss(ret, tgt.double())
        loss.backward()
        grads = _oracle_grads(orc)
        # the reference algorithm's own FP32 error on this batch (same step in
        # FP32): the FP32 bars are max(1e-5, 3x this)
        orc32 = OracleFine(model32, dtype=torch.float32)
        del model32
        torch.cuda.empty_cache()
        train_loss(orc32(ro, rd, vd, global_step=1, **RK), tgt).backward()
        ref32 = {k: _rel_l2(v, grads[k]) for k, v in _oracle_grads(orc32).items()}
        tv_add_grad(orc32.sdf_grid, 1e-4 / SUB, world_max, True)
        tv_add_grad(orc32.k0_grid, 1e-4 / SUB, world_max, True)
        UtilsAdam([([orc32.sdf_grid], 1e-3), ([orc32.k0_grid], 1e-3), (list(orc32.rgbnet.parameters()), 1e-3),
                   (list(orc32.k_rgbnet.parameters()), 1e-3)], betas=(0.9, 0.99)).step()
        after32 = _params(orc32.sdf_grid, orc32.k0_grid, orc32.rgbnet, orc32.k_rgbnet)
        del orc32
        tv_add_grad(orc.sdf_grid, 1e-4 / SUB, world_max, True)
        tv_add_grad(orc.k0_grid, 1e-4 / SUB, world_max, True)
        opt = UtilsAdam([([orc.sdf_grid], 1e-3), ([orc.k0_grid], 1e-3), (list(orc.rgbnet.parameters()), 1e-3),
                         (list(orc.k_rgbnet.parameters()), 1e-3)], betas=(0.9, 0.99))
        opt.step()
        after = _params(orc.sdf_grid, orc.k0_grid, orc.rgbnet, orc.k_rgbnet)
        delta = {k: after[k] - before[k] for k in before}
        # the reference algorithm's own FP32 update error, measured like the
        # GPU's (against the FP64 update rounded to FP32 storage)
        ref32_update = {k: _rel_l2(after32[k] - before[k], (before[k] + delta[k]).float().double() - before[k])
                        for k in before}
        return {"ret": {k: (v.detach() if torch.is_tensor(v) else v) for k, v in ret.items()},
                "loss": float(loss.item()), "grads": grads, "ref32": ref32, "ref32_update": ref32_update,
                "before": before, "delta": delta, "relu_ties": ties}

    return {"rays": rays, "full": full, "oracle": _Lazy(run)}


def test_fine256_fp32_step_matches_fp64_oracle(cuda, fine256):
    model = configs.build_fine_model(256, "fp32", device=cuda, seed=0, mask_voxels=6.4)
    # the bench's full 8192-ray forward: its first 384 rays equal the oracle's
    # (rays are independent until the loss)
    full = [torch.from_numpy(a).to(cuda) for a in fine256["full"][:3]]
    with torch.no_grad():
        g = model(*full, global_step=1, **RK)
    rgb_full = g["rgb_marched"][:SUB].double().cpu()
    del g
    tr = FineTrainer(model, n_rays=SUB)
    grads = {}
    _grab_grads(tr, grads)
    ro, rd, vd, tgt = (torch.from_numpy(a).to(cuda) for a in fine256["rays"])
    loss, ret = tr.step(ro, rd, vd, tgt, RK, global_step=1)
    torch.cuda.synchronize()
    o = fine256["oracle"].get(_device_relu(model))
    fo = o
    o = fo["ret"]
    err = (rgb_full - o["rgb_marched"]).abs().max().item()
    assert err <= 1e-5, err
    assert ret["weights"].numel() == o["weights"].numel() > 2000
    assert torch.equal(ret["ray_id"].long().cpu(), o["ray_id"])
    assert torch.equal(model._last_frame.step2.long().cpu(), o["step_id"])
    for key in ("rgb_marched", "rgb_marched0"):
        err = (ret[key].double().detach().cpu() - o[key]).abs().max().item()
        assert err <= 1e-5, (key, err)
    assert abs(float(loss) - fo["loss"]) <= 1e-6 * abs(fo["loss"])
    errs = {name: _rel_l2(grads[name], ref) for name, ref in fo["grads"].items()}
    print("fp32 step vs FP64 (256^3 bench workload):", errs, "reference fp32:", fo["ref32"])
    for name, err in errs.items():
        assert err <= max(1e-5, 3 * fo["ref32"][name]), (name, err, fo["ref32"][name])
    # the update of the whole step, against the oracle's updated parameters
    # rounded to the FP32 storage both sides keep them in (otherwise one ulp
    # of a parameter near 1, 6e-8, would count against a 1e-3 Adam step)
    after = _params(model.sdf.grid, model.k0.grid, model.rgbnet, model.k_rgbnet)
    uerr = {}
    for name, ref in fo["delta"].items():
        p0 = fo["before"][name]
        uerr[name] = _rel_l2(after[name] - p0, (p0 + ref).float().double() - p0)
    print("fp32 update vs FP64:", uerr, "reference fp32:", fo["ref32_update"])
    for name, err in uerr.items():
        assert err <= max(1e-5, 3 * fo["ref32_update"][name]), ("update", name, err)


# Bounds of the BF16 graph-replayed step against FP64 on this batch, about
# 2-3x the measured errors (RGB 1.5e-4, loss 3.5e-6, SDF gradient 7.4e-4, k0
# gradient 4.4e-2, MLP weight gradients <= 2.1e-2): the k0 grid and the MLP
# run in BF16 with FP32 accumulation, the SDF grid, alpha and normals in
# FP32; the k0 gradient sums many BF16 input gradients of either sign.
BF16_BOUNDS = {"rgb": 1e-3, "loss": 1e-5, "sdf": 2e-3, "k0": 1e-1, "mlp": 5e-2}


def test_fine256_bf16_graphed_step_vs_fp64_oracle(cuda, fine256):
    model = configs.build_fine_model(256, "bf16", device=cuda, seed=0, mask_voxels=6.4)
    ro, rd, vd, tgt = (torch.from_numpy(a).to(cuda) for a in fine256["rays"])
    with torch.no_grad():
        g = model(ro, rd, vd, global_step=1, **RK)
    fo = fine256["oracle"].get()
    o = fo["ret"]
    errs = {"rgb": (g["rgb_marched"].double().cpu() - o["rgb_marched"]).abs().max().item()}
    tr = FineTrainer(model, n_rays=SUB, graphed=True)
    grads = {}
    _grab_grads(tr, grads)
    loss, _ = tr.step(ro, rd, vd, tgt, RK, global_step=1)
    torch.cuda.synchronize()
    errs["loss"] = abs(float(loss) - fo["loss"]) / abs(fo["loss"])
    for name, ref in fo["grads"].items():
        errs[name] = _rel_l2(grads[name], ref)
    print("bf16 graphed step vs FP64 (256^3 bench workload):", errs)
    assert errs["rgb"] <= BF16_BOUNDS["rgb"]
    assert errs["loss"] <= BF16_BOUNDS["loss"]
    assert errs["sdf"] <= BF16_BOUNDS["sdf"]
    assert errs["k0"] <= BF16_BOUNDS["k0"]
    for name in fo["grads"]:
        if "rgbnet" in name:
            assert errs[name] <= BF16_BOUNDS["mlp"], (name, errs[name])


LONG_R = 384


def _long_ray_subset():
    """64 rays of the 384^3 bench batch that march more than 512 samples and
    32 that march fewer (or miss the bbox)."""
    from oracle.ops import RenderUtilsOracle

    o, d, v, t = _bench_batch(65536, 8, 11)
    stepdist = float(np.float32(0.25) * np.float32(2.0 / LONG_R))   # stepsize x voxel size
    n_steps = RenderUtilsOracle.sample_pts_on_rays(torch.from_numpy(o[:4096]), torch.from_numpy(d[:4096]),
                                                   torch.tensor([-1.0] * 3), torch.tensor([1.0] * 3), 0.1, 1e9,
                                                   stepdist)[4].numpy()
    long_ = np.nonzero(n_steps > 512)[0][:64]
    short = np.nonzero(n_steps <= 512)[0][:32]
    assert len(long_) == 64 and len(short) == 32
    idx = np.sort(np.concatenate([long_, short]))
    return tuple(np.ascontiguousarray(a[idx]) for a in (o, d, v, t))


def _long_model(cuda, precision):
    return configs.build_fine_model(LONG_R, precision, device=cuda, seed=7, scene="spheres64",
                                    mask_voxels=0.05 / (2.0 / LONG_R))


@pytest.fixture(scope="module")
def long384(cuda):
    """The FP64 oracle's forward + backward on the long-ray subset of the
    384^3 bench workload (global_step 0: s-density 0.05)."""
    rays = _long_ray_subset()
    rk = dict(RK, stepsize=0.25)

    def run(relu_device):
        model = _long_model(cuda, "fp32")
        orc = OracleFine(model, dtype=torch.float64)
        del model
        torch.cuda.empty_cache()
        o = orc(*(torch.from_numpy(a) for a in rays[:3]), global_step=0, relu_device=relu_device, **rk)
        ties = orc.relu_ties
        assert _relu_ties_ok(orc), (orc.relu_ties, orc.relu_examined)
        ol = train_loss(o, torch.from_numpy(rays[3]).double())
        ol.backward()
        grads = {"sdf": orc.sdf_grid.grad, "k0": orc.k0_grid.grad,
                 "rgbnet": [q.grad for q in orc.rgbnet.parameters()],
                 "k_rgbnet": [q.grad for q in orc.k_rgbnet.parameters()]}
        del orc
        # the reference algorithm's own FP32 error on this batch
        model = _long_model(cuda, "fp32")
        orc32 = OracleFine(model, dtype=torch.float32)
        del model
        torch.cuda.empty_cache()
        train_loss(orc32(*(torch.from_numpy(a) for a in rays[:3]), global_step=0, **rk),
                   torch.from_numpy(rays[3])).backward()
        ref32 = {"sdf": _rel_l2(orc32.sdf_grid.grad, grads["sdf"]),
                 "k0": _rel_l2(orc32.k0_grid.grad, grads["k0"])}
        for net in ("rgbnet", "k_rgbnet"):
            for (n, q), r in zip(getattr(orc32, net).named_parameters(), grads[net]):
                ref32[net + "." + n] = _rel_l2(q.grad, r)
        return {"ret": {k: (v.detach() if torch.is_tensor(v) else v) for k, v in o.items()},
                "grads": grads, "ref32": ref32, "relu_ties": ties}

    return {"rays": rays, "rk": rk, "oracle": _Lazy(run)}


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_long_rays_384_vs_fp64_oracle(cuda, precision, long384):
    model = _long_model(cuda, precision)
    rays, rk = long384["rays"], long384["rk"]
    T = lambda a: torch.from_numpy(a).to(cuda)  # noqa: E731
    g = model(T(rays[0]), T(rays[1]), T(rays[2]), global_step=0, **rk)
    gl = train_loss(g, T(rays[3]))
    gl.backward()
    torch.cuda.synchronize()
    lo = long384["oracle"].get(_device_relu(model) if precision == "fp32" else None)
    o, og = lo["ret"], lo["grads"]
    err = (g["rgb_marched"].detach().double().cpu() - o["rgb_marched"]).abs().max().item()
    errs = {"rgb": err, "sdf": _rel_l2(model.sdf.grid.grad, og["sdf"]), "k0": _rel_l2(model.k0.grid.grad, og["k0"])}
    for net in ("rgbnet", "k_rgbnet"):
        for (n, p), q in zip(getattr(model, net).named_parameters(), og[net]):
            errs[net + "." + n] = _rel_l2(p.grad, q)
    print(precision, "384^3 long rays vs FP64:", errs, "shaded", o["weights"].numel(), "reference fp32:",
          lo["ref32"], "relu ties", lo["relu_ties"])
    assert o["weights"].numel() > 1000
    if precision == "fp32":
        assert torch.equal(g["ray_id"].long().cpu(), o["ray_id"])
        assert err <= 1e-5
        for k, v in errs.items():
            if k != "rgb":
                assert v <= max(1e-5, 3 * lo["ref32"][k]), (k, v, lo["ref32"][k])
    else:
        assert err <= 1e-3
        assert errs["sdf"] <= BF16_BOUNDS["sdf"] and errs["k0"] <= BF16_BOUNDS["k0"]
        for k, v in errs.items():
            if "rgbnet" in k:
                assert v <= BF16_BOUNDS["mlp"], (k, v)


@pytest.mark.parametrize("precision,rgb_tol,loss_tol,grad_tol", [("fp32", 1e-5, 1e-6, 1e-5),
                                                                  ("bf16", 1e-3, 2e-3, 5e-2)])
def test_coarse_eikonal_bench_batch_vs_fp64_oracle(cuda, precision, rgb_tol, loss_tol, grad_tol):
    """The differentiation workload at the bench's 32768-ray batch (96^3
    coarse grids and MLP, eikonal 0.1): RGB, loss, eikonal term and every
    gradient against the FP64 oracle on the whole batch; the gradient bars
    are grad_tol or 3x the reference algorithm's own FP32 error, whichever is
    larger (the k0 gradient sums many cancelling per-sample terms)."""
    from voxurf_gb300.train import eikonal_loss, fine_loss

    n = 32768
    model = configs.build_coarse_model(96, precision, device=cuda, seed=0)
    ro, rd, vd, tgt = _bench_batch(n, 8, 13)
    rk = dict(configs.COARSE_RENDER_KWARGS)
    T = lambda a: torch.from_numpy(a).to(cuda)  # noqa: E731
    g = model(T(ro), T(rd), T(vd), global_step=1, **rk)
    g_eik = eikonal_loss(g["gradient"])
    gl = fine_loss(g, T(tgt)) + 0.1 * g_eik
    gl.backward()
    fr = model._last_frame
    keep = set(zip(fr.ray2.long().cpu().tolist(), fr.step2.long().cpu().tolist()))
    from voxurf_gb300.mlp import last_relu_masks

    dev_relu = last_relu_masks(model.rgbnet) if precision == "fp32" else None
    dev_relu = [m.cpu() for m in dev_relu] if dev_relu is not None else None

    def run_oracle(dtype):
        # threshold ties: FP32 and FP64 decide a weight within 1e-3 (relative)
        # of fast_color_thres differently (behind a nearly opaque sample FP32
        # keeps 1 - alpha only to ~1e-4, so T does too); a few per thousand
        # rays at most.  The FP32 run of the reference algorithm (the baseline
        # of the gradient bars) computes the NeuS alpha with cancellation: its
        # own weights near the threshold lie up to ~5e-4 from the FP64 ones on
        # an x86 host and more than 1e-3 on an Arm host (the two round
        # differently), so it takes the device's decision within 1e-2.
        tie_rel = 1e-3 if dtype == torch.float64 else 1e-2
        orc = OracleCoarse(model, dtype=dtype)
        o = orc(*(torch.from_numpy(a) for a in (ro, rd, vd)), global_step=1, device_keep=keep, tie_rel=tie_rel,
                relu_device=dev_relu if dtype == torch.float64 else None, **rk)
        assert _relu_ties_ok(orc), (orc.relu_ties, orc.relu_examined)
        o_eik = ((o["gradient"].norm(dim=-1) - 1.0) ** 2).mean()
        ol = train_loss(o, torch.from_numpy(tgt).to(dtype), weight_rgb0=0) + 0.1 * o_eik
        ol.backward()
        if dtype == torch.float64:
            assert orc.ties <= max(4, n // 256), orc.ties
        got = set(zip(o["ray_id"].tolist(), o["step_id"].tolist()))
        assert got == keep, (sorted(got - keep)[:8], sorted(keep - got)[:8])
        grads = {"sdf": orc.sdf_grid.grad, "k0": orc.k0_grid.grad}
        for nm, q in orc.rgbnet.named_parameters():
            grads["rgbnet." + nm] = q.grad
        return o, o_eik, ol, grads, orc.ties

    o, o_eik, ol, ograds, ties = run_oracle(torch.float64)
    errs = {"rgb_max_abs": (g["rgb_marched"].double().detach().cpu() - o["rgb_marched"].detach()).abs().max().item(),
            "ties": ties, "loss_rel": abs(gl.item() - ol.item()) / abs(ol.item()),
            "eikonal_rel": abs(g_eik.item() - o_eik.item()) / abs(o_eik.item()),
            "sdf": _rel_l2(model.sdf.grid.grad, ograds["sdf"]), "k0": _rel_l2(model.k0.grid.grad, ograds["k0"])}
    for nm, p in model.rgbnet.named_parameters():
        errs["rgbnet." + nm] = _rel_l2(p.grad, ograds["rgbnet." + nm])
    _, _, _, grads32, _ = run_oracle(torch.float32)
    ref32 = {k: _rel_l2(v, ograds[k]) for k, v in grads32.items()}
    print(precision, "coarse 96^3 x 32768 rays vs FP64:", errs, "reference fp32:", ref32)
    assert len(keep) > 100000
    assert errs["rgb_max_abs"] <= rgb_tol
    assert errs["loss_rel"] <= loss_tol and errs["eikonal_rel"] <= loss_tol
    for k, v in ref32.items():
        assert errs[k] <= max(grad_tol, 3 * v), (k, errs[k], v)
