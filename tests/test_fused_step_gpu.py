"""The graph-replayed training step (fused_step.GraphedFineStep) against the
eager autograd step (FineTrainer) on identical models and batches.

Both run the same kernels; the differences are the GEMM row counts (the
graphed step pads to a row bucket), the padded first-layer GEMMs and the
explicit loss gradient, so per-step gradients must agree to rel-L2 1e-5 in
FP32 (5e-2 in BF16, whose GEMM outputs are rounded to 8 mantissa bits and
whose GEMM kernels differ with the padded shapes).
Bucket changes and captures happen along the way (small bucket size).
"""
import numpy as np
import pytest
import torch

from voxurf_gb300 import configs, synthetic
from voxurf_gb300.train import FineTrainer

pytestmark = pytest.mark.gpu

RK = dict(configs.FINE_RENDER_KWARGS)


def _rel(a, b):
    a, b = a.detach().double().reshape(-1), b.detach().double().reshape(-1)
    return float((a - b).norm() / (b.norm() + 1e-30))


def _grab(tr, store):
    model = tr.model
    named = [("sdf", model.sdf.grid), ("k0", model.k0.grid)] + \
        [("rgbnet." + n, p) for n, p in model.rgbnet.named_parameters()] + \
        [("k_rgbnet." + n, p) for n, p in model.k_rgbnet.named_parameters()]
    orig = tr.optimizer.step

    def step(*a, **k):
        store.append({n: p.grad.detach().clone() for n, p in named})
        return orig(*a, **k)

    tr.optimizer.step = step


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("bf16", 5e-2)])
def test_graphed_step_matches_eager(cuda, precision, tol):
    n_rays, steps = 512, 6
    models = [configs.build_fine_model(32, precision, device=cuda, seed=3, mask_voxels=3.0, width=64)
              for _ in range(2)]
    eager = FineTrainer(models[0], n_rays=n_rays)
    graphed = FineTrainer(models[1], n_rays=n_rays, graphed=True)
    ge, gg = [], []
    _grab(eager, ge)
    _grab(graphed, gg)
    rays = [torch.from_numpy(a).to(cuda) for a in synthetic.random_rays(n_rays * steps, seed=5)]
    tgt = torch.from_numpy(configs.train_targets(n_rays * steps, 5)).to(cuda)
    for i in range(steps):
        sl = slice(i * n_rays, (i + 1) * n_rays)
        batch = [r[sl].contiguous() for r in rays] + [tgt[sl].contiguous()]
        le, _ = eager.step(*batch, RK)
        lg, _ = graphed.step(*batch, RK)
        if i == 0:
            graphed._engine.bucket = 256      # small buckets from now on: several captures
        torch.cuda.synchronize()
        assert abs(float(le) - float(lg)) <= 1e-5 * max(1.0, abs(float(le))), (i, float(le), float(lg))
        for name in ge[-1]:
            err = _rel(gg[-1][name], ge[-1][name])
            assert err <= tol, (i, name, err)
    assert len(graphed._engine.graphs) >= 2
    for (n, p), (_, q) in zip(models[0].named_parameters(), models[1].named_parameters()):
        assert _rel(q, p) <= (1e-4 if precision == "fp32" else 1e-2), n


def test_graphed_step_replays_without_host_work(cuda):
    """Once the buckets are captured, part B adds no host-side launches: the
    library's launch counter grows only by part A and the optimizer."""
    from voxurf_gb300 import _native

    n_rays = 256
    model = configs.build_fine_model(32, "bf16", device=cuda, seed=4, mask_voxels=3.0, width=64)
    tr = FineTrainer(model, n_rays=n_rays, graphed=True)
    rays = [torch.from_numpy(a).to(cuda) for a in synthetic.random_rays(n_rays, seed=9)]
    tgt = torch.from_numpy(configs.train_targets(n_rays, 9)).to(cuda)
    for _ in range(3):                        # same batch: same S2, one bucket
        tr.step(*rays, tgt, RK)
    torch.cuda.synchronize()
    c0 = _native.launch_count()
    tr.step(*rays, tgt, RK)
    torch.cuda.synchronize()
    # smoothing 1-2, march 1, scan <= 3, optimizer sweeps 2 + multi-tensor Adam 1
    assert _native.launch_count() - c0 <= 10
    assert np.isfinite(float(tr._engine.graphs[next(iter(tr._engine.graphs))]["loss"]))
