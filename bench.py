#!/usr/bin/env python
"""Benchmark of the Voxurf fine-stage training step on GB300.

Workload (the 256^3 fine configuration): SDF grid 256^3 FP32 (sphere r=0.45
union torus R=0.6 r=0.15, noise 0.005, seeded), k0 256^3 x 12 ~ N(0,0.1),
mask |SDF| < 0.05, rgbnet 70->192x3->3 and k_rgbnet 60->192x3->3, Gaussian
smoothing 5^3 sigma 0.8, stepsize 0.5 voxel, 8192 rays per step drawn from
49 cameras (1600x1200, f = 1.2 W) on the radius-3 sphere, targets U(0,1).
One step = forward + loss + hand-written backward + TV (weight 1e-4 on sdf
and k0) + Adam (lr 1e-3) on both grids and both MLPs.

`value` is train rays/s of the plain FP32 path with ray batches resident in
HBM; `e2e` is the same step through the public API with each batch copied
from pinned host memory and the loss read back inside the timed region;
`fused_bf16` repeats the step with k0 sampled from BF16 and both MLPs in
BF16 (FP32 accumulation).  The working set (~10 GB of grids and Adam state
swept every step) is far larger than L2, so no flush is needed.

--impl reference times the reference algorithm on the host CPU (the oracle's
torch restatement of the reference step, FP32, all host threads) on the
same workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "train rays/s (fine stage fwd+bwd+TV+Adam, 256^3, 8192 rays/step)"
UNIT = "rays/s"
R = 256
N_RAYS = 8192
MASK_VOXELS = 6.4  # |SDF| < 0.05 at voxel size 2/256

# Dominant kernel: the fused TV + Adam sweep over the k0 grid.  Algorithmic
# bytes per element: read p_old, grad, exp_avg, exp_avg_sq (16 B) + write
# p_new, exp_avg, exp_avg_sq (12 B) = 28 B (TV neighbour reads hit L1/L2).
K0_ELEMS = R ** 3 * 12
SWEEP_BYTES_PER_ELEM = 28
# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one k0 sweep
# launch, captured at 256^3 (the FP32 step's <12,1,1,0> launch: 3,222.35 MB
# read + 2,363.16 MB written for 201.3M elements; a single-pass capture).
SWEEP_NCU_TRAFFIC = 3222352128 + 2363156480 if R == 256 else None


def bench_config() -> dict:
    """The workload, identical in both arms."""
    return {"workload": "voxurf fine stage train step: SDF 256^3 f32 + k0 256^3x12 f32, 8192 rays/step, "
                        "stepsize 0.5, mask |SDF|<0.05, MLP 192x4 (x2), TV 1e-4, Adam 1e-3",
            "rays_per_step": N_RAYS, "grid": R,
            "l2": "no flush: ~10 GB of grids + Adam state swept per step (> 129 MB L2)"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-bf16", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-render", action="store_true", help="skip the render-server measurement")
    p.add_argument("--no-long", action="store_true", help="skip the long-ray (384^3, stepsize 0.25) measurement")
    p.add_argument("--no-eikonal", action="store_true",
                   help="skip the eikonal-training (coarse 96^3, 8192/32768 rays) measurement")
    p.add_argument("--no-mesh", action="store_true", help="skip the 512^3 mesh-extraction field measurement")
    p.add_argument("--no-womask", action="store_true", help="skip the maskless (womask) model's training step")
    p.add_argument("--no-background", action="store_true",
                   help="skip the background-sample generator measurement (scenes without an object mask)")
    p.add_argument("--micro", choices=["smooth", "mlp_tc", "background", "train_fp32", "train_bf16",
                                       "train_bf16_nograph"], default=None,
                   help="single-kernel timing instead of the step (profiling): the Gaussian smoothing sweep "
                        "on a --grid^3 grid, the fused tensor-core MLP against the GEMM path, or the "
                        "background-sample generator and cumdist_thres")
    p.add_argument("--render-requests", type=int, default=120)
    p.add_argument("--render-only", action="store_true", help="only the render-server measurement (profiling)")
    p.add_argument("--render-plain", type=int, default=8, help="requests rendered by the plain per-request path")
    p.add_argument("--render-grid", type=int, default=256, help="scene grid size (256 is the benchmark)")
    p.add_argument("--render-tick", type=int, default=1 << 21, help="rays packed per tick")
    p.add_argument("--render-staging", type=int, default=-1, choices=[-1, 0, 1],
                   help="row assembly of the features kernel (serve.RenderServer staging)")
    p.add_argument("--grid", type=int, default=256, help="grid resolution (256 is the benchmark; smaller sizes "
                                                         "serve profiler captures)")
    args = p.parse_args()
    global R, K0_ELEMS, MASK_VOXELS, SWEEP_NCU_TRAFFIC
    if args.grid != R:
        R = args.grid
        K0_ELEMS = R ** 3 * 12
        MASK_VOXELS = 0.05 / (2.0 / R)
        SWEEP_NCU_TRAFFIC = None
    return args


def dist_setup(args):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if (torch.cuda.is_available() and args.impl == "ours") else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    elif torch.cuda.is_available() and args.impl == "ours":
        torch.cuda.set_device(local)
    return world, rank, local


def rank_barrier(world, dev):
    """All replicas reach this point, with their device work finished."""
    import torch

    if world > 1:
        torch.distributed.barrier()
    if dev.type == "cuda":
        torch.cuda.synchronize(dev)


def max_over_ranks_of(x: float, world: int, dev) -> float:
    """The slowest replica's time (max over ranks; gloo on CPU, NCCL on GPU)."""
    import torch

    if world > 1:
        t = torch.tensor([x], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())
    return x


def whole_job_rays_per_s(world: int, rays_per_step: int, steps: int, t_max: float) -> float:
    """Rays of all replicas over the slowest replica's timed region."""
    return world * rays_per_step * steps / t_max


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def make_batches(n_batches, seed=0):
    import numpy as np

    from voxurf_gb300 import configs, synthetic

    o, d, v = synthetic.random_rays(N_RAYS * n_batches, seed=seed)
    t = configs.train_targets(N_RAYS * n_batches, seed)
    return [np.ascontiguousarray(a.reshape(n_batches, N_RAYS, 3)) for a in (o, d, v, t)]


def run_ours(args, world, rank, local):
    import torch

    from voxurf_gb300 import _native, configs
    from voxurf_gb300.train import FineTrainer

    dev = torch.device("cuda", local)
    if args.render_only:
        print(json.dumps({"render": run_render(args, dev)}))
        return
    if args.micro:
        print(json.dumps({"micro": run_micro(args, dev)}))
        return
    rk = dict(configs.FINE_RENDER_KWARGS)
    n_b = args.warmup + args.steps
    host = make_batches(n_b, seed=rank)
    dev_batches = [torch.from_numpy(a).to(dev) for a in host]

    def build(precision, graphed=False):
        model = configs.build_fine_model(R, precision, device=dev, seed=0, mask_voxels=MASK_VOXELS)
        return model, FineTrainer(model, n_rays=N_RAYS, graphed=graphed)

    def barrier():
        rank_barrier(world, dev)

    def max_over_ranks(x):
        return max_over_ranks_of(x, world, dev)

    # ---- plain FP32, device-resident batches ---------------------------------
    model, tr = build("fp32")
    sweep_ms = []
    orig_grid_step = tr.optimizer._grid_step

    def timed_grid_step(p, *a, **k):
        if p is model.k0.grid and timing["on"]:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            orig_grid_step(p, *a, **k)
            e1.record()
            timing["events"].append((e0, e1))
        else:
            orig_grid_step(p, *a, **k)

    timing = {"on": False, "events": []}
    tr.optimizer._grid_step = timed_grid_step
    for i in range(args.warmup):
        tr.step(dev_batches[0][i], dev_batches[1][i], dev_batches[2][i], dev_batches[3][i], rk)
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    timing["on"] = True
    l0 = _native.launch_count()
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_start.record()
    for i in range(args.warmup, n_b):
        tr.step(dev_batches[0][i], dev_batches[1][i], dev_batches[2][i], dev_batches[3][i], rk)
    e_end.record()
    barrier()
    launches = _native.launch_count() - l0
    timing["on"] = False
    ms = e_start.elapsed_time(e_end)
    clk = clocks.stop()
    sweep_ms = [a.elapsed_time(b) for a, b in timing["events"]]
    t_total = max_over_ranks(ms / 1000.0)
    value = whole_job_rays_per_s(world, N_RAYS, args.steps, t_total)
    shaded = int(model._last_frame.S2)

    # ---- e2e: same step, batches from pinned host memory, loss read back -------
    e2e, h2d = None, 0
    if not args.no_e2e:
        pinned = [torch.from_numpy(a).pin_memory() for a in host]
        barrier()
        w0 = time.perf_counter()
        e2e_losses = []
        for i in range(args.warmup, n_b):
            xs = [p[i].to(dev, non_blocking=True) for p in pinned]
            loss, _ = tr.step(xs[0], xs[1], xs[2], xs[3], rk)
            e2e_losses.append(float(loss.item()))
        barrier()
        t_e2e = max_over_ranks(time.perf_counter() - w0)
        e2e = whole_job_rays_per_s(world, N_RAYS, args.steps, t_e2e)
        h2d = sum(p[0].numel() * p[0].element_size() for p in pinned)
    del tr, model
    torch.cuda.empty_cache()

    # ---- fused BF16 variant --------------------------------------------------
    bf16 = None
    if not args.no_bf16:
        # k0 sampled from BF16, both MLPs in BF16 (FP32 accumulation), the
        # step replayed from CUDA graphs (fused_step.GraphedFineStep)
        model, tr = build("bf16", graphed=True)
        for i in range(args.warmup):
            tr.step(dev_batches[0][i], dev_batches[1][i], dev_batches[2][i], dev_batches[3][i], rk)
        barrier()
        l0 = _native.launch_count() + tr._engine.launches_replayed
        b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b0.record()
        for i in range(args.warmup, n_b):
            tr.step(dev_batches[0][i], dev_batches[1][i], dev_batches[2][i], dev_batches[3][i], rk)
        b1.record()
        barrier()
        tb = max_over_ranks(b0.elapsed_time(b1) / 1000.0)
        bf16 = {"value": world * N_RAYS * args.steps / tb, "unit": UNIT, "ms_per_step": 1000 * tb / args.steps,
                "speedup_vs_fp32": (world * N_RAYS * args.steps / tb) / value,
                "execution": "cuda graphs per shaded-row bucket (8192 rows)", "graphs": len(tr._engine.graphs),
                "gpu_launches": int(_native.launch_count() + tr._engine.launches_replayed - l0)}
        del tr, model
        torch.cuda.empty_cache()

    peak, peak_src = measured_peaks()
    sweep_avg = sum(sweep_ms) / max(len(sweep_ms), 1)
    alg_bytes = K0_ELEMS * SWEEP_BYTES_PER_ELEM
    achieved = alg_bytes / (sweep_avg / 1000.0) / 1e9 if sweep_avg > 0 else None
    roofline = {"kernel": "grid_tv_adam_kernel (k0 TV+Adam sweep)", "bound": "hbm", "achieved": achieved,
                "peak": peak, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                else "fallback 6800 GB/s", "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                "bytes_per_launch": alg_bytes, "launch_ms": sweep_avg,
                "traffic": SWEEP_NCU_TRAFFIC, "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                "one 256^3 launch" if SWEEP_NCU_TRAFFIC else None}

    render = None
    if not args.no_render:
        render = run_render(args, dev)
    long_rays = None
    if not args.no_long and R == 256:
        long_rays = run_long_rays(args, dev)
    eikonal = None
    if not args.no_eikonal and R == 256:
        eikonal = run_eikonal(args, dev)
    womask = womask_coarse = None
    if not args.no_womask and R == 256:
        womask = run_womask(args, dev)
        womask_coarse = run_womask_coarse(args, dev)
    mesh = None
    if not args.no_mesh and R == 256:
        mesh = run_mesh_query(args, dev)
    bg_samples = None
    if not args.no_background and R == 256:
        bg_samples = run_background(args, dev)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_total * 1000 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(),
            "parallelism": f"replicas x{world}", "shaded_samples_last_step": shaded,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 4},
            "fused_bf16": bf16,
            "render": render,
            "long_rays": long_rays,
            "eikonal_train": eikonal,
            "womask_train": womask,
            "womask_coarse_train": womask_coarse,
            "mesh_query": mesh,
            "background_samples": bg_samples,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": int(launches),
            # the sub-results that matter most, last (a reader of the output's
            # tail sees them)
            "headline": headline(value, e2e, bf16, render, long_rays),
        }
        print(json.dumps(line))


def headline(value, e2e, bf16, render, long_rays) -> dict:
    h = {"fp32_rays_s": value, "fp32_e2e_rays_s": e2e}
    if bf16:
        h["bf16_rays_s"] = bf16["value"]
        h["bf16_ms_per_step"] = bf16["ms_per_step"]
        h["bf16_speedup_vs_fp32"] = bf16["speedup_vs_fp32"]
    if render:
        h["render_saturated_mpix_s"] = render["saturated"]["mpix_s"]
        h["render_poisson_p99_ms_800x600"] = render["poisson_50_req_s"].get("p99_ms_800x600")
        h["render_poisson_p50_ms"] = render["poisson_50_req_s"].get("p50_ms")
    if long_rays:
        h["long_rays_bf16_speedup_vs_fp32"] = long_rays["speedup_bf16_vs_fp32"]
    return h


LONG_R = 384               # long-ray workload: 64 spheres, stepsize 0.25, 65536 rays, s = 0.05
LONG_RAYS = 65536
LONG_STEPS = 5


def run_long_rays(args, dev):
    """Long-ray stress workload (SDF 384^3 holding 64 random spheres + noise,
    k0 384^3 x 12, 65536 rays per step at stepsize 0.25 voxel = up to ~2660
    samples per ray, s-density 0.05): the plain FP32 step against the fused
    BF16 graph-replayed step, both full training steps."""
    import numpy as np
    import torch

    from voxurf_gb300 import configs, synthetic
    from voxurf_gb300.train import FineTrainer

    rk = dict(configs.FINE_RENDER_KWARGS, stepsize=0.25)
    n_b = 3 + LONG_STEPS
    o, d, v = synthetic.random_rays(LONG_RAYS * n_b, seed=11)
    t = configs.train_targets(LONG_RAYS * n_b, 11)
    batches = [torch.from_numpy(np.ascontiguousarray(a.reshape(n_b, LONG_RAYS, 3))).to(dev) for a in (o, d, v, t)]
    out = {"workload": f"SDF {LONG_R}^3 64 spheres + k0 {LONG_R}^3x12, {LONG_RAYS} rays/step, stepsize 0.25, "
                       "s 0.05, mask |SDF|<0.05", "rays_per_step": LONG_RAYS}
    for name, precision, graphed in (("fp32", "fp32", False), ("bf16_graphed", "bf16", True)):
        model = configs.build_fine_model(LONG_R, precision, device=dev, seed=7, scene="spheres64",
                                         mask_voxels=0.05 / (2.0 / LONG_R))
        tr = FineTrainer(model, n_rays=LONG_RAYS, graphed=graphed)
        for i in range(3):
            tr.step(batches[0][i], batches[1][i], batches[2][i], batches[3][i], rk, global_step=0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(3, n_b):
            tr.step(batches[0][i], batches[1][i], batches[2][i], batches[3][i], rk, global_step=0)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / LONG_STEPS
        out[name] = {"rays_per_s": LONG_RAYS / (ms / 1000.0), "ms_per_step": ms}
        if not graphed:
            fr = model._last_frame
            out["shaded_rows_last_step"] = int(fr.S2)
            out["max_steps_bound"] = int(fr.max_steps)
        del tr, model
        torch.cuda.empty_cache()
    out["speedup_bf16_vs_fp32"] = out["bf16_graphed"]["rays_per_s"] / out["fp32"]["rays_per_s"]
    return out


def _event_ms(fn, warmup, steps):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def run_micro_train(args, dev):
    """Training steps of one arm alone (profiling driver): `train_fp32` = the
    plain FP32 step, `train_bf16` = the graph-replayed BF16 step,
    `train_bf16_nograph` = the same BF16 step launched eagerly (every kernel
    a separate launch, which profilers can attribute); --grid^3 grids,
    8192 rays, --warmup untimed steps then --steps timed ones (no minimum)."""
    import torch

    from voxurf_gb300 import configs
    from voxurf_gb300.fused_step import GraphedFineStep
    from voxurf_gb300.train import FineTrainer

    rk = dict(configs.FINE_RENDER_KWARGS)
    n_b = args.warmup + args.steps
    batches = [torch.from_numpy(a).to(dev) for a in make_batches(n_b, seed=0)]
    prec = "fp32" if args.micro == "train_fp32" else "bf16"
    model = configs.build_fine_model(args.grid, prec, device=dev, seed=0, mask_voxels=MASK_VOXELS)
    tr = FineTrainer(model, n_rays=N_RAYS, graphed=prec == "bf16")
    if args.micro == "train_bf16_nograph":
        tr._engine = GraphedFineStep(tr, rk, use_graphs=False)

    def step(i):
        return tr.step(batches[0][i], batches[1][i], batches[2][i], batches[3][i], rk)

    for i in range(args.warmup):
        step(i)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(args.warmup, n_b):
        loss, _ = step(i)
    e1.record()
    torch.cuda.synchronize()
    return {"kind": args.micro, "grid": args.grid, "rays": N_RAYS, "steps": args.steps,
            "ms_per_step": e0.elapsed_time(e1) / max(args.steps, 1), "loss": float(loss)}


def run_micro(args, dev):
    """One kernel in isolation (CUDA events on the launching stream, warm-up
    launches first): `smooth` = vx_smooth3d / vx_smooth3d_adjoint (5^3,
    sigma 0.8) on a --grid^3 FP32 grid, 8 algorithmic bytes per voxel (12
    with accumulation); `mlp_tc` = the fused tcgen05 colour MLP
    (70(80) -> 192 x3 -> 3, BF16 rows; one and two tiles in flight per CTA)
    against torch's BF16 GEMMs (its cuBLAS) with the head kernel, at 131,072
    and 2,097,152 rows."""
    import numpy as np
    import torch
    import torch.nn as nn

    from voxurf_gb300 import _abi
    from voxurf_gb300._torch import ptr, stream_ptr

    W, S = max(args.warmup, 3), max(args.steps, 10)
    out = {"kind": args.micro}
    if args.micro.startswith("train_"):
        return run_micro_train(args, dev)
    if args.micro == "background":
        from voxurf_gb300 import ub360_utils_cuda

        out["generator"] = run_background(args, dev)
        d = torch.rand((N_RAYS, 890), device=dev, generator=torch.Generator(dev).manual_seed(1)) * 0.02
        ms = _event_ms(lambda: ub360_utils_cuda.cumdist_thres(d, 0.0208), W, S)
        out["cumdist_thres"] = {"shape": [N_RAYS, 890], "ms": ms, "gbs": d.numel() * 5 / (ms / 1000.0) / 1e9}
        print(json.dumps({"micro": out}))
        return
    if args.micro == "smooth":
        from voxurf_gb300.voxurf_fine import gaussian_taps, smooth_grid, smooth_grid_adjoint

        R = args.grid
        a = torch.randn((R, R, R), device=dev, generator=torch.Generator(dev).manual_seed(0))
        o = torch.empty_like(a)
        taps = gaussian_taps(5, 0.8)
        for name, fn, b in (("forward", lambda: smooth_grid(a, taps), 8),
                            ("adjoint", lambda: smooth_grid_adjoint(a, taps, out=o), 8),
                            ("adjoint_accumulate", lambda: smooth_grid_adjoint(a, taps, out=o, accumulate=True), 12)):
            ms = _event_ms(fn, W, S)
            out[name] = {"us": ms * 1000, "gbs": R ** 3 * b / ms / 1e6}
        out["grid"] = R
        return out
    gen = torch.Generator().manual_seed(0)
    net = nn.Sequential(nn.Linear(70, 192), nn.ReLU(), nn.Sequential(nn.Linear(192, 192), nn.ReLU()),
                        nn.Sequential(nn.Linear(192, 192), nn.ReLU()), nn.Linear(192, 3))
    for m in net.modules():
        if isinstance(m, nn.Linear):
            m.weight.data = torch.randn(m.weight.shape, generator=gen) * (1.0 / np.sqrt(m.in_features))
            m.bias.data = torch.randn(m.bias.shape, generator=gen) * 0.1
    net = net.to(dev)
    from voxurf_gb300.mlp import TensorCoreMLP

    tc = TensorCoreMLP(net, 80)
    lin = [m for m in net.modules() if isinstance(m, nn.Linear)]
    W0 = torch.zeros((192, 80), dtype=torch.bfloat16, device=dev)
    W0[:, :70] = lin[0].weight.to(torch.bfloat16)
    Ws = [W0, lin[1].weight.to(torch.bfloat16), lin[2].weight.to(torch.bfloat16)]
    bs = [m.bias.to(torch.bfloat16) for m in lin[:3]]
    Wh, bh = lin[3].weight.float().contiguous(), lin[3].bias.float().contiguous()
    for n in (131072, 2097152):
        X = torch.zeros((n, 80), dtype=torch.bfloat16, device=dev)
        X[:, :70] = torch.randn((n, 70), generator=gen).to(dev, torch.bfloat16)
        res = torch.empty((n, 3), device=dev)

        def gemm():
            h = X
            for Wl, bl in zip(Ws, bs):
                h = torch._addmm_activation(bl, h, Wl.t())
            _abi.call("vx_mlp_head", ptr(h), n, 192, 192, 1, ptr(Wh), ptr(bh), None, ptr(res), None, 0, 0,
                      stream_ptr())

        flops = n * 2 * (80 * 192 + 2 * 192 * 192 + 3 * 192)
        row = {}
        for name, fn in (("gemm", gemm), ("tc_one_tile", lambda: tc.forward(X, res, pipeline=0)),
                         ("tc", lambda: tc.forward(X, res, pipeline=1))):
            ms = _event_ms(fn, W, S)
            row[name] = {"ms": ms, "tflops": flops / ms / 1e9}
        out[f"rows_{n}"] = row
    return out


MESH_R = 512               # extract_geometry resolution of the reference's final mesh (run.py:798-799)


def run_mesh_query(args, dev):
    """Dense field for mesh extraction on the 256^3 fine model: the 512^3
    lattice over the bbox (smoothing of the SDF grid + one field launch,
    537 MB written), CUDA events around model.extract_fields."""
    import torch

    from voxurf_gb300 import configs

    model = configs.build_fine_model(R, "fp32", device=dev, seed=0, mask_voxels=MASK_VOXELS)
    bmin, bmax = model.xyz_min, model.xyz_max
    ms = _event_ms(lambda: model.extract_fields(bmin, bmax, MESH_R), 2, 5)
    grid = model.mesh_sdf_grid()
    from voxurf_gb300.voxurf_fine import extract_fields

    ms_field = _event_ms(lambda: extract_fields(grid, model.xyz_min, model.xyz_max, bmin, bmax, MESH_R), 2, 5)
    peak, _ = measured_peaks()
    field_bytes = MESH_R ** 3 * 4
    del model, grid
    torch.cuda.empty_cache()
    return {"workload": f"extract_fields {MESH_R}^3 over the bbox of the 256^3 fine model (-smoothed SDF)",
            "ms": ms, "field_ms": ms_field, "points_per_s": MESH_R ** 3 / (ms / 1000.0),
            "field_write_gbs": field_bytes / (ms_field / 1000.0) / 1e9,
            "field_frac_of_hbm": field_bytes / (ms_field / 1000.0) / 1e9 / peak}


def run_background(args, dev):
    """Background samples of a scene without an object mask (the womask
    fine model's sample_ray_ori + inversion + cumdist_thres + compaction) for
    8192 training rays (with jitter) on the 256^3 grid's 891 candidates per
    ray: count launch, device scan, one 8-byte read of the total, fill
    launch; CUDA events around the public call."""
    import numpy as np
    import torch

    from voxurf_gb300 import background, synthetic

    o, d, _ = synthetic.random_rays(N_RAYS, seed=21)
    o, d = torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev)
    jit = torch.rand(N_RAYS, device=dev, generator=torch.Generator(dev).manual_seed(0))
    vs = np.float32(2.0 / R)
    S = background.n_samples_for([R, R, R], 0.5)
    mn, mx = [-1.0] * 3, [1.0] * 3
    fn = lambda: background.background_samples(o, d, mn, mx, 0.2, 1e9, 0.5, vs, S, jit)  # noqa: E731
    ms = _event_ms(fn, 3, 10)
    kept = int(fn()[0].shape[0])
    return {"workload": f"womask background samples: {N_RAYS} rays x {S} candidates (256^3 grid, stepsize 0.5, "
                        "jitter), inversion + cumdist_thres + compaction",
            "ms": ms, "candidates_per_s": N_RAYS * S / (ms / 1000.0), "kept_samples": kept,
            "bytes_written": kept * 64}


EIK_R = 96                 # differentiation workload: coarse grids/MLP, eikonal 0.1
EIK_RAYS = (8192, 32768)
EIK_STEPS = 5
EIK_WEIGHT = 0.1


def run_eikonal(args, dev):
    """Differentiation workload: the coarse model (SDF 96^3 f32, k0 96^3x12,
    MLP 75 -> 128 x3 -> 3, Gaussian smoothing 5^3) trained with an eikonal
    term 0.1 * mean((|grad| - 1)^2) on the sampled points' finite-difference
    SDF gradient, at 8192 and 32768 rays per step: plain FP32 against BF16
    k0 + MLP (FP32 accumulation), both through the hand-written backward
    and full Adam steps.  Also the BF16 run's RGB / loss deviation from the
    FP32 run on the same batch (the FP64-oracle errors of both are checked
    by the test suite)."""
    import numpy as np
    import torch

    from voxurf_gb300 import configs, synthetic
    from voxurf_gb300.train import FineTrainer

    rk = dict(configs.COARSE_RENDER_KWARGS)
    n_b = 3 + EIK_STEPS
    out = {"workload": f"coarse SDF {EIK_R}^3 f32 + k0 {EIK_R}^3x12, MLP 75->128x3->3, sphere r=0.5, "
                       f"smoothing 5^3 s=0.8, eikonal {EIK_WEIGHT}, TV 1e-4, Adam 1e-3"}
    for n in EIK_RAYS:
        o, d, v = synthetic.random_rays(n * n_b, seed=13)
        t = configs.train_targets(n * n_b, 13)
        batches = [torch.from_numpy(np.ascontiguousarray(a.reshape(n_b, n, 3))).to(dev) for a in (o, d, v, t)]
        res, first = {}, {}
        for precision in ("fp32", "bf16"):
            model = configs.build_coarse_model(EIK_R, precision, device=dev, seed=0)
            tr = FineTrainer(model, n_rays=n, weight_eikonal=EIK_WEIGHT)
            loss, ret = tr.step(batches[0][0], batches[1][0], batches[2][0], batches[3][0], rk, global_step=1)
            first[precision] = (float(loss), ret["rgb_marched"].detach().clone())
            for i in range(1, 3):
                tr.step(batches[0][i], batches[1][i], batches[2][i], batches[3][i], rk, global_step=i + 1)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for i in range(3, n_b):
                tr.step(batches[0][i], batches[1][i], batches[2][i], batches[3][i], rk, global_step=i + 1)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / EIK_STEPS
            res[precision] = {"rays_per_s": n / (ms / 1000.0), "ms_per_step": ms,
                              "shaded_rows_last_step": int(ret["weights"].numel())}
            del tr, model, ret
            torch.cuda.empty_cache()
        res["speedup_bf16_vs_fp32"] = res["bf16"]["rays_per_s"] / res["fp32"]["rays_per_s"]
        res["bf16_vs_fp32_rgb_max_abs"] = float((first["bf16"][1] - first["fp32"][1]).abs().max())
        res["bf16_vs_fp32_loss_rel"] = abs(first["bf16"][0] - first["fp32"][0]) / max(abs(first["fp32"][0]), 1e-30)
        out[f"rays_{n}"] = res
    return out


WM_R = 256


def run_womask(args, dev):
    """Maskless fine model (foreground NeuS SDF inside the unit sphere,
    inverted-sphere background density grid): SDF + k0 256^3, bg_density +
    bg_k0 256^3, rgbnet / k_rgbnet 192 wide x4, bg_rgbnet 72 -> 192 x2 -> 3,
    8192 rays per step, full steps (forward, loss, backward, Adam) through
    the autograd path (foreground and background sample generation,
    boolean selections and MLP row counts read back by the host each step):
    FP32 and BF16."""
    import numpy as np
    import torch

    from voxurf_gb300 import configs, synthetic
    from voxurf_gb300.train import FineTrainer

    rk = dict(configs.FINE_RENDER_KWARGS)
    W, S = 3, 10
    o, d, v = synthetic.random_rays(N_RAYS * (W + S), seed=21)
    t = configs.train_targets(N_RAYS * (W + S), 21)
    b = [torch.from_numpy(np.ascontiguousarray(a.reshape(W + S, N_RAYS, 3))).to(dev) for a in (o, d, v, t)]
    out = {"workload": f"womask fine: SDF/k0 {WM_R}^3, bg_density/bg_k0 {WM_R}^3, rgbnet/k_rgbnet 192x4, "
                       f"bg_rgbnet 72->192x3->3, {N_RAYS} rays/step, sphere r=0.5 foreground"}
    for precision in ("fp32", "bf16"):
        model = configs.build_womask_model(WM_R, precision, device=dev, seed=0, width=192)
        tr = FineTrainer(model, n_rays=N_RAYS)
        for i in range(W):
            loss, ret = tr.step(b[0][i], b[1][i], b[2][i], b[3][i], rk, global_step=i + 2)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(W, W + S):
            loss, ret = tr.step(b[0][i], b[1][i], b[2][i], b[3][i], rk, global_step=i + 2)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / S
        out[precision] = {"ms_per_step": ms, "rays_per_s": N_RAYS / (ms / 1000.0),
                          "fg_rows_last_step": int(ret["weights"].numel()),
                          "bg_rows_last_step": int(ret["bg_weights"].numel()), "loss": float(loss)}
        del tr, model, ret
        torch.cuda.empty_cache()
    out["speedup_bf16_vs_fp32"] = out["fp32"]["ms_per_step"] / out["bf16"]["ms_per_step"]
    return out


WC_R = 96


def run_womask_coarse(args, dev):
    """Maskless coarse model with the dtu_e2e_womask coarse settings: SDF +
    k0 96^3, bg_density 96^3, rgbnet 75 -> 128 -> 3, bg_rgbnet 60 -> 128 x3
    -> 3, 8192 rays per step; full steps (forward, loss, the ori_tv loss
    terms: 0.01 x (sdf_tv 0.1 + smooth_grad_tv 0.05) + 0.01 x k0 TV,
    backward, Adam with the config's learning rates) through the autograd
    path: FP32 and BF16."""
    import numpy as np
    import torch

    from voxurf_gb300 import configs, synthetic
    from voxurf_gb300.train import FineTrainer

    rk = dict(configs.COARSE_RENDER_KWARGS)
    W, S = 3, 10
    o, d, v = synthetic.random_rays(N_RAYS * (W + S), seed=23)
    t = configs.train_targets(N_RAYS * (W + S), 23)
    b = [torch.from_numpy(np.ascontiguousarray(a.reshape(W + S, N_RAYS, 3))).to(dev) for a in (o, d, v, t)]
    out = {"workload": f"womask coarse: SDF/k0 {WC_R}^3, bg_density {WC_R}^3, rgbnet 75->128->3, "
                       f"bg_rgbnet 60->128x3->3, {N_RAYS} rays/step, ori_tv loss terms, sphere r=0.5 foreground"}
    for precision in ("fp32", "bf16"):
        model = configs.build_womask_coarse_model(WC_R, precision, device=dev, seed=0, width=128)
        tr = FineTrainer(model, lr_sdf=0.1, lr_k0=0.1, lr_rgbnet=1e-3, lr_bg=0.1, n_rays=N_RAYS,
                         loss_weights=(1.0, 0.0, 0.0), weight_tv_density=0.01, smooth_grad_tv=0.05, ori_tv=True,
                         sdf_tv=0.1, weight_tv_k0=0.01)
        for i in range(W):
            loss, ret = tr.step(b[0][i], b[1][i], b[2][i], b[3][i], rk, global_step=i + 2)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(W, W + S):
            loss, ret = tr.step(b[0][i], b[1][i], b[2][i], b[3][i], rk, global_step=i + 2)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / S
        out[precision] = {"ms_per_step": ms, "rays_per_s": N_RAYS / (ms / 1000.0),
                          "fg_rows_last_step": int(ret["weights"].numel()),
                          "bg_rows_last_step": int(ret["bg_weights"].numel()), "loss": float(loss)}
        del tr, model, ret
        torch.cuda.empty_cache()
    out["speedup_bf16_vs_fp32"] = out["fp32"]["ms_per_step"] / out["bf16"]["ms_per_step"]
    return out


RENDER_SCENES = 4
RENDER_RATE = 50.0          # requests per second (Poisson)
MLP_FLOPS_PER_ROW = 347136  # rgbnet + k_rgbnet forward FLOPs per shaded sample (70/60 -> 192 x3 -> 3)


def run_render(args, dev):
    """Render server on 4 resident 256^3 scenes (SDF FP32 + k0 BF16, MLPs
    BF16): a Poisson stream at 50 req/s and a saturated stream (all requests
    at t = 0), resolutions uniform over 160x120 .. 1600x1200, random poses
    on the radius-3 sphere; latency is arrival -> RGB + depth in host memory.
    Beside it, the plain per-request FP32 render (8192-ray chunks through
    Voxurf.forward) of the first requests of the same stream."""
    import numpy as np
    import torch

    from voxurf_gb300 import configs, serve

    RR = args.render_grid
    models = configs.build_serve_models(RR, "bf16", device=dev, n=RENDER_SCENES, mask_voxels=0.05 / (2.0 / RR))
    s_val = configs.trained_s_val()
    scenes = [serve.ResidentScene(m, s_val=s_val, precision="bf16") for m in models]
    for m in models:
        m.s_val = torch.ones(1) * s_val
        m.precision = "fp32"   # the plain render path
        m._k0_shadow = None
    server = serve.RenderServer(scenes, tick_rays=args.render_tick, arena_pixels=32 << 20,
                                staging=args.render_staging)
    torch.cuda.synchronize()
    serve.run_stream(server, serve.request_stream(6, float("inf"), RENDER_SCENES, seed=99))  # warm-up
    n = args.render_requests
    poisson = serve.run_stream(server, serve.request_stream(n, RENDER_RATE, RENDER_SCENES, seed=1))
    rows0 = server.rows_shaded
    saturated = serve.run_stream(server, serve.request_stream(n, float("inf"), RENDER_SCENES, seed=2))
    rows = server.rows_shaded - rows0
    sat_wall = saturated["wall_s"]
    # host time per tick by server method, on a second saturated stream
    # (timed wrappers around the methods: not part of the figures above)
    host = {"_front": 0.0, "_back": 0.0, "_row_bounds": 0.0, "poll": 0.0}

    def timed(name, fn):
        def call(*a, **k):
            t0 = time.perf_counter()
            try:
                return fn(*a, **k)
            finally:
                host[name] += time.perf_counter() - t0
        return call

    for name in host:
        setattr(server, name, timed(name, getattr(server, name)))
    ticks0 = server.ticks
    probe = serve.run_stream(server, serve.request_stream(n, float("inf"), RENDER_SCENES, seed=3))
    for name in host:
        delattr(server, name)   # back to the class methods
    ticks = max(server.ticks - ticks0, 1)
    saturated["host_ms_per_tick_probe"] = {
        "ticks": ticks, "wall": probe["wall_s"] * 1e3 / ticks, "probe_mpix_s": probe["mpix_s"],
        "launch_front": host["_front"] * 1e3 / ticks, "launch_back": host["_back"] * 1e3 / ticks,
        "harvest": host["poll"] * 1e3 / ticks, "wait_row_counts": host["_row_bounds"] * 1e3 / ticks}

    # plain per-request FP32 render of the first requests of the saturated stream
    stream = serve.request_stream(n, float("inf"), RENDER_SCENES, seed=2)[:args.render_plain]
    torch.cuda.synchronize()
    lat, px = [], 0
    w0 = time.perf_counter()
    err = None
    for t, s, c2w, H, W in stream:
        a = time.perf_counter()
        rgb, depth = serve.plain_render(models[s], c2w, H, W)
        rgb_h = rgb.cpu().numpy()
        lat.append(time.perf_counter() - a)
        px += H * W
        if (H, W) == (600, 800) and err is None:
            mine, _ = server.render(s, c2w, H, W)
            err = float(np.abs(mine - rgb_h).max())
    plain_wall = time.perf_counter() - w0
    plain = None
    if stream:
        plain = {"requests": len(stream), "mpix_s": px / plain_wall / 1e6,
                 "p50_ms": float(np.percentile(np.array(lat) * 1000, 50)),
                 "p99_ms": float(np.percentile(np.array(lat) * 1000, 99))}
    bf16_peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16_peak = float(json.load(f)["bf16_tflops"])
    except (OSError, KeyError, ValueError):
        bf16_peak = 1900.0
    mlp_tflops = rows * MLP_FLOPS_PER_ROW / sat_wall / 1e12
    del server, scenes, models
    torch.cuda.empty_cache()
    return {
        "metric": "render Mpix/s and p50/p99 latency (4 resident 256^3 scenes)",
        "workload": f"4 scenes sdf {RR}^3 f32 + k0 {RR}^3x12 bf16 + MLP bf16 (fused tcgen05), mask |SDF|<0.05, "
                    "s_val at step 20000, poses on r=3 sphere, res uniform {160x120,400x300,800x600,1600x1200}, "
                    f"tick {args.render_tick} rays",
        "poisson_50_req_s": poisson,
        "saturated": saturated,
        "plain_fp32_per_request": plain,
        "speedup_vs_plain": saturated["mpix_s"] / plain["mpix_s"] if plain else None,
        "shaded_rows_per_pixel": rows / saturated["pixels"],
        "mlp_tflops": mlp_tflops, "mlp_frac_of_bf16_peak": mlp_tflops / bf16_peak,
        "rgb_max_abs_vs_plain_fp32_800x600": err,
    }


def cpu_baseline():
    """The reference step on the host CPU (oracle restatement, FP32, all
    threads), a bounded sample of the benchmark workload: one warm-up and
    three timed full steps of 8192 rays on the 256^3 grids (~20 s)."""
    import torch

    from oracle.bench_cpu import time_reference_steps

    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    res = time_reference_steps(R, N_RAYS, 1, 3)
    return {"value": res["rays_per_s"], "unit": UNIT, "cores": cores, "kind": "port", "sample": res["sample"]}


def run_reference(args, world, rank):
    """The reference arm: --warmup untimed and --steps timed full reference
    steps (8192 rays on the 256^3 grids each, ~5 s of CPU per step) on all
    host cores, rank 0 only."""
    if rank != 0:
        return
    import torch

    from oracle.bench_cpu import time_reference_steps

    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    res = time_reference_steps(R, N_RAYS, args.warmup, args.steps)
    v = res["rays_per_s"]
    t_total = sum(res["times"])
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * t_total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": bench_config(),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": res["sample"]},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
