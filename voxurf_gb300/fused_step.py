"""The fine-stage training step replayed from CUDA graphs.

FineTrainer.step runs the forward through two torch.autograd.Functions and
lets autograd drive the hand-written backward: ~150 launches per step whose
host-side cost (Python, autograd, allocation) exceeds the GPU time of the
BF16 step.  GraphedFineStep runs the same kernels in the same order on
static buffers:

  part A (eager, 4 launches): Gaussian smoothing of the SDF grid, the ray
      march, the scan of the per-ray shaded counts, then the one host sync
      of the step (the shaded-row count S2, which sizes the MLP GEMMs);
  part B (one CUDA graph per row bucket): compaction, MLP input rows,
      rgbnet and k_rgbnet forward, compositing, the run.py loss and its
      gradient, compositing backward, MLP backward, the march/feature
      backward into the grid gradients and the smoothing adjoint;
  optimizer (eager, 3 launches): the fused TV + Adam sweeps of the two
      grids and one multi-tensor Adam launch for the MLPs.

Part B is captured for a row capacity rounded up to `bucket_rows`; kernels
that work per row read S2 from the device (s2_off[N]) and skip the rest,
the MLP engines too.  inv_s (which
changes every step with s_val) reaches the captured backward through a
device scalar refreshed from pinned host memory by the graph's first node.
The first time a capacity is seen, part B runs eagerly (on a side stream),
is captured, and is replayed; re-running part B is idempotent because it
clears its accumulators first.

The colour MLPs run on the engines of mlp.py (the tcgen05 kernels for BF16
rows, the FP32 CUDA-core kernels for FP32 rows); their input rows are padded
to the engine's row stride, and the rgbnet forward writes its logits straight
into the k-branch rows (k_res).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _abi, _native
from . import grid as grid_mod
from ._torch import ptr, stream_ptr
from .mlp import F32TrainMLP, TcTrainMLP, row_stride
from .voxurf_fine import _feature_cfg, max_steps_bound


def _round_up(x: int, m: int) -> int:
    return (x + m - 1) // m * m


class GraphedFineStep:
    def __init__(self, trainer, render_kwargs: dict, bucket_rows: int = 8192, use_graphs: bool = True):
        model = trainer.model
        if trainer.weight_eikonal > 0 or (trainer.weight_tv_density > 0 and (trainer.smooth_grad_tv > 0
                                                                               or trainer.ori_tv)):
            raise NotImplementedError("graphed step: eikonal / smooth_grad_tv / ori_tv terms run on the eager path")
        if not model.use_rgb_k:
            raise NotImplementedError("graphed step: the k-branch configuration (use_rgb_k) only")
        self.tr, self.model, self.rk = trainer, model, dict(render_kwargs)
        self.bucket = int(bucket_rows)
        self.use_graphs = use_graphs
        dev = model.sdf.grid.device
        self.dev = dev
        N = trainer.n_rays
        self.N = N
        X, Y, Z = (int(s) for s in model.sdf.grid.shape[2:])
        self.XYZ = (X, Y, Z)
        self.bf16 = model.precision == "bf16"
        self.xdt = torch.bfloat16 if self.bf16 else torch.float32
        xyz_min, xyz_max = grid_mod.host_values(model.xyz_min), grid_mod.host_values(model.xyz_max)
        self.geom = grid_mod.grid_geom((X, Y, Z), xyz_min, xyz_max)
        vs = model.voxel_size.float()
        self.stepdist = float(self.rk["stepsize"] * vs)
        self.voxel_size = float(vs)
        self.near = float(self.rk["near"])
        self.bg = float(self.rk["bg"])
        self.thres = float(model.fast_color_thres)
        self.max_steps = max_steps_bound(xyz_min, xyz_max, self.stepdist)
        self.taps = np.ascontiguousarray(model.smooth_taps, np.float32) if model.smooth_sdf else None
        self.cfg = _feature_cfg(model)
        self.d1 = model.dim0
        self.k_res = bool(model.k_res)
        self.d2a = model.k_dim0 - (3 if self.k_res else 0)
        self.ld1 = row_stride(self.d1, self.xdt)
        self.ld2 = row_stride(self.d2a + (3 if self.k_res else 0), self.xdt)
        f32, i32, i64 = torch.float32, torch.int32, torch.int64
        # inputs
        self.inp = torch.empty((4, N, 3), dtype=f32, device=dev)   # rays_o, rays_d, viewdirs, target
        # part A
        self.sdf_s = torch.empty((X, Y, Z), dtype=f32, device=dev)
        self.rec = torch.empty((N * self.max_steps, 4), dtype=f32, device=dev)
        self.dw_slot = torch.empty(N * self.max_steps, dtype=f32, device=dev)
        self.n1 = torch.empty(N, dtype=i32, device=dev)
        self.n2 = torch.empty(N, dtype=i32, device=dev)
        self.alast = torch.empty(N, dtype=f32, device=dev)
        self.s2_off = torch.empty(N + 1, dtype=i64, device=dev)
        self.scan_bytes = int(_native.load().vx_scan_scratch_bytes(N))
        self.scan_tmp = torch.empty(max(self.scan_bytes, 16), dtype=torch.uint8, device=dev)
        _abi._declare()
        self.loss_scratch_bytes = int(_native.load().vx_fine_composite_loss_scratch_bytes(N))
        # gradients (the optimizer's p.grad) and per-step device scalars
        self.d_sdf_s = torch.empty((X, Y, Z), dtype=f32, device=dev)
        self.d_sdf = torch.zeros_like(model.sdf.grid)
        self.d_k0 = torch.zeros_like(model.k0.grid)          # channels_last_3d like the parameter
        # marks of the k0 voxels the backward scatters to: part B resets only
        # those gradient rows, the optimizer sweep reads only those
        self.k0_touched = torch.zeros(_round_up(X * Y * Z, 16), dtype=torch.uint8, device=dev)
        self.k0_group = next(g for g in trainer.optimizer.param_groups if g.get("name") == "k0")
        self.dyn_host = torch.zeros(4, dtype=f32, pin_memory=True)
        self.dyn = torch.zeros(4, dtype=f32, device=dev)
        # the MLP engines (their operand buffers follow the FP32 parameters)
        if self.bf16:
            self.eng1 = TcTrainMLP(model.rgbnet, self.ld1)
            self.eng2 = TcTrainMLP(model.k_rgbnet, self.ld2)
        else:
            self.eng1 = F32TrainMLP(model.rgbnet)
            self.eng2 = F32TrainMLP(model.k_rgbnet)
        self.rgb_params = list(model.rgbnet.parameters())
        self.k_params = list(model.k_rgbnet.parameters())
        # static FP32 gradients (the optimizer's p.grad) and per-capacity
        # engine state (saved activations, backward scratch)
        self.g1 = self.eng1.grad_buffers()
        self.g2 = self.eng2.grad_buffers()
        self.mlp_state = {}
        self.cap = 0
        self.graphs = {}
        self.S2 = 0
        # library kernels executed by graph replays (the launch counter of
        # the C library only sees launches issued through its entry points)
        self.launches_replayed = 0

    # ---- buffers read beyond S2 (GEMM operands): static, zero-initialised --
    def _ensure_rows(self, cap: int) -> None:
        if cap <= self.cap:
            return
        cap = _round_up(int(cap * 1.25), self.bucket)
        self.X1 = torch.zeros((cap, self.ld1), dtype=self.xdt, device=self.dev)
        self.X2 = torch.zeros((cap, self.ld2), dtype=self.xdt, device=self.dev)
        self.cap = cap
        self.graphs.clear()   # captured graphs point at the old buffers
        self.mlp_state.clear()

    # ---- one step -------------------------------------------------------------
    def step(self, rays_o, rays_d, viewdirs, target, global_step=None):
        tr, model = self.tr, self.model
        if global_step is None:
            tr.global_step += 1
            global_step = tr.global_step
        _, inv_s = model.neus_s_val(global_step)
        for i, t in enumerate((rays_o, rays_d, viewdirs, target)):
            self.inp[i].copy_(t)
        S2 = self._part_a(inv_s)
        self.S2 = S2
        kptr = 0 if self.bf16 else model.k0.grid.data_ptr()
        cap = self._pick_capacity(S2, kptr)
        self._ensure_rows(cap)
        self.dyn_host[0] = inv_s
        key = (cap, kptr)
        entry = self.graphs.get(key)
        if entry is None:
            entry = self._build(cap, key)
        else:
            entry["graph"].replay()
            self.launches_replayed += entry["lib_launches"]
        model.sdf.grid.grad = self.d_sdf
        model.k0.grid.grad = self.d_k0
        for p, g in zip(self.rgb_params + self.k_params, entry["grads"]):
            p.grad = g
        self.k0_group["touched"] = self.k0_touched
        # the k0 sweep (TV + Adam) resets the touched gradient rows (part B
        # clears the marks); without a TV weight k0 takes the plain Adam
        # update, so reset the rows here
        sweep_resets = bool(self.k0_group.get("tv_weight", 0.0))
        try:
            tr.optimizer.step(zero_grad=True)
        finally:
            self.k0_group.pop("touched", None)
        if not sweep_resets:
            X, Y, Z = self.XYZ
            _native.call("vx_grid_clear_touched", ptr(self.d_k0), ptr(self.k0_touched), X * Y * Z, 12,
                         stream_ptr(self.dev))
        return entry["loss"], S2

    def _pick_capacity(self, S2: int, kptr: int) -> int:
        """Row capacity for S2 shaded rows: the smallest captured capacity in
        [S2, 1.3 S2 + bucket] (S2 drifts by a few percent between steps, and a
        capture costs tens of milliseconds), else S2 + 8% rounded up to the
        bucket, so that the next steps reuse the new graph."""
        fits = [c for (c, p) in self.graphs if p == kptr and S2 <= c <= 1.3 * S2 + self.bucket]
        if fits:
            return min(fits)
        return max(_round_up(int(S2 * 1.08) + 1, self.bucket), self.bucket)

    def _build(self, cap, key):
        if not self.use_graphs:
            return self._part_b(cap)
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):
            self._part_b(cap)            # warm-up
            # the k0 gradient accumulates over the touched voxels and is reset
            # by the optimizer sweep: undo the warm-up's contribution before
            # the replay (the sdf gradient buffer is cleared by part B itself)
            X, Y, Z = self.XYZ
            _native.call("vx_grid_clear_touched", ptr(self.d_k0), ptr(self.k0_touched), X * Y * Z, 12,
                         stream_ptr(self.dev))
        torch.cuda.current_stream(self.dev).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        c0 = _native.launch_count()
        with torch.cuda.graph(g):
            out = self._part_b(cap)
        out["lib_launches"] = _native.launch_count() - c0   # library kernels in the graph
        g.replay()
        self.launches_replayed += out["lib_launches"]
        out["graph"] = g
        self.graphs[key] = out
        return out

    # ---- part A: smoothing, march, scan, S2 ------------------------------------
    def _part_a(self, inv_s: float) -> int:
        model = self.model
        st = stream_ptr(self.dev)
        X, Y, Z = self.XYZ
        N = self.N
        sdf = model.sdf.grid
        if self.taps is not None:
            _abi.call("vx_smooth3d", ptr(sdf), ptr(self.sdf_s), None, None, X, Y, Z,
                      self.taps.ctypes.data, len(self.taps), st)
        else:
            self.sdf_s.copy_(sdf.reshape(X, Y, Z))
        a = _abi.FineMarchArgs()
        a.rays_o, a.rays_d, a.viewdirs = ptr(self.inp[0]), ptr(self.inp[1]), ptr(self.inp[2])
        a.n_rays, a.near, a.stepdist = N, self.near, self.stepdist
        a.grid = self.geom
        a.sdf_smooth = ptr(self.sdf_s)
        a.voxel_size = self.voxel_size
        if model.mask_cache is not None:
            model.mask_cache.fill_march(a)
        a.inv_s, a.dist, a.fast_color_thres = inv_s, self.stepdist, self.thres
        a.max_steps = self.max_steps
        a.rec, a.dw_slot, a.n1, a.n2, a.alphainv_last = ptr(self.rec), ptr(self.dw_slot), ptr(self.n1), \
            ptr(self.n2), ptr(self.alast)
        _abi.call_struct("vx_fine_march", a, st)
        _native.call("vx_exclusive_scan_i32", ptr(self.n2), N, ptr(self.s2_off), ptr(self.scan_tmp),
                     self.scan_bytes, st)
        return int(self.s2_off[N].item())

    # ---- part B: everything that depends on the shaded rows -------------------
    def _part_b(self, cap: int) -> dict:
        model = self.model
        dev, N, xdt = self.dev, self.N, self.xdt
        st = stream_ptr(self.dev)
        f32, i32 = torch.float32, torch.int32
        n_rows_dev = self.s2_off[N:]          # device S2
        self.dyn.copy_(self.dyn_host, non_blocking=True)
        self.d_sdf_s.zero_()
        # the marks of the previous step's scatter (its gradient rows were
        # reset by the optimizer sweep, which reads the marks)
        self.k0_touched.zero_()
        X, Y, Z = self.XYZ
        o, d, v, target = self.inp[0], self.inp[1], self.inp[2], self.inp[3]
        # compaction
        ray2 = torch.empty(cap, dtype=i32, device=dev)
        step2 = torch.empty(cap, dtype=i32, device=dev)
        slot2 = torch.empty(cap, dtype=i32, device=dev)
        w2 = torch.empty(cap, dtype=f32, device=dev)
        alpha2 = torch.empty(cap, dtype=f32, device=dev)
        pts2 = torch.empty((cap, 3), dtype=f32, device=dev)
        c = _abi.FineCompactArgs()
        c.rays_o, c.rays_d, c.n_rays, c.near, c.stepdist = ptr(o), ptr(d), N, self.near, self.stepdist
        for i in range(3):
            c.xyz_min[i] = self.geom.xyz_min[i]
            c.xyz_max[i] = self.geom.xyz_max[i]
        c.max_steps, c.rec, c.n1, c.s2_off = self.max_steps, ptr(self.rec), ptr(self.n1), ptr(self.s2_off)
        c.ray2, c.step2, c.slot2, c.w2, c.alpha2, c.pts2 = ptr(ray2), ptr(step2), ptr(slot2), ptr(w2), \
            ptr(alpha2), ptr(pts2)
        _abi.call_struct("vx_fine_compact", c, st)
        # MLP input rows
        X1, X2 = self.X1[:cap], self.X2[:cap]
        f = _abi.FineFeaturesArgs()
        f.n_rows, f.ray2, f.pts2, f.viewdirs = cap, ptr(ray2), ptr(pts2), ptr(v)
        f.grid, f.sdf_smooth, f.voxel_size = self.geom, ptr(self.sdf_s), self.voxel_size
        if self.bf16:
            f.k0_bf16 = ptr(model._k0_shadow)
        else:
            f.k0_f32 = ptr(model.k0.grid)
        f.cfg = self.cfg
        f.ld1, f.ld2 = self.ld1, self.ld2
        f.X1, f.X2, f.out_bf16 = ptr(X1), ptr(X2), int(self.bf16)
        f.n_rows_dev = ptr(n_rows_dev)
        _abi.call_struct("vx_fine_features", f, st)
        # colour MLPs: one pack launch for both engines' operands, then the
        # rgbnet forward (its logits also land in the k-branch rows, k_res)
        # and the k_rgbnet forward, over the device row count S2
        sv = self.mlp_state.setdefault(cap, ({}, {}, {}, {}))
        TcTrainMLP.pack_many([self.eng1, self.eng2], st)
        cols = X2[:, self.d2a:self.d2a + 3] if self.k_res else None
        logit, st1 = self.eng1.forward(X1, train=True, cols=cols, n_rows_dev=n_rows_dev, saved=sv[0])
        kout, st2 = self.eng2.forward(X2, train=True, n_rows_dev=n_rows_dev, saved=sv[1])
        # compositing, loss (run.py:604-610, 627, fine dtu_e2e weights) and the
        # compositing backward in one pass; rows at or beyond S2 stay unwritten
        # (the tensor-core MLP backward reads S2 rows; the FP32 engine runs
        # over the capacity and needs zeros there)
        wm, we, w0 = self.tr.loss_weights
        rgb0 = torch.empty((N, 3), dtype=f32, device=dev)
        rgbk = torch.empty((N, 3), dtype=f32, device=dev)
        loss = torch.empty(1, dtype=f32, device=dev)
        rows_alloc = torch.empty if self.bf16 else torch.zeros
        d_logit = rows_alloc((cap, 3), dtype=f32, device=dev)
        d_klogit = rows_alloc((cap, 3), dtype=f32, device=dev)
        d_w2 = torch.empty(cap, dtype=f32, device=dev)
        d_last = torch.empty(N, dtype=f32, device=dev)
        nb = self.loss_scratch_bytes
        scratch = torch.empty(nb, dtype=torch.uint8, device=dev)
        a = _abi.FineCompositeLossArgs()
        a.n_rays, a.s2_off, a.w2 = N, ptr(self.s2_off), ptr(w2)
        a.logit, a.kout, a.alphainv_last, a.target, a.bg = ptr(logit), ptr(kout), ptr(self.alast), ptr(target), \
            self.bg
        a.w_main, a.w_rgb0, a.w_entropy_last = wm, w0, we
        a.rgb0, a.rgbk, a.d_logit, a.d_kout, a.d_w2, a.d_last = ptr(rgb0), ptr(rgbk), ptr(d_logit), \
            ptr(d_klogit), ptr(d_w2), ptr(d_last)
        a.loss, a.scratch, a.scratch_bytes = ptr(loss), ptr(scratch), nb
        a.k_into_logit = int(not model.k_detach_2)
        _abi.call_struct("vx_fine_composite_loss", a, st)
        # MLP backward (k-branch first: its logit input may feed d_logit)
        if self.bf16:
            # both input-gradient chains, then the weight-gradient passes of
            # both MLPs in one launch and their sums in another
            dX2, g2, pend2 = self.eng2.backward_chain(st2, d_klogit, dx_dtype=xdt, grads=self.g2, work=sv[3])
            if self.k_res and not model.k_detach_1:
                d_logit = d_logit + dX2[:, self.d2a:self.d2a + 3].float()
            dX1, g1, pend1 = self.eng1.backward_chain(st1, d_logit, dx_dtype=xdt, grads=self.g1, work=sv[2])
            TcTrainMLP.weight_gradients([pend2, pend1], st)
        else:
            dX2, g2 = self.eng2.backward(st2, d_klogit, dx_dtype=xdt, grads=self.g2, work=sv[3])
            if self.k_res and not model.k_detach_1:
                d_logit = d_logit + dX2[:, self.d2a:self.d2a + 3].float()
            dX1, g1 = self.eng1.backward(st1, d_logit, dx_dtype=xdt, grads=self.g1, work=sv[2])
        # march / feature backward into the grid gradients
        bw = _abi.FineBackwardArgs()
        bw.n_rays, bw.n_rows = N, cap
        bw.rays_o, bw.rays_d, bw.viewdirs = ptr(o), ptr(d), ptr(v)
        bw.near, bw.stepdist, bw.grid = self.near, self.stepdist, self.geom
        bw.sdf_smooth, bw.voxel_size, bw.inv_s, bw.dist = ptr(self.sdf_s), self.voxel_size, 1.0, self.stepdist
        bw.max_steps, bw.rec, bw.dw_slot, bw.n1 = self.max_steps, ptr(self.rec), ptr(self.dw_slot), ptr(self.n1)
        bw.alphainv_last, bw.d_last = ptr(self.alast), ptr(d_last)
        bw.pts2, bw.slot2, bw.dw2 = ptr(pts2), ptr(slot2), ptr(d_w2)
        bw.cfg, bw.ld1, bw.ld2 = self.cfg, self.ld1, self.ld2
        bw.dX1, bw.dX2, bw.in_bf16 = ptr(dX1), ptr(dX2), int(self.bf16)
        bw.d_sdf_smooth, bw.d_k0 = ptr(self.d_sdf_s), ptr(self.d_k0)
        bw.n_rows_dev, bw.inv_s_dev = ptr(n_rows_dev), ptr(self.dyn)
        bw.k0_touched = ptr(self.k0_touched)
        _abi.call_struct("vx_fine_backward", bw, st)
        if self.taps is not None:
            _abi.call("vx_smooth3d_adjoint", ptr(self.d_sdf_s), ptr(self.d_sdf), None, None,
                      X, Y, Z, self.taps.ctypes.data, len(self.taps), 0, st)
        else:
            self.d_sdf.view(X, Y, Z).copy_(self.d_sdf_s)
        return {"loss": loss[0], "grads": g1 + g2, "S2_cap": cap}
