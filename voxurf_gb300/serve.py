"""Render server: several trained fine-stage scenes resident in HBM,
novel-view requests of any resolution, continuous batching in ticks.

The reference renders views one scene per process, 8192 rays per
Voxurf.forward call (run.py:81-126, render_viewpoints).  Here each tick
packs rays from every admitted request (oldest first, up to ``tick_rays``)
and runs the inference form of the forward (voxurf_fine.py:620-802 with
global_step=None) over them with one launch per stage for all scenes
(vx_serve_rays / _march / _rows / _features / _composite); only the colour
MLPs are issued per scene, on the scene's contiguous rows: for BF16 scenes
the fused tcgen05 kernel (vx_mlp_tc_forward, hidden activations never leave
the SM), otherwise the MLP engines of mlp.py (tcgen05 training kernels for
BF16 rows, FP32 CUDA-core kernels for FP32 rows) in inference mode.  With a bool mask, a thread-per-ray pass over the
mask's block occupancy starts each ray's march at its first sample that can
lie in the mask.  The composite writes straight into each request's range
of an output arena.

A tick has a front half (rays, march, row scan, rows, features; on the
front stream) and a back half (the MLPs and compositing; on the back
stream), and the two halves of consecutive ticks overlap: the host
launches the front half of tick t+1 and the back half of tick t, then
waits for tick t+1's row counts (the tick's one host synchronisation,
taken right after the scan: the features kernel reads the row count on the
device).  So the march and feature gathers of one tick (load/store and
integer work, many warps) run beside the tensor-core MLPs of the previous
one (one CTA of 9 warps per SM).  Two workspace slots alternate between
ticks, each with its own MLP input rows; a slot is reused once its
previous tick's compositing is done (an event).

Admission is by device memory: a request is admitted once the arena (sized
from free HBM when the server starts) has room for its pixels and fewer
than ``max_active`` requests are in flight; until then it waits in FIFO
order.  A request that is admitted while others are being rendered joins
the very next tick, so work of different requests overlaps on the device.
Each scene keeps its own s_val (it is not part of a checkpoint: the
reference's eval uses whatever the module holds, voxurf_fine.py:61).
"""
from __future__ import annotations

import bisect
import ctypes
import math
import time
from collections import deque

import numpy as np
import torch

from . import _abi
from . import grid as grid_mod
from ._torch import ptr, scratch, stream_ptr
from .mlp import TensorCoreMLP, engine_for
from .voxurf_fine import _feature_cfg, max_steps_bound, smooth_grid

_BYTES_PER_PIXEL = 16  # rgb f32 + depth f32 (device and pinned host)


def _round_up(x: int, m: int) -> int:
    return (x + m - 1) // m * m


def inv_s_of(s_val: float) -> float:
    """1/s_val as the model computes it (FP32 division, voxurf_fine.py:476)."""
    return float((torch.ones(1) / torch.tensor([s_val], dtype=torch.float32)).item())


class ResidentScene:
    """One scene in the render layout: smoothed SDF (FP32), k0 channel-last
    (BF16 or FP32), optional mask, the two colour MLPs (hidden layers in the
    compute dtype, output layers FP32) and the scene's s_val."""

    def __init__(self, model, s_val: float | None = None, stepsize: float = 0.5, near: float = 0.1,
                 bg: float = 0.0, precision: str = "bf16", skip_block: int = 16):
        """skip_block > 0 builds the block occupancy of a bool mask (blocks of
        skip_block^3 voxels, widened by one voxel): a thread-per-ray pass finds
        each ray's first sample that can lie in the mask and the march starts
        there (exact: rays that miss the mask do no march work); 0 disables it.
        A MaskCache (density) mask has no occupancy grid."""
        if precision not in ("bf16", "fp32"):
            raise ValueError(precision)
        dev = model.sdf.grid.device
        self.precision = precision
        self.dtype = torch.bfloat16 if precision == "bf16" else torch.float32
        with torch.no_grad():
            sdf = model.sdf.grid.detach().float()
            if model.smooth_sdf:
                self.sdf = smooth_grid(sdf.contiguous(), model.smooth_taps)
            else:
                self.sdf = sdf[0, 0].contiguous()
            k0 = model.k0.grid.detach()[0].permute(1, 2, 3, 0)  # [X,Y,Z,12]
            self.k0 = k0.to(self.dtype).contiguous()
        self.s_val = float(model.s_val.float().item()) if s_val is None else float(s_val)
        xyz_min = grid_mod.host_values(model.xyz_min)
        xyz_max = grid_mod.host_values(model.xyz_max)
        vs = float(model.voxel_size.float())
        self.stepdist = float(stepsize * model.voxel_size.float())
        self.max_steps = max_steps_bound(xyz_min, xyz_max, self.stepdist)
        self.cfg = _feature_cfg(model)
        self.d1 = model.dim0
        self.k_res = bool(model.k_res)
        self.use_rgb_k = bool(model.use_rgb_k)
        self.d2a = model.k_dim0 - (3 if self.k_res else 0)
        # MLP input rows padded to 16 columns (the tensor-core K step)
        self.ld1 = _round_up(self.d1, 16)
        self.ld2 = _round_up(self.d2a + 3, 16)
        # MLP engines (operands packed once: the weights of a served scene
        # do not change); used when the fused inference kernel does not apply
        self.engines = (engine_for(model.rgbnet, self.dtype, self.ld1),
                        engine_for(model.k_rgbnet, self.dtype, self.ld2) if self.use_rgb_k else None)
        for e in self.engines:
            if e is not None:
                e.pack()
        # fused tcgen05 forward of both MLPs (BF16 scenes of the 192-wide layout)
        self.tc = None
        if precision == "bf16" and self.use_rgb_k and TensorCoreMLP.supports(model.rgbnet, self.ld1) \
                and TensorCoreMLP.supports(model.k_rgbnet, self.ld2):
            self.tc = (TensorCoreMLP(model.rgbnet, self.ld1), TensorCoreMLP(model.k_rgbnet, self.ld2))

        d = _abi.SceneDesc()
        d.grid = grid_mod.grid_geom(self.sdf.shape, xyz_min, xyz_max)
        d.sdf_smooth = self.sdf.data_ptr()
        d.k0 = self.k0.data_ptr()
        d.k0_bf16 = int(precision == "bf16")
        d.voxel_size = vs
        self.mask = None
        self.occ = None
        if isinstance(model.mask_cache, grid_mod.MaskCache):
            # trilinear density mask: evaluated per sample, no block skipping
            self.mask = model.mask_cache.density
            model.mask_cache.fill_march(d)
        elif model.mask_cache is not None:
            mc = model.mask_cache
            self.mask = mc.mask.contiguous()
            d.mask = self.mask.data_ptr()
            d.mask_X, d.mask_Y, d.mask_Z = (int(s) for s in self.mask.shape)
            sc, sh = grid_mod.host_values(mc.xyz2ijk_scale), grid_mod.host_values(mc.xyz2ijk_shift)
            for a in range(3):
                d.mask_scale[a] = float(sc[a])
                d.mask_shift[a] = float(sh[a])
            if skip_block:
                # block occupancy of the mask: the march jumps over empty blocks
                B = int(skip_block)
                oshape = tuple(-(-int(s) // B) + 2 for s in self.mask.shape)
                self.occ = torch.empty(oshape, dtype=torch.uint8, device=dev)
                _abi.call("vx_mask_occupancy", ptr(self.mask), *self.mask.shape, B, ptr(self.occ), stream_ptr(dev))
                d.occ = self.occ.data_ptr()
                d.occ_X, d.occ_Y, d.occ_Z = oshape
                d.occ_block = B
        d.inv_s = inv_s_of(self.s_val)
        d.stepdist = self.stepdist
        d.near = float(near)
        d.bg = float(bg)
        d.fast_color_thres = float(model.fast_color_thres)
        self.desc = d
        self.device = dev

    def nbytes(self) -> int:
        ts = [self.sdf, self.k0] + ([self.mask] if self.mask is not None else [])
        for e in self.engines:
            if e is not None:
                ts += [t for t in vars(e).values() if isinstance(t, torch.Tensor)]
                ts += [t for v in vars(e).values() if isinstance(v, list) for t in v if isinstance(t, torch.Tensor)]
        return sum(t.numel() * t.element_size() for t in ts)


class RenderRequest:
    """A novel view: scene index, camera-to-world (3x4 or 4x4), resolution,
    pinhole intrinsics (OpenCV axes by default)."""

    def __init__(self, rid: int, scene: int, c2w, H: int, W: int, focal: float | None, inverse_y: bool,
                 arrival: float):
        self.id = rid
        self.scene = scene
        self.c2w = np.asarray(c2w, np.float32)[:3, :4].copy()
        self.H, self.W = int(H), int(W)
        f = 1.2 * W if focal is None else float(focal)
        self.fx = self.fy = f
        self.cx, self.cy = W / 2.0, H / 2.0
        self.inverse_y = bool(inverse_y)
        self.arrival = arrival
        self.n_pix = self.H * self.W
        self.next_pix = 0
        self.off = None          # arena offset once admitted
        self.t_admit = None
        self.t_done = None
        self.event = None
        self.rgb = None          # [H, W, 3] float32 (host) when done
        self.depth = None        # [H, W] float32

    @property
    def latency(self) -> float | None:
        return None if self.t_done is None else self.t_done - self.arrival


class OutputArena:
    """First-fit allocator over [0, capacity) pixels."""

    def __init__(self, capacity: int):
        self.capacity = int(capacity)
        self.free = [(0, self.capacity)]  # sorted (start, length)

    def alloc(self, n: int) -> int | None:
        for i, (s, ln) in enumerate(self.free):
            if ln >= n:
                if ln == n:
                    self.free.pop(i)
                else:
                    self.free[i] = (s + n, ln - n)
                return s
        return None

    def release(self, s: int, n: int) -> None:
        i = bisect.bisect_left(self.free, (s, 0))
        self.free.insert(i, (s, n))
        merged = []
        for a, ln in self.free:
            if merged and merged[-1][0] + merged[-1][1] == a:
                merged[-1] = (merged[-1][0], merged[-1][1] + ln)
            else:
                merged.append((a, ln))
        self.free = merged

    def used(self) -> int:
        return self.capacity - sum(ln for _, ln in self.free)


class _TickSlot:
    """Device workspace of one tick in flight (rays, per-ray sample records,
    row offsets, the MLP input rows) and its pinned host staging."""

    def __init__(self, N: int, max_steps: int, scan_bytes: int, max_chunks: int, dev):
        self.rays = torch.empty((3, N, 3), dtype=torch.float32, device=dev)
        self.ray_scene = torch.empty(N, dtype=torch.int32, device=dev)
        self.ray_out = torch.empty(N, dtype=torch.int64, device=dev)
        self.n2 = torch.empty(N, dtype=torch.int32, device=dev)
        self.alast = torch.empty(N, dtype=torch.float32, device=dev)
        self.s2_off = torch.empty(N + 1, dtype=torch.int64, device=dev)
        self.scan_tmp = scratch(scan_bytes, dev)
        self.rec = torch.empty(N * max_steps * 8, dtype=torch.uint8, device=dev)
        self.chunk_host = torch.empty(max_chunks * ctypes.sizeof(_abi.ViewChunk), dtype=torch.uint8,
                                      pin_memory=True)
        self.chunk_dev = torch.empty_like(self.chunk_host, device=dev)
        self.chunk_ready = torch.cuda.Event()
        self.bounds_host = torch.empty(16, dtype=torch.int64, pin_memory=True)
        self.idx_host = torch.empty(16, dtype=torch.int64, pin_memory=True)   # scene bounds, staged
        self.idx_dev = torch.empty(16, dtype=torch.int64, device=dev)
        self.ev_back = None   # recorded after the back half of the slot's last tick
        self.rows_cap = 0     # shaded rows the slot's ray2 / X1 / X2 hold
        self.ray2 = self.X1 = self.X2 = None


class _Tick:
    """One tick between its front and back halves."""

    def __init__(self, slot: int):
        self.slot = slot
        self.N = 0
        self.S2 = 0
        self.scene_ids: list[int] = []
        self.bounds: list[int] = []
        self.row_bounds: list[int] = []
        self.finished: list = []
        self.ev_bounds = None   # row counts in pinned memory
        self.ev_front = None    # front half done (MLP input rows written)


class RenderServer:
    def __init__(self, scenes: list[ResidentScene], tick_rays: int = 1 << 19, arena_pixels: int | None = None,
                 hbm_reserve: int = 8 << 30, max_active: int = 64, device=None, mem_info=None, mlp: str = "tc",
                 staging: int = -1, rows_per_ray: float = 8.0):
        """staging: the features kernel's row assembly (vx_serve_features: 0
        stores each row from its thread and needs no dynamic shared memory,
        so its CTAs fit on the SMs beside the tensor-core MLP of the other
        tick; 1 stages rows in shared memory; -1 chooses 1 where it fits).
        rows_per_ray: the initial shaded-row capacity of a slot per tick ray
        (a slot grows when a tick has more).
        mlp: "tc" runs each scene's two colour MLPs as fused tcgen05
        launches where the scene supports it (BF16, 192-wide), "layers" on the
        MLP engines of mlp.py (one kernel per layer)."""
        if not 1 <= len(scenes) <= 8:
            raise ValueError("1 to 8 resident scenes")
        if not all(s.use_rgb_k and s.k_res for s in scenes):
            raise NotImplementedError("render server: fine models with the k-branch (use_rgb_k, k_res)")
        c0 = bytes(scenes[0].cfg)
        if any(bytes(s.cfg) != c0 or s.precision != scenes[0].precision for s in scenes):
            raise ValueError("resident scenes must share the feature layout and precision")
        self.scenes = scenes
        self.device = torch.device(device) if device is not None else scenes[0].device
        self.dtype = scenes[0].dtype
        self.bf16 = scenes[0].precision == "bf16"
        self.tick_rays = int(tick_rays)
        self.max_active = int(max_active)
        self.mem_info = mem_info or (lambda: torch.cuda.mem_get_info(self.device))
        self.max_steps = max(s.max_steps for s in scenes)
        self.table = (_abi.SceneDesc * len(scenes))(*[s.desc for s in scenes])
        self.cfg = scenes[0].cfg
        self.d1 = scenes[0].d1
        self.d2a = scenes[0].d2a
        self.ld1 = scenes[0].ld1
        self.ld2 = scenes[0].ld2
        if mlp not in ("tc", "layers"):
            raise ValueError(mlp)
        self.mlp = mlp
        if staging not in (-1, 0, 1):
            raise ValueError(staging)
        self.staging = int(staging)
        dev = self.device
        N = self.tick_rays
        # per-tick workspace (fixed size), two slots: while the back half of
        # tick t (features, MLPs, compositing) runs on the back stream, the
        # front half of tick t+1 (rays, march, scan) runs on the front stream
        lib = _abi._native.load()
        self.scan_bytes = int(lib.vx_scan_scratch_bytes(N))
        self.max_chunks = 4 * max_active + 8
        self.slots = [_TickSlot(N, self.max_steps, self.scan_bytes, self.max_chunks, dev) for _ in range(2)]
        torch.cuda.current_stream(dev).synchronize()   # scene uploads are complete
        self.front_stream = torch.cuda.Stream(dev)
        self.back_stream = torch.cuda.Stream(dev)
        self.pending = None   # the tick whose back half is not launched yet
        self.rows_cap = 0     # logit rows
        self._grow_rows(N * 6)
        for sl in self.slots:
            self._grow_slot_rows(sl, int(N * rows_per_ray))
        # output arena (device) and its pinned host mirror
        if arena_pixels is None:
            free, _ = self.mem_info()
            arena_pixels = max(0, (free - hbm_reserve)) // (2 * _BYTES_PER_PIXEL)
            arena_pixels = min(arena_pixels, 64 << 20)
        self.arena = OutputArena(arena_pixels)
        self.out_rgb = torch.empty((arena_pixels, 3), dtype=torch.float32, device=dev)
        self.out_depth = torch.empty(arena_pixels, dtype=torch.float32, device=dev)
        self.host_rgb = torch.empty((arena_pixels, 3), dtype=torch.float32, pin_memory=True)
        self.host_depth = torch.empty(arena_pixels, dtype=torch.float32, pin_memory=True)
        self.queue: deque[RenderRequest] = deque()   # waiting for admission
        self.active: list[RenderRequest] = []        # admitted, pixels left to launch
        self.finishing: list[RenderRequest] = []     # all pixels launched, copy in flight
        self.reaped: list[RenderRequest] = []        # in the pinned arena, host copy pending
        self.done: list[RenderRequest] = []
        self._next_id = 0
        self.ticks = 0
        self.rays_launched = 0
        self.rows_shaded = 0

    # ---- requests ---------------------------------------------------------
    def submit(self, scene: int, c2w, H: int, W: int, focal: float | None = None, inverse_y: bool = True,
               arrival: float | None = None) -> RenderRequest:
        if not 0 <= scene < len(self.scenes):
            raise ValueError(f"unknown scene {scene}")
        if H * W > self.arena.capacity:
            raise ValueError(f"{H}x{W} exceeds the output arena ({self.arena.capacity} pixels)")
        r = RenderRequest(self._next_id, scene, c2w, H, W, focal, inverse_y,
                          time.perf_counter() if arrival is None else arrival)
        self._next_id += 1
        self.queue.append(r)
        return r

    def _admit(self) -> None:
        while self.queue and len(self.active) + len(self.finishing) < self.max_active:
            r = self.queue[0]
            off = self.arena.alloc(r.n_pix)
            if off is None:
                return  # FIFO: wait for memory to free up
            self.queue.popleft()
            r.off = off
            r.t_admit = time.perf_counter()
            self.active.append(r)

    def _reap(self) -> None:
        """Requests whose results have reached the pinned arena give back
        their arena range and their seat (an event query each; no copy).
        Their pinned range stays intact until poll() copies it out: a request
        admitted into it now is copied to host memory only after it has been
        rendered, ticks later."""
        still = []
        for r in self.finishing:
            if r.event.query():
                self.arena.release(r.off, r.n_pix)
                r.event = None
                self.reaped.append(r)
            else:
                still.append(r)
        self.finishing = still

    def poll(self) -> list[RenderRequest]:
        """Completes the requests whose results have reached host memory."""
        self._reap()
        out = self.reaped
        self.reaped = []
        for r in out:
            a, b = r.off, r.off + r.n_pix
            r.rgb = self.host_rgb[a:b].numpy().reshape(r.H, r.W, 3).copy()
            r.depth = self.host_depth[a:b].numpy().reshape(r.H, r.W).copy()
            r.t_done = time.perf_counter()
        self.done.extend(out)
        return out

    def idle(self) -> bool:
        return not (self.queue or self.active or self.finishing or self.reaped or self.pending)

    def has_work(self) -> bool:
        return bool(self.queue or self.active or self.pending)

    # ---- one tick -----------------------------------------------------------
    def tick(self) -> int:
        """Frees the seats and arena ranges of finished requests, admits what
        fits, launches the front half of one tick of rays and the back half
        of the previous tick, then copies finished requests out of the pinned
        arena (those host copies overlap the launched work).
        Returns the number of rays launched."""
        self._reap()
        self._admit()
        budget = self.tick_rays
        batch = []
        for r in self.active:
            if budget == 0 or len(batch) == self.max_chunks:
                break
            n = min(r.n_pix - r.next_pix, budget)
            if n > 0:
                batch.append((r, r.next_pix, n))
                r.next_pix += n
                budget -= n
        new = self._front(batch) if batch else None
        if new is not None:
            new.finished = [r for r in self.active if r.next_pix == r.n_pix]
            self.active = [r for r in self.active if r.next_pix < r.n_pix]
        if self.pending is not None:
            self._back(self.pending)
        self.pending = None
        # completed requests are copied out of the pinned arena while the
        # GPU runs what was just launched
        self.poll()
        if new is None:
            return 0
        self._row_bounds(new)   # the tick's one host sync (front stream only)
        self.pending = new
        self.ticks += 1
        self.rays_launched += new.N
        return new.N

    def run_until_idle(self, sleep: float = 0.0) -> None:
        while not self.idle():
            if self.has_work():
                self.tick()
            else:
                self.poll()
                if sleep:
                    time.sleep(sleep)

    def render(self, scene: int, c2w, H: int, W: int, **kw):
        """Renders one view synchronously (alone, or with whatever is queued)."""
        r = self.submit(scene, c2w, H, W, **kw)
        while r.t_done is None:
            if self.has_work():
                self.tick()
            else:
                self.poll()
        return r.rgb, r.depth

    # ---- device work ------------------------------------------------------------
    def _grow_rows(self, n: int) -> None:
        """The logit buffers (shared by the ticks: only the back stream uses
        them)."""
        n = _round_up(max(n, 1), 1 << 16)
        if n <= self.rows_cap:
            return
        dev = self.device
        if self.rows_cap:
            self.back_stream.synchronize()   # the old rows are no longer read
        self.rows_cap = n
        self.logit = torch.empty((n, 3), dtype=torch.float32, device=dev)
        self.klogit = torch.empty((n, 3), dtype=torch.float32, device=dev)

    def _grow_slot_rows(self, sl: _TickSlot, n: int) -> None:
        """A slot's MLP input rows; the caller has made sure no queued work
        reads the old ones."""
        n = _round_up(max(n, 1), 1024)
        if n <= sl.rows_cap:
            return
        dev = self.device
        sl.ray2 = sl.X1 = sl.X2 = None
        sl.rows_cap = n
        sl.ray2 = torch.empty(n, dtype=torch.int32, device=dev)
        sl.X1 = torch.empty((n, self.ld1), dtype=self.dtype, device=dev)
        sl.X2 = torch.empty((n, self.ld2), dtype=self.dtype, device=dev)

    def _rows_and_features(self, t: "_Tick", st: int) -> None:
        """ray2 and the MLP input rows of a tick, sized on the device (the
        row count is s2_off[N]); rows beyond the slot's capacity are skipped
        and redone by _row_bounds after it grows the slot."""
        sl = self.slots[t.slot]
        o, d, v = sl.rays[0], sl.rays[1], sl.rays[2]
        N = t.N
        _abi.call("vx_serve_rows", ptr(sl.s2_off), N, ptr(sl.ray2), sl.rows_cap, st)
        _abi.call("vx_serve_features", self.table, len(self.scenes), ctypes.byref(self.cfg), ptr(o), ptr(d), ptr(v),
                  ptr(sl.ray_scene), self.max_steps, ptr(sl.rec), ptr(sl.s2_off), ptr(sl.ray2), sl.rows_cap,
                  ptr(sl.s2_off[N:]), self.ld1, self.ld2, ptr(sl.X1), ptr(sl.X2), int(self.bf16), self.staging, st)

    def _front(self, batch) -> "_Tick":
        """Rays, march and the row scan of one tick on the front stream."""
        batch = sorted(batch, key=lambda t: t[0].scene)   # rows grouped by scene
        t = _Tick(self.ticks % 2)
        sl = self.slots[t.slot]
        fs = self.front_stream
        if sl.ev_back is not None:
            fs.wait_event(sl.ev_back)   # the slot's previous tick is composited
        st = fs.cuda_stream
        chunks = (_abi.ViewChunk * len(batch))()
        ray0 = 0
        bounds, scene_ids = [0], []
        for i, (r, pix0, n) in enumerate(batch):
            c = chunks[i]
            for q in range(12):
                c.c2w[q] = float(r.c2w.reshape(-1)[q])
            c.fx, c.fy, c.cx, c.cy = r.fx, r.fy, r.cx, r.cy
            c.W = r.W
            c.inverse_y = int(r.inverse_y)
            c.scene = r.scene
            c.pix0, c.ray0, c.out0 = pix0, ray0, r.off + pix0
            ray0 += n
            if scene_ids and scene_ids[-1] == r.scene:
                bounds[-1] = ray0
            else:
                scene_ids.append(r.scene)
                bounds.append(ray0)
        t.N, t.scene_ids, t.bounds = ray0, scene_ids, bounds
        N = ray0
        nbytes = ctypes.sizeof(chunks)
        with torch.cuda.stream(fs):
            sl.chunk_ready.synchronize()   # the slot's pinned staging is free again
            ctypes.memmove(sl.chunk_host.data_ptr(), ctypes.addressof(chunks), nbytes)
            sl.chunk_dev[:nbytes].copy_(sl.chunk_host[:nbytes], non_blocking=True)
            nb = len(bounds)
            sl.idx_host[:nb].copy_(torch.tensor(bounds, dtype=torch.int64))
            sl.idx_dev[:nb].copy_(sl.idx_host[:nb], non_blocking=True)
            sl.chunk_ready.record(fs)
            o, d, v = sl.rays[0], sl.rays[1], sl.rays[2]
            tab, ns = self.table, len(self.scenes)
            _abi.call("vx_serve_rays", ptr(sl.chunk_dev), len(batch), N, ptr(o), ptr(d), ptr(v),
                      ptr(sl.ray_scene), ptr(sl.ray_out), st)
            _abi.call("vx_serve_march", tab, ns, ptr(o), ptr(d), ptr(v), ptr(sl.ray_scene), N, self.max_steps,
                      ptr(sl.rec), ptr(sl.n2), ptr(sl.alast), st)
            _abi.call("vx_exclusive_scan_i32", ptr(sl.n2), N, ptr(sl.s2_off), ptr(sl.scan_tmp), self.scan_bytes,
                      st)
            sl.bounds_host[:nb].copy_(sl.s2_off.index_select(0, sl.idx_dev[:nb]), non_blocking=True)
            t.ev_bounds = torch.cuda.Event()
            t.ev_bounds.record(fs)
            self._rows_and_features(t, st)
            t.ev_front = torch.cuda.Event()
            t.ev_front.record(fs)
        return t

    def _row_bounds(self, t: "_Tick") -> None:
        t.ev_bounds.synchronize()
        t.row_bounds = self.slots[t.slot].bounds_host[:len(t.bounds)].tolist()
        t.S2 = t.row_bounds[-1]
        self.rows_shaded += t.S2
        sl = self.slots[t.slot]
        if t.S2 > sl.rows_cap:
            # more shaded rows than the slot holds: grow it and redo the
            # tick's rows and features (the skipped rows were not written)
            fs = self.front_stream
            fs.synchronize()
            self._grow_slot_rows(sl, t.S2 + t.S2 // 4)
            with torch.cuda.stream(fs):
                self._rows_and_features(t, fs.cuda_stream)
                t.ev_front = torch.cuda.Event()
                t.ev_front.record(fs)

    def _back(self, t: "_Tick") -> None:
        """Rows, features, MLPs and compositing of a tick on the back stream,
        then the copies of the requests it finished."""
        sl = self.slots[t.slot]
        bs = self.back_stream
        st = bs.cuda_stream
        with torch.cuda.stream(bs):
            bs.wait_event(t.ev_front)
            S2, N = t.S2, t.N
            tab, ns = self.table, len(self.scenes)
            if S2 > self.rows_cap:
                self._grow_rows(S2)
            if S2 > 0:
                with torch.no_grad():
                    for g, sc in enumerate(t.scene_ids):
                        a, b = t.row_bounds[g], t.row_bounds[g + 1]
                        if b > a:
                            self._shade(self.scenes[sc], sl, a, b, st)
            use_k = self.scenes[0].use_rgb_k
            _abi.call("vx_serve_composite", tab, ns, ptr(sl.ray_scene), N, self.max_steps, ptr(sl.rec),
                      ptr(sl.s2_off), ptr(self.logit), ptr(self.klogit) if use_k else None, ptr(sl.alast),
                      ptr(sl.ray_out), ptr(self.out_rgb), ptr(self.out_depth), st)
            sl.ev_back = torch.cuda.Event()
            sl.ev_back.record(bs)
            for r in t.finished:
                a, b = r.off, r.off + r.n_pix
                self.host_rgb[a:b].copy_(self.out_rgb[a:b], non_blocking=True)
                self.host_depth[a:b].copy_(self.out_depth[a:b], non_blocking=True)
                r.event = torch.cuda.Event()
                r.event.record(bs)
                self.finishing.append(r)

    def _shade(self, s: ResidentScene, sl: _TickSlot, a: int, b: int, st: int) -> None:
        X1, X2 = sl.X1, sl.X2
        if s.tc is not None and self.mlp == "tc":
            # rgbnet -> logits (also into the k_rgbnet input's last columns), then
            # k_rgbnet with the logits as residual, each one fused tcgen05 launch
            s.tc[0].forward(X1[a:b], self.logit[a:b], cols=X2[a:b, self.d2a:], ld_cols=self.ld2)
            s.tc[1].forward(X2[a:b], self.klogit[a:b], add=self.logit[a:b])
            return
        cols = X2[a:b, self.d2a:self.d2a + 3] if s.k_res else None
        s.engines[0].forward(X1[a:b], out=self.logit[a:b], train=False, cols=cols)
        if s.use_rgb_k:
            kout, _ = s.engines[1].forward(X2[a:b], train=False)
            torch.add(self.logit[a:b], kout, out=self.klogit[a:b])


def plain_render(model, c2w, H: int, W: int, focal: float | None = None, chunk: int = 8192,
                 render_kwargs: dict | None = None):
    """A view rendered the reference's way (run.py:81-126): camera rays,
    then Voxurf.forward(global_step=None) over 8192-ray chunks, one request
    at a time.  Returns (rgb [H,W,3], depth [H,W]) as device tensors."""
    from .configs import FINE_RENDER_KWARGS

    rk = dict(FINE_RENDER_KWARGS if render_kwargs is None else render_kwargs)
    rk["render_depth"] = True
    dev = model.sdf.grid.device
    f = 1.2 * W if focal is None else float(focal)
    o = torch.empty((H * W, 3), dtype=torch.float32, device=dev)
    d = torch.empty_like(o)
    v = torch.empty_like(o)
    m = (ctypes.c_float * 12)(*np.asarray(c2w, np.float32)[:3, :4].reshape(-1))
    _abi.call("vx_camera_rays", m, f, f, W / 2.0, H / 2.0, H, W, int(rk.get("inverse_y", True)), ptr(o), ptr(d),
              ptr(v), stream_ptr(dev))
    rgb, depth = [], []
    with torch.no_grad():
        for i in range(0, H * W, chunk):
            ret = model(o[i:i + chunk], d[i:i + chunk], v[i:i + chunk], global_step=None, **rk)
            rgb.append(ret["rgb_marched"])
            depth.append(ret["depth"])
    return torch.cat(rgb).reshape(H, W, 3), torch.cat(depth).reshape(H, W)


RESOLUTIONS = [(120, 160), (300, 400), (600, 800), (1200, 1600)]  # (H, W)


def request_stream(n: int, rate: float, n_scenes: int, seed: int = 0, resolutions=RESOLUTIONS):
    """n requests: Poisson arrivals at `rate` per second (rate = inf: all at
    t = 0), a uniform scene, a random pose on the radius-3 sphere and a
    resolution uniform over `resolutions`.  Returns [(t, scene, c2w, H, W)]."""
    rng = np.random.default_rng(seed)
    t = np.zeros(n) if math.isinf(rate) else np.cumsum(rng.exponential(1.0 / rate, size=n))
    out = []
    for i in range(n):
        H, W = resolutions[int(rng.integers(len(resolutions)))]
        out.append((float(t[i]), int(rng.integers(n_scenes)), random_pose(rng), H, W))
    return out


def run_stream(server: RenderServer, stream) -> dict:
    """Feeds a request stream to the server in real time (each request is
    submitted at its arrival time) and runs ticks until all are done.
    Latency = arrival -> result in host memory."""
    t0 = time.perf_counter()
    reqs = []
    i, n = 0, len(stream)
    while i < n or not server.idle():
        now = time.perf_counter() - t0
        while i < n and stream[i][0] <= now:
            t, s, c2w, H, W = stream[i]
            reqs.append(server.submit(s, c2w, H, W, arrival=t0 + t))
            i += 1
        if server.has_work():
            server.tick()
        else:
            server.poll()
            if server.idle() and i < n:
                time.sleep(max(0.0, stream[i][0] - (time.perf_counter() - t0)))
    t_end = max(r.t_done for r in reqs)
    return summarize(reqs, t_end - t0)


def summarize(reqs, wall: float) -> dict:
    lat = np.array([r.latency for r in reqs]) * 1000.0
    px = sum(r.n_pix for r in reqs)
    out = {"requests": len(reqs), "pixels": int(px), "wall_s": wall, "mpix_s": px / wall / 1e6,
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}
    for H, W in sorted({(r.H, r.W) for r in reqs}):
        sel = np.array([r.latency for r in reqs if (r.H, r.W) == (H, W)]) * 1000.0
        out[f"p50_ms_{W}x{H}"] = float(np.percentile(sel, 50))
        out[f"p99_ms_{W}x{H}"] = float(np.percentile(sel, 99))
    return out


def random_pose(rng: np.random.Generator, radius: float = 3.0) -> np.ndarray:
    """Camera on a sphere of the given radius looking at the origin (OpenCV)."""
    z = rng.uniform(-1.0, 1.0)
    phi = rng.uniform(0.0, 2.0 * math.pi)
    r = math.sqrt(max(0.0, 1.0 - z * z))
    pos = radius * np.array([r * math.cos(phi), r * math.sin(phi), z])
    fwd = -pos / np.linalg.norm(pos)
    up = np.array([0.0, 0.0, 1.0]) if abs(fwd[2]) < 0.99 else np.array([0.0, 1.0, 0.0])
    right = np.cross(fwd, up)
    right /= np.linalg.norm(right)
    down = np.cross(fwd, right)
    c2w = np.eye(4)
    c2w[:3, 0], c2w[:3, 1], c2w[:3, 2], c2w[:3, 3] = right, down, fwd, pos
    return c2w
