"""Host-side mirror of the optimizer and checkpoint parts of lib/utils.py
(load_checkpoint / load_model read run.py's checkpoints into these models).

``Adam`` keeps the reference's interface (utils.py:54-151: param groups with
``lr``, ``betas``, ``eps``, per-voxel learning rate through
``set_pervoxel_lr(count)``) and update rule (utils.py:154-199), computed by
one sm_103a kernel per parameter instead of ~6 torch launches.

Extension used by the fused training step: a param group may carry
``tv_weight`` (the weight a caller would pass to
DenseGrid.total_variation_add_grad, already scaled) and ``tv_dense``; for
such 5-D grid parameters the step runs TV add-grad + Adam + gradient reset
in a single sweep (vx_grid_tv_adam_step), reading the old parameter buffer
and writing a second one that is swapped in (ping-pong), and refreshes a
BF16 shadow copy when ``shadow`` (a tensor) is given.  A group may also
carry ``touched``: uint8 marks of the voxels where the gradient can be
nonzero (vx_grid_tv_adam_step_touched reads the gradient only there).
"""
from __future__ import annotations

import ctypes
import math

import torch
import torch.nn as nn

from ._torch import call, ptr, stream_ptr


class Adam(torch.optim.Optimizer):
    def __init__(self, params, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, weight_decay=0, amsgrad=False):
        if not 0.0 <= lr:
            raise ValueError(f"Invalid learning rate: {lr}")
        if not 0.0 <= eps:
            raise ValueError(f"Invalid epsilon value: {eps}")
        if not 0.0 <= betas[0] < 1.0 or not 0.0 <= betas[1] < 1.0:
            raise ValueError(f"Invalid beta parameters: {betas}")
        if weight_decay != 0 or amsgrad:
            raise NotImplementedError("weight_decay/amsgrad are not used by the Voxurf configs")
        defaults = dict(lr=lr, betas=betas, eps=eps, weight_decay=weight_decay, amsgrad=amsgrad)
        self.per_lr = None
        super().__init__(params, defaults)

    def set_pervoxel_lr(self, count):
        """utils.py:78-80."""
        assert self.param_groups[0]["params"][0].shape == count.shape
        self.per_lr = (count.float() / count.max()).contiguous()

    @torch.no_grad()
    def step(self, closure=None, zero_grad: bool = False):
        """One update of every parameter with a gradient.  zero_grad=True
        also drops the gradients afterwards (set_to_none), so the next
        backward writes fresh ones instead of accumulating."""
        loss = None
        if closure is not None:
            with torch.enable_grad():
                loss = closure()
        st = stream_ptr()
        batch = []  # small tensors without per-voxel lr: one multi-tensor launch
        for group in self.param_groups:
            beta1, beta2 = group["betas"]
            for p in group["params"]:
                if p.grad is None:
                    continue
                state = self.state[p]
                if len(state) == 0:
                    state["step"] = 0
                    state["exp_avg"] = torch.zeros_like(p, memory_format=torch.preserve_format)
                    state["exp_avg_sq"] = torch.zeros_like(p, memory_format=torch.preserve_format)
                state["step"] += 1
                g = p.grad
                if g.stride() != p.stride():
                    g = g.contiguous(memory_format=_fmt(p))
                per_lr = self.per_lr if (self.per_lr is not None and p.shape == self.per_lr.shape) else None
                if per_lr is not None and per_lr.stride() != p.stride():
                    per_lr = per_lr.contiguous(memory_format=_fmt(p))
                tv_w = group.get("tv_weight", 0.0)
                if p.dim() == 5 and tv_w:
                    self._grid_step(p, g, state, per_lr, group, tv_w, zero_grad, st)
                elif per_lr is None and group.get("shadow") is None and p.is_contiguous() and g.is_contiguous() \
                        and group["betas"] == self.param_groups[0]["betas"] \
                        and group["eps"] == self.param_groups[0]["eps"]:
                    batch.append((p, g, state, float(group["lr"])))
                    continue
                else:
                    call("vx_adam_step", ptr(p), ptr(g), ptr(state["exp_avg"]), ptr(state["exp_avg_sq"]),
                         ptr(per_lr), p.numel(), float(group["lr"]), float(beta1), float(beta2),
                         float(group["eps"]), int(state["step"]), 0, st)
                    shadow = group.get("shadow")
                    if shadow is not None:
                        shadow.copy_(p.detach())
                if zero_grad:
                    p.grad = None
        if batch:
            b1, b2 = self.param_groups[0]["betas"]
            eps = float(self.param_groups[0]["eps"])
            for i in range(0, len(batch), 48):
                part = batch[i:i + 48]
                n = len(part)
                P = ctypes.c_void_p * n
                call("vx_adam_step_multi", n, P(*[p.data_ptr() for p, _, _, _ in part]),
                     P(*[g.data_ptr() for _, g, _, _ in part]),
                     P(*[s["exp_avg"].data_ptr() for _, _, s, _ in part]),
                     P(*[s["exp_avg_sq"].data_ptr() for _, _, s, _ in part]),
                     (ctypes.c_int64 * n)(*[p.numel() for p, _, _, _ in part]),
                     (ctypes.c_double * n)(*[lr for _, _, _, lr in part]),
                     (ctypes.c_int64 * n)(*[int(s["step"]) for _, _, s, _ in part]),
                     float(b1), float(b2), eps, st)
            if zero_grad:
                for p, _, _, _ in batch:
                    p.grad = None
        return loss

    def _grid_step(self, p, g, state, per_lr, group, tv_w, zero_grad, st):
        beta1, beta2 = group["betas"]
        spare = state.get("spare")
        if spare is None or spare.shape != p.shape:
            spare = torch.empty_like(p, memory_format=torch.preserve_format)
        C, X, Y, Z = p.size(1), p.size(2), p.size(3), p.size(4)
        cl = C > 1 and not p.is_contiguous()
        shadow = group.get("shadow")
        touched = group.get("touched")
        # with a touched map, zero_grad also resets the marked gradient rows in
        # the same sweep (the gradient buffer is then reused by the next
        # step's scatter); without one, the gradient is dropped
        reset = int(bool(zero_grad) and touched is not None)
        args = (ptr(p), ptr(spare), ptr(g), ptr(state["exp_avg"]), ptr(state["exp_avg_sq"]), ptr(per_lr),
                ptr(shadow), C, X, Y, Z, int(cl), 1, float(tv_w), int(bool(group.get("tv_dense", True))),
                float(group["lr"]), float(beta1), float(beta2), float(group["eps"]), int(state["step"]), reset)
        if touched is not None:
            # the gradient is zero outside the marked voxels (the fused step's scatter)
            call("vx_grid_tv_adam_step_touched", *args, ptr(touched), st)
        else:
            call("vx_grid_tv_adam_step", *args, st)
        old = p.data
        p.data = spare
        state["spare"] = old


def _fmt(p):
    return torch.channels_last_3d if (p.dim() == 5 and p.size(1) > 1 and not p.is_contiguous()) else \
        torch.contiguous_format


def create_optimizer_or_freeze_model(model, cfg_train, global_step):
    """utils.py:202-229: one param group per `lrate_<name>` key."""
    decay_steps = cfg_train.lrate_decay * 1000
    decay_factor = 0.1 ** (global_step / decay_steps)
    param_group = []
    for k in cfg_train.keys():
        if not k.startswith("lrate_"):
            continue
        k = k[len("lrate_"):]
        if not hasattr(model, k):
            continue
        param = getattr(model, k)
        if param is None:
            continue
        lr = getattr(cfg_train, f"lrate_{k}") * decay_factor
        if lr > 0:
            if isinstance(param, nn.Module):
                param = param.parameters()
            param_group.append({"params": param, "lr": lr, "name": k})
        else:
            param.requires_grad = False
    return Adam(param_group, betas=(0.9, 0.99))


# ---- checkpoints (utils.py:234-300) -------------------------------------------
def _load_ckpt(ckpt_path):
    # run.py stores numpy arrays in model_kwargs / MaskCache_kwargs
    return torch.load(ckpt_path, map_location="cpu", weights_only=False)


def _load_state(model, state, strict):
    """load_state_dict that keeps the model's storage (channel-last grids,
    device) and, when not strict, skips keys the model does not hold (the
    reference registers `nonempty_mask` as a buffer; here it is recomputed)."""
    own = model.state_dict()
    if strict:
        model.load_state_dict(state, strict=True)
        return
    model.load_state_dict({k: v for k, v in state.items() if k in own and own[k].shape == v.shape}, strict=False)


def load_checkpoint(model, optimizer, ckpt_path, no_reload_optimizer, strict=True):
    """utils.py:234-250: model (and optimizer) state from a run.py checkpoint;
    a narrower rgbnet input layer in the checkpoint is zero-padded."""
    ckpt = _load_ckpt(ckpt_path)
    start = ckpt["global_step"]
    sd = dict(ckpt["model_state_dict"])
    w = sd.get("rgbnet.0.weight")
    if w is not None and model.rgbnet[0].weight.shape != w.shape:
        tmp = torch.zeros(model.rgbnet[0].weight.shape)
        tmp[:, :w.shape[-1]] = w
        sd["rgbnet.0.weight"] = tmp
    model.load_state_dict(sd, strict=strict)
    if not no_reload_optimizer:
        try:
            optimizer.load_state_dict(ckpt["optimizer_state_dict"])
        except Exception:
            if strict:
                raise ValueError("failed to load the optimizer state dict")
    return model, optimizer, start


def load_model(model_class, ckpt_path, new_kwargs=None, strict=False):
    """utils.py:279-300: model_class(**ckpt['model_kwargs'] updated by
    new_kwargs) with the checkpoint's state (a MaskCache named by
    mask_cache_path is loaded from its own checkpoint on construction)."""
    ckpt = _load_ckpt(ckpt_path)
    kwargs = dict(ckpt["model_kwargs"])
    if new_kwargs is not None:
        kwargs.update(new_kwargs)
    model = model_class(**kwargs)
    try:
        _load_state(model, ckpt["model_state_dict"], strict=True)
    except RuntimeError:
        if strict:
            raise
        _load_state(model, ckpt["model_state_dict"], strict=False)
    return model
