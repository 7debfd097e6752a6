"""Colour-MLP forward/backward for rgbnet / k_rgbnet (lib/voxurf_fine.py:
132-187, lib/voxurf_coarse.py:116-123): Linear -> ReLU stacks applied to the
feature rows written by the feature kernels.

The GEMMs are cuBLAS calls (FP32, or BF16 with FP32 accumulation); the
hidden layers use cuBLASLt's bias+ReLU epilogue (torch._addmm_activation);
the backward fuses ReLU-backward with the bias gradient in one sm_103a pass
(vx_relu_bwd_colsum) instead of torch's threshold_backward plus a strided
column reduction.  Parameters stay FP32 masters; in BF16 mode they are cast
per call and the weight gradients are returned in FP32.
"""
from __future__ import annotations

import os

import torch
import torch.nn as nn

from ._torch import call, ptr, stream_ptr

# FP32 backward GEMMs: "native" = cuBLAS SGEMM through the library's own
# handle (vx_gemm_f32; 20% faster training steps than torch.matmul's choice
# of kernels for these shapes), "emulated" = the same call in cuBLAS's BF16x9
# FP32 emulation on the tensor cores (another 5%; meets the FP32 parity
# bars), "torch" = torch.matmul.
FP32_GEMM = os.environ.get("VX_FP32_GEMM", "native")


def _gemm_f32(dz: torch.Tensor, other: torch.Tensor, wgrad: bool) -> torch.Tensor:
    """Row-major FP32 products of the MLP backward through vx_gemm_f32:
    wgrad: dz^T @ h ([N_out, K_in]); else dz @ W ([S, K_in])."""
    emulate = int(FP32_GEMM == "emulated")
    S, n_out = dz.shape
    dev = dz.device
    if wgrad:
        h = other
        k_in = h.shape[1]
        out = torch.empty((n_out, k_in), dtype=torch.float32, device=dev)
        # column-major: out^T (k_in x n_out) = h^T (k_in x S) . dz (S x n_out)
        call("vx_gemm_f32", 0, 1, k_in, n_out, S, 1.0, ptr(h), k_in, ptr(dz), n_out, 0.0, ptr(out), k_in, emulate,
             None, 0, stream_ptr(dev))
    else:
        W = other
        k_in = W.shape[1]
        out = torch.empty((S, k_in), dtype=torch.float32, device=dev)
        # column-major: out^T (k_in x S) = W^T (k_in x n_out) . dz^T (n_out x S)
        call("vx_gemm_f32", 0, 0, k_in, S, n_out, 1.0, ptr(W), k_in, ptr(dz), n_out, 0.0, ptr(out), k_in, emulate,
             None, 0, stream_ptr(dev))
    return out


def _colsum(dh: torch.Tensor, h: torch.Tensor | None, dz: torch.Tensor | None,
            out: torch.Tensor | None = None) -> torch.Tensor:
    M, N = dh.shape
    if out is None:
        out = torch.zeros(N, dtype=torch.float32, device=dh.device)
    dtype = 1 if dh.dtype == torch.bfloat16 else 0
    call("vx_relu_bwd_colsum", ptr(dh), ptr(h), M, N, dtype, ptr(dz), ptr(out), stream_ptr())
    return out


def _head_layer(Ws, hs_last) -> bool:
    """The last layer is a colour head (3 outputs from a ReLU layer of at
    most 256 columns in 16-byte row chunks) that the fused head kernels take."""
    W = Ws[-1]
    N = W.shape[1]
    per = 8 if hs_last.dtype == torch.bfloat16 else 4
    return (len(Ws) >= 2 and W.shape[0] == 3 and N <= 256 and N % per == 0 and hs_last.is_contiguous()
            and hs_last.data_ptr() % 16 == 0)


def mlp_forward(x: torch.Tensor, Ws, bs) -> list[torch.Tensor]:
    """Linear/ReLU stack on rows x (weights already in x's dtype): returns
    the activations [x, h1, ..., logits].  A 3-output last layer runs in
    vx_mlp_head (FP32 accumulation and FP32 logits) instead of a GEMM with a
    3-wide dimension."""
    n = len(Ws)
    hs = [x]
    h = x
    for i in range(n):
        if i < n - 1:
            h = torch._addmm_activation(bs[i], h, Ws[i].t())
        elif _head_layer(Ws, h):
            M, N = h.shape
            out = torch.empty((M, 3), dtype=torch.float32, device=h.device)
            W, b = Ws[i].float().contiguous(), bs[i].float().contiguous()
            call("vx_mlp_head", ptr(h), M, N, N, int(h.dtype == torch.bfloat16), ptr(W), ptr(b), None, ptr(out),
                 None, 0, 0, stream_ptr(h.device))
            h = out
        else:
            h = torch.addmm(bs[i], h, Ws[i].t())
        hs.append(h)
    return hs


def mlp_backward(dy: torch.Tensor, hs, Ws, need_dx: bool):
    """Gradients of mlp_forward: (dx or None, [dW1, db1, ..., dWn, dbn]) with
    FP32 weight gradients; ReLU backward and the bias gradient are one pass
    (vx_relu_bwd_colsum); a 3-output head's weight and bias gradients, its
    input gradient and the ReLU backward below it are one pass
    (vx_mlp_head_backward)."""
    n = len(Ws)
    grads = [None] * (2 * n)
    dx = None
    top = n
    head = _head_layer(Ws, hs[n - 1])
    # every accumulator of the pass (head dW, dbh, db; the bias gradients of
    # the layers below) comes from one zero-filled buffer, 16-byte aligned
    sizes = [3 * hs[n - 1].shape[1], 3, hs[n - 1].shape[1]] if head else [dy.shape[1]]
    sizes += [Ws[i].shape[1] for i in reversed(range(1, n - 1 if head else n))]
    offs, total = [], 0
    for sz in sizes:
        offs.append(total)
        total += (sz + 3) // 4 * 4
    acc = torch.zeros(total, dtype=torch.float32, device=dy.device)
    views = iter([acc[o:o + sz] for o, sz in zip(offs, sizes)])
    if head:
        h = hs[n - 1]
        M, N = h.shape
        dev = h.device
        dW = next(views).view(3, N)
        dbh = next(views)
        db = next(views)
        dz = torch.empty_like(h)
        W = Ws[n - 1].float().contiguous()
        dout = dy.float().contiguous()  # kept alive until the kernel is enqueued
        call("vx_mlp_head_backward", ptr(dout), ptr(h), ptr(W), M, N, int(h.dtype == torch.bfloat16), ptr(dz),
             ptr(dW), ptr(dbh), ptr(db), stream_ptr(dev))
        grads[2 * (n - 1)] = dW
        grads[2 * (n - 1) + 1] = dbh
        top = n - 1
    else:
        dz = dy.to(hs[0].dtype).contiguous()
        db = _colsum(dz, None, None, next(views))
    lib_gemm = dz.dtype == torch.float32 and FP32_GEMM != "torch"
    for i in reversed(range(top)):
        if lib_gemm:
            h, W = hs[i].contiguous(), Ws[i].contiguous()
            grads[2 * i] = _gemm_f32(dz, h, True)
        else:
            grads[2 * i] = (dz.t() @ hs[i]).float()
        grads[2 * i + 1] = db
        if i > 0:
            dh = _gemm_f32(dz, W, False) if lib_gemm else dz @ Ws[i]
            dz_prev = torch.empty_like(dh)
            db = _colsum(dh, hs[i], dz_prev, next(views))
            dz = dz_prev
        elif need_dx:
            dx = _gemm_f32(dz, W, False) if lib_gemm else dz @ Ws[0]
    return dx, grads


class _MLP(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, *params):
        n = len(params) // 2
        dt = x.dtype
        Ws = [params[2 * i].detach().to(dt) for i in range(n)]
        bs = [params[2 * i + 1].detach().to(dt) for i in range(n)]
        hs = mlp_forward(x, Ws, bs)
        ctx.save_for_backward(*hs, *Ws)
        ctx.n = n
        return hs[-1]

    @staticmethod
    def backward(ctx, dy):
        n = ctx.n
        saved = ctx.saved_tensors
        hs, Ws = saved[: n + 1], saved[n + 1:]
        dx, grads = mlp_backward(dy, hs, Ws, ctx.needs_input_grad[0])
        return (dx, *grads)


def mlp_params(net: nn.Sequential) -> list[torch.Tensor]:
    """W1, b1, ..., Wn, bn of a Linear/ReLU stack (reference layout)."""
    return list(net.parameters())


def apply_mlp(net: nn.Sequential, x: torch.Tensor) -> torch.Tensor:
    """net(x) with the fused backward; x float32 or bfloat16 (compute dtype)."""
    return _MLP.apply(x.contiguous(), *mlp_params(net))


class TensorCoreMLP:
    """A rgbnet / k_rgbnet stack (Linear(K,192), ReLU, 2 x [Linear(192,192),
    ReLU], Linear(192,3)) packed for the fused tcgen05 forward
    (vx_mlp_tc_forward): hidden weights BF16 in the operand layout, first
    layer K zero-padded to K0 (multiple of 16), biases rounded to BF16 like
    the GEMM path, the FP32 output layer as BF16 hi + lo rows of a 16-wide
    tensor-core tile.  Inference only (no autograd)."""

    WIDTH = 192

    @staticmethod
    def supports(net: nn.Sequential, K0: int) -> bool:
        lin = [m for m in net.modules() if isinstance(m, nn.Linear)]
        return (len(lin) == 4 and all(m.out_features == TensorCoreMLP.WIDTH for m in lin[:3])
                and lin[3].out_features == 3 and lin[0].in_features <= K0 <= 80 and K0 % 16 == 0)

    def __init__(self, net: nn.Sequential, K0: int):
        if not self.supports(net, K0):
            raise ValueError("the fused tensor-core MLP needs Linear(K<=80,192), 2 x Linear(192,192), "
                             "Linear(192,3)")
        lin = [m for m in net.modules() if isinstance(m, nn.Linear)]
        dev = lin[0].weight.device
        st = stream_ptr(dev)
        self.K0 = K0
        self.packed = []
        for i, m in enumerate(lin[:3]):
            Kp = K0 if i == 0 else self.WIDTH
            out = torch.empty((Kp // 8) * self.WIDTH * 8, dtype=torch.bfloat16, device=dev)
            W = m.weight.detach().float().contiguous()
            call("vx_mlp_tc_pack", ptr(W), self.WIDTH, W.shape[1], Kp, ptr(out), st)
            self.packed.append(out)
        self.biases = [m.bias.detach().to(torch.bfloat16).float().contiguous() for m in lin[:3]]
        # output layer on the tensor cores: FP32 weights as BF16 hi + lo parts
        Wh = lin[3].weight.detach().float()
        hi = Wh.to(torch.bfloat16).float()
        lo = (Wh - hi).to(torch.bfloat16).float()
        Wsplit = torch.zeros((16, self.WIDTH), dtype=torch.float32, device=dev)
        Wsplit[0:3] = hi
        Wsplit[3:6] = lo
        self.Whp = torch.empty(16 * self.WIDTH, dtype=torch.bfloat16, device=dev)
        call("vx_mlp_tc_pack", ptr(Wsplit), 16, self.WIDTH, self.WIDTH, ptr(self.Whp), st)
        self._Wsplit = Wsplit  # kept alive until the pack kernel has run
        self.bh = lin[3].bias.detach().float().contiguous()

    def forward(self, X: torch.Tensor, out: torch.Tensor, add: torch.Tensor | None = None,
                cols: torch.Tensor | None = None, ld_cols: int = 0) -> None:
        """out[i] = MLP(X[i, :K0]) (+ add[i]); X [n, ldx] BF16 rows, out [n,3] FP32."""
        from . import _abi

        a = _abi.MlpTcArgs()
        a.X, a.ldx, a.K0, a.n_rows, a.width = ptr(X), X.stride(0), self.K0, X.shape[0], self.WIDTH
        a.W0p, a.W1p, a.W2p = (ptr(t) for t in self.packed)
        a.b0, a.b1, a.b2 = (ptr(t) for t in self.biases)
        a.Whp, a.bh, a.add, a.out = ptr(self.Whp), ptr(self.bh), ptr(add), ptr(out)
        a.cols, a.ld_cols = ptr(cols), ld_cols
        _abi.call_struct("vx_mlp_tc_forward", a, stream_ptr(X.device))
