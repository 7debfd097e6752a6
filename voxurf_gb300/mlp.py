"""Colour-MLP forward/backward for rgbnet / k_rgbnet (lib/voxurf_fine.py:
132-187, applied at :718-752) and the coarse rgbnet (lib/voxurf_coarse.py:
116-123): Linear -> ReLU stacks applied to the feature rows written by the
feature kernels, then a 3-wide output layer.

Two native engines, both hand-written sm_103a kernels:
* BF16 rows (the mixed-precision path): TcTrainMLP, the tcgen05 tensor-core
  kernels of mlp_train.cu (BF16 operands, FP32 accumulation);
* FP32 rows (the plain path): F32TrainMLP, FP32 CUDA-core kernels
  (mlp_f32.cu) for the hidden layers and the fused output-layer kernels of
  mlp_ops.cu (vx_mlp_head, vx_mlp_head_backward).
Parameters stay FP32 masters (the reference's nn.Linear parameters, same
names and shapes); each forward refreshes the engine's operand copies of
them with one pack launch, and the backward returns FP32 gradients.
"""
from __future__ import annotations

import weakref

import torch
import torch.nn as nn

from ._torch import call, ptr, stream_ptr


def _round_up(x: int, m: int) -> int:
    return (x + m - 1) // m * m


def _pad_width(n: int) -> int:
    """Column counts of the FP32 kernels' tiles."""
    for p in (32, 64, 80, 128, 192):
        if n <= p:
            return p
    raise ValueError(f"MLP layer width {n} above 192")


def row_stride(d_in: int, dtype: torch.dtype) -> int:
    """Row stride of MLP input rows of d_in features for the engine of dtype
    (zero columns beyond d_in): a multiple of 16 elements for the tensor-core
    engine (its MMA K step), of 4 for the FP32 engine (16-byte rows)."""
    return _round_up(d_in, 16 if dtype == torch.bfloat16 else 4)


class _TrainMLP(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, eng, cols, *params):
        train = any(ctx.needs_input_grad)
        eng.pack()
        logits, st = eng.forward(x, train=train, cols=cols)
        ctx.eng, ctx.st = eng, st
        ctx.x_dtype = x.dtype
        return logits

    @staticmethod
    def backward(ctx, dy):
        dX, grads = ctx.eng.backward(ctx.st, dy.float().contiguous(), dx_dtype=ctx.x_dtype)
        ctx.st = None
        return (dX if ctx.needs_input_grad[0] else None, None, None, *grads)


# engines per module, kept beside the module (a deep copy of the module,
# e.g. an FP64 copy for checking, must not carry the engine's buffers along)
_ENGINES: "weakref.WeakKeyDictionary[nn.Module, dict]" = weakref.WeakKeyDictionary()


def engine_for(net: nn.Sequential, dtype: torch.dtype, ld: int):
    """The engine of `net` for input rows of `dtype` with row stride `ld`
    (cached per module; its operand buffers follow the parameters)."""
    cache = _ENGINES.setdefault(net, {})
    key = (dtype, ld)
    eng = cache.get(key)
    lin = _linears(net)
    if eng is None or eng.lin[0].weight.data_ptr() != lin[0].weight.data_ptr():
        eng = TcTrainMLP(net, ld) if dtype == torch.bfloat16 else F32TrainMLP(net)
        cache[key] = eng
    return eng


def apply_mlp(net: nn.Sequential, x: torch.Tensor, cols: torch.Tensor | None = None) -> torch.Tensor:
    """net(x) -> FP32 logits [S, 3] with the hand-written backward.  x: rows
    [S, ld] FP32 or BF16 (the compute dtype), ld = row_stride(in_features,
    dtype) or more, zero beyond in_features (pad columns are never written
    back).  cols: optional [S, >=3] view (row stride given by the tensor) that
    also receives the logits in x's dtype (the k-branch input columns)."""
    lin = _linears(net)
    d_in = lin[0].in_features
    ld = x.shape[1]
    if x.stride(1) != 1 or ld < d_in:
        raise ValueError("MLP rows must be row-contiguous with at least in_features columns")
    if x.dtype == torch.bfloat16 and ld % 16:
        ld = _round_up(ld, 16)
        x = torch.nn.functional.pad(x, (0, ld - x.shape[1]))
    eng = engine_for(net, x.dtype, ld)
    return _TrainMLP.apply(x, eng, cols, *net.parameters())


def mlp_params(net: nn.Sequential) -> list[torch.Tensor]:
    """W1, b1, ..., Wn, bn of a Linear/ReLU stack (reference layout)."""
    return list(net.parameters())


def last_relu_masks(net: nn.Sequential) -> list[torch.Tensor] | None:
    """ReLU decisions (post-ReLU activation > 0) of each hidden layer in the
    last training forward of `net` through the FP32 engine, [S, W] bool each
    (rows in the order of the MLP input), or None."""
    for eng in _ENGINES.get(net, {}).values():
        if isinstance(eng, F32TrainMLP) and eng.last_hs is not None:
            return [h > 0 for h in eng.last_hs]
    return None


class F32TrainMLP:
    """Plain-FP32 engine: the hidden layers as FP32 CUDA-core GEMMs with
    fused epilogues (vx_mlp_f32_rowgemm: +bias and ReLU forward; ReLU mask and
    bias-gradient column sums backward), their weight gradients summed over
    rows per CTA (vx_mlp_f32_wgrad) and in a fixed order (vx_mlp_f32_reduce),
    the 3-wide output layer in vx_mlp_head / vx_mlp_head_backward."""

    def __init__(self, net: nn.Sequential):
        from . import _abi

        lin = _linears(net)
        W = lin[0].out_features
        if not (len(lin) >= 2 and lin[-1].out_features == 3 and W % 4 == 0 and W <= 192
                and all(m.in_features == W and m.out_features == W for m in lin[1:-1])
                and lin[-1].in_features == W and lin[0].in_features <= 192):
            raise ValueError("FP32 MLP engine: Linear(K<=192, W), (L-1) x Linear(W, W), Linear(W, 3), W <= 192")
        for m in lin:
            if not (m.weight.is_contiguous() and m.bias.is_contiguous() and m.weight.dtype == torch.float32):
                raise ValueError("MLP parameters must be contiguous FP32")
        self.lin, self.W, self.L, self.d_in = lin, W, len(lin) - 1, lin[0].in_features
        self.Wp = _pad_width(W)
        if self.Wp != W:
            raise ValueError("FP32 MLP engine: hidden width must be 32, 64, 80, 128 or 192")
        dev = lin[0].weight.device
        self.device = dev
        J = _abi.MlpPackJob
        self.Bf, self.Bb, jobs = [], [], []
        for l in range(self.L):
            k_in = lin[l].in_features
            bf = torch.empty((_round_up(k_in, 16), W), dtype=torch.float32, device=dev)       # Bt[k][n] = W_l[n][k]
            bb = torch.empty((W, _pad_width(k_in)), dtype=torch.float32, device=dev)          # Bt[k][n] = W_l[k][n]
            jobs.append(J(lin[l].weight.data_ptr(), k_in, W, k_in, W, bf.shape[0], 1, 3, bf.data_ptr()))
            jobs.append(J(lin[l].weight.data_ptr(), k_in, k_in, W, bb.shape[1], W, 0, 3, bb.data_ptr()))
            self.Bf.append(bf)
            self.Bb.append(bb)
        self.jobs = (J * len(jobs))(*jobs)
        self.last_hs = None

    def pack(self, stream: int | None = None) -> None:
        from . import _abi

        _abi.call("vx_mlp_train_pack", self.jobs, len(self.jobs), stream_ptr(self.device) if stream is None else stream)

    def grad_buffers(self) -> list[torch.Tensor]:
        out = []
        for m in self.lin:
            out += [torch.empty_like(m.weight), torch.empty_like(m.bias)]
        return out

    def _rowgemm(self, mode, A, K, Bt, Np, C, n_store, bias=None, H=None, colsum=None, n_rows_dev=None):
        from . import _abi

        g = _abi.MlpF32RowGemmArgs()
        g.M, g.m_dev, g.K, g.A, g.lda = A.shape[0], ptr(n_rows_dev), K, ptr(A), A.stride(0)
        g.Bt, g.Np, g.mode = ptr(Bt), Np, mode
        g.bias, g.H, g.ldh = ptr(bias), ptr(H), 0 if H is None else H.stride(0)
        g.C, g.ldc, g.n_store = ptr(C), C.stride(0), n_store
        g.colsum, g.colsum_cap = ptr(colsum), 0 if colsum is None else colsum.numel()
        _abi.call_struct("vx_mlp_f32_rowgemm", g, stream_ptr(A.device))

    def forward(self, X: torch.Tensor, out: torch.Tensor | None = None, train: bool = True,
                cols: torch.Tensor | None = None, n_rows_dev: torch.Tensor | None = None,
                saved: dict | None = None):
        if X.dtype != torch.float32 or X.stride(1) != 1 or X.shape[1] < self.d_in:
            raise ValueError("rows must be FP32 with >= in_features columns")
        n, dev, W = X.shape[0], X.device, self.W
        if out is None:
            out = torch.empty((n, 3), dtype=torch.float32, device=dev)
        st = saved if saved is not None else {}
        if "hs" not in st:
            st["hs"] = [torch.empty((n, W), dtype=torch.float32, device=dev) for _ in range(self.L)]
        h, k = X, self.d_in
        for l in range(self.L):
            self._rowgemm(0, h, k, self.Bf[l], W, st["hs"][l], W, bias=self.lin[l].bias, n_rows_dev=n_rows_dev)
            h, k = st["hs"][l], W
        lh = self.lin[-1]
        cols_ptr, ld_cols, cols_bf16 = None, 0, 0
        if cols is not None:
            cols_ptr, ld_cols, cols_bf16 = ptr(cols), cols.stride(0), int(cols.dtype == torch.bfloat16)
        call("vx_mlp_head", ptr(h), n, W, W, 0, lh.weight.data_ptr(), lh.bias.data_ptr(), None, ptr(out), cols_ptr,
             ld_cols, cols_bf16, stream_ptr(dev))
        st.update(n=n, X=X, n_rows_dev=n_rows_dev)
        self.last_hs = st["hs"] if train else None
        return out, (st if train else None)

    def backward(self, st: dict, dY: torch.Tensor, dx_dtype=torch.float32, grads: list | None = None,
                 dX: torch.Tensor | None = None, work: dict | None = None):
        from . import _abi, _native

        lib = _native.load()
        _abi._declare()
        n, X, hs = st["n"], st["X"], st["hs"]
        W, L, dev = self.W, self.L, dY.device
        stp = stream_ptr(dev)
        nrd = st["n_rows_dev"]
        if grads is None:
            grads = self.grad_buffers()
        w = work if work is not None else {}
        g_rows = int(lib.vx_mlp_f32_rowgemm_grid(n))
        g_wg = int(lib.vx_mlp_f32_wgrad_grid(n))
        Np0 = _pad_width(self.d_in)
        if "dz" not in w:
            w["dz"] = [torch.empty((n, W), dtype=torch.float32, device=dev) for _ in range(2)]
            w["part"] = [torch.empty(g_wg * W * W, dtype=torch.float32, device=dev) for _ in range(L - 1)]
            w["part0"] = torch.empty(g_wg * W * Np0, dtype=torch.float32, device=dev)
            w["colsum"] = [torch.empty(g_rows * W, dtype=torch.float32, device=dev) for _ in range(L - 1)]
        if dX is None:
            dX = torch.empty((n, X.shape[1]), dtype=torch.float32, device=dev)
        # the output-layer kernel accumulates dWh, dbh and db_{L-1}
        dWh, dbh, dbL = grads[2 * L], grads[2 * L + 1], grads[2 * (L - 1) + 1]
        for t in (dWh, dbh, dbL):
            t.zero_()
        lh = self.lin[-1]
        dz = w["dz"][0]
        call("vx_mlp_head_backward", ptr(dY), ptr(hs[-1]), lh.weight.data_ptr(), n, W, 0, ptr(dz), ptr(dWh),
             ptr(dbh), ptr(dbL), stp)
        sums = []
        S = _abi.MlpSumJob

        def wgrad(A, B, N, part):
            g = _abi.MlpF32WgradArgs()
            g.rows, g.rows_dev, g.A, g.lda, g.B, g.ldb = n, ptr(nrd), ptr(A), A.stride(0), ptr(B), B.stride(0)
            g.M, g.N, g.part, g.part_cap = W, N, ptr(part), part.numel()
            _abi.call_struct("vx_mlp_f32_wgrad", g, stp)

        for l in range(L - 1, 0, -1):        # dW_l = dz_{l+1}^T h_l; dz_l = (dz_{l+1} W_l) * [h_l > 0]
            wgrad(dz, hs[l - 1], W, w["part"][l - 1])
            sums.append(S(w["part"][l - 1].data_ptr(), g_wg, W * W, W, W, W, grads[2 * l].data_ptr(), W))
            nxt = w["dz"][(L - l) % 2]
            self._rowgemm(1, dz, W, self.Bb[l], W, nxt, W, H=hs[l - 1], colsum=w["colsum"][l - 1], n_rows_dev=nrd)
            sums.append(S(w["colsum"][l - 1].data_ptr(), g_rows, W, W, 1, W, grads[2 * (l - 1) + 1].data_ptr(), W))
            dz = nxt
        wgrad(dz, X, self.d_in, w["part0"])  # dW_0 = dz_1^T X
        sums.append(S(w["part0"].data_ptr(), g_wg, W * Np0, Np0, W, self.d_in, grads[0].data_ptr(), self.d_in))
        self._rowgemm(2, dz, W, self.Bb[0], Np0, dX, self.d_in, n_rows_dev=nrd)   # dX = dz_1 W_0
        arr = (S * len(sums))(*sums)
        _abi.call("vx_mlp_f32_reduce", arr, len(sums), stp)
        return dX, grads


class TensorCoreMLP:
    """A rgbnet / k_rgbnet stack (Linear(K,192), ReLU, 2 x [Linear(192,192),
    ReLU], Linear(192,3)) packed for the fused tcgen05 forward
    (vx_mlp_tc_forward): hidden weights BF16 in the operand layout, first
    layer K zero-padded to K0 (multiple of 16), biases rounded to BF16 like
    the GEMM path, the FP32 output layer as BF16 hi + lo rows of a 16-wide
    tensor-core tile.  Inference only (no autograd)."""

    WIDTH = 192
    pipeline = 1   # two 128-row tiles in flight per CTA (vx_mlp_tc_args.pipeline)

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
                cols: torch.Tensor | None = None, ld_cols: int = 0, pipeline: int | None = None) -> None:
        """out[i] = MLP(X[i, :K0]) (+ add[i]); X [n, ldx] BF16 rows, out [n,3] FP32.
        pipeline: tiles in flight per CTA minus one (0 or 1; default
        self.pipeline); both give the same results."""
        from . import _abi

        a = _abi.MlpTcArgs()
        a.pipeline = self.pipeline if pipeline is None else int(pipeline)
        a.X, a.ldx, a.K0, a.n_rows, a.width = ptr(X), X.stride(0), self.K0, X.shape[0], self.WIDTH
        a.W0p, a.W1p, a.W2p = (ptr(t) for t in self.packed)
        a.b0, a.b1, a.b2 = (ptr(t) for t in self.biases)
        a.Whp, a.bh, a.add, a.out = ptr(self.Whp), ptr(self.bh), ptr(add), ptr(out)
        a.cols, a.ld_cols = ptr(cols), ld_cols
        _abi.call_struct("vx_mlp_tc_forward", a, stream_ptr(X.device))


def _linears(net: nn.Sequential) -> list:
    return [m for m in net.modules() if isinstance(m, nn.Linear)]


class TcTrainMLP:
    """A Linear/ReLU colour MLP (hidden width 32/64/128/192, 2 or 3 hidden
    layers, 3 outputs) trained on the tensor cores: BF16 operands, FP32
    accumulation, FP32 master weights and FP32 gradients (vx_mlp_train_*).

    K0 is the padded first-layer width (a multiple of 16 >= the Linear's
    in_features); input rows must have at least K0 columns, zero beyond
    in_features.  pack() refreshes the BF16 operands from the FP32 masters
    (one launch); forward() keeps the hidden activations (T-tiles) and ReLU
    bits for backward(); backward() returns the input gradient and writes the
    FP32 gradients of every weight and bias.
    """

    @staticmethod
    def supports(net: nn.Sequential, K0: int) -> bool:
        lin = _linears(net)
        if len(lin) not in (3, 4):
            return False
        W = lin[0].out_features
        return (W in (32, 64, 128, 192) and all(m.out_features == W and m.in_features == W for m in lin[1:-1])
                and lin[-1].out_features == 3 and lin[-1].in_features == W and lin[0].in_features <= K0 <= 80
                and K0 % 16 == 0)

    def __init__(self, net: nn.Sequential, K0: int):
        if not self.supports(net, K0):
            raise ValueError("tensor-core training MLP: Linear(K<=80, W), (1 or 2) x Linear(W, W), Linear(W, 3) "
                             "with W in 32/64/128/192")
        from . import _abi

        lin = _linears(net)
        self.lin = lin
        self.W = W = lin[0].out_features
        self.L = L = len(lin) - 1
        self.d_in = lin[0].in_features
        self.K0 = K0
        dev = lin[0].weight.device
        self.device = dev
        bf, f32 = torch.bfloat16, torch.float32
        self.W0p = torch.empty(K0 * W, dtype=bf, device=dev)
        self.Wp = torch.empty(max(L - 1, 1) * W * W, dtype=bf, device=dev)
        self.bias = torch.empty(L * W, dtype=f32, device=dev)
        self.Whp = torch.empty(16 * W, dtype=bf, device=dev)
        self.W0Tp = torch.empty(W * K0, dtype=bf, device=dev)
        self.WTp = torch.empty(max(L - 1, 1) * W * W, dtype=bf, device=dev)
        J = _abi.MlpPackJob

        def job(src, ld, N, K, Np, Kp, transpose, mode, dst):
            return J(src.data_ptr(), ld, N, K, Np, Kp, transpose, mode, dst)

        w0 = lin[0].weight
        jobs = [job(w0, self.d_in, W, self.d_in, W, K0, 0, 0, self.W0p.data_ptr()),
                job(w0, self.d_in, self.d_in, W, K0, W, 1, 0, self.W0Tp.data_ptr()),
                job(lin[L].weight, W, 3, W, 16, W, 0, 1, self.Whp.data_ptr())]
        for l in range(1, L):
            off = (l - 1) * W * W * 2
            jobs.append(job(lin[l].weight, W, W, W, W, W, 0, 0, self.Wp.data_ptr() + off))
            jobs.append(job(lin[l].weight, W, W, W, W, W, 1, 0, self.WTp.data_ptr() + off))
        for l in range(L):
            jobs.append(job(lin[l].bias, W, 1, W, 1, W, 0, 2, self.bias.data_ptr() + l * W * 4))
        for m in lin:
            if not (m.weight.is_contiguous() and m.bias.is_contiguous() and m.weight.dtype == f32):
                raise ValueError("MLP parameters must be contiguous FP32")
        self.jobs = (J * len(jobs))(*jobs)

    def pack(self, stream: int | None = None) -> None:
        from . import _abi

        _abi.call("vx_mlp_train_pack", self.jobs, len(self.jobs), stream_ptr(self.device) if stream is None else stream)

    @staticmethod
    def pack_many(mlps, stream: int | None = None) -> None:
        """One launch for the operands of several MLPs (up to 32 jobs)."""
        from . import _abi

        jobs = [j for m in mlps for j in m.jobs]
        arr = (_abi.MlpPackJob * len(jobs))(*jobs)
        _abi.call("vx_mlp_train_pack", arr, len(jobs), stream_ptr(mlps[0].device) if stream is None else stream)

    def grad_buffers(self) -> list[torch.Tensor]:
        """FP32 gradient buffers in parameter order [W0, b0, ..., Wh, bh]."""
        out = []
        for m in self.lin:
            out += [torch.empty_like(m.weight), torch.empty_like(m.bias)]
        return out

    def forward(self, X: torch.Tensor, out: torch.Tensor | None = None, train: bool = True,
                cols: torch.Tensor | None = None, n_rows_dev: torch.Tensor | None = None,
                saved: dict | None = None) -> tuple[torch.Tensor, dict | None]:
        """logits [n, 3] FP32 of X [n, >= K0] BF16 rows.  train: also returns
        the state backward() needs (hidden T-tiles, ReLU bits); `saved` may
        pass preallocated ones (graph capture).  cols: optional BF16 view
        [n, >= 3] that also receives the logits."""
        from . import _abi

        n = X.shape[0]
        if X.dtype != torch.bfloat16 or X.shape[1] < self.K0 or X.stride(1) != 1:
            raise ValueError("rows must be BF16 with >= K0 columns")
        cap = (n + 127) // 128 * 128
        dev = X.device
        if out is None:
            out = torch.empty((n, 3), dtype=torch.float32, device=dev)
        st = None
        if train:
            st = saved if saved is not None else {}
            if "H" not in st:
                st["H"] = torch.empty(self.L * cap * self.W, dtype=torch.bfloat16, device=dev)
                st["relu"] = torch.empty(self.L * cap * (self.W // 16), dtype=torch.int16, device=dev)
            st["cap"], st["n"], st["X"], st["n_rows_dev"] = cap, n, X, n_rows_dev
        a = _abi.MlpTrainFwdArgs()
        a.n_rows, a.n_rows_dev, a.rows_cap = n, ptr(n_rows_dev), cap
        a.width, a.n_hidden, a.K0 = self.W, self.L, self.K0
        a.X, a.ldx = ptr(X), X.stride(0)
        a.W0p, a.Wp, a.bias, a.Whp = ptr(self.W0p), ptr(self.Wp), ptr(self.bias), ptr(self.Whp)
        a.bh, a.out = self.lin[-1].bias.data_ptr(), ptr(out)
        if cols is not None and cols.dtype != torch.bfloat16:
            raise ValueError("cols must be BF16 for BF16 rows")
        a.cols, a.ld_cols = ptr(cols), (cols.stride(0) if cols is not None else 0)
        if train:
            a.H, a.relu = ptr(st["H"]), ptr(st["relu"])
        _abi.call_struct("vx_mlp_train_forward", a, stream_ptr(dev))
        return out, st

    def backward(self, st: dict, dY: torch.Tensor, dx_dtype=torch.bfloat16, grads: list | None = None,
                 dX: torch.Tensor | None = None, work: dict | None = None) -> tuple[torch.Tensor, list]:
        """dX [n, K0] (dx_dtype) and the FP32 gradients [dW0, db0, ..., dWh, dbh]
        (written into `grads` when given).  `work` may pass preallocated
        scratch (graph capture)."""
        dX, grads, pending = self.backward_chain(st, dY, dx_dtype, grads, dX, work)
        TcTrainMLP.weight_gradients([pending], stream_ptr(dY.device))
        return dX, grads

    def backward_chain(self, st: dict, dY: torch.Tensor, dx_dtype=torch.bfloat16, grads: list | None = None,
                       dX: torch.Tensor | None = None, work: dict | None = None):
        """The input-gradient chain alone: dX and the dz T-tiles of every
        layer.  Returns (dX, grads, pending); the weight gradients are
        written into grads by weight_gradients([pending, ...]), which runs
        the weight-gradient passes of several MLPs in one launch."""
        from . import _abi, _native

        lib = _native.load()
        _abi._declare()
        n, cap, X = st["n"], st["cap"], st["X"]
        W, L, K0 = self.W, self.L, self.K0
        dev = dY.device
        stp = stream_ptr(dev)
        if dY.dtype != torch.float32 or not dY.is_contiguous() or dY.shape[0] != n:
            raise ValueError("dY must be contiguous FP32 [n, 3]")
        grid = int(lib.vx_mlp_wgrad_grid(n))
        w = work if work is not None else {}
        if "dZ" not in w:
            w["dZ"] = torch.empty(L * cap * W, dtype=torch.bfloat16, device=dev)
            w["dYT"] = torch.empty(cap * 16, dtype=torch.bfloat16, device=dev)
            w["dbh"] = torch.empty(grid * 4, dtype=torch.float32, device=dev)
            w["part"] = [torch.empty(grid * W * (W + 16), dtype=torch.float32, device=dev) for _ in range(L - 1)]
            w["part0"] = torch.empty(grid * W * (K0 + 16), dtype=torch.float32, device=dev)
            w["parth"] = torch.empty(grid * W * 16, dtype=torch.float32, device=dev)
        if dX is None:
            dX = torch.empty((n, K0), dtype=dx_dtype, device=dev)
        if grads is None:
            grads = self.grad_buffers()
        b = _abi.MlpTrainBwdArgs()
        b.n_rows, b.n_rows_dev, b.rows_cap = n, ptr(st["n_rows_dev"]), cap
        b.width, b.n_hidden, b.K0 = W, L, K0
        b.dY, b.Wh, b.relu = ptr(dY), self.lin[-1].weight.data_ptr(), ptr(st["relu"])
        b.WTp, b.W0Tp, b.dZ, b.dYT = ptr(self.WTp), ptr(self.W0Tp), ptr(w["dZ"]), ptr(w["dYT"])
        b.dX, b.ld_dx, b.dx_bf16 = ptr(dX), dX.stride(0), int(dX.dtype == torch.bfloat16)
        b.dbh_part, b.dbh_part_cap = ptr(w["dbh"]), grid
        _abi.call_struct("vx_mlp_train_backward", b, stp)
        H, dZ = st["H"].data_ptr(), w["dZ"].data_ptr()
        lay = cap * W * 2   # bytes per layer of T-tiles
        R = _abi.MlpReduceJob
        pending = []   # (pass arguments, reduce job of its n_part partials)

        def wgrad(A, WA, B, WB, ldb, b_rows, ones, part, job):
            g = _abi.MlpWgradArgs()
            g.n_rows, g.n_rows_dev, g.A, g.WA, g.B, g.WB, g.ldb = n, ptr(st["n_rows_dev"]), A, WA, B, WB, ldb
            g.b_rows, g.ones, g.part, g.part_cap = b_rows, ones, ptr(part), part.numel()
            pending.append((g, job))

        for l in range(1, L):   # dW_l = dz_{l+1}^T h_l
            pl = w["part"][l - 1]
            wgrad(dZ + l * lay, W, H + (l - 1) * lay, W, 0, 0, 1, pl,
                  lambda k, pl=pl, l=l: R(pl.data_ptr(), k, W, W + 16, 0, 0, W, W, grads[2 * l].data_ptr(),
                                          grads[2 * l + 1].data_ptr(), None, 0))
        wgrad(dZ, W, X.data_ptr(), K0, X.stride(0), 1, 1, w["part0"],      # dW_0 = dz_1^T X
              lambda k: R(w["part0"].data_ptr(), k, W, K0 + 16, 0, 0, K0, self.d_in, grads[0].data_ptr(),
                          grads[1].data_ptr(), None, 0))
        wgrad(H + (L - 1) * lay, W, w["dYT"].data_ptr(), 16, 0, 0, 0, w["parth"],   # dWh = dy^T h_L
              lambda k: R(w["parth"].data_ptr(), k, W, 16, 1, 0, 16, 3, grads[2 * L].data_ptr(),
                          grads[2 * L + 1].data_ptr(), w["dbh"].data_ptr(), grid))
        return dX, grads, pending

    @staticmethod
    def weight_gradients(pendings: list, stream: int) -> None:
        """Every weight-gradient pass of the given backward_chain results in
        one launch per 8 passes (the SMs split over the passes in proportion
        to their bytes), then their ordered sums in one launch per 8."""
        import ctypes

        from . import _abi, _native

        lib = _native.load()
        _abi._declare()
        items = [it for p in pendings for it in p]
        for i in range(0, len(items), 8):
            grp = items[i:i + 8]
            k = len(grp)
            arr = (_abi.MlpWgradArgs * k)(*[g for g, _ in grp])
            ctas = (ctypes.c_int32 * k)()
            _native.check(lib.vx_mlp_wgrad_split(arr, k, ctas), "vx_mlp_wgrad_split")
            _native.check(lib.vx_mlp_train_wgrad_multi(arr, ctas, k, stream), "vx_mlp_train_wgrad_multi")
            jobs = [mk(int(ctas[j])) for j, (_, mk) in enumerate(grp)]
            _abi.call("vx_mlp_train_reduce", (_abi.MlpReduceJob * k)(*jobs), k, stream)

