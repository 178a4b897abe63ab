"""Tensor-core BF16 GEMM and the closure MLP over the libbbdg C ABI (bb_gemm_bf16, bb_mlp_*).

No counterpart in the reference (BernsteinBasis.jl has no learned part). Every call runs the
library's own kernels: the tcgen05 GEMM (TMA-fed shared-memory ring, TMEM accumulator, fused
bias / GELU / GELU' / transpose / column-sum epilogue), the loss, Adam and transpose kernels.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .context import get_context, ptr, require_cuda, stream_handle


def _ctx_of(t: torch.Tensor):
    return get_context(t.device)


def gemm_bf16(A: torch.Tensor, B: torch.Tensor, *, alpha: float = 1.0, bias=None, act: int = 0,
              pre=None, out_f32=None, out_bf16=None, out_t=None, bias_grad=None, kt_per: int = 0,
              stream=None):
    """C = alpha A B^T (A [M, K], B [N, K], BF16) with the fused epilogue of bb_gemm_bf16.

    Outputs are caller tensors (out_f32 [M, N] float32, out_bf16 [M, N] bfloat16, out_t [N, M]
    bfloat16, bias_grad [N] float32, pre [M, N] float32); returns out_f32. kt_per > 0 splits
    K into chunks of kt_per x 64 whose partial products are added into out_f32 (zero it first;
    no other output allowed)."""
    require_cuda(A, B)
    if A.dtype != torch.bfloat16 or B.dtype != torch.bfloat16:
        raise TypeError("operands must be bfloat16")
    M, K = A.shape
    N, K2 = B.shape
    if K != K2:
        raise ValueError("A and B must share K")
    for t in (bias, pre, out_f32, out_bf16, out_t, bias_grad):
        if t is not None:
            require_cuda(t)
    ldc = N
    ldt = M
    ctx = _ctx_of(A)
    ctx.check(_lib.load().bb_gemm_bf16(
        ctx.handle, M, N, K, ptr(A), ptr(B), float(alpha), ptr(bias), int(act), ptr(pre),
        ptr(out_f32), ptr(out_bf16), ptr(out_t), ptr(bias_grad), ldc, ldt, int(kt_per),
        stream_handle(stream)), "bb_gemm_bf16")
    return out_f32


def device_status(device=None, stream=None) -> int:
    ctx = get_context(device)
    out = ctypes.c_int()
    ctx.check(_lib.load().bb_device_status(ctx.handle, stream_handle(stream), ctypes.byref(out)),
              "bb_device_status")
    return out.value


def transpose_bf16(X: torch.Tensor, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    require_cuda(X)
    rows, cols = X.shape
    out = torch.empty((cols, rows), dtype=torch.bfloat16, device=X.device) if out is None else out
    ctx = _ctx_of(X)
    ctx.check(_lib.load().bb_transpose_bf16(ctx.handle, rows, cols, ptr(X), ptr(out),
                                            stream_handle(stream)), "bb_transpose_bf16")
    return out


class MLP:
    """bb_mlp: nin -> h1 -> h2 -> nout, GELU, BF16 weights, FP32 master copy and Adam."""

    def __init__(self, dims=(840, 512, 512, 336), max_batch: int = 24576, seed: int = 0,
                 device=None):
        self.dims = tuple(int(d) for d in dims)
        self.max_batch = int(max_batch)
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        self.ctx = get_context(self.device)
        h = ctypes.c_void_p()
        self.ctx.check(_lib.load().bb_mlp_create(self.ctx.handle, *self.dims, self.max_batch,
                                                 int(seed), ctypes.byref(h)), "bb_mlp_create")
        self.handle = h
        self.num_params = int(_lib.load().bb_mlp_num_params(h))
        self._loss = torch.zeros(1, dtype=torch.float64, device=self.device)

    def params(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        self.ctx.check(_lib.load().bb_mlp_get_params(
            self.handle, out.ctypes.data_as(ctypes.c_void_p), stream_handle()), "get_params")
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.num_params:
            raise ValueError(f"expected {self.num_params} parameters")
        self.ctx.check(_lib.load().bb_mlp_set_params(
            self.handle, p.ctypes.data_as(ctypes.c_void_p), stream_handle()), "set_params")

    def grads(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        self.ctx.check(_lib.load().bb_mlp_get_grads(
            self.handle, out.ctypes.data_as(ctypes.c_void_p), stream_handle()), "get_grads")
        return out

    def forward(self, X: torch.Tensor, XT: torch.Tensor | None = None, train: bool = False,
                out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        require_cuda(X)
        B = X.shape[0]
        Y = torch.empty((B, self.dims[3]), dtype=torch.float32, device=X.device) \
            if out is None else out
        self.ctx.check(_lib.load().bb_mlp_fwd(self.handle, B, ptr(X), ptr(XT), ptr(Y),
                                              int(bool(train)), stream_handle(stream)),
                       "bb_mlp_fwd")
        return Y

    def backward(self, Y: torch.Tensor, T: torch.Tensor, stream=None) -> torch.Tensor:
        """Stores the gradients; returns the loss as a one-element device tensor."""
        require_cuda(Y, T)
        self.ctx.check(_lib.load().bb_mlp_bwd(self.handle, Y.shape[0], ptr(Y), ptr(T),
                                              ptr(self._loss), stream_handle(stream)),
                       "bb_mlp_bwd")
        return self._loss

    def step(self, lr: float = 1e-3, betas=(0.9, 0.999), eps: float = 1e-8, stream=None):
        self.ctx.check(_lib.load().bb_mlp_step(self.handle, float(lr), float(betas[0]),
                                               float(betas[1]), float(eps),
                                               stream_handle(stream)), "bb_mlp_step")

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.load().bb_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def closure_features(N: int, nf: int, conn: torch.Tensor, q: torch.Tensor, scale: float,
                     X: torch.Tensor | None = None, XT: torch.Tensor | None = None,
                     transpose: bool = False, stream=None):
    """BF16 features [K, nf Np + 4 nf Nfp] of every element of q [nf, K, Np] (and X^T)."""
    from .ordering import np2, np3
    require_cuda(conn, q)
    K = q.shape[1]
    nin = nf * np3(N) + 4 * nf * np2(N)
    if X is None:
        X = torch.empty((K, nin), dtype=torch.bfloat16, device=q.device)
    if transpose and XT is None:
        XT = torch.empty((nin, K), dtype=torch.bfloat16, device=q.device)
    ctx = _ctx_of(q)
    dt = _lib.BB_F64 if q.dtype == torch.float64 else _lib.BB_F32
    ctx.check(_lib.load().bb_closure_features(ctx.handle, N, K, nf, ptr(conn), dt, ptr(q),
                                              float(scale), ptr(X),
                                              ptr(XT if transpose else None),
                                              stream_handle(stream)), "bb_closure_features")
    return X, XT


def closure_apply(N: int, nf: int, alpha: float, Y: torch.Tensor, q: torch.Tensor, stream=None):
    """q[f, e, p] += alpha * Y[e, f Np + p]."""
    require_cuda(Y, q)
    ctx = _ctx_of(q)
    dt = _lib.BB_F64 if q.dtype == torch.float64 else _lib.BB_F32
    ctx.check(_lib.load().bb_closure_apply(ctx.handle, N, q.shape[1], nf, dt, float(alpha),
                                           ptr(Y), ptr(q), stream_handle(stream)),
              "bb_closure_apply")
