"""Reference-element operator types with the reference's ``mul!`` API, on the GPU.

Mirrors the exports of src/BernsteinBasis.jl:19-23:
  BernsteinDerivativeMatrix_3D_r/_s/_t   (src/BernsteinDerivativeMatrix_3D.jl:9-44)
  BernsteinLift                          (src/BernsteinLift.jl:12-27)
  ElevationMatrix                        (src/ElevationMatrix.jl:11-24)
  mul_(out, op, x)                       LinearAlgebra.mul! (:134,:176,:218,:222-231 and
                                         src/BernsteinLift.jl:191-220,264-269)
plus the helpers the reference tests call: elevation_multiply_, reduction_multiply_,
face_lift_multiply_.

Operands are CUDA tensors. A row-major (K, Np) tensor has exactly the memory layout of
Julia's column-major Np x K matrix (one column per element); a 1-D tensor is one element.
Every operation runs in the CUDA library; there is no CPU path.
"""
from __future__ import annotations

import torch

from . import _lib
from .context import dtype_code, get_context, ptr, require_cuda, stream_handle
from .ordering import MAX_N, np2, np3, tri_offsets, tet_offsets


def _check_degree(N: int) -> int:
    N = int(N)
    if not 1 <= N <= MAX_N:
        raise ValueError(f"degree N={N} is outside 1..{MAX_N}")
    return N


class _Derivative:
    axis = 0

    def __init__(self, N: int):
        self.N = _check_degree(N)
        self.tri_offsets = tri_offsets(self.N)
        self.tet_offsets = tet_offsets(self.N)

    @property
    def shape(self):
        n = np3(self.N)
        return (n, n)

    def __repr__(self):
        return f"{type(self).__name__}({self.N})"


class BernsteinDerivativeMatrix_3D_r(_Derivative):
    """d/dr in the degree-N Bernstein basis (<= 7 nonzeros per row)."""
    axis = 0


class BernsteinDerivativeMatrix_3D_s(_Derivative):
    """d/ds in the degree-N Bernstein basis."""
    axis = 1


class BernsteinDerivativeMatrix_3D_t(_Derivative):
    """d/dt in the degree-N Bernstein basis."""
    axis = 2


class BernsteinLift:
    """Bernstein lift [L1 | L2 | L3 | L4] of degree N (4*Nfp face values -> Np).

    Unlike the reference struct (src/BernsteinLift.jl:12-20) it holds no scratch vectors:
    the kernels keep their intermediates in on-chip memory, so an instance is reentrant.
    """

    def __init__(self, N: int, dtype: torch.dtype | None = None):
        self.N = _check_degree(N)
        self.dtype = dtype

    @property
    def shape(self):
        return (np3(self.N), 4 * np2(self.N))

    def __repr__(self):
        return f"BernsteinLift({self.N})"


class ElevationMatrix:
    """2D degree elevation N-1 -> N (ElevationMatrix.jl); apply with mul_."""

    def __init__(self, N: int):
        self.N = _check_degree(N)

    @property
    def shape(self):
        return (np2(self.N), np2(self.N - 1))


def _columns(x: torch.Tensor, rows: int, name: str) -> int:
    if x.dim() == 1:
        if x.shape[0] != rows:
            raise ValueError(f"{name} has {x.shape[0]} entries, expected {rows}")
        return 1
    if x.dim() == 2:
        if x.shape[1] != rows:
            raise ValueError(f"{name} must be (K, {rows}), got {tuple(x.shape)}")
        return x.shape[0]
    raise ValueError(f"{name} must be 1-D or 2-D")


def _prep(out, x):
    require_cuda(out, x)
    if out.dtype != x.dtype:
        raise TypeError("out and x must share a dtype")
    if out.device != x.device:
        raise ValueError("out and x must be on the same device")
    return get_context(x.device), dtype_code(x.dtype)


def mul_(out: torch.Tensor, op, x: torch.Tensor, stream=None) -> torch.Tensor:
    """out = op * x, like LinearAlgebra.mul!(out, op, x); returns out."""
    if isinstance(op, _Derivative):
        n = np3(op.N)
        K = _columns(x, n, "x")
        if _columns(out, n, "out") != K:
            raise ValueError("out and x must have the same number of columns")
        ctx, dt = _prep(out, x)
        if out.data_ptr() == x.data_ptr():
            raise ValueError("out must not alias x")
        ctx.check(_lib.load().bb_deriv_apply(ctx.handle, op.axis, op.N, K, dt, ptr(x), ptr(out),
                                             stream_handle(stream)), "bb_deriv_apply")
        return out
    if isinstance(op, BernsteinLift):
        K = _columns(x, 4 * np2(op.N), "x")
        if _columns(out, np3(op.N), "out") != K:
            raise ValueError("out and x must have the same number of columns")
        ctx, dt = _prep(out, x)
        ctx.check(_lib.load().bb_lift_apply(ctx.handle, op.N, K, dt, ptr(x), ptr(out),
                                            stream_handle(stream)), "bb_lift_apply")
        return out
    if isinstance(op, ElevationMatrix):
        return elevation_multiply_(out, op.N - 1, x, stream=stream)
    raise TypeError(f"unsupported operator {type(op).__name__}")


def elevation_multiply_(out, N: int, x, stream=None):
    """elevation_multiply! (src/BernsteinLift.jl:100-125): degree N -> N+1 per column."""
    if not 0 <= N < MAX_N:
        raise ValueError("degree out of range")
    K = _columns(x, np2(N), "x")
    if _columns(out, np2(N + 1), "out") != K:
        raise ValueError("column mismatch")
    ctx, dt = _prep(out, x)
    if N == 0:
        # degree 0 -> 1 is the constant copied to all three coefficients
        out.view(K, 3).copy_(x.view(K, 1).expand(K, 3))
        return out
    ctx.check(_lib.load().bb_elevation_apply(ctx.handle, N, K, dt, ptr(x), ptr(out),
                                             stream_handle(stream)), "bb_elevation_apply")
    return out


def reduction_multiply_(out, N: int, x, stream=None):
    """reduction_multiply! (src/BernsteinLift.jl:66-90): degree N -> N-1 per column."""
    N = _check_degree(N)
    K = _columns(x, np2(N), "x")
    if _columns(out, np2(N - 1), "out") != K:
        raise ValueError("column mismatch")
    ctx, dt = _prep(out, x)
    ctx.check(_lib.load().bb_reduction_apply(ctx.handle, N, K, dt, ptr(x), ptr(out),
                                             stream_handle(stream)), "bb_reduction_apply")
    return out


def face_lift_multiply_(out, L: BernsteinLift, x, stream=None):
    """face_lift_multiply! (src/BernsteinLift.jl:139-164): one face, Nfp -> Np per column."""
    K = _columns(x, np2(L.N), "x")
    if _columns(out, np3(L.N), "out") != K:
        raise ValueError("column mismatch")
    ctx, dt = _prep(out, x)
    ctx.check(_lib.load().bb_face_lift_apply(ctx.handle, L.N, K, dt, ptr(x), ptr(out),
                                             stream_handle(stream)), "bb_face_lift_apply")
    return out


def grad_(dr, ds, dt_, N: int, x, stream=None):
    """Dr x, Ds x, Dt x from one read of x."""
    N = _check_degree(N)
    K = _columns(x, np3(N), "x")
    for o in (dr, ds, dt_):
        if _columns(o, np3(N), "out") != K:
            raise ValueError("column mismatch")
    require_cuda(dr, ds, dt_)
    ctx, code = _prep(dr, x)
    ctx.check(_lib.load().bb_grad_apply(ctx.handle, N, K, code, ptr(x), ptr(dr), ptr(ds),
                                        ptr(dt_), stream_handle(stream)), "bb_grad_apply")
    return dr, ds, dt_


def fused_apply_(dr, ds, dt_, lift_out, N: int, x, faces, stream=None):
    """Dr x, Ds x, Dt x and L faces in one launch."""
    N = _check_degree(N)
    K = _columns(x, np3(N), "x")
    if _columns(faces, 4 * np2(N), "faces") != K:
        raise ValueError("column mismatch")
    require_cuda(dr, ds, dt_, lift_out, faces)
    ctx, code = _prep(dr, x)
    ctx.check(_lib.load().bb_fused_apply(ctx.handle, N, K, code, ptr(x), ptr(faces), ptr(dr),
                                         ptr(ds), ptr(dt_), ptr(lift_out),
                                         stream_handle(stream)), "bb_fused_apply")
    return dr, ds, dt_, lift_out
