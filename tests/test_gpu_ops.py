"""GPU parity of the reference-element operators (through the C ABI) vs the CPU oracle.

Tolerances (relative l2 over each output): FP64 1e-12, FP32 1e-5.
"""
import ctypes
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-12, "f32": 1e-5}
DEGREES = [1, 2, 3, 4, 5, 7, 9, 10, 12, 15]


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def torch_dtype(name):
    import torch
    return torch.float64 if name == "f64" else torch.float32


@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("N", DEGREES)
def test_derivative_matches_oracle(cuda, bb, oracle_cpu, N, dt):
    import torch
    rng = np.random.default_rng(N)
    K, Np = 37, bb.np3(N)
    x = rng.uniform(-1, 1, (K, Np))
    xd = torch.tensor(x, dtype=torch_dtype(dt), device=cuda)
    outs = [torch.empty_like(xd) for _ in range(3)]
    for axis, D in enumerate((bb.BernsteinDerivativeMatrix_3D_r(N), bb.BernsteinDerivativeMatrix_3D_s(N),
                              bb.BernsteinDerivativeMatrix_3D_t(N))):
        bb.mul_(outs[axis], D, xd)
        want = oracle_cpu.deriv(axis, N, x)
        assert rel(outs[axis].cpu().numpy(), want) < TOL[dt], (N, axis)
    g = [torch.empty_like(xd) for _ in range(3)]
    bb.grad_(g[0], g[1], g[2], N, xd)
    for a in range(3):
        assert torch.equal(g[a], outs[a])


@pytest.mark.parametrize("K", [29, 1000])
@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("N", range(1, 21))
def test_lift_matches_oracle(cuda, bb, oracle_cpu, N, dt, K):
    """FP32 degrees 1..15 run the degree-specialised register-chain kernels, FP64 and FP32
    16..20 the level-parallel one; K = 29 leaves a ragged last tile, K = 1000 spans many
    tiles."""
    import torch
    rng = np.random.default_rng(50 + N)
    Np, Nfp = bb.np3(N), bb.np2(N)
    x = rng.uniform(-1, 1, (K, 4 * Nfp))
    xd = torch.tensor(x, dtype=torch_dtype(dt), device=cuda)
    out = torch.empty((K, Np), dtype=xd.dtype, device=cuda)
    bb.mul_(out, bb.BernsteinLift(N), xd)
    assert rel(out.cpu().numpy(), oracle_cpu.lift(N, x)) < TOL[dt]
    # single face (face_lift_multiply!)
    xf = torch.tensor(x[:, :Nfp].copy(), dtype=xd.dtype, device=cuda)
    of = torch.empty((K, Np), dtype=xd.dtype, device=cuda)
    bb.face_lift_multiply_(of, bb.BernsteinLift(N), xf)
    want = np.stack([oracle_cpu.face_lift(N, x[e, :Nfp]) for e in range(K)])
    assert rel(of.cpu().numpy(), want) < TOL[dt]


@pytest.mark.parametrize("N", range(1, 16))
def test_deriv_fp32_many_tiles_and_misaligned(cuda, bb, oracle_cpu, N):
    """About 12 M inputs give more tiles than the grid of the degree-specialised FP32
    derivative kernel has blocks at every degree (each degree has its own block shape and
    tile), so blocks alternate between their two shared buffers; K is odd, so for odd Np the
    last tile is ragged and its inputs end inside a float4. A sample of columns is checked
    against the oracle for each axis, the fused gradient equals the single-axis results
    bitwise, and misaligned columns (the generic kernel) agree."""
    import torch
    rng = np.random.default_rng(110 + N)
    Np = bb.np3(N)
    K = max(20011, (12_000_000 // Np) | 1)
    x = rng.uniform(-1, 1, (K, Np)).astype(np.float32)
    xd = torch.tensor(x, device=cuda)
    cols = np.r_[0:30, K // 2:K // 2 + 30, K - 30:K]
    outs = []
    for axis, D in enumerate((bb.BernsteinDerivativeMatrix_3D_r, bb.BernsteinDerivativeMatrix_3D_s,
                              bb.BernsteinDerivativeMatrix_3D_t)):
        o = torch.empty_like(xd)
        bb.mul_(o, D(N), xd)
        outs.append(o)
        want = oracle_cpu.deriv(axis, N, x[cols].astype(np.float64))
        assert rel(o.cpu().numpy()[cols], want) < TOL["f32"], axis
    g = [torch.empty_like(xd) for _ in range(3)]
    bb.grad_(g[0], g[1], g[2], N, xd)
    for a in range(3):
        assert torch.equal(g[a], outs[a])
    Km = 257
    xb = torch.tensor(np.concatenate([[0.0], x[:Km].ravel()]).astype(np.float32), device=cuda)
    xm = xb[1:].view(Km, Np)
    assert xm.data_ptr() % 16 != 0
    om = torch.empty((Km, Np), dtype=torch.float32, device=cuda)
    bb.mul_(om, bb.BernsteinDerivativeMatrix_3D_s(N), xm)
    assert rel(om.cpu().numpy(), outs[1][:Km].cpu().numpy()) < TOL["f32"]


@pytest.mark.parametrize("N", [3, 9, 10, 11, 12, 13, 15])
def test_lift_fp32_many_tiles_and_misaligned(cuda, bb, oracle_cpu, N):
    """K = 20011 gives more tiles (8, 4 or 2 elements) than the grid has blocks, so every
    block works through several tiles (the register-prefetch path for N <= 9, the bulk-copy
    path above) and ends on a ragged one; a sample of columns is checked against the oracle.
    Inputs and outputs that are not 16-byte aligned take the generic kernel and agree with
    it."""
    import torch
    rng = np.random.default_rng(90 + N)
    K = 20011
    Np, Nfp = bb.np3(N), bb.np2(N)
    x = rng.uniform(-1, 1, (K, 4 * Nfp)).astype(np.float32)
    xd = torch.tensor(x, device=cuda)
    out = torch.empty((K, Np), dtype=torch.float32, device=cuda)
    bb.mul_(out, bb.BernsteinLift(N), xd)
    cols = np.r_[0:40, K // 2:K // 2 + 40, K - 40:K]
    want = oracle_cpu.lift(N, x[cols].astype(np.float64))
    assert rel(out.cpu().numpy()[cols], want) < TOL["f32"]
    # misaligned views (offset by one float) run the generic kernel
    Km = 300
    xb = torch.tensor(np.concatenate([[0.0], x[:Km].ravel()]).astype(np.float32), device=cuda)
    ob = torch.empty(Km * Np + 1, dtype=torch.float32, device=cuda)
    xm, om = xb[1:].view(Km, 4 * Nfp), ob[1:].view(Km, Np)
    assert xm.data_ptr() % 16 != 0
    bb.mul_(om, bb.BernsteinLift(N), xm)
    assert rel(om.cpu().numpy(), out[:Km].cpu().numpy()) < TOL["f32"]


@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("N", [1, 2, 5, 9, 14, 19])
def test_elevation_reduction_match_oracle(cuda, bb, oracle_cpu, N, dt):
    import torch
    rng = np.random.default_rng(70 + N)
    K = 11
    x = rng.uniform(-1, 1, (K, bb.np2(N)))
    xd = torch.tensor(x, dtype=torch_dtype(dt), device=cuda)
    up = torch.empty((K, bb.np2(N + 1)), dtype=xd.dtype, device=cuda)
    dn = torch.empty((K, bb.np2(N - 1)), dtype=xd.dtype, device=cuda)
    bb.elevation_multiply_(up, N, xd)
    bb.reduction_multiply_(dn, N, xd)
    assert rel(up.cpu().numpy(), np.stack([oracle_cpu.elevation(N, r) for r in x])) < TOL[dt]
    assert rel(dn.cpu().numpy(), np.stack([oracle_cpu.reduction(N, r) for r in x])) < TOL[dt]


@pytest.mark.parametrize("N", [3, 9])
def test_fused_operator_pass(cuda, bb, N):
    import torch
    rng = np.random.default_rng(90 + N)
    K = 23
    x = torch.tensor(rng.uniform(-1, 1, (K, bb.np3(N))), device=cuda)
    f = torch.tensor(rng.uniform(-1, 1, (K, 4 * bb.np2(N))), device=cuda)
    dr, ds, dt_, li = (torch.empty_like(x) for _ in range(4))
    bb.fused_apply_(dr, ds, dt_, li, N, x, f)
    ref = [torch.empty_like(x) for _ in range(4)]
    bb.grad_(ref[0], ref[1], ref[2], N, x)
    bb.mul_(ref[3], bb.BernsteinLift(N), f)
    # the separate derivative calls use the factored form (w at degree N-1), the fused pass
    # the reference's per-row form: equal up to rounding; the lift is the same kernel
    for a, b in zip((dr, ds, dt_), ref[:3]):
        assert rel(a.cpu().numpy(), b.cpu().numpy()) < 1e-14
    assert torch.equal(li, ref[3])


@pytest.mark.parametrize("N", [3, 9, 12, 15])
def test_fused_operator_pass_fp32(cuda, bb, oracle_cpu, N):
    """FP32 (N <= 15): the fused pass is the gradient and lift calls back to back and equals
    them bitwise; it matches the oracle at 1e-5."""
    import torch
    rng = np.random.default_rng(95 + N)
    K = 301
    xh = rng.uniform(-1, 1, (K, bb.np3(N)))
    fh = rng.uniform(-1, 1, (K, 4 * bb.np2(N)))
    x = torch.tensor(xh, dtype=torch.float32, device=cuda)
    f = torch.tensor(fh, dtype=torch.float32, device=cuda)
    dr, ds, dt_, li = (torch.empty_like(x) for _ in range(4))
    bb.fused_apply_(dr, ds, dt_, li, N, x, f)
    ref = [torch.empty_like(x) for _ in range(4)]
    bb.grad_(ref[0], ref[1], ref[2], N, x)
    bb.mul_(ref[3], bb.BernsteinLift(N), f)
    for a, b in zip((dr, ds, dt_, li), ref):
        assert torch.equal(a, b)
    for axis, a in enumerate((dr, ds, dt_)):
        assert rel(a.cpu().numpy(), oracle_cpu.deriv(axis, N, xh)) < TOL["f32"]
    assert rel(li.cpu().numpy(), oracle_cpu.lift(N, fh)) < TOL["f32"]


def _golden():
    path = os.path.join(os.path.dirname(__file__), "golden", "operators_exact.json")
    with open(path) as fh:
        return json.load(fh)["cases"]


@pytest.mark.parametrize("case", _golden(), ids=lambda c: f"{c['op']}-N{c['N']}")
def test_gpu_matches_exact_golden(cuda, bb, case):
    import torch
    N = case["N"]
    x = torch.tensor(case["x"]["float"], dtype=torch.float64, device=cuda)
    y = np.array(case["y"]["float"])
    out = torch.empty(len(y), dtype=torch.float64, device=cuda)
    op = case["op"]
    if op[0] == "D":
        D = getattr(bb, f"BernsteinDerivativeMatrix_3D_{op[1]}")(N)
        bb.mul_(out, D, x)
    elif op == "elevation":
        bb.elevation_multiply_(out, N, x)
    elif op == "reduction":
        bb.reduction_multiply_(out, N, x)
    elif op == "face_lift":
        bb.face_lift_multiply_(out, bb.BernsteinLift(N), x)
    else:
        bb.mul_(out, bb.BernsteinLift(N), x)
    assert rel(out.cpu().numpy(), y) < 1e-13


def test_bad_arguments_return_status(cuda, bb):
    import torch
    from bbdg import _lib
    from bbdg.context import get_context
    L = _lib.load()
    ctx = get_context(0)
    x = torch.zeros(20, dtype=torch.float64, device=cuda)
    p = ctypes.c_void_p(x.data_ptr())
    assert L.bb_deriv_apply(ctx.handle, 0, 0, 1, 1, p, p, None) == _lib.BB_ERR_ARG
    assert L.bb_deriv_apply(ctx.handle, 0, 21, 1, 1, p, p, None) == _lib.BB_ERR_ARG
    assert L.bb_deriv_apply(ctx.handle, 3, 3, 1, 1, p, p, None) == _lib.BB_ERR_ARG
    assert L.bb_deriv_apply(ctx.handle, 0, 3, 1, 7, p, p, None) == _lib.BB_ERR_ARG
    assert L.bb_lift_apply(ctx.handle, 3, 1, 1, None, p, None) == _lib.BB_ERR_ARG
    with pytest.raises(ValueError):
        bb.mul_(torch.empty(20, device=cuda, dtype=torch.float64), bb.BernsteinDerivativeMatrix_3D_r(3),
                torch.empty(21, device=cuda, dtype=torch.float64))
    with pytest.raises(ValueError):
        bb.mul_(torch.empty(20, dtype=torch.float64), bb.BernsteinDerivativeMatrix_3D_r(3),
                torch.empty(20, dtype=torch.float64))
