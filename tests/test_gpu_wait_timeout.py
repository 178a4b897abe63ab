"""Bounded device-side waits: a wait that runs out is reported and leaves the context usable.

The bulk-copy pipelines of the degree-specialised stage kernel and of the tensor-core GEMM
wait on mbarriers. Every wait gives up after a bounded number of polls (about a second by
default), sets a status bit, lets the kernel's own copies in flight land and returns. Here the
limit is lowered to 2^14 polls (milliseconds) and the test-only fault mode arms one copy's
barrier without issuing the copy, so that one barrier phase never completes: the kernel must
return, the host must see BB_ERR_TIMEOUT (solver) or status bit 1 (GEMM), and the next normal
calls on the same context must give the same results as before. Nothing faults or hangs: the
left-out copy is never issued, so no transfer is in flight when the kernel exits.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 1 << 14


def test_stage_kernel_wait_runs_out_and_the_solver_recovers(cuda, bb):
    import torch
    from bbdg import _lib
    from bbdg.context import get_context
    ctx = get_context(0)
    m = bb.uniform_tet_mesh(8)                     # K = 3072: 768 tiles of 4 elements
    s = bb.DGSolver(m, 9, "wave", dtype=torch.float32, tau=1.0)
    s.set_kernel("specialised")
    s.set_tile(4, 288)
    assert s.kernel == "specialised"
    zero = lambda x, y, z: 0 * x  # noqa: E731
    q0 = s.project([bb.gaussian_pulses(1), zero, zero, zero])
    dt = s.dt_cfl()
    qa, ra = q0.clone(), torch.zeros_like(q0)
    s.run(qa, ra, dt, 2, graph=False)
    s.check()
    try:
        ctx.set_wait_limit(LIMIT)
        ctx.set_test_fault(1)
        qb, rb = q0.clone(), torch.zeros_like(q0)
        t0 = time.perf_counter()
        s.run(qb, rb, dt, 1, graph=False)
        with pytest.raises(_lib.BBError) as err:
            s.check()
        assert err.value.status == _lib.BB_ERR_TIMEOUT
        assert time.perf_counter() - t0 < 30.0
    finally:
        ctx.set_test_fault(0)
        ctx.set_wait_limit(0)
    # the same solver and context, normal mode again, with and without a CUDA graph
    for graph in (False, True):
        qc, rc = q0.clone(), torch.zeros_like(q0)
        s.run(qc, rc, dt, 2, graph=graph)
        s.check()
        assert torch.equal(qc, qa) and torch.equal(rc, ra)
    s.close()


def test_gemm_wait_runs_out_and_the_context_recovers(cuda):
    import torch
    from bbdg import mlp
    from bbdg.context import get_context
    ctx = get_context(0)
    g = torch.Generator(device="cuda").manual_seed(9)
    M, N, K = 512, 256, 256                        # 4 K-blocks of 64 per output tile
    A = torch.randn(M, K, generator=g, device=cuda).to(torch.bfloat16)
    B = torch.randn(N, K, generator=g, device=cuda).to(torch.bfloat16)
    want = A.double() @ B.double().t()
    assert ctx.device_status() == 0
    C = torch.empty(M, N, device=cuda)
    try:
        ctx.set_wait_limit(LIMIT)
        ctx.set_test_fault(1)
        mlp.gemm_bf16(A, B, out_f32=C)
        assert ctx.device_status() & 2
    finally:
        ctx.set_test_fault(0)
        ctx.set_wait_limit(0)
    for _ in range(2):
        C.fill_(float("nan"))
        mlp.gemm_bf16(A, B, out_f32=C)
        assert ctx.device_status() == 0
        err = (C.double() - want).abs().max().item() / want.abs().max().item()
        assert np.isfinite(err) and err < 1e-5, err
