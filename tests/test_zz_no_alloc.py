"""bb_norms_noalloc: the allocation-free variant of the FP64 norm reduction.

Some callers cannot allocate device memory: a host runtime whose device memory belongs to its
own pool allocator (CUDA.jl's pool, PyTorch's caching allocator), or a stepping loop that
must not stall on cudaFree. This entry point keeps its partial sums in a fixed file-scope
device array instead of context scratch and writes its result to a device buffer the caller
passes. The test calls it through the C ABI twice in a row and compares each result with
bb_norms, the allocating entry point, within the reduction tolerance (1e-12 relative; the two
differ only in summation order). This file is collected last, and it builds everything it
uses, so it also runs alone.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_norms_noalloc_matches_norms_twice_in_a_row(cuda, bb):
    import torch
    from bbdg import _lib
    from bbdg.context import get_context
    L = _lib.load()
    ctx = get_context(0)
    N, K = 5, 1234
    Np = bb.np3(N)
    rng = np.random.default_rng(2024)
    for call, (nf, dtype) in enumerate([(4, torch.float32), (6, torch.float64)]):
        a = torch.tensor(rng.standard_normal((nf, K, Np)), dtype=dtype, device=cuda)
        b = torch.tensor(rng.standard_normal((nf, K, Np)), dtype=dtype, device=cuda)
        code = _lib.BB_F32 if dtype == torch.float32 else _lib.BB_F64
        want = (ctypes.c_double * (3 * nf))()
        assert L.bb_norms(ctx.handle, N, K, nf, code, ctypes.c_void_p(a.data_ptr()),
                          ctypes.c_void_p(b.data_ptr()), want, None) == 0
        out = torch.full((3 * nf,), float("nan"), dtype=torch.float64, device=cuda)
        stream = torch.cuda.current_stream()
        rc = L.bb_norms_noalloc(N, K, nf, code, ctypes.c_void_p(a.data_ptr()),
                                ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, np.array(want[:]), rtol=1e-12, atol=0)


def test_norms_noalloc_rejects_too_many_fields(cuda, bb):
    import torch
    from bbdg import _lib
    L = _lib.load()
    a = torch.zeros((9, 2, bb.np3(1)), dtype=torch.float64, device=cuda)
    out = torch.zeros(27, dtype=torch.float64, device=cuda)
    rc = L.bb_norms_noalloc(1, 2, 9, _lib.BB_F64, ctypes.c_void_p(a.data_ptr()), None,
                            ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.BB_ERR_ARG


def test_norms_noalloc_without_b_gives_zero_difference_sums(cuda, bb):
    import torch
    from bbdg import _lib
    from bbdg.context import get_context
    L = _lib.load()
    ctx = get_context(0)
    N, K, nf = 3, 777, 2
    a = torch.tensor(np.random.default_rng(7).standard_normal((nf, K, bb.np3(N))),
                     dtype=torch.float64, device=cuda)
    want = (ctypes.c_double * (3 * nf))()
    assert L.bb_norms(ctx.handle, N, K, nf, _lib.BB_F64, ctypes.c_void_p(a.data_ptr()), None,
                      want, None) == 0
    out = torch.full((3 * nf,), float("nan"), dtype=torch.float64, device=cuda)
    assert L.bb_norms_noalloc(N, K, nf, _lib.BB_F64, ctypes.c_void_p(a.data_ptr()), None,
                              ctypes.c_void_p(out.data_ptr()), None) == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(nf, 3)
    np.testing.assert_allclose(got[:, 0], np.array(want[:]).reshape(nf, 3)[:, 0], rtol=1e-12)
    assert np.all(got[:, 1:] == 0)
