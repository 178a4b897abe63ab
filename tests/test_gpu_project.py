"""FP64 degree reduction (bb_project) vs the dense projection operator of the oracle."""
import numpy as np
import pytest

from oracle import dense

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,M", [(3, 2), (5, 3), (10, 5)])
def test_projection_matches_dense_operator(cuda, bb, N, M):
    import ctypes
    import torch
    from bbdg import _lib
    from bbdg.context import get_context
    ctx = get_context(0)
    K, nf = 77, 6
    rng = np.random.default_rng(N * 10 + M)
    x = rng.standard_normal((nf, K, bb.np3(N)))
    want = np.einsum("ab,fkb->fka", dense.projection_dense(N, M), x)
    for din, dout in ((torch.float64, torch.float64), (torch.float32, torch.float64)):
        xin = torch.tensor(x, dtype=din, device=cuda)
        out = torch.empty((nf, K, bb.np3(M)), dtype=dout, device=cuda)
        code = lambda t: _lib.BB_F64 if t == torch.float64 else _lib.BB_F32
        ctx.check(_lib.load().bb_project(ctx.handle, N, M, K, nf, code(din),
                                         ctypes.c_void_p(xin.data_ptr()), code(dout),
                                         ctypes.c_void_p(out.data_ptr()), None))
        got = out.cpu().numpy()
        ref = want if din == torch.float64 else np.einsum(
            "ab,fkb->fka", dense.projection_dense(N, M), xin.cpu().double().numpy())
        assert np.abs(got - ref).max() < 1e-11 * np.abs(ref).max(), (din, dout)
