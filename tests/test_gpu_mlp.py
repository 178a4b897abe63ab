"""GPU: tcgen05 BF16 GEMM, closure MLP forward/backward/Adam and the feature gather, through
the C ABI, against torch FP32 (GEMM) and the CPU oracle (oracle/mlp.py, meshdata.mapP).

Tolerances: the GEMM multiplies exact BF16 products and accumulates in FP32, so it matches an
FP64 product of the same BF16 inputs to ~1e-6 relative (tested at 1e-5). The MLP oracle
rounds to BF16 where the GPU does; the remaining difference is FP32 accumulation order plus
the BF16 rounding flips it causes (about one stored activation in 2,000 lands on the other
side of a rounding boundary, a 2^-8 relative change each), tested at 1e-3 relative for the
output and 2e-3 per parameter block.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


# shapes cover both tile widths (BN 256 when it pads no more than 128), ragged M, N and K,
# and more tiles than SMs (persistent CTAs cycling both TMEM accumulators)
@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (300, 200, 840), (1000, 512, 512),
                                   (130, 336, 24), (4096, 840, 512), (8192, 1024, 192),
                                   (8192, 336, 520), (24576, 512, 840)])
def test_gemm_plain(cuda, M, N, K):
    import torch
    from bbdg import mlp
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N)
    A = torch.randn((M, K), generator=g, device=cuda).bfloat16()
    B = torch.randn((N, K), generator=g, device=cuda).bfloat16()
    C = torch.empty((M, N), device=cuda)
    mlp.gemm_bf16(A, B, alpha=0.5, out_f32=C)
    ref = 0.5 * (A.double() @ B.double().T)
    torch.cuda.synchronize()
    assert _rel(C.cpu(), ref.cpu()) < 1e-5
    assert mlp.device_status() == 0


@pytest.mark.parametrize("M,N,K", [(512, 512, 8192), (336, 512, 24576)])
def test_gemm_split_k_through_mlp_shapes(cuda, M, N, K):
    """Weight-gradient shapes (K = batch): the split-K path adds partial tiles atomically."""
    import torch
    from bbdg import mlp
    g = torch.Generator(device="cuda").manual_seed(K)
    A = torch.randn((M, K), generator=g, device=cuda).bfloat16()
    B = torch.randn((N, K), generator=g, device=cuda).bfloat16()
    C = torch.zeros((M, N), device=cuda)
    mlp.gemm_bf16(A, B, out_f32=C, kt_per=16)
    ref = A.double() @ B.double().T
    torch.cuda.synchronize()
    assert _rel(C.cpu(), ref.cpu()) < 1e-5


def test_gemm_epilogues(cuda):
    import torch
    from bbdg import mlp
    M, N, K = 520, 264, 136
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn((M, K), generator=g, device=cuda).bfloat16()
    B = torch.randn((N, K), generator=g, device=cuda).bfloat16()
    bias = torch.randn(N, generator=g, device=cuda)
    pre = torch.empty((M, N), device=cuda)
    C = torch.empty((M, N), device=cuda)
    Cb = torch.empty((M, N), device=cuda, dtype=torch.bfloat16)
    CT = torch.empty((N, M), device=cuda, dtype=torch.bfloat16)
    bg = torch.zeros(N, device=cuda)
    # act 1: bias + GELU, pre-activation kept
    mlp.gemm_bf16(A, B, bias=bias, act=1, pre=pre, out_f32=C, out_bf16=Cb, out_t=CT,
                  bias_grad=bg)
    z = A.double() @ B.double().T + bias.double()
    y = torch.nn.functional.gelu(z)
    torch.cuda.synchronize()
    assert _rel(pre.cpu(), z.cpu()) < 1e-5
    assert _rel(C.cpu(), y.cpu()) < 1e-5
    assert torch.equal(Cb, C.bfloat16())
    assert torch.equal(CT, C.bfloat16().T.contiguous())
    assert _rel(bg.cpu(), y.sum(0).cpu()) < 1e-5
    # act 2: multiply by GELU'(pre)
    D = torch.empty((M, N), device=cuda)
    mlp.gemm_bf16(A, B, act=2, pre=pre, out_f32=D)
    zz = pre.double()
    dg = 0.5 * (1 + torch.erf(zz / np.sqrt(2))) + zz * torch.exp(-0.5 * zz * zz) / np.sqrt(2 * np.pi)
    want = (A.double() @ B.double().T) * dg
    torch.cuda.synchronize()
    assert _rel(D.cpu(), want.cpu()) < 1e-5


@pytest.mark.parametrize("N", [264, 203])
def test_gemm_fixed_epilogues(cuda, N):
    """The compile-time epilogues the MLP uses, with 16-byte row starts (N = 264) and without
    (N = 203: scalar stores inside the same variant)."""
    import torch
    from bbdg import mlp
    M, K = 520, 136
    g = torch.Generator(device="cuda").manual_seed(N)
    A = torch.randn((M, K), generator=g, device=cuda).bfloat16()
    B = torch.randn((N, K), generator=g, device=cuda).bfloat16()
    bias = torch.randn(N, generator=g, device=cuda)
    z = A.double() @ B.double().T
    # bias + GELU, pre-activation and BF16 output (the hidden layers' training forward)
    pre = torch.empty((M, N), device=cuda)
    Hb = torch.empty((M, N), device=cuda, dtype=torch.bfloat16)
    HT = torch.empty((N, M), device=cuda, dtype=torch.bfloat16)
    mlp.gemm_bf16(A, B, bias=bias, act=1, pre=pre, out_bf16=Hb, out_t=HT)
    torch.cuda.synchronize()
    zb = z + bias.double()
    assert _rel(pre.cpu(), zb.cpu()) < 1e-5
    want = torch.nn.functional.gelu(zb)
    assert _rel(Hb.double().cpu(), want.cpu()) < 5e-3          # BF16 output
    assert torch.equal(HT, Hb.T.contiguous())
    # bias + FP32 output (the output layer)
    C = torch.empty((M, N), device=cuda)
    mlp.gemm_bf16(A, B, bias=bias, out_f32=C)
    torch.cuda.synchronize()
    assert _rel(C.cpu(), zb.cpu()) < 1e-5
    # GELU' with BF16 output and bias gradient (the backward through a hidden layer)
    D = torch.empty((M, N), device=cuda, dtype=torch.bfloat16)
    bg = torch.zeros(N, device=cuda)
    mlp.gemm_bf16(A, B, act=2, pre=pre, out_bf16=D, bias_grad=bg)
    torch.cuda.synchronize()
    p64 = pre.double()
    dg = 0.5 * (1 + torch.erf(p64 / np.sqrt(2))) + p64 * torch.exp(-0.5 * p64 * p64) / np.sqrt(2 * np.pi)
    want = z * dg
    assert _rel(D.double().cpu(), want.cpu()) < 5e-3
    assert _rel(bg.cpu(), want.sum(0).cpu()) < 1e-5
    # BF16-only output
    E = torch.empty((M, N), device=cuda, dtype=torch.bfloat16)
    mlp.gemm_bf16(A, B, out_bf16=E)
    torch.cuda.synchronize()
    assert _rel(E.double().cpu(), z.cpu()) < 5e-3


def test_gemm_rejects_bad_arguments(cuda):
    import torch
    from bbdg import mlp, BBError
    A = torch.zeros((64, 20), device=cuda, dtype=torch.bfloat16)   # K % 8 != 0
    B = torch.zeros((64, 20), device=cuda, dtype=torch.bfloat16)
    with pytest.raises(BBError):
        mlp.gemm_bf16(A, B, out_f32=torch.empty((64, 64), device=cuda))
    A = torch.zeros((64, 16), device=cuda, dtype=torch.bfloat16)
    B = torch.zeros((64, 16), device=cuda, dtype=torch.bfloat16)
    with pytest.raises(BBError):
        mlp.gemm_bf16(A, B, act=2, out_f32=torch.empty((64, 64), device=cuda))  # no pre


def test_transpose(cuda):
    import torch
    from bbdg import mlp
    X = torch.randn((1000, 840), device=cuda).bfloat16()
    assert torch.equal(mlp.transpose_bf16(X), X.T.contiguous())


@pytest.mark.parametrize("dims,B", [((64, 128, 128, 48), 256), ((840, 512, 512, 336), 1024)])
def test_mlp_gradients_match_oracle(cuda, dims, B):
    import torch
    from bbdg import mlp
    from oracle import mlp as omlp
    rng = np.random.default_rng(11)
    p = omlp.init_params(dims, seed=3).astype(np.float32)
    X = rng.standard_normal((B, dims[0])).astype(np.float32)
    T = rng.standard_normal((B, dims[3])).astype(np.float32) * 0.5
    net = mlp.MLP(dims, max_batch=B, seed=1)
    net.set_params(p)
    assert np.array_equal(net.params(), p)
    Xd = torch.tensor(X, device=cuda).bfloat16()
    XT = mlp.transpose_bf16(Xd)
    Y = net.forward(Xd, XT, train=True)
    loss = net.backward(Y, torch.tensor(T, device=cuda))
    torch.cuda.synchronize()
    g = net.grads()
    l_ref, g_ref = omlp.backward(p.astype(np.float64), dims, X.astype(np.float64),
                                 T.astype(np.float64), emulate=True)
    Y_ref, _ = omlp.forward(p.astype(np.float64), dims, X.astype(np.float64), emulate=True)
    assert _rel(Y.cpu().numpy(), Y_ref) < 1e-3
    assert abs(loss.item() - l_ref) / l_ref < 1e-3
    lay, _ = omlp.layout(dims)
    for l, (ow, ob) in enumerate(lay):
        n_out = dims[l + 1]
        assert _rel(g[ow:ob], g_ref[ow:ob]) < 2e-3, f"W{l + 1}"
        assert _rel(g[ob:ob + n_out], g_ref[ob:ob + n_out]) < 2e-3, f"b{l + 1}"
    # inference path (no saved activations) gives the same output
    Y2 = net.forward(Xd)
    torch.cuda.synchronize()
    assert torch.equal(Y, Y2)
    assert mlp.device_status() == 0


def test_mlp_training_reduces_loss(cuda):
    """Adam on a smooth synthetic regression: the loss falls by more than 10x."""
    import torch
    from bbdg import mlp
    dims, B = (64, 128, 128, 32), 2048
    g = torch.Generator(device="cuda").manual_seed(2)
    X = torch.randn((B, dims[0]), generator=g, device=cuda)
    Wt = torch.randn((dims[3], dims[0]), generator=g, device=cuda) / 8
    T = torch.tanh(X @ Wt.T)
    Xb = X.bfloat16()
    XT = mlp.transpose_bf16(Xb)
    net = mlp.MLP(dims, max_batch=B, seed=4)
    losses = []
    for it in range(300):
        Y = net.forward(Xb, XT, train=True)
        loss = net.backward(Y, T)
        net.step(lr=2e-3)
        if it % 50 == 0 or it == 299:
            losses.append(loss.item())
    assert losses[-1] < losses[0] / 10, losses


def test_mlp_rejects_bad_arguments(cuda):
    import torch
    from bbdg import mlp, BBError
    with pytest.raises(BBError):
        mlp.MLP((840, 500, 512, 336), max_batch=64)   # width not a multiple of 8
    net = mlp.MLP((64, 64, 64, 64), max_batch=64)
    X = torch.zeros((128, 64), device=cuda, dtype=torch.bfloat16)
    with pytest.raises(BBError):
        net.forward(X)                                  # batch above max_batch
    Y = torch.zeros((64, 64), device=cuda)
    with pytest.raises(BBError):
        net.backward(Y, Y)                              # no training forward first


def _face_nodes(N, f):
    """Volume index of face f's node m (face-local (a, b), b outer), kernel ordering."""
    from oracle import dense
    idx = {t[:3]: n for n, t in enumerate(dense.lut3(N))}
    out = []
    for b in range(N + 1):
        for a in range(N + 1 - b):
            ijk = ((a, 0, b), (N - a - b, a, b), (0, a, b), (a, b, 0))[f]
            out.append(idx[ijk])
    return out


@pytest.mark.parametrize("N,nf", [(2, 6), (5, 6), (3, 4)])
def test_closure_features_match_mapP(cuda, bb, N, nf):
    import torch
    from bbdg import mlp
    from oracle import meshdata
    mesh = bb.uniform_tet_mesh(2)
    md = meshdata.build(mesh, N)
    K, Np, Nfp = mesh.K, bb.np3(N), bb.np2(N)
    rng = np.random.default_rng(N)
    q = rng.standard_normal((nf, K, Np))
    conn = torch.tensor(mesh.conn.reshape(-1), dtype=torch.int32, device=cuda)
    X, XT = mlp.closure_features(N, nf, conn, torch.tensor(q, device=cuda), 0.5, transpose=True)
    torch.cuda.synchronize()
    # oracle: exterior values through mapP (coordinate-matched), reordered to kernel face order
    Fm = md.Fmask.reshape(4, Nfp)
    want = np.zeros((K, nf * Np + 4 * nf * Nfp))
    want[:, :nf * Np] = q.transpose(1, 0, 2).reshape(K, -1)
    for f in range(4):
        pos = [int(np.where(Fm[f] == v)[0][0]) for v in _face_nodes(N, f)]
        for e in range(K):
            for m, j in enumerate(pos):
                gP = md.mapP[e * 4 * Nfp + f * Nfp + j]
                eP, jP = divmod(int(gP), 4 * Nfp)
                vP = md.Fmask[jP]
                for fld in range(nf):
                    want[e, nf * Np + (f * nf + fld) * Nfp + m] = q[fld, eP, vP]
    want = torch.tensor(want * 0.5, dtype=torch.float32).bfloat16()
    assert torch.equal(X.cpu(), want)
    assert torch.equal(XT.cpu(), want.T.contiguous())


def test_closure_apply(cuda):
    import torch
    from bbdg import mlp
    N, nf, K = 5, 6, 100
    Np = 56
    q = torch.randn((nf, K, Np), device=cuda)
    Y = torch.randn((K, nf * Np), device=cuda)
    want = q + 0.25 * Y.reshape(K, nf, Np).permute(1, 0, 2)
    mlp.closure_apply(N, nf, 0.25, Y, q)
    torch.cuda.synchronize()
    assert torch.allclose(q, want, rtol=0, atol=1e-6)
