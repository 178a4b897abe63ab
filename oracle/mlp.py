"""CPU oracle of the closure MLP -- TEST INFRASTRUCTURE ONLY (imported by tests/, never by the
product path).

The network is nin -> h1 -> h2 -> nout with GELU (exact erf form) after the two hidden layers
and the loss L = 1/(B nout) sum (Y - T)^2. Parameters are one flat vector in the library's
layout: W1[h1][nin], b1, W2[h2][h1], b2, W3[nout][h2], b3 (weights out x in, row-major).

`forward`/`backward` evaluate in FP64. With emulate=True they round to BF16 at exactly the
points where the GPU path stores BF16 -- the weights, the input, H1, H2, dY, dP2, dP1 -- so
the remaining difference to the GPU is FP32 accumulation order; with emulate=False they are
the plain FP64 network (pinned by finite differences in the tests). The reference
(BernsteinBasis.jl) has no learned part: there is nothing upstream to pin this against.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def layout(dims):
    """Offsets (W, b) of each layer in the flat parameter vector, and its length."""
    off, out = 0, []
    for l in range(3):
        nw = dims[l + 1] * dims[l]
        out.append((off, off + nw))
        off += nw + dims[l + 1]
    return out, off


def unpack(p, dims):
    lay, _ = layout(dims)
    Ws, bs = [], []
    for l, (ow, ob) in enumerate(lay):
        Ws.append(np.asarray(p[ow:ob], dtype=np.float64).reshape(dims[l + 1], dims[l]))
        bs.append(np.asarray(p[ob:ob + dims[l + 1]], dtype=np.float64))
    return Ws, bs


def forward(p, dims, X, emulate=True):
    """Returns Y and the activations needed by `backward`."""
    r = bf16 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    Ws, bs = unpack(p, dims)
    Wr = [r(W) for W in Ws]
    A0 = r(X)
    pre1 = A0 @ Wr[0].T + bs[0]
    H1 = r(gelu(pre1))
    pre2 = H1 @ Wr[1].T + bs[1]
    H2 = r(gelu(pre2))
    Y = H2 @ Wr[2].T + bs[2]
    return Y, dict(A0=A0, pre1=pre1, H1=H1, pre2=pre2, H2=H2, Wr=Wr)


def loss(Y, T):
    return float(np.mean((np.asarray(Y) - np.asarray(T)) ** 2))


def backward(p, dims, X, T, emulate=True):
    """(loss, flat gradient) of L = mean((Y - T)^2)."""
    r = bf16 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    Y, c = forward(p, dims, X, emulate)
    B, nout = Y.shape
    dYf = 2.0 * (Y - T) / (B * nout)
    dY = r(dYf)
    g = np.zeros(layout(dims)[1])
    lay, _ = layout(dims)
    Wr = c["Wr"]
    gW3 = dY.T @ c["H2"]
    gb3 = dYf.sum(0)
    dP2f = (dY @ Wr[2]) * gelu_grad(c["pre2"])
    dP2 = r(dP2f)
    gW2 = dP2.T @ c["H1"]
    gb2 = dP2f.sum(0)
    dP1f = (dP2 @ Wr[1]) * gelu_grad(c["pre1"])
    dP1 = r(dP1f)
    gW1 = dP1.T @ c["A0"]
    gb1 = dP1f.sum(0)
    for (ow, ob), gw, gb in zip(lay, (gW1, gW2, gW3), (gb1, gb2, gb3)):
        g[ow:ob] = gw.reshape(-1)
        g[ob:ob + gb.size] = gb
    return loss(Y, T), g


def init_params(dims, seed):
    """Deterministic parameters for tests (not the library's own initialisation)."""
    rng = np.random.default_rng(seed)
    lay, n = layout(dims)
    p = np.zeros(n)
    for l, (ow, ob) in enumerate(lay):
        a = 1.0 / np.sqrt(dims[l])
        p[ow:ob] = rng.uniform(-a, a, ob - ow)
        p[ob:ob + dims[l + 1]] = rng.uniform(-0.1, 0.1, dims[l + 1])
    return p
