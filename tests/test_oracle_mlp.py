"""CPU: the closure-MLP oracle pinned by finite differences and torch's BF16 rounding."""
import numpy as np
import pytest

from oracle import mlp as omlp


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(10000) * 10.0 ** rng.integers(-8, 8, 10000),
                        [0.0, -0.0, 1.0, 1.00390625, 1.01171875, 65504.0, 1e-40]])
    want = torch.tensor(x, dtype=torch.float32).bfloat16().double().numpy()
    assert np.array_equal(omlp.bf16(x), want)


def test_backward_matches_finite_differences():
    dims, B = (8, 16, 16, 8), 5
    rng = np.random.default_rng(1)
    p = omlp.init_params(dims, seed=2)
    X = rng.standard_normal((B, dims[0]))
    T = rng.standard_normal((B, dims[3]))
    _, g = omlp.backward(p, dims, X, T, emulate=False)
    h = 1e-6
    idx = rng.choice(p.size, 60, replace=False)
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (omlp.loss(omlp.forward(pp, dims, X, False)[0], T) -
              omlp.loss(omlp.forward(pm, dims, X, False)[0], T)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-6 * abs(fd), (i, fd, g[i])


def test_emulated_rounding_changes_little():
    """The BF16 emulation is a small perturbation of the FP64 network (sanity of the points
    where it rounds)."""
    dims, B = (64, 128, 128, 48), 64
    rng = np.random.default_rng(3)
    p = omlp.init_params(dims, seed=4)
    X = rng.standard_normal((B, dims[0]))
    T = rng.standard_normal((B, dims[3]))
    l0, g0 = omlp.backward(p, dims, X, T, emulate=False)
    l1, g1 = omlp.backward(p, dims, X, T, emulate=True)
    assert abs(l1 - l0) / l0 < 1e-2
    assert np.linalg.norm(g1 - g0) / np.linalg.norm(g0) < 3e-2


def test_gelu_grad_is_derivative():
    x = np.linspace(-6, 6, 1001)
    h = 1e-6
    fd = (omlp.gelu(x + h) - omlp.gelu(x - h)) / (2 * h)
    assert np.abs(fd - omlp.gelu_grad(x)).max() < 1e-8
