"""The face-lift recursion the CUDA kernels run, restated in numpy and checked against the
oracle (src/BernsteinLift.jl:139-164, face_lift_multiply!) for every degree up to the
library's maximum, in float64 and float32 arithmetic (no GPU).

The kernels apply L0 as the 7-point stencil of (N+1)^2/2 R_{N+1} E_{N->N+1} and carry the
layer weights l_d = (-1)^d C(N,d)/(d+1) in the reduction itself:
F_0 = L0 x, F_d = -1/(d+1) [(i+1) F_{d-1}(i+1,j) + (j+1) F_{d-1}(i,j+1) + (N-d+1-i-j) F_{d-1}(i,j)],
where the reference forms E_d = R_{N-d+1} E_{d-1} and writes l_d E_d. The GPU suite checks
the kernels up to N = 15; this pins the algebra, and its rounding in both precisions, up to
N = 20, where the level-parallel lift serves FP32 and FP64.
"""
import numpy as np
import pytest

MAX_N = 20
TOL = {np.float64: 1e-12, np.float32: 1e-5}


def tri_off(n, j):
    return j * (2 * n + 3 - j) // 2


def tet_off(n, k):
    a, b = n + 1, n + 1 - k
    return (a * (a + 1) * (a + 2) - b * (b + 1) * (b + 2)) // 6


def ijk3(n, i, j, k):
    return i + tri_off(n, j) + tet_off(n, k) - j * k


def folded_face_lift(N, x, dt):
    """x: (K, Nfp) face coefficients (2D order j outer, i inner) -> (K, Np), arithmetic in dt."""
    K = x.shape[0]
    X = np.zeros((K, N + 3, N + 3), dt)  # X[:, i + 1, j + 1] = x(i, j), zero outside
    for j in range(N + 1):
        for i in range(N + 1 - j):
            X[:, i + 1, j + 1] = x[:, i + tri_off(N, j)]

    def xv(i, j):
        return X[:, i + 1, j + 1]

    Np = (N + 1) * (N + 2) * (N + 3) // 6
    out = np.zeros((K, Np), dt)
    E = np.zeros((K, N + 2, N + 2), dt)
    half = dt(0.5)
    for j in range(N + 1):
        for i in range(N + 1 - j):
            k = N - i - j
            v = ((i + 1) ** 2 + (j + 1) ** 2 + (k + 1) ** 2) * xv(i, j)
            v = v + ((i + 1) * j) * xv(i + 1, j - 1) + ((i + 1) * k) * xv(i + 1, j)
            v = v + ((j + 1) * i) * xv(i - 1, j + 1) + ((j + 1) * k) * xv(i, j + 1)
            v = v + ((k + 1) * i) * xv(i - 1, j) + ((k + 1) * j) * xv(i, j - 1)
            E[:, i, j] = half * v
            out[:, ijk3(N, i, j, 0)] = E[:, i, j]
    for d in range(1, N + 1):
        n = N - d + 1
        c = dt(-1.0 / (d + 1))
        F = np.zeros_like(E)
        for j in range(n):
            for i in range(n - j):
                F[:, i, j] = ((i + 1) * E[:, i + 1, j] + (j + 1) * E[:, i, j + 1]
                              + (n - i - j) * E[:, i, j]) * c
                out[:, ijk3(N, i, j, d)] = F[:, i, j]
        E = F
    return out


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("N", range(1, MAX_N + 1))
def test_folded_lift_recursion_matches_oracle(oracle_cpu, N, dt):
    rng = np.random.default_rng(700 + N)
    Nfp = (N + 1) * (N + 2) // 2
    x = rng.uniform(-1, 1, (6, Nfp))
    got = folded_face_lift(N, x.astype(dt), dt).astype(np.float64)
    want = np.stack([oracle_cpu.face_lift(N, x[e]) for e in range(x.shape[0])])
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err < TOL[dt], err


def test_lift_weight_ratio():
    """l_d / (l_{d-1} (N-d+1)) = -1/(d+1) for the reference's l_j (constants.jl:10-12)."""
    from bbdg.ordering import l_j
    for N in range(1, MAX_N + 1):
        lj = (1.0,) + tuple(l_j(N))  # l_0 = 1
        for d in range(1, N + 1):
            assert lj[d] / (lj[d - 1] * (N - d + 1)) == pytest.approx(-1.0 / (d + 1), rel=1e-14)
