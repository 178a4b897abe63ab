"""CPU oracle pinned against the reference's own tests (test/runtests.jl), restated.

Each test names the testset it restates. Inputs are seeded (the reference uses unseeded
rand); comparisons use the reference's default isapprox tolerance sqrt(eps) ~ 1.5e-8 unless
noted. Also checks the oracle against the exact rational golden vectors in tests/golden.
"""
import json
import os

import numpy as np
import pytest

from oracle import dense, meshdata

RTOL = 1.5e-8  # isapprox default for Float64


def close(a, b, rtol=RTOL):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


@pytest.mark.parametrize("N", range(1, 13))
def test_derivative_vector_mul(oracle_cpu, N):
    """runtests.jl:7-17 Matrix-vector mul! of BernsteinDerivativeMatrix_3D."""
    rng = np.random.default_rng(N)
    Np = (N + 1) * (N + 2) * (N + 3) // 6
    x = rng.random(Np)
    for axis in range(3):
        D = dense.to_float(dense.deriv_dense(N, axis))
        assert close(D @ x, oracle_cpu.deriv(axis, N, x[None])[0])


@pytest.mark.parametrize("N", range(1, 7))
def test_derivative_matrix_mul(oracle_cpu, N):
    """runtests.jl:19-29 Matrix-matrix mul! (column loop over elements)."""
    rng = np.random.default_rng(100 + N)
    Np = (N + 1) * (N + 2) * (N + 3) // 6
    X = rng.random((Np, Np))          # Julia Np x Np, column e = row e here
    for axis in range(3):
        D = dense.to_float(dense.deriv_dense(N, axis))
        assert close((D @ X.T).T, oracle_cpu.deriv(axis, N, X))


@pytest.mark.parametrize("N", range(1, 10))
def test_face_lift_vs_naive(oracle_cpu, N):
    """runtests.jl:31-48 face_lift_multiply vs. a more naive algorithm."""
    rng = np.random.default_rng(200 + N)
    x = rng.random((N + 1) * (N + 2) // 2)
    Lf = dense.to_float(dense.face_lift_dense(N))
    assert close(Lf @ x, oracle_cpu.face_lift(N, x))


@pytest.mark.parametrize("N", range(1, 21))
def test_index_ordering(oracle_cpu, bb, N):
    """runtests.jl:51-80 2D and 3D index ordering (oracle and host tables)."""
    tri, tet = oracle_cpu.offsets(N)
    assert tuple(tri) == bb.tri_offsets(N) and tuple(tet) == bb.tet_offsets(N)
    index = 1
    for j in range(N + 1):
        for i in range(N - j + 1):
            assert bb.ij_to_linear(i, j, tri) == index
            index += 1
    index = 1
    for k in range(N + 1):
        for j in range(N - k + 1):
            for i in range(N - j - k + 1):
                assert bb.ijk_to_linear(i, j, k, tri, tet) == index
                index += 1


@pytest.mark.parametrize("N", range(1, 21))
def test_elevation_vs_matrix(oracle_cpu, N):
    """runtests.jl:82-90 Elevation multiply vs. ElevationMatrix."""
    rng = np.random.default_rng(300 + N)
    x = rng.random((N + 1) * (N + 2) // 2)
    E = dense.to_float(dense.elevation_dense(N + 1))
    assert close(E @ x, oracle_cpu.elevation(N, x))


@pytest.mark.parametrize("N", range(1, 10))
def test_L0_from_elevation_reduction(oracle_cpu, N):
    """runtests.jl:92-106 L0 = (N+1)^2/2 E'E via elevation then reduction."""
    rng = np.random.default_rng(400 + N)
    x = rng.random((N + 1) * (N + 2) // 2)
    E1 = dense.to_float(dense.elevation_dense(N + 1))
    L0 = (N + 1) ** 2 / 2 * E1.T @ E1
    y = oracle_cpu.reduction(N + 1, oracle_cpu.elevation(N, x)) * (N + 1) ** 2 / 2
    assert close(L0 @ x, y)


@pytest.mark.parametrize("N", range(1, 9))
def test_lift_vs_mass_matrix_lift(oracle_cpu, N):
    """runtests.jl:108-117 lift mul! vs get_bernstein_lift, restated as M^{-1}[M^f]."""
    rng = np.random.default_rng(500 + N)
    Nfp = (N + 1) * (N + 2) // 2
    L = dense.lift_from_mass(N)
    X = rng.random(4 * Nfp)
    Y = rng.random((2, 4 * Nfp))
    assert close(L @ X, oracle_cpu.lift(N, X[None])[0])
    assert close((L @ Y.T).T, oracle_cpu.lift(N, Y))


@pytest.mark.parametrize("N", range(1, 10))
def test_derivative_vs_vandermonde(N):
    """runtests.jl:128-141 D = V^{-1} Dr_nodal V, restated with exact basis derivatives."""
    Dv = dense.deriv_from_vandermonde(N, seed=N)
    for axis in range(3):
        D = dense.to_float(dense.deriv_dense(N, axis))
        assert np.abs(Dv[axis] - D).max() < 1e-8 * max(1.0, np.abs(D).max())


def _golden():
    path = os.path.join(os.path.dirname(__file__), "golden", "operators_exact.json")
    with open(path) as fh:
        return json.load(fh)["cases"]


@pytest.mark.parametrize("case", _golden(), ids=lambda c: f"{c['op']}-N{c['N']}")
def test_oracle_matches_exact_golden(oracle_cpu, case):
    """Fast oracle operators vs exact rational golden vectors (1e-14 relative)."""
    N, x, y = case["N"], np.array(case["x"]["float"]), np.array(case["y"]["float"])
    op = case["op"]
    if op[0] == "D":
        got = oracle_cpu.deriv("rst".index(op[1]), N, x[None])[0]
    elif op == "elevation":
        got = oracle_cpu.elevation(N, x)
    elif op == "reduction":
        got = oracle_cpu.reduction(N, x)
    elif op == "face_lift":
        got = oracle_cpu.face_lift(N, x)
    else:
        got = oracle_cpu.lift(N, x[None])[0]
    assert close(got, y, 1e-14), op


def test_lj_constants(oracle_cpu, bb):
    """constants.jl:10-12 l_j table."""
    for N in range(1, 21):
        lj = bb.l_j(N)
        for j in range(1, 21):
            assert oracle_cpu.l_j(N, j) == pytest.approx(lj[j - 1], rel=1e-15, abs=0)


@pytest.mark.parametrize("phys", [0, 1])
@pytest.mark.parametrize("tau", [0.0, 1.0])
def test_example_analytic_solution(oracle_cpu, bb, phys, tau):
    """The examples' end check (3d_wave.jl:140-145, 3d_maxwell.jl:141-150): L-inf error of
    the discrete solution vs the analytic standing wave at T = 0.05, N = 7, 4^3 hex mesh."""
    m = bb.uniform_tet_mesh(4)
    N = 7
    md = meshdata.build(m, N)
    X = bb.element_domain_points(m, N)
    x, y, z = X[..., 0], X[..., 1], X[..., 2]
    T = 0.05
    nsteps = 26 if tau > 0 else 200
    zero = lambda x, y, z: 0 * x
    if phys == 0:
        f0 = lambda x, y, z: np.cos(np.pi * x) * np.cos(np.pi * y) * np.cos(np.pi * z)
        q = bb.project_fields(m, N, [f0, zero, zero, zero])
        s3 = np.sqrt(3)
        ex = [np.cos(np.pi * x) * np.cos(np.pi * y) * np.cos(np.pi * z) * np.cos(s3 * np.pi * T),
              np.sin(np.pi * x) * np.cos(np.pi * y) * np.cos(np.pi * z) * np.sin(s3 * np.pi * T) / s3,
              np.cos(np.pi * x) * np.sin(np.pi * y) * np.cos(np.pi * z) * np.sin(s3 * np.pi * T) / s3,
              np.cos(np.pi * x) * np.cos(np.pi * y) * np.sin(np.pi * z) * np.sin(s3 * np.pi * T) / s3]
    else:
        f5 = lambda x, y, z: np.sin(np.pi * x) * np.sin(np.pi * y)
        q = bb.project_fields(m, N, [zero] * 5 + [f5])
        s2 = np.sqrt(2)
        ex = [-np.sin(np.pi * x) * np.cos(np.pi * y) * np.sin(np.pi * s2 * T) / s2,
              np.cos(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * s2 * T) / s2,
              0 * x, 0 * x, 0 * x,
              np.sin(np.pi * x) * np.sin(np.pi * y) * np.cos(np.pi * s2 * T)]
    qT, _ = oracle_cpu.lsrk(phys, N, q, md, T / nsteps, nsteps, tau=tau)
    V = bb.bernstein_basis_tet(N, *(2 * bb.mesh.reference_domain_points(N)[:, [1, 2, 3]].T - 1))
    u = np.einsum("pn,fkn->fkp", V, qT)
    err = max(np.abs(u[i] - ex[i]).max() for i in range(len(ex)))
    assert err < 5e-4, err


def test_projection_operator_definition():
    """P = M_MM^-1 E^T M_NN reproduces degree-M polynomials and is the L2-orthogonal map."""
    for N, M in ((3, 2), (5, 3), (10, 5)):
        P = dense.projection_dense(N, M)
        E = dense.elevation3_dense(M, N)
        assert np.allclose(P @ E, np.eye(P.shape[0]), atol=1e-10)     # exact on degree M
        MN = np.array(dense.mass(N))
        rng = np.random.default_rng(N)
        c = rng.standard_normal(MN.shape[0])
        r = c - E @ (P @ c)                                           # residual is orthogonal
        assert np.abs(E.T @ MN @ r).max() < 1e-10 * np.abs(c).max()


def test_advection_example_analytic_solution(oracle_cpu, bb):
    """examples/3d_advec_scalar.jl end check: u0 = sin(pi x) sin(pi y) sin(pi z) advected in x
    with unit speed on the periodic 4^3 hex mesh, N = 7, T = 0.1; L-inf error vs u0(x - T)."""
    m = bb.uniform_tet_mesh(4)
    N = 7
    md = meshdata.build(m, N)
    f0 = lambda x, y, z: np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z)
    q = bb.project_fields(m, N, [f0])
    T, nsteps = 0.1, 100
    qT, _ = oracle_cpu.lsrk(2, N, q, md, T / nsteps, nsteps)
    X = bb.element_domain_points(m, N)
    x, y, z = X[..., 0], X[..., 1], X[..., 2]
    V = bb.bernstein_basis_tet(N, *(2 * bb.mesh.reference_domain_points(N)[:, [1, 2, 3]].T - 1))
    u = np.einsum("pn,kn->kp", V, qT[0])
    ex = np.sin(np.pi * (x - T)) * np.sin(np.pi * y) * np.sin(np.pi * z)
    assert np.abs(u - ex).max() < 1e-3


def test_three_component_advection_oracle(oracle_cpu, bb):
    """examples/3d_advec.jl: q = (u, v, w), fx(q) = (u, 0, 0), the scalar example's flux on
    every component. The u component equals the scalar example bitwise; v and w, which have
    no volume term, follow the lifted interface flux alone (zero data stays zero); the
    example's end check (u0 = (sin sin sin, 0, 0), N = 7, 4^3 hexes, T = 0.1) holds."""
    m = bb.uniform_tet_mesh(3)
    N = 4
    md = meshdata.build(m, N)
    rng = np.random.default_rng(17)
    q = rng.uniform(-1, 1, (3, m.K, bb.np3(N)))
    r3 = oracle_cpu.rhs(3, N, q, md)
    r1 = oracle_cpu.rhs(2, N, q[:1], md)
    assert np.array_equal(r3[0], r1[0])
    assert np.abs(r3[1]).max() > 0 and np.abs(r3[2]).max() > 0
    # v alone, with u = w = 0: only the lifted flux of v acts, linear in v
    qv = np.zeros_like(q)
    qv[1] = q[1]
    rv = oracle_cpu.rhs(3, N, qv, md)
    assert np.abs(rv[0]).max() == 0 and np.abs(rv[2]).max() == 0
    np.testing.assert_allclose(oracle_cpu.rhs(3, N, 2 * qv, md)[1], 2 * rv[1], rtol=1e-13,
                               atol=1e-13)
    m4 = bb.uniform_tet_mesh(4)
    N = 7
    md4 = meshdata.build(m4, N)
    f0 = lambda x, y, z: np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z)
    zero = lambda x, y, z: 0 * x
    q0 = bb.project_fields(m4, N, [f0, zero, zero])
    T, nsteps = 0.1, 100
    qT, _ = oracle_cpu.lsrk(3, N, q0, md4, T / nsteps, nsteps)
    X = bb.element_domain_points(m4, N)
    x, y, z = X[..., 0], X[..., 1], X[..., 2]
    V = bb.bernstein_basis_tet(N, *(2 * bb.mesh.reference_domain_points(N)[:, [1, 2, 3]].T - 1))
    u = np.einsum("pn,kn->kp", V, qT[0])
    ex = np.sin(np.pi * (x - T)) * np.sin(np.pi * y) * np.sin(np.pi * z)
    assert np.abs(u - ex).max() < 1e-3
    assert np.abs(qT[1:]).max() == 0
