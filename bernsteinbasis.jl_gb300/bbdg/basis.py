"""Bernstein Vandermonde matrices and nodal-to-Bernstein conversion (host side, FP64).

Mirrors ``src/utility.jl:8-107`` (cartesian_to_barycentric, bernstein_basis,
bernstein_basis_from_barycentric). These run once per degree at set-up; the result is the
Bernstein coefficient array that both the CUDA path and the CPU oracle start from
(the examples' ``modal_u0 = inv(vande) * u0``, examples/3d_wave.jl:111-113).
"""
from __future__ import annotations

from functools import lru_cache
from math import factorial

import numpy as np

from .ordering import linear_to_ijkl_lookup, bernstein_2d_multiindex
from .mesh import TetMesh, element_domain_points, reference_domain_points


def cartesian_to_barycentric_tet(r, s, t):
    """utility.jl:23-29."""
    r, s, t = (np.asarray(a, dtype=np.float64) for a in (r, s, t))
    return (1 + r) / 2, (1 + s) / 2, (1 + t) / 2, -(1 + r + s + t) / 2


def cartesian_to_barycentric_tri(r, s):
    """utility.jl:15-21."""
    r, s = (np.asarray(a, dtype=np.float64) for a in (r, s))
    return (r + 1) / 2, (s + 1) / 2, -(r + s) / 2


def bernstein_basis_from_barycentric_tet(N, l0, l1, l2, l3):
    """utility.jl:97-99: V[m, n] = psi_n(point m), columns in storage order."""
    cols = []
    for (i, j, k, l) in linear_to_ijkl_lookup(N):
        c = factorial(N) / (factorial(i) * factorial(j) * factorial(k) * factorial(l))
        cols.append(c * l0 ** i * l1 ** j * l2 ** k * l3 ** l)
    return np.stack(cols, axis=-1)


def bernstein_basis_from_barycentric_tri(N, l0, l1, l2):
    """utility.jl:88-89."""
    cols = []
    for (i, j, k) in bernstein_2d_multiindex(N):
        c = factorial(N) / (factorial(i) * factorial(j) * factorial(k))
        cols.append(c * l0 ** i * l1 ** j * l2 ** k)
    return np.stack(cols, axis=-1)


def bernstein_basis_tet(N, r, s, t):
    """utility.jl:62-63."""
    return bernstein_basis_from_barycentric_tet(N, *cartesian_to_barycentric_tet(r, s, t))


def bernstein_basis_tri(N, r, s):
    """utility.jl:59-60."""
    return bernstein_basis_from_barycentric_tri(N, *cartesian_to_barycentric_tri(r, s))


@lru_cache(maxsize=None)
def _interp_matrix(N: int) -> np.ndarray:
    """Inverse Bernstein Vandermonde at the degree-N domain points (equispaced lattice)."""
    W = reference_domain_points(N)            # weights on X1..X4
    lam = (W[:, 1], W[:, 2], W[:, 3], W[:, 0])  # lambda0..lambda3
    V = bernstein_basis_from_barycentric_tet(N, *lam)
    return np.linalg.inv(V)


def nodal_to_bernstein(values: np.ndarray, N: int) -> np.ndarray:
    """Coefficients (K, Np) interpolating values (K, Np) given at the domain points."""
    return values @ _interp_matrix(N).T


def project_fields(mesh: TetMesh, N: int, fields) -> np.ndarray:
    """Bernstein coefficients (nf, K, Np) of callables f(x, y, z), FP64."""
    X = element_domain_points(mesh, N)
    out = np.empty((len(fields), mesh.K, X.shape[1]))
    for m, f in enumerate(fields):
        v = np.broadcast_to(np.asarray(f(X[..., 0], X[..., 1], X[..., 2]), dtype=np.float64),
                            X.shape[:2])
        out[m] = nodal_to_bernstein(v, N)
    return out


def gaussian_pulses(seed: int, count: int = 8):
    """Sum of Gaussian pulses: centres U[-0.8,0.8]^3, widths U[0.1,0.3], amplitudes N(0,1).

    Returns f(x, y, z) = sum_g a_g exp(-|x - c_g|^2 / w_g^2).
    """
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-0.8, 0.8, size=(count, 3))
    widths = rng.uniform(0.1, 0.3, size=count)
    amps = rng.standard_normal(count)

    def f(x, y, z):
        acc = np.zeros(np.broadcast(x, y, z).shape)
        for c, w, a in zip(centres, widths, amps):
            acc += a * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / w ** 2)
        return acc
    return f


def evaluate_at_points(mesh: TetMesh, N: int, q: np.ndarray, pts: np.ndarray,
                       chunk: int = 16384) -> np.ndarray:
    """Values (nf, P) of the degree-N Bernstein fields q (nf, K, Np) of a uniform_tet_mesh at
    points pts (P, 3) in [-1, 1]^3 (host, FP64). Each point is located in its hexahedron
    (periodic wrap) and in the one of the hexahedron's six tetrahedra where its barycentric
    coordinates are all >= 0 (the largest minimum, for points on shared faces)."""
    if mesh.n < 1 or mesh.K != 6 * mesh.n ** 3:
        raise ValueError("point location needs a uniform_tet_mesh")
    q = np.asarray(q, dtype=np.float64)
    n, h = mesh.n, mesh.h
    X1 = mesh.EVX[:, 0, :]
    G = np.stack([mesh.EVX[:, m, :] - X1 for m in (1, 2, 3)], axis=2)   # (K, 3, 3)
    Ginv = np.linalg.inv(G)
    lut = np.array(linear_to_ijkl_lookup(N))                           # (Np, 4): i, j, k, l
    coef = np.array([factorial(N) / (factorial(i) * factorial(j) * factorial(k) * factorial(l))
                     for (i, j, k, l) in lut])
    out = np.empty((q.shape[0], pts.shape[0]))
    for p0 in range(0, pts.shape[0], chunk):
        P = np.asarray(pts[p0:p0 + chunk], dtype=np.float64)
        cell = np.clip(np.floor((P + 1.0) / h).astype(np.int64), 0, n - 1)
        hexid = cell[:, 0] + n * (cell[:, 1] + n * cell[:, 2])
        best_e = np.zeros(P.shape[0], np.int64)
        best_l = np.zeros((P.shape[0], 4))
        best_m = np.full(P.shape[0], -np.inf)
        for t in range(6):
            e = 6 * hexid + t
            # vertex X1 of the element may sit in a neighbouring cell of the unwrapped lattice
            lam3 = np.einsum("pij,pj->pi", Ginv[e], P - X1[e])             # weights on X2..X4
            lam = np.concatenate([1.0 - lam3.sum(axis=1, keepdims=True), lam3], axis=1)
            m = lam.min(axis=1)
            better = m > best_m
            best_m = np.where(better, m, best_m)
            best_e = np.where(better, e, best_e)
            best_l = np.where(better[:, None], lam, best_l)
        # coefficient (i, j, k, l) carries lambda_X2^i lambda_X3^j lambda_X4^k lambda_X1^l
        L1, L2, L3, L4 = (best_l[:, c] for c in range(4))                 # X1, X2, X3, X4
        B = coef[None, :] * (L2[:, None] ** lut[:, 0] * L3[:, None] ** lut[:, 1] *
                             L4[:, None] ** lut[:, 2] * L1[:, None] ** lut[:, 3])
        for f in range(q.shape[0]):
            out[f, p0:p0 + chunk] = np.einsum("pn,pn->p", B, q[f][best_e])
    return out
