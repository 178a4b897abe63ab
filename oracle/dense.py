"""Dense operator definitions the reference's tests check against -- TEST INFRASTRUCTURE ONLY.

  deriv_dense        BernsteinDerivativeMatrix_3D.jl:61-94 (getindex / get_coeff)
  elevation_dense    ElevationMatrix.jl:11-24
  face_lift_dense    test/runtests.jl:34-40 ([L0; l_i E^T ... L0] with L0 = (N+1)^2/2 E'E)
  mass / face_mass   closed-form Bernstein mass matrices on the reference tetrahedron
                     (volume 4/3) and reference faces (triangle area 2, StartUpDG's face
                     quadrature measure); lift_from_mass = M^{-1} [M^1 | M^2 | M^3 | M^4]
                     restates get_bernstein_lift (utility.jl:157-180) without StartUpDG
  vandermonde_tet    utility.jl:97-107 and its barycentric derivatives (:109-138)
All functions accept a ``num`` conversion so tests/golden can run them in exact rationals.
"""
from __future__ import annotations

from fractions import Fraction
from math import comb, factorial

import numpy as np


def lut3(N):
    return [(i, j, k, N - i - j - k)
            for k in range(N + 1) for j in range(N + 1 - k) for i in range(N + 1 - j - k)]


def lut2(N):
    return [(i, j, N - i - j) for j in range(N + 1) for i in range(N + 1 - j)]


def _get_coeff(a, b):
    """BernsteinDerivativeMatrix_3D.jl:61-67."""
    i1, j1, k1, l1 = a
    if a == b:
        return i1
    if (i1 + 1, j1 - 1, k1, l1) == b:
        return j1
    if (i1 + 1, j1, k1 - 1, l1) == b:
        return k1
    if (i1 + 1, j1, k1, l1 - 1) == b:
        return l1
    return 0


def deriv_dense(N, axis, num=float):
    """Dense Dr/Ds/Dt (axis 0/1/2) from the getindex definitions (:69-94)."""
    L = lut3(N)
    half = num(1) / num(2)
    M = [[None] * len(L) for _ in L]
    for m, (i1, j1, k1, l1) in enumerate(L):
        for n, (i2, j2, k2, l2) in enumerate(L):
            d3 = _get_coeff((l1, j1, k1, i1), (l2, j2, k2, i2))
            if axis == 0:
                d = _get_coeff((i1, j1, k1, l1), (i2, j2, k2, l2))
            elif axis == 1:
                d = _get_coeff((j1, i1, k1, l1), (j2, i2, k2, l2))
            else:
                d = _get_coeff((k1, j1, i1, l1), (k2, j2, i2, l2))
            M[m][n] = half * num(d - d3)
    return M


def elevation_dense(N, num=float):
    """ElevationMatrix{N}: degree N-1 -> N, size np2(N) x np2(N-1) (ElevationMatrix.jl:17-24)."""
    A, B = lut2(N), lut2(N - 1)
    M = [[num(0)] * len(B) for _ in A]
    for m, a in enumerate(A):
        for n, (i2, j2, k2) in enumerate(B):
            if a == (i2 + 1, j2, k2):
                M[m][n] = num(i2 + 1) / num(N)
            elif a == (i2, j2 + 1, k2):
                M[m][n] = num(j2 + 1) / num(N)
            elif a == (i2, j2, k2 + 1):
                M[m][n] = num(k2 + 1) / num(N)
    return M


def _mm(A, B):
    return [[sum(A[i][k] * B[k][j] for k in range(len(B))) for j in range(len(B[0]))]
            for i in range(len(A))]


def _tr(A):
    return [list(r) for r in zip(*A)]


def face_lift_dense(N, num=float):
    """test/runtests.jl:34-40: Lf = [L0; l_1 E_N' L0; l_2 (E_N E_{N-1})' L0; ...]."""
    E1 = elevation_dense(N + 1, num)
    L0 = [[num((N + 1) ** 2) / num(2) * v for v in row] for row in _mm(_tr(E1), E1)]
    rows = [list(r) for r in L0]
    E = None
    for i in range(1, N + 1):
        Ei = elevation_dense(N + 1 - i, num)
        E = Ei if E is None else _mm(E, Ei)
        c = num((-1) ** i * comb(N, i)) / num(1 + i)
        blk = _mm(_tr(E), L0)
        rows += [[c * v for v in r] for r in blk]
    return rows


def _multinom(alpha):
    n = sum(alpha)
    out = factorial(n)
    for a in alpha:
        out //= factorial(a)
    return out


def mass(N, num=float):
    """Bernstein mass matrix on the reference tetrahedron (volume 4/3)."""
    L = lut3(N)
    scale = num(4) / num(3) / num(comb(2 * N + 3, 3))
    return [[scale * num(_multinom(a) * _multinom(b)) / num(
        _multinom(tuple(x + y for x, y in zip(a, b)))) for b in L] for a in L]


def _face_coords(f, alpha):
    """Face-local barycentric (a, b, c) of a 3D multi-index on face f (zero index dropped)."""
    i, j, k, l = alpha
    return ((i, k, l), (j, k, i), (j, k, l), (i, j, l))[f]


def _on_face(f, alpha):
    i, j, k, l = alpha
    return (j, l, i, k)[f] == 0


def face_mass(N, f, num=float):
    """int_face B_alpha phi_a over reference face f (measure of the reference triangle, 2)."""
    L, F = lut3(N), lut2(N)
    scale = num(2) / num(comb(2 * N + 2, 2))
    out = [[num(0)] * len(F) for _ in L]
    for m, a in enumerate(L):
        if not _on_face(f, a):
            continue
        a2 = _face_coords(f, a)
        for n, b in enumerate(F):
            out[m][n] = scale * num(_multinom(a2) * _multinom(b)) / num(
                _multinom(tuple(x + y for x, y in zip(a2, b))))
    return out


def _solve(A, B):
    """Gauss-Jordan solve A X = B (works for floats and Fractions)."""
    n = len(A)
    M = [list(A[i]) + list(B[i]) for i in range(n)]
    for c in range(n):
        p = max(range(c, n), key=lambda r: abs(M[r][c]))
        M[c], M[p] = M[p], M[c]
        piv = M[c][c]
        M[c] = [v / piv for v in M[c]]
        for r in range(n):
            if r != c and M[r][c] != 0:
                fct = M[r][c]
                M[r] = [vr - fct * vc for vr, vc in zip(M[r], M[c])]
    return [row[n:] for row in M]


def lift_from_mass(N, num=float):
    """M^{-1} [M^1 | M^2 | M^3 | M^4], shape Np x 4 Nfp (get_bernstein_lift semantics)."""
    if num is float:
        M = np.array(mass(N), dtype=np.float64)
        Mf = np.concatenate([np.array(face_mass(N, f), dtype=np.float64) for f in range(4)], 1)
        return np.linalg.solve(M, Mf)
    M = mass(N, num)
    Mf = [sum((face_mass(N, f, num)[r] for f in range(4)), []) for r in range(len(M))]
    return _solve(M, Mf)


def vandermonde_tet(N, l0, l1, l2, l3):
    """utility.jl:97-107: V and the four barycentric derivative matrices Vi, Vj, Vk, Vl."""
    L = lut3(N)
    V = np.zeros((len(l0), len(L)))
    D = [np.zeros_like(V) for _ in range(4)]
    lam = (l0, l1, l2, l3)
    for n, a in enumerate(L):
        V[:, n] = _multinom(a) * np.prod([lam[m] ** a[m] for m in range(4)], axis=0)
        for d in range(4):
            if a[d] > 0:
                b = list(a)
                b[d] -= 1
                D[d][:, n] = (factorial(N) / np.prod([factorial(x) for x in b])) * np.prod(
                    [lam[m] ** b[m] for m in range(4)], axis=0)
    return V, D


def deriv_from_vandermonde(N, seed=0):
    """V^{-1} dV/dr (and s, t) at random points: the runtests.jl:128-141 identity."""
    rng = np.random.default_rng(seed)
    Np = len(lut3(N))
    lam = rng.dirichlet(np.ones(4), size=Np).T
    V, (Vi, Vj, Vk, Vl) = vandermonde_tet(N, *lam)
    # lambda0 = (1+r)/2, lambda1 = (1+s)/2, lambda2 = (1+t)/2, lambda3 = -(1+r+s+t)/2
    return [np.linalg.solve(V, (Vd - Vl) / 2) for Vd in (Vi, Vj, Vk)]


def elevation3_dense(M, N):
    """3D degree elevation E (Np(N) x Np(M)): B^M_a = sum_g E[g, a] B^N_g."""
    LM, LN = lut3(M), lut3(N)
    E = np.zeros((len(LN), len(LM)))
    for a, al in enumerate(LM):
        for g, ga in enumerate(LN):
            d = tuple(x - y for x, y in zip(ga, al))
            if min(d) >= 0:
                E[g, a] = _multinom(al) * _multinom(d) / _multinom(ga)
    return E


def projection_dense(N, M):
    """L2 projection from degree N to M: P = M_MM^{-1} E_{M->N}^T M_NN (Np(M) x Np(N))."""
    E = elevation3_dense(M, N)
    return np.linalg.solve(np.array(mass(M)), E.T @ np.array(mass(N)))


def to_float(M):
    return np.array([[float(v) for v in row] for row in M], dtype=np.float64)


FR = Fraction
