"""Multi-index ordering and lift-chain constants (host side).

Mirrors ``src/ordering.jl:6-39`` and ``src/constants.jl:10-16`` of BernsteinBasis.jl.
The Julia functions are 1-based; the ``*_to_linear`` functions here keep that convention so
that code written against the reference reads the same, and ``*_to_linear0`` give 0-based
indices for array work. Degrees up to 20 are supported, as in the reference tables.
"""
from __future__ import annotations

from functools import lru_cache
from math import comb

import numpy as np

MAX_N = 20


def np2(N: int) -> int:
    """Number of 2D Bernstein coefficients of degree N: (N+1)(N+2)/2."""
    return (N + 1) * (N + 2) // 2


def np3(N: int) -> int:
    """Number of 3D Bernstein coefficients of degree N: (N+1)(N+2)(N+3)/6."""
    return (N + 1) * (N + 2) * (N + 3) // 6


@lru_cache(maxsize=None)
def tri_offsets(N: int) -> tuple:
    """ordering.jl:8-16: 21 running row offsets of the degree-N triangle."""
    tup, count = [0], 0
    for i in range(1, 21):
        count += N + 2 - i
        tup.append(count)
    return tuple(tup)


@lru_cache(maxsize=None)
def tet_offsets(N: int) -> tuple:
    """ordering.jl:18-26: 21 running layer offsets of the degree-N tetrahedron."""
    tup, count = [0], 0
    for i in range(1, 21):
        count += (N + 2 - i) * (N + 3 - i) // 2
        tup.append(count)
    return tuple(tup)


def ij_to_linear(i: int, j: int, tri_offset) -> int:
    """ordering.jl:6 (1-based result)."""
    return i + tri_offset[j] + 1


def ijk_to_linear(i: int, j: int, k: int, tri_offset, tet_offset) -> int:
    """ordering.jl:32-35 (1-based result)."""
    return i + tri_offset[j] + 1 + tet_offset[k] - j * k


def ij_to_linear0(i: int, j: int, tri_offset) -> int:
    return i + tri_offset[j]


def ijk_to_linear0(i: int, j: int, k: int, tri_offset, tet_offset) -> int:
    return i + tri_offset[j] + tet_offset[k] - j * k


@lru_cache(maxsize=None)
def linear_to_ijkl_lookup(N: int) -> tuple:
    """ordering.jl:37-39: (i, j, k, l) of every 3D coefficient, in storage order."""
    return tuple((i, j, k, N - i - j - k)
                 for k in range(N + 1) for j in range(N + 1 - k) for i in range(N + 1 - j - k))


@lru_cache(maxsize=None)
def bernstein_2d_multiindex(N: int) -> tuple:
    """ordering.jl:47-51 (first return value): (i, j, k) of every 2D coefficient."""
    return tuple((i, j, N - i - j) for j in range(N + 1) for i in range(N + 1 - j))


def l_j(N: int) -> tuple:
    """constants.jl:10-12: the 20 lift-chain scalars (-1)^j C(N,j)/(1+j), zero past N."""
    return tuple(((-1.0 if j % 2 else 1.0) * comb(N, j) / (1.0 + j)) if j <= N else 0.0
                 for j in range(1, 21))


@lru_cache(maxsize=None)
def face_node_volume_index(N: int) -> np.ndarray:
    """0-based volume index of every face node, faces in reference order (4, Nfp).

    Face f's node (a, b) (b outer, a inner) sits on the face where one barycentric index is
    zero; the maps follow the index permutations of BernsteinLift.jl:207-218:
    f1: (a, 0, b), f2: (N-a-b, a, b), f3: (0, a, b), f4: (a, b, 0) as (i, j, k).
    The same node list is StartUpDG's Fmask for the Bernstein coefficients.
    """
    to, te = tri_offsets(N), tet_offsets(N)
    out = np.zeros((4, np2(N)), dtype=np.int32)
    for n, (a, b, _c) in enumerate(bernstein_2d_multiindex(N)):
        out[0, n] = ijk_to_linear0(a, 0, b, to, te)
        out[1, n] = ijk_to_linear0(N - a - b, a, b, to, te)
        out[2, n] = ijk_to_linear0(0, a, b, to, te)
        out[3, n] = ijk_to_linear0(a, b, 0, to, te)
    return out
