"""StartUpDG-style MeshData for the oracle -- TEST INFRASTRUCTURE ONLY.

Restates what the reference examples take from StartUpDG (examples/3d_wave.jl:89-97 and the
``md`` fields used at :41-83): ``Fmask`` (face nodes in volume-index order, faces
s=-1, r+s+t=-1, r=-1, t=-1), ``mapP`` (the neighbour's face node at the same physical point,
periodic), the affine metric terms ``rxJ..tzJ``, scaled normals ``nxJ, nyJ, nzJ`` and ``J``.
mapP is found here by matching node coordinates, independently of the compact
face/orientation connectivity the product kernels use.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def _lut(N):
    return [(i, j, k, N - i - j - k)
            for k in range(N + 1) for j in range(N + 1 - k) for i in range(N + 1 - j - k)]


def fmask(N: int) -> np.ndarray:
    """Face node volume indices (4*Nfp,), StartUpDG face order, ascending within a face."""
    lut = _lut(N)
    faces = [[n for n, (i, j, k, l) in enumerate(lut) if j == 0],   # s = -1
             [n for n, (i, j, k, l) in enumerate(lut) if l == 0],   # r + s + t = -1
             [n for n, (i, j, k, l) in enumerate(lut) if i == 0],   # r = -1
             [n for n, (i, j, k, l) in enumerate(lut) if k == 0]]   # t = -1
    return np.array(sum(faces, []), dtype=np.int32)


# Scaled reference normals of the four faces (nrJ, nsJ, ntJ).
_NREF = np.array([(0, -1, 0), (1, 1, 1), (-1, 0, 0), (0, 0, -1)], dtype=np.float64)


@dataclass
class MeshData:
    N: int
    K: int
    Fmask: np.ndarray   # (4*Nfp,) int32
    mapP: np.ndarray    # (K*4*Nfp,) int64 global face-node index
    geo9: np.ndarray    # (K, 9) rxJ, sxJ, txJ, ryJ, syJ, tyJ, rzJ, szJ, tzJ
    nJ: np.ndarray      # (K, 4*Nfp, 3) nxJ, nyJ, nzJ at every face node
    J: float            # md.J[1,1]
    Jall: np.ndarray    # (K,) per-element Jacobian


def geometric_factors(EVX: np.ndarray):
    """Affine metric terms (cofactor form) for vertices in StartUpDG order."""
    X1, X2, X3, X4 = (EVX[:, m, :] for m in range(4))
    xr, yr, zr = ((X2 - X1) / 2).T
    xs, ys, zs = ((X3 - X1) / 2).T
    xt, yt, zt = ((X4 - X1) / 2).T
    J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt)
    rxJ, ryJ, rzJ = ys * zt - zs * yt, -(xs * zt - zs * xt), xs * yt - ys * xt
    sxJ, syJ, szJ = -(yr * zt - zr * yt), xr * zt - zr * xt, -(xr * yt - yr * xt)
    txJ, tyJ, tzJ = yr * zs - zr * ys, -(xr * zs - zr * xs), xr * ys - yr * xs
    geo9 = np.stack([rxJ, sxJ, txJ, ryJ, syJ, tyJ, rzJ, szJ, tzJ], axis=1)
    return geo9, J


def build(mesh, N: int) -> MeshData:
    """MeshData of a periodic lattice mesh (vertex lattice coordinates mesh.EVI, period n)."""
    K, n = mesh.K, mesh.n
    Fm = fmask(N)
    Nfp = (N + 1) * (N + 2) // 2
    NfpT = 4 * Nfp
    lut = np.array(_lut(N), dtype=np.int64)            # (Np, 4) i, j, k, l
    # lattice coordinate (units h/N) of node (i,j,k,l): i*X2 + j*X3 + k*X4 + l*X1
    W = np.stack([lut[:, 3], lut[:, 0], lut[:, 1], lut[:, 2]], axis=1)   # weights on X1..X4
    P = np.einsum("pm,kmc->kpc", W, mesh.EVI)          # (K, Np, 3)
    Pf = P[:, Fm, :]                                   # (K, NfpT, 3)
    period = n * N
    Pw = np.mod(Pf, period)
    # face pairing: faces are matched by the wrapped lattice coordinates of their centroid
    cent = np.mod(Pf.reshape(K, 4, Nfp, 3).sum(axis=2) * 3, 3 * Nfp * period)
    ckey = (cent[..., 0] * (3 * Nfp * period) + cent[..., 1]) * (3 * Nfp * period) + cent[..., 2]
    flat = ckey.reshape(-1)
    order = np.argsort(flat, kind="stable")
    assert np.all(flat[order][0::2] == flat[order][1::2]), "unpaired face"
    partner = np.empty_like(order)
    partner[order[0::2]] = order[1::2]
    partner[order[1::2]] = order[0::2]
    # node matching inside each face pair by wrapped lattice coordinates
    nkey = (Pw[..., 0] * period + Pw[..., 1]) * period + Pw[..., 2]   # (K, NfpT)
    nkey = nkey.reshape(K * 4, Nfp)
    mine = nkey
    theirs = nkey[partner]
    pos_m = np.argsort(mine, axis=1)
    pos_t = np.argsort(theirs, axis=1)
    assert np.all(np.take_along_axis(mine, pos_m, 1) == np.take_along_axis(theirs, pos_t, 1))
    match = np.empty_like(pos_m)                       # node a of face side -> node of partner
    rows = np.arange(K * 4)[:, None]
    match[rows, pos_m] = pos_t
    mapP = (partner[:, None] // 4) * NfpT + (partner[:, None] % 4) * Nfp + match
    geo9, Jall = geometric_factors(mesh.EVX)
    nJ = np.empty((K, NfpT, 3))
    for f in range(4):
        nr, ns, nt = _NREF[f]
        for c in range(3):
            nJ[:, f * Nfp:(f + 1) * Nfp, c] = (geo9[:, 3 * c] * nr + geo9[:, 3 * c + 1] * ns
                                                + geo9[:, 3 * c + 2] * nt)[:, None]
    return MeshData(N=N, K=K, Fmask=Fm, mapP=np.ascontiguousarray(mapP.reshape(-1), np.int64),
                    geo9=np.ascontiguousarray(geo9), nJ=np.ascontiguousarray(nJ),
                    J=float(Jall[0]), Jall=Jall)


@dataclass
class LatticeMesh:
    """Vertex arrays of an affine tetrahedral mesh on a periodic vertex lattice: the fields
    `build` reads (K, n, EVI lattice coordinates, EVX physical coordinates)."""
    n: int
    K: int
    h: float
    EVI: np.ndarray
    EVX: np.ndarray


_EVEN_PERMS = [p for p in __import__("itertools").permutations(range(4))
               if sum(p[i] > p[j] for i in range(4) for j in range(i + 1, 4)) % 2 == 0]


def scrambled(mesh, seed: int, jitter: float = 0.15) -> LatticeMesh:
    """A mesh that is not the generator's own: each element's vertices re-listed by a random
    even permutation (so faces meet in every orientation), the elements shuffled, and every
    lattice vertex moved by a random offset of up to jitter*h per coordinate (the same offset
    for a vertex and its periodic images, so the mesh stays conforming and periodic; the
    elements stay affine but differ in size and shape)."""
    rng = np.random.default_rng(seed)
    K, n, h = mesh.K, mesh.n, 2.0 / mesh.n
    perm = np.array(_EVEN_PERMS)[rng.integers(0, len(_EVEN_PERMS), K)]     # (K, 4)
    EVI = np.take_along_axis(mesh.EVI, perm[:, :, None], axis=1)
    order = rng.permutation(K)
    EVI = EVI[order]
    w = np.mod(EVI, n)
    vid = w[..., 0] + n * (w[..., 1] + n * w[..., 2])
    delta = rng.uniform(-jitter * h, jitter * h, (n ** 3, 3))
    EVX = -1.0 + h * EVI.astype(np.float64) + delta[vid]
    return LatticeMesh(n=n, K=K, h=h, EVI=np.ascontiguousarray(EVI), EVX=EVX)
