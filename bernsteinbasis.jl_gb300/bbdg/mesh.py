"""Affine tetrahedral meshes, face connectivity and geometric factors (host side).

The reference takes its mesh from StartUpDG (``uniform_mesh(Tet(), n)`` with
``is_periodic=true``, examples/3d_wave.jl:95-97). This module builds the same kind of mesh
directly: the cube [-1, 1]^3 cut into n^3 hexahedra, each split into the 6 Kuhn tetrahedra
that share the hexahedron's main diagonal, periodic in x, y and z.

Element vertices follow StartUpDG's reference order: X1..X4 sit at reference coordinates
(-1,-1,-1), (1,-1,-1), (-1,1,-1), (-1,-1,1). Faces follow the reference face order
(s=-1, r+s+t=-1, r=-1, t=-1). Face f's node (a, b) with c = N-a-b is the domain point
(a*A + b*B + c*C)/N of the face's vertices (A, B, C) = FACE_VERTS[f].

Connectivity is stored compactly, one 32-bit word per face side:
``neighbour_element << 5 | neighbour_face << 3 | orientation``, where the orientation
indexes PERMS: face vertex m of this side is face vertex PERMS[o][m] of the neighbour side.
The kernels turn it into node indices on the fly, replacing StartUpDG's per-node ``mapP``.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass

import numpy as np

from .ordering import linear_to_ijkl_lookup

# Face-local vertices (A, B, C) of each reference face, as element-vertex numbers (0-based,
# StartUpDG order). f1: j=0, f2: l=0, f3: i=0, f4: k=0.
FACE_VERTS = ((1, 3, 0), (2, 3, 1), (2, 3, 0), (1, 2, 0))
# Scaled outward reference normals (nrJ, nsJ, ntJ) of the four faces.
REF_NORMALS = np.array([(0.0, -1.0, 0.0), (1.0, 1.0, 1.0), (-1.0, 0.0, 0.0), (0.0, 0.0, -1.0)])
PERMS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))
# Per-element geometry record: 9 scaled metric terms, 1/J, J, pad, 12 scaled face normals.
GEO_STRIDE = 24
GEO_RXJ, GEO_INVJ, GEO_J, GEO_NX, GEO_NY, GEO_NZ = 0, 9, 10, 12, 16, 20
MAX_K = 1 << 27


@dataclass
class TetMesh:
    n: int                 # hexahedra per direction
    K: int                 # elements
    h: float               # hexahedron edge length
    EVI: np.ndarray        # (K, 4, 3) int64 vertex lattice coordinates (units of h, unwrapped)
    EVX: np.ndarray        # (K, 4, 3) float64 vertex coordinates
    nbr: np.ndarray        # (K, 4) int64 neighbour element
    nbr_face: np.ndarray   # (K, 4) int64 neighbour face
    orient: np.ndarray     # (K, 4) int64 orientation code (index into PERMS)
    conn: np.ndarray       # (K, 4) int32 packed connectivity
    geo: np.ndarray        # (K, GEO_STRIDE) float64 geometry records

    @property
    def J(self) -> np.ndarray:
        return self.geo[:, GEO_J]


def _kuhn_tets():
    """Six Kuhn tetrahedra of the unit cube as 4 lattice corners each, positively oriented."""
    e = np.eye(3, dtype=np.int64)
    tets = []
    for p in itertools.permutations(range(3)):
        P0 = np.zeros(3, np.int64)
        P1 = e[p[0]]
        P2 = e[p[0]] + e[p[1]]
        P3 = np.ones(3, np.int64)
        X = [P0, P1, P2, P3]
        if np.linalg.det(np.stack([X[1] - X[0], X[2] - X[0], X[3] - X[0]], axis=1)) < 0:
            X[2], X[3] = X[3], X[2]
        tets.append(np.stack(X))
    return np.stack(tets)  # (6, 4, 3)


def _wrapped_vertex_ids(EVI, n):
    w = np.mod(EVI, n)
    return w[..., 0] + n * (w[..., 1] + n * w[..., 2])


def connect_faces(EVI: np.ndarray, n: int):
    """Match every face side with its periodic partner; return (nbr, nbr_face, orient)."""
    K = EVI.shape[0]
    vid = _wrapped_vertex_ids(EVI, n)                          # (K, 4)
    fv = np.stack([vid[:, list(FACE_VERTS[f])] for f in range(4)], axis=1)  # (K, 4, 3)
    # faces pair up by their lattice centroid A+B+C, wrapped by the period (exact integers;
    # distinct faces of a conforming mesh have distinct centroids)
    csum = np.stack([EVI[:, list(FACE_VERTS[f]), :].sum(axis=1) for f in range(4)], axis=1)
    cw = np.mod(csum, 3 * n)                                   # (K, 4, 3)
    P = np.int64(3 * n)
    key = (cw[..., 0] * P + cw[..., 1]) * P + cw[..., 2]       # (K, 4)
    flat = key.reshape(-1)
    order = np.argsort(flat, kind="stable")
    sk = flat[order]
    if sk.size % 2 or np.any(sk[0::2] != sk[1::2]) or (sk.size > 2 and np.any(sk[2::2] == sk[1:-1:2])):
        raise ValueError("mesh faces do not pair up; periodic meshes need n >= 2")
    a, b = order[0::2], order[1::2]
    partner = np.empty_like(order)
    partner[a] = b
    partner[b] = a
    nbr = (partner // 4).reshape(K, 4)
    nbr_face = (partner % 4).reshape(K, 4)
    # orientation: vertex m of this side equals vertex sigma[m] of the neighbour side
    mine = fv.reshape(-1, 3)
    theirs = fv.reshape(-1, 3)[partner]
    sigma = np.argmax(mine[:, :, None] == theirs[:, None, :], axis=2)  # (K*4, 3)
    ok = np.all(np.take_along_axis(theirs, sigma, axis=1) == mine, axis=1)
    if not np.all(ok):
        raise ValueError("face vertex sets of a face pair disagree")
    code = np.full(sigma.shape[0], -1, np.int64)
    for o, p in enumerate(PERMS):
        code[np.all(sigma == np.array(p), axis=1)] = o
    orient = code.reshape(K, 4)
    return nbr, nbr_face, orient


def pack_connectivity(nbr, nbr_face, orient) -> np.ndarray:
    if nbr.shape[0] >= MAX_K:
        raise ValueError(f"at most {MAX_K - 1} elements")
    return ((nbr.astype(np.int64) << 5) | (nbr_face.astype(np.int64) << 3)
            | orient.astype(np.int64)).astype(np.int32)


def geometric_factors(EVX: np.ndarray) -> np.ndarray:
    """Affine metric terms and scaled face normals, StartUpDG conventions (FP64)."""
    K = EVX.shape[0]
    X1, X2, X3, X4 = (EVX[:, m, :] for m in range(4))
    # d(x,y,z)/d(r,s,t): columns xr, xs, xt of the affine map x = X1 + sum (Xm - X1)(1+r)/2
    G = np.stack([(X2 - X1) / 2, (X3 - X1) / 2, (X4 - X1) / 2], axis=2)  # (K, 3, 3): G[:, c, rst]
    J = np.linalg.det(G)
    if np.any(J <= 0):
        raise ValueError("elements must be positively oriented")
    Ginv = np.linalg.inv(G)  # Ginv[:, rst, c] = d(rst)/d(xyz)
    geo = np.zeros((K, GEO_STRIDE))
    # (rxJ, sxJ, txJ, ryJ, syJ, tyJ, rzJ, szJ, tzJ)
    for c in range(3):          # x, y, z
        for r in range(3):      # r, s, t
            geo[:, GEO_RXJ + 3 * c + r] = Ginv[:, r, c] * J
    geo[:, GEO_INVJ] = 1.0 / J
    geo[:, GEO_J] = J
    for f in range(4):
        nr, ns, nt = REF_NORMALS[f]
        for c, base in enumerate((GEO_NX, GEO_NY, GEO_NZ)):
            geo[:, base + f] = (geo[:, 3 * c + 0] * nr + geo[:, 3 * c + 1] * ns
                                + geo[:, 3 * c + 2] * nt)
    return geo


def uniform_tet_mesh(n: int) -> TetMesh:
    """n^3 hexahedra on [-1,1]^3, 6 Kuhn tetrahedra each, periodic in x, y, z."""
    if n < 2:
        raise ValueError("n must be >= 2")
    tets = _kuhn_tets()                                              # (6, 4, 3)
    iz, iy, ix = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1)   # hex h = ix + n(iy + n iz)
    EVI = (base[:, None, None, :] + tets[None]).reshape(-1, 4, 3).astype(np.int64)
    h = 2.0 / n
    EVX = -1.0 + h * EVI.astype(np.float64)
    nbr, nbr_face, orient = connect_faces(EVI, n)
    return TetMesh(n=n, K=EVI.shape[0], h=h, EVI=EVI, EVX=EVX, nbr=nbr, nbr_face=nbr_face,
                   orient=orient, conn=pack_connectivity(nbr, nbr_face, orient),
                   geo=geometric_factors(EVX))


def reference_domain_points(N: int) -> np.ndarray:
    """Barycentric weights (Np, 4) of the degree-N domain points on vertices X1..X4.

    Coefficient (i, j, k, l) sits at lambda0 = i/N (vertex X2), lambda1 = j/N (X3),
    lambda2 = k/N (X4), lambda3 = l/N (X1).
    """
    lut = np.array(linear_to_ijkl_lookup(N), dtype=np.float64) / N   # (Np, 4): i, j, k, l
    return np.stack([lut[:, 3], lut[:, 0], lut[:, 1], lut[:, 2]], axis=1)


def element_domain_points(mesh: TetMesh, N: int) -> np.ndarray:
    """Physical coordinates (K, Np, 3) of every element's degree-N domain points."""
    W = reference_domain_points(N)                     # (Np, 4) on X1..X4
    return np.einsum("pm,kmc->kpc", W, mesh.EVX)


def from_meshdata(N: int, Fmask: np.ndarray, mapP: np.ndarray, rst9: np.ndarray,
                  nJ: np.ndarray, J: np.ndarray, h: float = 0.0) -> TetMesh:
    """A TetMesh from StartUpDG MeshData-shaped arrays (0-based): rd.Fmask (4*Nfp), md.mapP
    (K*4*Nfp, element-major), per-element metric terms (K, 9) in the order rxJ, sxJ, txJ,
    ryJ, syJ, tyJ, rzJ, szJ, tzJ, face-constant scaled normals (K, 4, 3) and J (K). The
    connectivity and geometry records are built by the library (bb_conn_from_mapP,
    bb_geo_from_meshdata); vertex arrays are not needed by the solver and are left empty."""
    import ctypes
    from . import _lib
    K = int(np.asarray(J).shape[0])
    fm = np.ascontiguousarray(Fmask, dtype=np.int32)
    mp = np.ascontiguousarray(mapP, dtype=np.int64).reshape(-1)
    conn = np.empty(K * 4, dtype=np.int32)
    L = _lib.load(build_if_missing=True)
    rc = L.bb_conn_from_mapP(int(N), K, fm.ctypes.data_as(ctypes.c_void_p),
                             mp.ctypes.data_as(ctypes.c_void_p),
                             conn.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise ValueError("mapP does not describe a conforming face pairing")
    r9 = np.ascontiguousarray(rst9, dtype=np.float64)
    n3 = np.ascontiguousarray(nJ, dtype=np.float64)
    jj = np.ascontiguousarray(J, dtype=np.float64)
    geo = np.empty((K, GEO_STRIDE), dtype=np.float64)
    rc = L.bb_geo_from_meshdata(K, _lib.BB_F64, r9.ctypes.data_as(ctypes.c_void_p),
                                n3.ctypes.data_as(ctypes.c_void_p),
                                jj.ctypes.data_as(ctypes.c_void_p),
                                geo.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise ValueError("bad geometry arrays")
    c64 = conn.astype(np.int64).reshape(K, 4)
    nbr, nbr_face, orient = c64 >> 5, (c64 >> 3) & 3, c64 & 7
    return TetMesh(n=0, K=K, h=h, EVI=np.zeros((K, 4, 3), np.int64),
                   EVX=np.zeros((K, 4, 3)), nbr=nbr, nbr_face=nbr_face, orient=orient,
                   conn=conn.reshape(K, 4), geo=geo)
