"""ctypes wrapper of the C++ oracle (bbdg_oracle.cpp) -- TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes

import numpy as np

from . import build as _build

_lib = None

_P = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        I, D, F = ctypes.c_int, ctypes.c_double, ctypes.c_float
        L.oracle_max_threads.restype = I
        L.oracle_offsets.argtypes = [I, _P, _P]
        L.oracle_l_j.argtypes = [I, I]
        L.oracle_l_j.restype = D
        for name in ("oracle_deriv_f64", "oracle_deriv_f32"):
            getattr(L, name).argtypes = [I, I, I, _P, _P]
        for name in ("oracle_elevation_f64", "oracle_reduction_f64", "oracle_face_lift_f64"):
            getattr(L, name).argtypes = [I, _P, _P]
        L.oracle_lift_f64.argtypes = [I, I, _P, _P, I]
        L.oracle_lift_f32.argtypes = [I, I, _P, _P, I]
        L.oracle_rhs_f64.argtypes = [I, I, I, _P, _P, _P, _P, _P, _P, D, _P, D, I]
        L.oracle_rhs_f32.argtypes = [I, I, I, _P, _P, _P, _P, _P, _P, F, _P, F, I]
        L.oracle_rhs_f64.restype = I
        L.oracle_rhs_f32.restype = I
        L.oracle_lsrk_f64.argtypes = [I, I, I, _P, _P, _P, _P, _P, _P, D, _P, D, D, I, I]
        L.oracle_lsrk_f32.argtypes = [I, I, I, _P, _P, _P, _P, _P, _P, F, _P, F, F, I, I]
        L.oracle_lsrk_f64.restype = I
        L.oracle_lsrk_f32.restype = I
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_P)


def max_threads() -> int:
    return lib().oracle_max_threads()


def offsets(N: int):
    tri = np.zeros(21, np.int32)
    tet = np.zeros(21, np.int32)
    lib().oracle_offsets(N, _ptr(tri), _ptr(tet))
    return tri, tet


def l_j(N: int, j: int) -> float:
    return lib().oracle_l_j(N, j)


def deriv(axis: int, N: int, x: np.ndarray) -> np.ndarray:
    """Dr/Ds/Dt (axis 0/1/2) applied column-wise to x of shape (K, Np) (Julia Np x K)."""
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    K = x.shape[0] if x.ndim == 2 else 1
    fn = lib().oracle_deriv_f64 if x.dtype == np.float64 else lib().oracle_deriv_f32
    fn(axis, N, K, _ptr(x), _ptr(out))
    return out


def elevation(N: int, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty((N + 2) * (N + 3) // 2)
    lib().oracle_elevation_f64(N, _ptr(x), _ptr(out))
    return out


def reduction(N: int, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty(N * (N + 1) // 2)
    lib().oracle_reduction_f64(N, _ptr(x), _ptr(out))
    return out


def face_lift(N: int, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty((N + 1) * (N + 2) * (N + 3) // 6)
    lib().oracle_face_lift_f64(N, _ptr(x), _ptr(out))
    return out


def lift(N: int, x: np.ndarray, nthreads: int = 1) -> np.ndarray:
    """BernsteinLift mul! column-wise: x (K, 4*Nfp) -> (K, Np)."""
    x = np.ascontiguousarray(x)
    K = x.shape[0] if x.ndim == 2 else 1
    Np = (N + 1) * (N + 2) * (N + 3) // 6
    out = np.empty((K, Np), dtype=x.dtype)
    fn = lib().oracle_lift_f64 if x.dtype == np.float64 else lib().oracle_lift_f32
    fn(N, K, _ptr(x), _ptr(out), nthreads)
    return out if x.ndim == 2 else out[0]


def soa_to_aos(q: np.ndarray) -> np.ndarray:
    """(nf, K, Np) -> reference layout (K, Np, nf)."""
    return np.ascontiguousarray(np.transpose(q, (1, 2, 0)))


def aos_to_soa(q: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.transpose(q, (2, 0, 1)))


def _jall(md, dt_, per_element_J):
    """Per-element Jacobians (kept alive by the caller) or None for the examples' md.J[1,1]."""
    if not per_element_J:
        return None, None
    a = np.ascontiguousarray(md.Jall, dtype=dt_)
    return a, _ptr(a)


def rhs(phys: int, N: int, q_soa: np.ndarray, md, tau: float = 0.0,
        nthreads: int = 0, per_element_J: bool = False) -> np.ndarray:
    """Example right-hand side (wave phys=0, Maxwell phys=1, scalar advection phys=2,
    examples/3d_advec_scalar.jl, three-component advection phys=3, examples/3d_advec.jl) on
    SoA state (nf, K, Np).

    tau <= 0 evaluates the examples' flux as written; tau > 0 scales the penalty by the
    face Jacobian (upwind penalty tau). per_element_J divides by each element's own J instead
    of the examples' md.J[1,1] (the two agree on uniform meshes).
    """
    nthreads = nthreads or max_threads()
    dt_ = q_soa.dtype
    q = soa_to_aos(q_soa)
    du = np.empty_like(q)
    geo9 = np.ascontiguousarray(md.geo9, dtype=dt_)
    nJ = np.ascontiguousarray(md.nJ, dtype=dt_)
    K = q.shape[0]
    fn = lib().oracle_rhs_f64 if dt_ == np.float64 else lib().oracle_rhs_f32
    jall, jp = _jall(md, dt_, per_element_J)
    rc = fn(phys, N, K, _ptr(q), _ptr(du), _ptr(md.Fmask), _ptr(md.mapP), _ptr(geo9),
            _ptr(nJ), float(md.J), jp, float(tau), nthreads)
    assert rc == 0
    return aos_to_soa(du)


def lsrk(phys: int, N: int, q_soa: np.ndarray, md, dt: float, nsteps: int, tau: float = 0.0,
         nthreads: int = 0, res_soa: np.ndarray | None = None, per_element_J: bool = False):
    """Advance nsteps LSRK45 steps; returns (q, res) in SoA layout."""
    nthreads = nthreads or max_threads()
    dt_ = q_soa.dtype
    q = soa_to_aos(q_soa)
    res = np.zeros_like(q) if res_soa is None else soa_to_aos(res_soa.astype(dt_))
    geo9 = np.ascontiguousarray(md.geo9, dtype=dt_)
    nJ = np.ascontiguousarray(md.nJ, dtype=dt_)
    K = q.shape[0]
    fn = lib().oracle_lsrk_f64 if dt_ == np.float64 else lib().oracle_lsrk_f32
    jall, jp = _jall(md, dt_, per_element_J)
    rc = fn(phys, N, K, _ptr(q), _ptr(res), _ptr(md.Fmask), _ptr(md.mapP), _ptr(geo9),
            _ptr(nJ), float(md.J), jp, float(tau), float(dt), nsteps, nthreads)
    assert rc == 0
    return aos_to_soa(q), aos_to_soa(res)
