"""Batched uneven solves: many wave / Maxwell problems in one persistent launch per stage.

Host side of bb_batch_* (include/bbdg.h). Each problem has its own mesh, degree, physics,
time step and state; the library advances all of them together. ``config4_problems`` draws
the benchmark's set of 48 problems (seed 2): wave or Maxwell with probability 1/2, degree
uniform in 4..11, an n^3-hexahedron cube with n uniform in 4..20, Gaussian-pulse initial
states, dt = 0.25 h/(N+1)^2.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .basis import gaussian_pulses, project_fields
from .context import dtype_code, get_context, stream_handle
from .mesh import uniform_tet_mesh
from .ordering import np3

PHYS_CODE = {"wave": _lib.BB_WAVE, "maxwell": _lib.BB_MAXWELL, "advection": _lib.BB_ADVECTION}
NFIELDS = {"wave": 4, "maxwell": 6, "advection": 1}


@dataclass
class ProblemSpec:
    physics: str
    N: int
    n: int           # hexahedra per direction
    seed: int        # initial-state seed
    tau: float = 1.0
    cfl: float = 0.25


def config4_problems(seed: int = 2, count: int = 48):
    rng = np.random.default_rng(seed)
    specs = []
    for p in range(count):
        physics = "wave" if rng.random() < 0.5 else "maxwell"
        N = int(rng.integers(4, 12))
        n = int(rng.integers(4, 21))
        specs.append(ProblemSpec(physics, N, n, seed=1000 * seed + p))
    return specs


def initial_state(spec: ProblemSpec, mesh) -> np.ndarray:
    """Gaussian-pulse sum in p (wave), E_z (Maxwell) or u (advection), the other fields zero
    (FP64)."""
    zero = lambda x, y, z: 0 * x  # noqa: E731
    f = gaussian_pulses(spec.seed)
    nf = NFIELDS[spec.physics]
    fields = {"wave": [f] + [zero] * 3, "maxwell": [zero] * 5 + [f], "advection": [f]}[spec.physics]
    assert len(fields) == nf
    return project_fields(mesh, spec.N, fields)


class BatchSolver:
    """All problems of ``specs`` on one device; states are (nf, K, Np) tensors in ``q``."""

    def __init__(self, specs, dtype: torch.dtype = torch.float32, device=None, states=None):
        self.specs = list(specs)
        self.dtype = dtype
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        self.ctx = get_context(self.device)
        self.meshes, self.q, self.res, self._keep = [], [], [], []
        probs = (_lib.BatchProblem * len(self.specs))()
        for p, spec in enumerate(self.specs):
            mesh = uniform_tet_mesh(spec.n)
            self.meshes.append(mesh)
            conn = torch.as_tensor(mesh.conn.reshape(-1), dtype=torch.int32).to(self.device)
            geo = torch.as_tensor(mesh.geo.reshape(-1), dtype=dtype).to(self.device)
            q0 = initial_state(spec, mesh) if states is None else states[p]
            q = torch.as_tensor(q0, dtype=dtype).to(self.device).contiguous()
            res = torch.zeros_like(q)
            self.q.append(q)
            self.res.append(res)
            self._keep += [conn, geo]
            probs[p] = _lib.BatchProblem(PHYS_CODE[spec.physics], spec.N, mesh.K,
                                         conn.data_ptr(), geo.data_ptr(), q.data_ptr(),
                                         res.data_ptr(), self.dt(p), spec.tau)
        h = ctypes.c_void_p()
        self.ctx.check(_lib.load().bb_batch_create(self.ctx.handle, len(self.specs), probs,
                                                   dtype_code(dtype), ctypes.byref(h)),
                       "bb_batch_create")
        self.handle = h

    def dt(self, p: int) -> float:
        s = self.specs[p]
        return s.cfl * self.meshes[p].h / (s.N + 1) ** 2

    def dofs(self) -> int:
        return sum(NFIELDS[s.physics] * np3(s.N) * m.K for s, m in zip(self.specs, self.meshes))

    def set_tile(self, physics: str, N: int, elems_per_block: int) -> None:
        self.ctx.check(_lib.load().bb_batch_set_tile(self.handle, PHYS_CODE[physics], int(N),
                                                     int(elems_per_block)), "bb_batch_set_tile")

    def tile(self, physics: str, N: int) -> int:
        e = ctypes.c_int()
        self.ctx.check(_lib.load().bb_batch_get_tile(self.handle, PHYS_CODE[physics], int(N),
                                                     ctypes.byref(e)), "bb_batch_get_tile")
        return e.value

    def run(self, nsteps: int, graph: bool = True, stream=None) -> None:
        self.ctx.check(_lib.load().bb_batch_run(self.handle, int(nsteps), int(bool(graph)),
                                                stream_handle(stream)), "bb_batch_run")

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.load().bb_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
