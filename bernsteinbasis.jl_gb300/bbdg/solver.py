"""DG solvers for the wave, Maxwell and scalar advection examples on the GPU.

Replaces the examples' ``rhs_matvec!`` + ``solve(ODEProblem(...), Tsit5())`` loop
(examples/3d_wave.jl:36-84,:133-134; examples/3d_maxwell.jl:36-93,:137-138;
examples/3d_advec_scalar.jl:17-42,:84-85) with a fused RHS + 5-stage low-storage RK kernel
per stage, replayed from a CUDA graph per step.

State layout: a (nf, K, Np) CUDA tensor; field m is the reference's Np x K matrix of that
component (p, u, v, w for the wave equation; Hx, Hy, Hz, Ex, Ey, Ez for Maxwell; u for
advection).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .basis import project_fields
from .context import dtype_code, get_context, ptr, require_cuda, stream_handle
from .mesh import TetMesh
from .ordering import np3

PHYSICS = {"wave": (_lib.BB_WAVE, 4), "maxwell": (_lib.BB_MAXWELL, 6),
           "advection": (_lib.BB_ADVECTION, 1), "advection3": (_lib.BB_ADVECTION3, 3)}


class DGSolver:
    """Bernstein DG solver on an affine tetrahedral mesh.

    tau <= 0 evaluates the examples' interface flux exactly as written; tau > 0 scales the
    penalty terms by the face Jacobian (upwind penalty tau), which keeps fixed time steps
    dt ~ h/(N+1)^2 stable on refined meshes.
    """

    def __init__(self, mesh: TetMesh, N: int, physics: str = "wave",
                 dtype: torch.dtype = torch.float32, tau: float = 1.0, device=None):
        if physics not in PHYSICS:
            raise ValueError(f"physics must be one of {sorted(PHYSICS)}")
        self.mesh = mesh
        self.N = int(N)
        self.Np = np3(self.N)
        self.physics = physics
        self.phys_code, self.nf = PHYSICS[physics]
        self.dtype = dtype
        self.tau = float(tau)
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        self.ctx = get_context(self.device)
        self.K = mesh.K
        self.conn = torch.as_tensor(mesh.conn.reshape(-1), dtype=torch.int32).to(self.device)
        self.geo = torch.as_tensor(mesh.geo.reshape(-1), dtype=dtype).to(self.device)
        h = ctypes.c_void_p()
        self.ctx.check(_lib.load().bb_solver_create(
            self.ctx.handle, self.phys_code, self.N, self.K, dtype_code(dtype), ptr(self.conn),
            ptr(self.geo), self.tau, ctypes.byref(h)), "bb_solver_create")
        self.handle = h

    # ---- state helpers ---------------------------------------------------------------
    def zeros(self) -> torch.Tensor:
        return torch.zeros((self.nf, self.K, self.Np), dtype=self.dtype, device=self.device)

    def project(self, fields) -> torch.Tensor:
        """Bernstein coefficients of callables f(x, y, z) (host FP64, then uploaded)."""
        if len(fields) != self.nf:
            raise ValueError(f"{self.physics} needs {self.nf} fields")
        q = project_fields(self.mesh, self.N, fields)
        return torch.as_tensor(q, dtype=self.dtype).to(self.device)

    def dt_cfl(self, cfl: float = 0.25) -> float:
        """Time step cfl * h / (N+1)^2, h the hexahedron edge."""
        return cfl * self.mesh.h / (self.N + 1) ** 2

    def _check_state(self, *ts):
        require_cuda(*ts)
        for t in ts:
            if t.shape != (self.nf, self.K, self.Np) or t.dtype != self.dtype:
                raise ValueError(f"state must be ({self.nf}, {self.K}, {self.Np}) {self.dtype}")

    # ---- tiling ------------------------------------------------------------------------
    def set_tile(self, elems_per_block: int, threads: int = 0) -> None:
        self.ctx.check(_lib.load().bb_solver_set_tile(self.handle, int(elems_per_block),
                                                      int(threads)), "bb_solver_set_tile")

    def set_kernel(self, kind: str) -> None:
        """'specialised' (default: degree-specialised kernel when one exists) or 'generic'."""
        if kind not in ("specialised", "generic"):
            raise ValueError("kind must be 'specialised' or 'generic'")
        self.ctx.check(_lib.load().bb_solver_set_kernel(self.handle, int(kind == "generic")),
                       "bb_solver_set_kernel")

    @property
    def kernel(self) -> str:
        return "specialised" if _lib.load().bb_solver_get_kernel(self.handle) == 0 else "generic"

    @property
    def tile(self):
        e, t = ctypes.c_int(), ctypes.c_int()
        self.ctx.check(_lib.load().bb_solver_get_tile(self.handle, ctypes.byref(e),
                                                      ctypes.byref(t)))
        return e.value, t.value

    # ---- compute -----------------------------------------------------------------------
    def rhs(self, q: torch.Tensor, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """One evaluation of rhs_matvec!."""
        self._check_state(q)
        out = torch.empty_like(q) if out is None else out
        self._check_state(out)
        self.ctx.check(_lib.load().bb_rhs(self.handle, ptr(q), ptr(out), stream_handle(stream)),
                       "bb_rhs")
        return out

    def ode_rhs(self):
        """f(t, q) -> dq/dt for external integrators (the OrdinaryDiffEq `rhs_matvec!(du, u,
        params, t)` role): one bb_rhs per call on a device state, t unused (autonomous)."""
        def f(t, q):
            return self.rhs(q)
        return f

    def run(self, q: torch.Tensor, res: torch.Tensor, dt: float, nsteps: int,
            graph: bool = True, stream=None) -> None:
        """Advance q (and the LSRK register res) by nsteps steps in place."""
        self._check_state(q, res)
        self.ctx.check(_lib.load().bb_lsrk_run(self.handle, float(dt), int(nsteps), ptr(q),
                                               ptr(res), int(bool(graph)),
                                               stream_handle(stream)), "bb_lsrk_run")

    def check(self, stream=None) -> None:
        """Waits for the stream and raises BBError if a kernel of this solver reported a
        problem since the last check (BB_ERR_TIMEOUT: a bounded device wait ran out;
        BB_ERR_DEVICE: corrupt connectivity)."""
        self.ctx.check(_lib.load().bb_solver_check(self.handle, stream_handle(stream)),
                       "bb_solver_check")

    def run_host(self, q_host_in: torch.Tensor, q_host_out: torch.Tensor, q_dev: torch.Tensor,
                 res_dev: torch.Tensor, dt: float, nsteps: int, graph: bool = True,
                 stream=None) -> None:
        """Host-in/host-out variant: copy q in, advance, copy q out (stream-ordered).

        bb_lsrk_run_host pipelines the copies with the stages over element chunks; pass
        page-locked tensors (``Tensor.pin_memory()``) for the copies to overlap and, with
        ``graph`` and one step, for the call to be captured once and replayed."""
        self._check_state(q_dev, res_dev)
        for t in (q_host_in, q_host_out):
            if t.is_cuda or t.shape != q_dev.shape or t.dtype != self.dtype or not t.is_contiguous():
                raise ValueError("host buffers must be contiguous CPU tensors like the state")
        self.ctx.check(_lib.load().bb_lsrk_run_host(
            self.handle, float(dt), int(nsteps), ctypes.c_void_p(q_host_in.data_ptr()),
            ctypes.c_void_p(q_host_out.data_ptr()), ptr(q_dev), ptr(res_dev), int(bool(graph)),
            stream_handle(stream)), "bb_lsrk_run_host")

    # ---- diagnostics -------------------------------------------------------------------
    def norms(self, a: torch.Tensor, b: torch.Tensor | None = None, stream=None) -> np.ndarray:
        """(nf, 3): sum a^2, sum (a-b)^2, sum b^2 per field (FP64 reductions)."""
        return norms(a, b, self.N, stream=stream)

    def mass_norms(self, a: torch.Tensor, b: torch.Tensor | None = None,
                   stream=None) -> np.ndarray:
        """Per field sum_e J_e (a-b)_e^T M (a-b)_e, M the Bernstein mass matrix."""
        self._check_state(a)
        if b is not None:
            self._check_state(b)
        out = (ctypes.c_double * self.nf)()
        self.ctx.check(_lib.load().bb_mass_norms(
            self.ctx.handle, self.N, self.K, self.nf, dtype_code(self.dtype), ptr(a), ptr(b),
            ptr(self.geo), out, stream_handle(stream)), "bb_mass_norms")
        return np.array(out[:])

    def energy(self, q: torch.Tensor) -> float:
        """0.5 * integral of the squared fields (the wave / Maxwell energy)."""
        return 0.5 * float(self.mass_norms(q).sum())

    # ---- checkpoints ---------------------------------------------------------------------
    def mesh_fingerprint(self) -> str:
        """Hash of the connectivity and geometry records: a checkpoint fits this mesh only."""
        import hashlib
        h = hashlib.sha1()
        h.update(np.ascontiguousarray(self.mesh.conn, dtype=np.int32).tobytes())
        h.update(np.ascontiguousarray(self.mesh.geo, dtype=np.float64).tobytes())
        return h.hexdigest()[:20]

    def save_state(self, path: str, q: torch.Tensor, res: torch.Tensor, t: float = 0.0,
                   step: int = 0, as_fp64: bool = False) -> None:
        """Writes q, the LSRK register res, the time and the step count to an .npz file,
        in the solver's dtype or (as_fp64) widened to FP64, so that a run can resume, or an
        FP64 state can seed FP32 checks from the same point."""
        self._check_state(q, res)
        cast = (lambda x: x.double()) if as_fp64 else (lambda x: x)
        np.savez(path, q=cast(q).cpu().numpy(), res=cast(res).cpu().numpy(), t=float(t),
                 step=int(step), N=self.N, physics=self.physics, tau=self.tau,
                 mesh=self.mesh_fingerprint(), dtype=str(self.dtype))

    def load_state(self, path: str):
        """Reads a checkpoint of save_state into new device tensors of this solver's dtype.
        Returns (q, res, t, step). Raises ValueError if it was written for another degree,
        physics, penalty or mesh."""
        z = np.load(path if path.endswith(".npz") else path + ".npz")
        want = (self.N, self.physics, self.tau, self.mesh_fingerprint())
        got = (int(z["N"]), str(z["physics"]), float(z["tau"]), str(z["mesh"]))
        if got != want:
            raise ValueError(f"checkpoint {got} does not match this solver {want}")
        q = torch.as_tensor(z["q"]).to(device=self.device, dtype=self.dtype).contiguous()
        res = torch.as_tensor(z["res"]).to(device=self.device, dtype=self.dtype).contiguous()
        self._check_state(q, res)
        return q, res, float(z["t"]), int(z["step"])

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.load().bb_solver_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def norms(a: torch.Tensor, b: torch.Tensor | None, N: int, stream=None) -> np.ndarray:
    """(nf, 3) FP64 sums for a state-shaped (nf, K, Np) tensor a (and optional b)."""
    require_cuda(a)
    if b is not None:
        require_cuda(b)
        if b.shape != a.shape or b.dtype != a.dtype:
            raise ValueError("a and b must match")
    nf, K, Np = a.shape
    if Np != np3(N):
        raise ValueError("last dimension must be Np")
    ctx = get_context(a.device)
    out = (ctypes.c_double * (3 * nf))()
    ctx.check(_lib.load().bb_norms(ctx.handle, int(N), int(K), int(nf), dtype_code(a.dtype),
                                   ptr(a), ptr(b), out, stream_handle(stream)), "bb_norms")
    return np.array(out[:]).reshape(nf, 3)


def relative_l2(a: torch.Tensor, b: torch.Tensor, N: int) -> np.ndarray:
    """Per-field relative l2 error ||a - b|| / ||b|| of Bernstein coefficients."""
    s = norms(a, b, N)
    return np.sqrt(s[:, 1] / np.maximum(s[:, 2], 1e-300))
