"""bbdg: GB300-native Bernstein DG hot path (host package over the libbbdg C ABI).

Drop-in for the hot path of vincentxwang/BernsteinBasis.jl: the operator types and their
mul! API (src/BernsteinBasis.jl:19-23), and the wave / Maxwell right-hand side and
low-storage RK time stepping of examples/3d_wave.jl and examples/3d_maxwell.jl. All compute
runs in libbbdg.so (hand-written CUDA for sm_103a); this package builds meshes and tables
on the host and passes device pointers through the C ABI.
"""
from .ordering import (MAX_N, np2, np3, tri_offsets, tet_offsets, ij_to_linear,
                       ijk_to_linear, linear_to_ijkl_lookup, bernstein_2d_multiindex, l_j)
from .mesh import TetMesh, uniform_tet_mesh, element_domain_points
from .basis import (bernstein_basis_tet, bernstein_basis_tri, nodal_to_bernstein,
                    project_fields, gaussian_pulses)
from ._lib import BBError


def __getattr__(name):
    # GPU-facing modules import torch lazily so the host-only parts stay light.
    if name in ("BernsteinDerivativeMatrix_3D_r", "BernsteinDerivativeMatrix_3D_s",
                "BernsteinDerivativeMatrix_3D_t", "BernsteinLift", "ElevationMatrix", "mul_",
                "elevation_multiply_", "reduction_multiply_", "face_lift_multiply_", "grad_",
                "fused_apply_"):
        from . import operators
        return getattr(operators, name)
    if name in ("DGSolver", "norms", "relative_l2"):
        from . import solver
        return getattr(solver, name)
    if name in ("Context", "get_context"):
        from . import context
        return getattr(context, name)
    raise AttributeError(name)
