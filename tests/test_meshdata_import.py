"""Import of a StartUpDG MeshData-shaped mesh that is not the generator's own.

StartUpDG hands the examples `rd.Fmask`, `md.mapP` and the affine metric terms
(examples/3d_wave.jl:89-97, `md.mapP` used at :45). A uniform Kuhn mesh exercises little of
that: every element has the same J, the same normals up to sign, and its faces meet in only
two of the six orientations. The mesh here is scrambled (oracle/meshdata.py::scrambled):
each element's vertices re-listed by a random even permutation, the elements shuffled, and
every lattice vertex moved by a random offset, so J, the metric terms and the normals vary per
element and all six orientation codes occur. `mapP` is matched by node coordinates in the
oracle, independently of the library; `bb_conn_from_mapP` and `bb_geo_from_meshdata` turn it
into the solver's records, and the GPU right-hand side and LSRK45 steps on that mesh are
checked against the oracle (dividing by each element's own J, where the examples divide by
the constant md.J[1,1] of their uniform meshes). Tolerances, relative l2 per field: 1e-12 in
FP64, 1e-5 in FP32.
"""
import numpy as np
import pytest

from oracle import meshdata


def _imported(bb, n, N, seed):
    from bbdg.mesh import from_meshdata
    lm = meshdata.scrambled(bb.uniform_tet_mesh(n), seed)
    md = meshdata.build(lm, N)
    nJ = md.nJ.reshape(lm.K, 4, bb.np2(N), 3)[:, :, 0, :]   # face-constant on affine faces
    return lm, md, from_meshdata(N, md.Fmask, md.mapP, md.geo9, nJ, md.Jall, h=lm.h)


@pytest.mark.parametrize("N", [2, 5])
def test_scrambled_import_has_every_orientation_and_exact_geometry(bb, N):
    from bbdg.mesh import geometric_factors
    lm, md, mesh = _imported(bb, 4, N, seed=11)
    assert set(np.unique(mesh.orient)) == set(range(6))
    K = mesh.K
    assert np.all(mesh.nbr[mesh.nbr, mesh.nbr_face] == np.arange(K)[:, None])
    assert np.all(mesh.nbr_face[mesh.nbr, mesh.nbr_face] == np.arange(4)[None, :])
    assert md.Jall.max() / md.Jall.min() > 1.5           # elements differ in size
    # cofactor geometry imported by the library == inverse-matrix geometry of the vertices
    assert np.allclose(mesh.geo, geometric_factors(lm.EVX), rtol=1e-12, atol=1e-13)


def per_field_rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.array([np.linalg.norm(a[f] - b[f]) / max(np.linalg.norm(b[f]), 1e-300)
                     for f in range(a.shape[0])])


@pytest.mark.gpu
@pytest.mark.parametrize("physics", ["wave", "maxwell"])
@pytest.mark.parametrize("N", [3, 5, 9])
def test_gpu_solver_on_scrambled_import_matches_oracle(cuda, bb, oracle_cpu, N, physics):
    import torch
    lm, md, mesh = _imported(bb, 4, N, seed=N)
    phys = 0 if physics == "wave" else 1
    rng = np.random.default_rng(100 + N)
    nf = 4 if physics == "wave" else 6
    q0 = rng.uniform(-1, 1, (nf, mesh.K, bb.np3(N)))
    dt = 0.1 * lm.h / (N + 1) ** 2
    want_rhs = oracle_cpu.rhs(phys, N, q0, md, tau=1.0, per_element_J=True)
    want_q, _ = oracle_cpu.lsrk(phys, N, q0, md, dt, 3, tau=1.0, per_element_J=True)
    cases = [(torch.float64, "generic", 1e-12), (torch.float32, "generic", 1e-5)]
    if N in (5, 9):
        cases.append((torch.float32, "specialised", 1e-5))
    for dtype, kind, tol in cases:
        s = bb.DGSolver(mesh, N, physics, dtype=dtype, tau=1.0)
        s.set_kernel(kind)
        assert s.kernel == kind
        qd = torch.tensor(q0, dtype=dtype, device=cuda)
        err = per_field_rel(s.rhs(qd).cpu().numpy(), want_rhs)
        assert np.all(err < tol), (str(dtype), kind, "rhs", err)
        rd = torch.zeros_like(qd)
        s.run(qd, rd, dt, 3)
        err = per_field_rel(qd.cpu().numpy(), want_q)
        assert np.all(err < tol), (str(dtype), kind, "lsrk", err)
        s.close()
