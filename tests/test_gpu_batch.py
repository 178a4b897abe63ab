"""Batched persistent solves (bb_batch_*) against single-problem solves and the oracle."""
import numpy as np
import pytest

from oracle import cpu, meshdata

pytestmark = pytest.mark.gpu


def specs():
    from bbdg.batch import ProblemSpec
    return [ProblemSpec("wave", 2, 2, seed=1), ProblemSpec("maxwell", 3, 2, seed=2),
            ProblemSpec("wave", 5, 3, seed=3), ProblemSpec("maxwell", 4, 2, seed=4),
            ProblemSpec("advection", 6, 2, seed=6), ProblemSpec("wave", 9, 2, seed=5)]


def test_batch_matches_single_solves_and_oracle(cuda, bb):
    import torch
    from bbdg.batch import BatchSolver
    B = BatchSolver(specs(), dtype=torch.float64)
    q0 = [q.clone() for q in B.q]
    B.set_tile("wave", 5, 2)          # a non-default tile for one degree
    B.run(3, graph=True)
    torch.cuda.synchronize()
    for p, spec in enumerate(B.specs):
        mesh = B.meshes[p]
        s = bb.DGSolver(mesh, spec.N, spec.physics, dtype=torch.float64, tau=spec.tau)
        s.set_kernel("generic")
        s.set_tile(B.tile(spec.physics, spec.N), 256)
        q = q0[p].clone()
        r = torch.zeros_like(q)
        s.run(q, r, B.dt(p), 3, graph=False)
        torch.cuda.synchronize()
        assert torch.equal(q, B.q[p]), p          # same tile code -> bitwise equal
        code = {"wave": 0, "maxwell": 1, "advection": 2}[spec.physics]
        want, _ = cpu.lsrk(code, spec.N, q0[p].cpu().numpy(),
                           meshdata.build(mesh, spec.N), B.dt(p), 3, tau=spec.tau)
        got = B.q[p].cpu().numpy()
        for f in range(got.shape[0]):
            if np.linalg.norm(want[f]) > 0:
                err = np.linalg.norm(got[f] - want[f]) / np.linalg.norm(want[f])
                assert err < 1e-12, (p, f, err)


def test_batch_graph_equals_stream_fp32(cuda, bb):
    import torch
    from bbdg.batch import BatchSolver
    A = BatchSolver(specs(), dtype=torch.float32)
    B = BatchSolver(specs(), dtype=torch.float32)
    A.run(4, graph=True)
    B.run(2, graph=False)
    B.run(2, graph=False)
    torch.cuda.synchronize()
    for qa, qb in zip(A.q, B.q):
        assert torch.equal(qa, qb)


def test_batch_fast_lanes_match_single_solves(cuda, bb):
    """FP32: problems with a degree-specialised kernel for their (N, physics, K) run it as
    fast lanes on side streams, the others the batched generic kernel; every problem ends
    bitwise equal to a single solver making the same kernel choice (graph replay)."""
    import torch
    from bbdg.batch import BatchSolver, ProblemSpec
    sp = specs() + [ProblemSpec("maxwell", 9, 2, seed=7), ProblemSpec("wave", 6, 3, seed=8),
                    ProblemSpec("wave", 7, 2, seed=9)]
    B = BatchSolver(sp, dtype=torch.float32)
    q0 = [q.clone() for q in B.q]
    B.run(3, graph=True)
    torch.cuda.synchronize()
    kinds = set()
    for p, spec in enumerate(B.specs):
        s = bb.DGSolver(B.meshes[p], spec.N, spec.physics, dtype=torch.float32, tau=spec.tau)
        if s.kernel == "generic":
            s.set_tile(B.tile(spec.physics, spec.N), 256)
        kinds.add(s.kernel)
        q = q0[p].clone()
        r = torch.zeros_like(q)
        s.run(q, r, B.dt(p), 3, graph=True)
        torch.cuda.synchronize()
        assert torch.equal(q, B.q[p]), (p, s.kernel)
    assert kinds == {"generic", "specialised"}
