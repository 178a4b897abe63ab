"""GPU parity of the fused DG right-hand side and LSRK stepping vs the CPU oracle.

The oracle restates examples/3d_wave.jl:36-84 and examples/3d_maxwell.jl:36-93 loop for
loop (AoS SVector layout, Fmask/mapP gather, 9 derivative applies, BernsteinLift mul!).
Tolerances, relative l2 per field: FP64 1e-12, FP32 1e-5 (FP32 is checked against the
FP64 oracle).
"""
import numpy as np
import pytest

from oracle import meshdata

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-12, "f32": 1e-5}


def per_field_rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.array([np.linalg.norm(a[f] - b[f]) / max(np.linalg.norm(b[f]), 1e-300)
                     for f in range(a.shape[0])])


def tdt(name):
    import torch
    return torch.float64 if name == "f64" else torch.float32


def random_state(rng, nf, K, Np):
    return rng.uniform(-1, 1, (nf, K, Np))


@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("tau", [0.0, 1.0])
@pytest.mark.parametrize("physics", ["wave", "maxwell"])
@pytest.mark.parametrize("N", [1, 2, 3, 5, 7, 9])
def test_rhs_matches_oracle(cuda, bb, oracle_cpu, N, physics, tau, dt):
    import torch
    m = bb.uniform_tet_mesh(3)
    md = meshdata.build(m, N)
    s = bb.DGSolver(m, N, physics, dtype=tdt(dt), tau=tau)
    rng = np.random.default_rng(N * 7 + len(physics))
    q = random_state(rng, s.nf, m.K, s.Np)
    qd = torch.tensor(q, dtype=tdt(dt), device=cuda)
    got = s.rhs(qd).cpu().numpy()
    want = oracle_cpu.rhs(0 if physics == "wave" else 1, N, q, md, tau=tau)
    err = per_field_rel(got, want)
    assert np.all(err < TOL[dt]), err


@pytest.mark.parametrize("epb", [1, 2, 4, 5, 6, 12, 18])
def test_tiling_does_not_change_results(cuda, bb, epb):
    import torch
    m = bb.uniform_tet_mesh(3)
    N = 4
    s = bb.DGSolver(m, N, "maxwell", dtype=torch.float64, tau=1.0)
    rng = np.random.default_rng(5)
    q0 = torch.tensor(random_state(rng, 6, m.K, s.Np), device=cuda)
    ref_rhs = s.rhs(q0)
    q_ref, r_ref = q0.clone(), torch.zeros_like(q0)
    s.run(q_ref, r_ref, 1e-3, 3, graph=False)
    s.set_tile(epb)
    assert s.tile[0] == epb
    assert torch.equal(s.rhs(q0), ref_rhs)
    q, r = q0.clone(), torch.zeros_like(q0)
    s.run(q, r, 1e-3, 3, graph=False)
    assert torch.equal(q, q_ref) and torch.equal(r, r_ref)


@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("physics", ["wave", "maxwell"])
@pytest.mark.parametrize("N", [2, 4, 6])
def test_lsrk_matches_oracle(cuda, bb, oracle_cpu, N, physics, dt):
    import torch
    m = bb.uniform_tet_mesh(3)
    md = meshdata.build(m, N)
    s = bb.DGSolver(m, N, physics, dtype=tdt(dt), tau=1.0)
    q0 = bb.project_fields(m, N, pulse_fields(s.nf))
    step = s.dt_cfl()
    nsteps = 5
    qd = torch.tensor(q0, dtype=tdt(dt), device=cuda)
    rd = torch.zeros_like(qd)
    s.run(qd, rd, step, nsteps, graph=True)
    q_or, r_or = oracle_cpu.lsrk(0 if physics == "wave" else 1, N, q0, md, step, nsteps, tau=1.0)
    err = per_field_rel(qd.cpu().numpy(), q_or)
    assert np.all(err < TOL[dt]), err


def test_graph_and_stream_paths_agree(cuda, bb):
    import torch
    m = bb.uniform_tet_mesh(3)
    N = 5
    s = bb.DGSolver(m, N, "wave", dtype=torch.float32, tau=1.0)
    q0 = s.project([bb.gaussian_pulses(1), lambda x, y, z: 0 * x, lambda x, y, z: 0 * x,
                    lambda x, y, z: 0 * x])
    qa, ra = q0.clone(), torch.zeros_like(q0)
    qb, rb = q0.clone(), torch.zeros_like(q0)
    s.run(qa, ra, s.dt_cfl(), 7, graph=False)
    s.run(qb, rb, s.dt_cfl(), 4, graph=True)
    s.run(qb, rb, s.dt_cfl(), 3, graph=True)
    torch.cuda.synchronize()
    assert torch.equal(qa, qb)
    # host-buffer path (copies inside the call) gives the same state
    hin = q0.cpu().pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    qd, rd = torch.empty_like(q0), torch.zeros_like(q0)
    s.run_host(hin, hout, qd, rd, s.dt_cfl(), 7)
    torch.cuda.synchronize()
    assert torch.equal(hout, qa.cpu())


@pytest.mark.parametrize("nsteps", [1, 2, 3])
@pytest.mark.parametrize("case", [("wave", 5, "f32"), ("maxwell", 9, "f32"), ("wave", 3, "f64")])
def test_pipelined_host_path_equals_the_device_path(cuda, bb, case, nsteps):
    """bb_lsrk_run_host runs the first and the last step chunk by chunk on one stream per
    stage, ordered by the chunks' neighbours, behind the uploads and ahead of the downloads;
    the result equals the device-resident run bitwise, with and without the step graph, for
    the specialised and the generic kernels (81 tiles: 10 chunks of 8 or 9 tiles on the
    periodic 3^3-hex mesh, whose chunk graph wraps around)."""
    import torch
    physics, N, dt_name = case
    m = bb.uniform_tet_mesh(3)
    s = bb.DGSolver(m, N, physics, dtype=tdt(dt_name), tau=1.0)
    rng = np.random.default_rng(31 + N + nsteps)
    q0 = torch.tensor(random_state(rng, s.nf, m.K, s.Np) * 1e-2, dtype=tdt(dt_name), device=cuda)
    step = s.dt_cfl()
    qa, ra = q0.clone(), torch.zeros_like(q0)
    s.run(qa, ra, step, nsteps, graph=False)
    for graph in (False, True):
        hin = q0.cpu().pin_memory()
        hout = torch.full_like(hin, float("nan")).pin_memory()
        qd, rd = torch.empty_like(q0), torch.zeros_like(q0)
        s.run_host(hin, hout, qd, rd, step, nsteps, graph=graph)
        torch.cuda.synchronize()
        assert torch.equal(hout, qa.cpu()) and torch.equal(rd, ra) and torch.equal(qd, qa)
    s.check()


@pytest.mark.parametrize("nsteps", [1, 3])
def test_host_path_24_chunks_on_the_headline_tile(cuda, bb, nsteps):
    """8^3 hexes x 6 tets (K = 3072) on the 4-element x 288-thread wave tile: 768 tiles in 24
    chunks of 32, five stage streams; bitwise equal to the device-resident run."""
    import torch
    m = bb.uniform_tet_mesh(8)
    s = bb.DGSolver(m, 9, "wave", dtype=torch.float32, tau=1.0)
    s.set_kernel("specialised")
    s.set_tile(4, 288)
    assert s.kernel == "specialised"
    rng = np.random.default_rng(77 + nsteps)
    q0 = torch.tensor(random_state(rng, s.nf, m.K, s.Np) * 1e-2, dtype=torch.float32, device=cuda)
    step = s.dt_cfl()
    qa, ra = q0.clone(), torch.zeros_like(q0)
    s.run(qa, ra, step, nsteps)
    hin = q0.cpu().pin_memory()
    hout = torch.full_like(hin, float("nan")).pin_memory()
    qd, rd = torch.empty_like(q0), torch.zeros_like(q0)
    for _ in range(2):  # the second call reuses the schedule (one step: its graph)
        s.run_host(hin, hout, qd, rd, step, nsteps)
        torch.cuda.synchronize()
        assert torch.equal(hout, qa.cpu()) and torch.equal(qd, qa) and torch.equal(rd, ra)
    # pageable host buffers take the direct path; a new pinned output buffer a new graph
    for out in (torch.full_like(hin, float("nan")), torch.full_like(hin, float("nan")).pin_memory()):
        s.run_host(hin.clone(), out, qd, rd, step, nsteps)
        torch.cuda.synchronize()
        assert torch.equal(out, qa.cpu())
    s.check()


def test_config1_anchor_fp64_and_fp32(cuda, bb, oracle_cpu):
    """Wave, N=7, 4^3 hexes x 6 tets (K=384), p0 = exp(-10 r^2), 100 LSRK45 steps,
    dt = 0.25 h/(N+1)^2: FP64 GPU within 1e-12 and FP32 GPU within 1e-5 of the FP64 oracle."""
    import torch
    m = bb.uniform_tet_mesh(4)
    N = 7
    md = meshdata.build(m, N)
    zero = lambda x, y, z: 0 * x
    q0 = bb.project_fields(m, N, [lambda x, y, z: np.exp(-10 * (x * x + y * y + z * z)),
                                  zero, zero, zero])
    dt = 0.25 * 0.5 / (N + 1) ** 2
    q_or, _ = oracle_cpu.lsrk(0, N, q0, md, dt, 100, tau=1.0)
    for name in ("f64", "f32"):
        s = bb.DGSolver(m, N, "wave", dtype=tdt(name), tau=1.0)
        qd = torch.tensor(q0, dtype=tdt(name), device=cuda)
        rd = torch.zeros_like(qd)
        s.run(qd, rd, dt, 100)
        err = per_field_rel(qd.cpu().numpy(), q_or)
        assert np.all(err < TOL[name]), (name, err)


def test_norms_and_mass_energy(cuda, bb):
    import torch
    from oracle import dense
    m = bb.uniform_tet_mesh(2)
    N = 3
    s = bb.DGSolver(m, N, "wave", dtype=torch.float64, tau=1.0)
    rng = np.random.default_rng(11)
    a = rng.standard_normal((4, m.K, s.Np))
    b = rng.standard_normal((4, m.K, s.Np))
    A, B = torch.tensor(a, device=cuda), torch.tensor(b, device=cuda)
    nrm = s.norms(A, B)
    assert np.allclose(nrm[:, 0], (a ** 2).sum(axis=(1, 2)), rtol=1e-12)
    assert np.allclose(nrm[:, 1], ((a - b) ** 2).sum(axis=(1, 2)), rtol=1e-12)
    assert np.allclose(nrm[:, 2], (b ** 2).sum(axis=(1, 2)), rtol=1e-12)
    M = np.array(dense.mass(N))
    want = np.einsum("fkn,nm,fkm,k->f", a - b, M, a - b, m.J)
    assert np.allclose(s.mass_norms(A, B), want, rtol=1e-11)


def test_corrupt_connectivity_is_reported(cuda, bb):
    import torch
    from bbdg import BBError
    m = bb.uniform_tet_mesh(2)
    m.conn = m.conn.copy()
    m.conn[3, 1] = np.int32((m.K + 5) << 5)   # neighbour index out of range
    s = bb.DGSolver(m, 2, "wave", dtype=torch.float64, tau=1.0)
    with pytest.raises(BBError) as ei:
        s.rhs(s.zeros())
    assert ei.value.status == 7


def test_corrupt_connectivity_is_reported_by_the_specialised_kernel(cuda, bb):
    """The degree-specialised FP32 kernel checks every neighbour index before any access:
    one out of range is skipped, flagged and reported as BB_ERR_DEVICE."""
    import torch
    from bbdg import BBError
    m = bb.uniform_tet_mesh(2)                     # K = 48, a multiple of the N=9 tile
    m.conn = m.conn.copy()
    m.conn[5, 2] = np.int32((m.K + 9) << 5)        # neighbour index out of range
    s = bb.DGSolver(m, 9, "wave", dtype=torch.float32, tau=1.0)
    assert s.kernel == "specialised"
    with pytest.raises(BBError) as ei:
        s.rhs(s.zeros())
    assert ei.value.status == 7


FAST_TILES = {("wave", 9): [(4, 288), (4, 160), (2, 160)],
              ("maxwell", 9): [(2, 192), (2, 256)],
              ("wave", 5): [(4, 160), (8, 320), (2, 96)],
              ("maxwell", 5): [(4, 224), (8, 448), (2, 128)],
              ("wave", 10): [(2, 160)],
              ("maxwell", 10): [(2, 192), (2, 256)],
              ("wave", 4): [(8, 320)],
              ("maxwell", 4): [(4, 224)],
              ("wave", 6): [(4, 160), (8, 320), (2, 160)],
              ("maxwell", 6): [(2, 192)],
              ("wave", 7): [(4, 288), (2, 160)],
              ("maxwell", 7): [(2, 192)],
              ("wave", 8): [(4, 288)],
              ("maxwell", 8): [(4, 224)],
              ("wave", 11): [(2, 224)],
              ("maxwell", 11): [(2, 256)]}


def pulse_fields(nf):
    """A different Gaussian-pulse sum in every field (all fields O(1))."""
    return [bb_pulses(seed=40 + m) for m in range(nf)]


def bb_pulses(seed):
    import bbdg
    return bbdg.gaussian_pulses(seed=seed)


@pytest.mark.parametrize("key", sorted(FAST_TILES))
def test_degree_specialised_kernels_match_oracle_and_generic(cuda, bb, oracle_cpu, key):
    """Every compiled FP32 (N, physics, tile) variant: RHS vs the FP64 oracle (1e-5) and a
    3-step LSRK run vs the FP64 oracle and the generic FP32 kernel (1e-5 per field)."""
    import torch
    physics, N = key
    m = bb.uniform_tet_mesh(4)          # K = 384, a multiple of every tile size
    md = meshdata.build(m, N)
    s = bb.DGSolver(m, N, physics, dtype=torch.float32, tau=1.0)
    rng = np.random.default_rng(123)
    q = random_state(rng, s.nf, m.K, s.Np)
    qd = torch.tensor(q, dtype=torch.float32, device=cuda)
    want = oracle_cpu.rhs(0 if physics == "wave" else 1, N, q, md, tau=1.0)
    q0 = bb.project_fields(m, N, pulse_fields(s.nf))
    q_or, _ = oracle_cpu.lsrk(0 if physics == "wave" else 1, N, q0, md, s.dt_cfl(), 3, tau=1.0)
    s.set_kernel("generic")
    s.set_tile(4, 256)
    assert s.kernel == "generic" and s.tile == (4, 256)
    qg = torch.tensor(q0, dtype=torch.float32, device=cuda)
    rg = torch.zeros_like(qg)
    s.run(qg, rg, s.dt_cfl(), 3)
    s.set_kernel("specialised")
    for epb, nt in FAST_TILES[key]:
        s.set_tile(epb, nt)
        assert s.kernel == "specialised" and s.tile == (epb, nt)
        err = per_field_rel(s.rhs(qd).cpu().numpy(), want)
        assert np.all(err < 1e-5), (epb, nt, err)
        qf = torch.tensor(q0, dtype=torch.float32, device=cuda)
        rf = torch.zeros_like(qf)
        s.run(qf, rf, s.dt_cfl(), 3)
        e1 = per_field_rel(qf.cpu().numpy(), q_or)
        e2 = per_field_rel(qf.cpu().numpy(), qg.cpu().numpy())
        assert np.all(e1 < 1e-5) and np.all(e2 < 1e-5), (epb, nt, e1, e2)


@pytest.mark.parametrize("key", sorted(FAST_TILES))
def test_degree_specialised_kernels_on_many_tiles(cuda, bb, key):
    """Every variant on a mesh with many more tiles than blocks (K = 3,072), where each block
    prefetches the neighbour traces of tiles ahead: equal to the generic kernel (1e-5)."""
    import torch
    physics, N = key
    m = bb.uniform_tet_mesh(8)
    s = bb.DGSolver(m, N, physics, dtype=torch.float32, tau=1.0)
    q0 = bb.project_fields(m, N, pulse_fields(s.nf))
    dt = s.dt_cfl()
    s.set_kernel("generic")
    s.set_tile(4, 256)
    qg = torch.tensor(q0, dtype=torch.float32, device=cuda)
    rg = torch.zeros_like(qg)
    s.run(qg, rg, dt, 2)
    s.set_kernel("specialised")
    for epb, nt in FAST_TILES[key]:
        s.set_tile(epb, nt)
        qf = torch.tensor(q0, dtype=torch.float32, device=cuda)
        rf = torch.zeros_like(qf)
        s.run(qf, rf, dt, 2)
        err = per_field_rel(qf.cpu().numpy(), qg.cpu().numpy())
        assert np.all(err < 1e-5), (epb, nt, err)


def test_specialised_kernel_falls_back_on_misaligned_state(cuda, bb, oracle_cpu):
    """A state tensor that does not start on a 16-byte boundary takes the generic kernel."""
    import torch
    m = bb.uniform_tet_mesh(4)
    N = 9
    md = meshdata.build(m, N)
    s = bb.DGSolver(m, N, "wave", dtype=torch.float32, tau=1.0)
    rng = np.random.default_rng(7)
    q = random_state(rng, 4, m.K, s.Np)
    buf = torch.empty(q.size + 1, dtype=torch.float32, device=cuda)
    qd = buf[1:].view(q.shape)
    qd.copy_(torch.tensor(q, dtype=torch.float32))
    assert qd.data_ptr() % 16 != 0
    err = per_field_rel(s.rhs(qd).cpu().numpy(), oracle_cpu.rhs(0, N, q, md, tau=1.0))
    assert np.all(err < 1e-5), err
    # aligned state, output that does not start on a 16-byte boundary: also the generic path
    qa = torch.tensor(q, dtype=torch.float32, device=cuda)
    obuf = torch.empty(q.size + 1, dtype=torch.float32, device=cuda)
    out = obuf[1:].view(q.shape)
    assert out.data_ptr() % 16 != 0
    s.rhs(qa, out=out)
    err = per_field_rel(out.cpu().numpy(), oracle_cpu.rhs(0, N, q, md, tau=1.0))
    assert np.all(err < 1e-5), err


# ---- scalar advection (examples/3d_advec_scalar.jl) ----------------------------------------

@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("N", [1, 2, 3, 5, 7, 9])
def test_advection_rhs_matches_oracle(cuda, bb, oracle_cpu, N, dt):
    import torch
    m = bb.uniform_tet_mesh(3)
    md = meshdata.build(m, N)
    s = bb.DGSolver(m, N, "advection", dtype=tdt(dt))
    rng = np.random.default_rng(300 + N)
    q = random_state(rng, 1, m.K, s.Np)
    got = s.rhs(torch.tensor(q, dtype=tdt(dt), device=cuda)).cpu().numpy()
    want = oracle_cpu.rhs(2, N, q, md)
    err = per_field_rel(got, want)
    assert np.all(err < TOL[dt]), err


@pytest.mark.parametrize("dt", ["f64", "f32"])
def test_advection_example_end_check(cuda, bb, oracle_cpu, dt):
    """The example's own end check (3d_advec_scalar.jl:88-93) on the GPU: N = 7, 4^3 hexes,
    T = 0.1; the GPU run equals the oracle run and both are within 1e-3 of u0(x - T)."""
    import torch
    m = bb.uniform_tet_mesh(4)
    N = 7
    md = meshdata.build(m, N)
    f0 = lambda x, y, z: np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z)
    q0 = bb.project_fields(m, N, [f0])
    s = bb.DGSolver(m, N, "advection", dtype=tdt(dt))
    T, nsteps = 0.1, 100
    q = torch.tensor(q0, dtype=tdt(dt), device=cuda)
    r = torch.zeros_like(q)
    s.run(q, r, T / nsteps, nsteps)
    got = q.cpu().numpy()
    want, _ = oracle_cpu.lsrk(2, N, q0, md, T / nsteps, nsteps)
    assert np.all(per_field_rel(got, want) < TOL[dt])
    X = bb.element_domain_points(m, N)
    x, y, z = X[..., 0], X[..., 1], X[..., 2]
    V = bb.bernstein_basis_tet(N, *(2 * bb.mesh.reference_domain_points(N)[:, [1, 2, 3]].T - 1))
    u = np.einsum("pn,kn->kp", V, got[0].astype(np.float64))
    ex = np.sin(np.pi * (x - T)) * np.sin(np.pi * y) * np.sin(np.pi * z)
    assert np.abs(u - ex).max() < 1e-3


# ---- three-component advection (examples/3d_advec.jl) -------------------------------------

@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("N", [1, 3, 5, 9])
def test_three_component_advection_matches_oracle(cuda, bb, oracle_cpu, N, dt):
    """RHS and 3 LSRK45 steps of 3d_advec.jl on random (u, v, w) against the oracle."""
    import torch
    m = bb.uniform_tet_mesh(3)
    md = meshdata.build(m, N)
    s = bb.DGSolver(m, N, "advection3", dtype=tdt(dt))
    assert s.nf == 3 and s.kernel == "generic"
    rng = np.random.default_rng(400 + N)
    q = random_state(rng, 3, m.K, s.Np)
    qd = torch.tensor(q, dtype=tdt(dt), device=cuda)
    err = per_field_rel(s.rhs(qd).cpu().numpy(), oracle_cpu.rhs(3, N, q, md))
    assert np.all(err < TOL[dt]), err
    step = 0.1 * m.h / (N + 1) ** 2
    rd = torch.zeros_like(qd)
    s.run(qd, rd, step, 3)
    want, _ = oracle_cpu.lsrk(3, N, q, md, step, 3)
    err = per_field_rel(qd.cpu().numpy(), want)
    assert np.all(err < TOL[dt]), err


def test_external_integrator_drives_the_rhs(cuda, bb, oracle_cpu):
    """An integrator outside the library (classical RK4 written here) through
    DGSolver.ode_rhs(), the OrdinaryDiffEq interop path, against the same RK4 loop on the
    oracle's right-hand side (FP64, 1e-12 per field)."""
    import torch
    m = bb.uniform_tet_mesh(3)
    N = 4
    md = meshdata.build(m, N)
    s = bb.DGSolver(m, N, "wave", dtype=torch.float64, tau=1.0)
    q0 = bb.project_fields(m, N, pulse_fields(4))
    dt, nsteps = s.dt_cfl(), 6

    def rk4(f, q):
        for i in range(nsteps):
            t = i * dt
            k1 = f(t, q)
            k2 = f(t + dt / 2, q + dt / 2 * k1)
            k3 = f(t + dt / 2, q + dt / 2 * k2)
            k4 = f(t + dt, q + dt * k3)
            q = q + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        return q

    got = rk4(s.ode_rhs(), torch.tensor(q0, device=cuda)).cpu().numpy()
    want = rk4(lambda t, q: oracle_cpu.rhs(0, N, q, md, tau=1.0), np.asarray(q0))
    err = per_field_rel(got, want)
    assert np.all(err < 1e-12), err


def test_checkpoint_resume_is_bitwise_and_fp64_dump_seeds_fp32(cuda, bb, tmp_path):
    """save_state / load_state: 3 steps, checkpoint, 4 more steps equals 7 steps in one go
    (bitwise); an FP64 checkpoint loads into an FP32 solver as the rounded state; a
    checkpoint of another degree or mesh is refused."""
    import torch
    m = bb.uniform_tet_mesh(3)
    s = bb.DGSolver(m, 4, "maxwell", dtype=torch.float32, tau=1.0)
    q0 = s.project([bb.gaussian_pulses(f + 1) for f in range(6)])
    dt = s.dt_cfl()
    qa, ra = q0.clone(), torch.zeros_like(q0)
    s.run(qa, ra, dt, 7)
    qb, rb = q0.clone(), torch.zeros_like(q0)
    s.run(qb, rb, dt, 3)
    s.save_state(str(tmp_path / "ck"), qb, rb, t=3 * dt, step=3)
    qc, rc, t, step = s.load_state(str(tmp_path / "ck.npz"))
    assert step == 3 and t == 3 * dt
    s.run(qc, rc, dt, 4)
    assert torch.equal(qc, qa) and torch.equal(rc, ra)
    s64 = bb.DGSolver(m, 4, "maxwell", dtype=torch.float64, tau=1.0)
    q64 = s64.project([bb.gaussian_pulses(f + 1) for f in range(6)])
    s64.save_state(str(tmp_path / "ck64"), q64, torch.zeros_like(q64), as_fp64=True)
    q32, _, _, _ = s.load_state(str(tmp_path / "ck64.npz"))
    assert torch.equal(q32, q64.float())
    other = bb.DGSolver(m, 5, "maxwell", dtype=torch.float32, tau=1.0)
    with pytest.raises(ValueError):
        other.load_state(str(tmp_path / "ck.npz"))


def test_autotuner_keeps_the_fastest_candidate_it_timed(cuda, bb):
    """tune() times every candidate that runs (every compiled specialised variant of the
    physics and degree that divides K, and the generic tiles) and keeps the fastest."""
    import torch
    from bbdg import autotune
    m = bb.uniform_tet_mesh(8)
    s = bb.DGSolver(m, 9, "wave", dtype=torch.float32, tau=1.0)
    (kind, epb, nt), table = autotune.tune(s, steps=2, use_cache=False)
    names = {f"{k}:{e}x{t}" for k, e, t in autotune.candidates(s)}
    assert {n for n in names if n.startswith("specialised")} <= set(table)
    best = min(table, key=table.get)
    assert best == f"{kind}:{epb}x{nt}"
    assert s.kernel == kind and s.tile == (epb, nt)
