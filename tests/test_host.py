"""Host-side logic (no GPU): mesh, compact connectivity vs coordinate-matched mapP,
geometric factors, projection, and the C-ABI library's exported symbols."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import meshdata

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "bbdg.h")).read()
    return re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(bb_\w+)\(", src, re.M)


def test_capi_library_exports_every_declared_symbol():
    from bbdg import _lib, _build
    path = _build.build()
    lib = ctypes.CDLL(path)
    names = header_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    # the Python binding covers the same set
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_generic_tile_lift_form_and_size():
    """bb_stage_tile_bytes (host arithmetic only): FP64 tiles always lift level by level, an
    FP32 tile takes the chain-per-thread lift exactly when that tile fits in 100 KB, and every
    size counts the degree tables in full (the stack-slot table included)."""
    from bbdg import _lib
    lib = _lib.load()
    b, c = ctypes.c_int64(), ctypes.c_int()

    def tile(phys, N, dtype, epb):
        assert lib.bb_stage_tile_bytes(phys, N, dtype, epb, ctypes.byref(b), ctypes.byref(c)) == 0
        return b.value, c.value

    def np3(n):
        return (n + 1) * (n + 2) * (n + 3) // 6

    def np2(n):
        return (n + 1) * (n + 2) // 2

    for phys in (0, 1, 2):
        for N in (1, 3, 9, 15, 20):
            words = (np3(N) + np3(N - 1) + (np3(N + 1) + 1) // 2 + (4 * np2(N) + 1) // 2
                     + (6 * np2(N) + 1) // 2 + (4 * np3(N) + 1) // 2 + (np3(N) + 1) // 2)
            for epb in (1, 2, 4, 8):
                b64, c64 = tile(phys, N, 1, epb)
                assert c64 == 0 and b64 >= 4 * words
                b32, c32 = tile(phys, N, 0, epb)
                assert b32 >= 4 * words
                if c32:
                    assert b32 <= 100 * 1024
    # the benchmark's degree: an FP32 2-element wave tile lifts chain per thread (two chains
    # per face), the FP64 one level by level
    assert tile(0, 9, 0, 2)[1] == 1 and tile(0, 9, 1, 2)[1] == 0
    assert lib.bb_stage_tile_bytes(0, 0, 0, 2, ctypes.byref(b), ctypes.byref(c)) != 0


def neighbour_node(N, o, a_idx):
    """Face node a of this side -> node index on the partner side (orientation o)."""
    from bbdg.mesh import PERMS
    pairs = [(a, b) for b in range(N + 1) for a in range(N + 1 - b)]
    a, b = pairs[a_idx]
    w = (a, b, N - a - b)
    wn = [0, 0, 0]
    for v in range(3):
        wn[PERMS[o][v]] = w[v]
    return pairs.index((wn[0], wn[1]))


@pytest.mark.parametrize("n,N", [(2, 1), (2, 3), (3, 2), (4, 4)])
def test_compact_connectivity_matches_mapP(bb, n, N):
    m = bb.uniform_tet_mesh(n)
    md = meshdata.build(m, N)
    Nfp = (N + 1) * (N + 2) // 2
    table = [[neighbour_node(N, o, a) for a in range(Nfp)] for o in range(6)]
    conn = m.conn.astype(np.int64)
    nbr, nface, orient = conn >> 5, (conn >> 3) & 3, conn & 7
    for e in range(m.K):
        for f in range(4):
            for a in range(Nfp):
                want = md.mapP[(e * 4 + f) * Nfp + a]
                got = (nbr[e, f] * 4 + nface[e, f]) * Nfp + table[orient[e, f]][a]
                assert got == want


def test_mesh_periodic_pairs_and_volume(bb):
    m = bb.uniform_tet_mesh(3)
    assert m.K == 6 * 27
    # pairing is an involution and never pairs a face with itself
    for e in range(m.K):
        for f in range(4):
            e2, f2 = m.nbr[e, f], m.nbr_face[e, f]
            assert (e2, f2) != (e, f)
            assert m.nbr[e2, f2] == e and m.nbr_face[e2, f2] == f
    vol = (4.0 / 3.0) * m.J.sum()
    assert vol == pytest.approx(8.0, rel=1e-13)


def test_geometry_matches_oracle_meshdata(bb):
    m = bb.uniform_tet_mesh(3)
    N = 2
    md = meshdata.build(m, N)
    from bbdg.mesh import GEO_NX, GEO_NY, GEO_NZ, GEO_INVJ, GEO_J
    assert np.allclose(m.geo[:, :9], md.geo9, rtol=1e-14, atol=1e-15)
    assert np.allclose(m.geo[:, GEO_J], md.Jall)
    assert np.allclose(m.geo[:, GEO_INVJ], 1 / md.Jall)
    Nfp = (N + 1) * (N + 2) // 2
    for f in range(4):
        for c, base in enumerate((GEO_NX, GEO_NY, GEO_NZ)):
            assert np.allclose(m.geo[:, base + f], md.nJ[:, f * Nfp, c], atol=1e-15)


@pytest.mark.parametrize("N", [1, 3, 6])
def test_projection_reproduces_polynomials(bb, N):
    m = bb.uniform_tet_mesh(2)
    f = lambda x, y, z: (1 + x + 2 * y - z) ** N
    q = bb.project_fields(m, N, [f])[0]
    # evaluate the Bernstein expansion at random points of every element
    rng = np.random.default_rng(N)
    lam = rng.dirichlet(np.ones(4), size=7)             # weights on lambda0..lambda3
    from oracle.dense import vandermonde_tet
    V, _ = vandermonde_tet(N, *lam.T)
    u = q @ V.T                                          # (K, 7)
    W = lam[:, [3, 0, 1, 2]]                             # weights on X1..X4
    X = np.einsum("pm,kmc->kpc", W, m.EVX)
    assert np.allclose(u, f(X[..., 0], X[..., 1], X[..., 2]), rtol=1e-9, atol=1e-9)


def test_face_node_tables_agree_with_oracle_fmask(bb):
    for N in range(1, 10):
        fv = bb.ordering.face_node_volume_index(N).reshape(-1)
        assert np.array_equal(fv, meshdata.fmask(N))


def test_product_rejects_bad_degree(bb):
    with pytest.raises(ValueError):
        bb.mesh.uniform_tet_mesh(1)


def test_config4_problem_set_is_seeded_and_in_range():
    from bbdg.batch import config4_problems
    a, b = config4_problems(), config4_problems()
    assert len(a) == 48 and a == b
    assert all(4 <= s.N <= 11 and 4 <= s.n <= 20 for s in a)
    assert {s.physics for s in a} == {"wave", "maxwell"}


@pytest.mark.parametrize("N", [1, 2, 4, 7])
def test_meshdata_import_rebuilds_connectivity_and_geometry(bb, N):
    """bb_conn_from_mapP / bb_geo_from_meshdata on StartUpDG-shaped arrays (the oracle's
    coordinate-matched mapP and cofactor geometry) reproduce the mesh's own records."""
    from bbdg.mesh import from_meshdata
    from oracle import meshdata
    m = bb.uniform_tet_mesh(3)
    md = meshdata.build(m, N)
    Nfp = bb.np2(N)
    nJ = md.nJ.reshape(m.K, 4, Nfp, 3)[:, :, 0, :]     # face-constant on affine faces
    got = from_meshdata(N, md.Fmask, md.mapP, md.geo9, nJ, md.Jall, h=m.h)
    assert np.array_equal(got.conn, m.conn)
    assert np.allclose(got.geo, m.geo, rtol=1e-13, atol=1e-13)


def test_meshdata_import_rejects_a_broken_mapP(bb):
    from bbdg.mesh import from_meshdata
    from oracle import meshdata
    m = bb.uniform_tet_mesh(2)
    md = meshdata.build(m, 2)
    bad = md.mapP.copy()
    bad[0], bad[1] = bad[1], bad[0] + 3 * bb.np2(2)    # two nodes of one face to different faces
    nJ = md.nJ.reshape(m.K, 4, bb.np2(2), 3)[:, :, 0, :]
    with pytest.raises(ValueError):
        from_meshdata(2, md.Fmask, bad, md.geo9, nJ, md.Jall)


def test_stack_slot_header_is_generated_and_injective():
    """The committed lift-stack slot table is what its generator produces, and every degree's
    slots are distinct and fit the stack stride the stage kernel reserves."""
    import re
    import subprocess
    import sys
    csrc = os.path.join(os.path.dirname(__file__), "..", "bernsteinbasis.jl_gb300", "csrc")
    with open(os.path.join(csrc, "bbdg_stack_slots.cuh")) as fh:
        committed = fh.read()
    produced = subprocess.run([sys.executable, os.path.join(csrc, "gen_stack_slots.py")],
                              capture_output=True, text=True, check=True).stdout
    assert produced == committed
    for block in re.findall(r"stack_slot<(\d+)>\(int q\) \{(.*?)\n\}", committed, re.S):
        N = int(block[0])
        NP = (N + 1) * (N + 2) * (N + 3) // 6
        table = dict((int(a), int(b)) for a, b in re.findall(r"case (\d+): return (\d+);", block[1]))
        slots = [table.get(q, q) for q in range(NP)]
        assert len(set(slots)) == NP
        span = int(re.search(rf"struct StackSlots<{N}> \{{\s*static constexpr int span = (\d+);",
                             committed).group(1))
        assert max(slots) + 1 == span
        nps = (max(NP, span) + 14) // 16 * 16 + 1
        assert span <= nps and nps % 16 == 1


def test_autotuner_candidates_come_from_the_compiled_registry(monkeypatch):
    """The autotuner's specialised candidates are the library's compiled variants (read
    through bb_fast_variant, no GPU needed), and its cache key changes with the library's
    content hash, so a rebuilt library is tuned again."""
    torch = pytest.importorskip("torch")
    from bbdg import autotune
    variants = autotune.compiled_variants()
    assert len(variants) >= 20 and len(set(variants)) == len(variants)
    header = open(os.path.join(os.path.dirname(__file__), "..", "bernsteinbasis.jl_gb300",
                               "csrc", "bbdg_stage_fast_variants.h")).read()
    listed = re.findall(r"X\((\d+), BB_(WAVE|MAXWELL), (\d+), (\d+)\)", header)
    assert [(int(n), p.lower(), int(e)) for n, p, e, _ in listed] == \
        [(n, p, e) for n, p, e, _ in variants]

    class FakeSolver:
        physics, N, dtype, K, device = "wave", 9, torch.float32, 3072, None
    monkeypatch.setattr(torch.cuda, "get_device_name", lambda d=None: "GPU")
    monkeypatch.setattr(autotune, "_LIB_HASH", "aaaa")
    k1 = autotune._key(FakeSolver)
    monkeypatch.setattr(autotune, "_LIB_HASH", "bbbb")
    assert autotune._key(FakeSolver) != k1
    cands = autotune.candidates(FakeSolver)
    spec = [c for c in cands if c[0] == "specialised"]
    assert spec == [("specialised", e, t) for n, p, e, t in variants
                    if n == 9 and p == "wave" and 3072 % e == 0]


def test_debug_index_checks_compile():
    """The debug build's index checks (-DBB_DEBUG_CHECKS) compile in the stage kernels: the
    generic tile (bbdg_solver.cu) and the degree-specialised N = 9 variants."""
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    csrc = os.path.join(os.path.dirname(__file__), "..", "bernsteinbasis.jl_gb300", "csrc")
    inc = os.path.join(os.path.dirname(__file__), "..", "include")
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        for src in ("bbdg_solver.cu", "bbdg_stage_fast_v9.cu"):
            r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O1",
                                "-std=c++17", "-I", inc, "--expt-relaxed-constexpr",
                                "-DBB_DEBUG_CHECKS", "-c", os.path.join(csrc, src), "-o",
                                os.path.join(tmp, src + ".o")], capture_output=True, text=True)
            assert r.returncode == 0, r.stderr[-2000:]
