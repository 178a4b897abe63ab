"""The chunk schedule of bb_lsrk_run_host, checked on the CPU (bb_host_schedule runs no CUDA).

bb_lsrk_run_host uploads element chunks, extracts each chunk's traces as it lands and runs
every LSRK stage chunk by chunk on its own stream, a launch waiting for one event of the
previous stage's stream. Those streams run their launches in order, so a launch of stage s
effectively waits for every launch of stage s-1 up to the largest index any launch of stage s
so far has waited for. The checker replays that and asserts, for every launch on chunk c:
  * read after write: stage s-1 has run on every chunk holding a face neighbour of an element
    of c (the traces stage s reads), and stage 0 runs only after those chunks' traces were
    extracted;
  * write after read: stage s-1 has run on every chunk with an element whose neighbour lies in
    c (those launches read the trace slots of c that stage s overwrites);
and that the chunks are whole-tile ranges covering every tile once, with the upload order and
each stage's order permutations of the chunks. Meshes: the periodic uniform mesh (its chunk
graph a ring that wraps) at several sizes and tiles, and the same mesh with its elements
shuffled (every chunk touching nearly every other). A schedule with a wait lowered by one,
planted here, must be rejected.
"""
import ctypes

import numpy as np
import pytest


def schedule(bb, conn, epb):
    from bbdg import _lib
    K = conn.shape[0]
    M = 24
    nch = ctypes.c_int(0)
    tiles = np.zeros(M + 1, np.int64)
    up = np.zeros(M, np.int32)
    order = np.zeros(5 * M, np.int32)
    ready0 = np.zeros(M, np.int32)
    wait = np.zeros(5 * M, np.int32)
    conn = np.ascontiguousarray(conn, np.int32)
    rc = _lib.load().bb_host_schedule(K, epb, conn.ctypes.data, ctypes.byref(nch), tiles.ctypes.data,
                                      up.ctypes.data, order.ctypes.data, ready0.ctypes.data,
                                      wait.ctypes.data)
    assert rc == 0
    C = nch.value
    return dict(C=C, tiles=tiles[:C + 1], up=up[:C], order=order.reshape(5, M)[:, :C],
                ready0=ready0[:C], wait=wait.reshape(5, M)[:, :C])


def violations(sch, conn, epb):
    """Every dependency the schedule fails to cover (empty when it is safe)."""
    K = conn.shape[0]
    C, tiles = sch["C"], sch["tiles"]
    ntiles = (K + epb - 1) // epb
    bad = []
    if tiles[0] != 0 or tiles[-1] != ntiles or np.any(np.diff(tiles) < min(8, ntiles)):
        bad.append("chunks are not whole-tile ranges covering every tile")
    for name, o in [("up", sch["up"])] + [(f"order{s}", sch["order"][s]) for s in range(5)]:
        if sorted(o.tolist()) != list(range(C)):
            bad.append(f"{name} is not a permutation")
    if bad:
        return bad
    ebounds = np.minimum(tiles * epb, K)
    chunk_of = np.searchsorted(ebounds, np.arange(K), side="right") - 1
    nbr = conn >> 5
    reads = [set() for _ in range(C)]      # chunks whose traces chunk c reads
    readers = [set() for _ in range(C)]    # chunks that read traces of chunk c
    for e in range(K):
        c = chunk_of[e]
        for f in range(4):
            n = int(nbr[e, f])
            if 0 <= n < K:
                reads[c].add(int(chunk_of[n]))
                readers[int(chunk_of[n])].add(c)
    for c in range(C):
        reads[c].add(c)
        readers[c].add(c)
    pos = np.empty(C, int)
    pos[sch["up"]] = np.arange(C)
    r0 = sch["ready0"]
    if np.any(np.diff(r0) < 0):
        bad.append("stage 0 launches out of upload order")
    for i, c in enumerate(sch["order"][0]):
        if max(pos[d] for d in reads[c]) > r0[i]:
            bad.append(f"stage 0 on chunk {c} before its neighbours' traces")
    for s in range(1, 5):
        idx = np.empty(C, int)
        idx[sch["order"][s - 1]] = np.arange(C)
        eff = -1
        for i, c in enumerate(sch["order"][s]):
            eff = max(eff, int(sch["wait"][s][i]))
            if max(idx[d] for d in reads[c]) > eff:
                bad.append(f"stage {s} on chunk {c} reads traces stage {s - 1} has not written")
            if max(idx[d] for d in readers[c]) > eff:
                bad.append(f"stage {s} on chunk {c} overwrites traces stage {s - 1} still reads")
    return bad


def shuffled(conn, seed):
    rng = np.random.default_rng(seed)
    K = conn.shape[0]
    new_of_old = rng.permutation(K)
    out = np.empty_like(conn)
    nb = conn >> 5
    out[new_of_old] = (new_of_old[nb] << 5) | (conn & 31)
    return out


@pytest.mark.parametrize("n,epb", [(3, 2), (4, 4), (8, 4), (8, 12), (12, 4)])
def test_schedule_of_the_uniform_mesh_is_safe(bb, n, epb):
    conn = bb.uniform_tet_mesh(n).conn.reshape(-1, 4)
    sch = schedule(bb, conn, epb)
    ntiles = (conn.shape[0] + epb - 1) // epb
    assert sch["C"] == min(24, max(1, ntiles // 8))
    assert violations(sch, conn, epb) == []


@pytest.mark.parametrize("seed", [1, 2])
def test_schedule_of_a_shuffled_mesh_is_safe(bb, seed):
    conn = shuffled(bb.uniform_tet_mesh(6).conn.reshape(-1, 4), seed)
    sch = schedule(bb, conn, 4)
    assert sch["C"] == 24
    assert violations(sch, conn, 4) == []


def test_the_checker_rejects_a_lowered_wait(bb):
    conn = bb.uniform_tet_mesh(8).conn.reshape(-1, 4)
    sch = schedule(bb, conn, 4)
    assert violations(sch, conn, 4) == []
    # the first launch of stage 2 whose wait is what lets it run: lower it by one
    w = sch["wait"][2]
    i = next(i for i in range(sch["C"]) if w[i] > 0 and (i == 0 or w[i] > w[:i].max()))
    planted = dict(sch, wait=sch["wait"].copy())
    planted["wait"][2][i] -= 1
    assert any("stage 2" in v for v in violations(planted, conn, 4))


def test_schedule_edge_cases(bb):
    """Fewer than 16 tiles: one chunk, and every order and wait degenerate; a tile that does
    not divide K (the generic kernel's ragged last tile): chunks still cover every tile;
    connectivity entries that name no element (which the kernels report) add no edge."""
    conn = bb.uniform_tet_mesh(2).conn.reshape(-1, 4)          # K = 48
    one = schedule(bb, conn, 4)                                # 12 tiles
    assert one["C"] == 1 and one["tiles"].tolist() == [0, 12]
    assert violations(one, conn, 4) == []
    conn3 = bb.uniform_tet_mesh(3).conn.reshape(-1, 4)         # K = 162
    ragged = schedule(bb, conn3, 5)                            # 33 tiles, the last of 2
    assert ragged["C"] == 4 and ragged["tiles"][-1] == 33
    assert violations(ragged, conn3, 5) == []
    bad = conn3.copy()
    bad[::7, 1] = (bad[::7, 1] & 31) | (1 << 26)               # neighbour index past K
    bad[::11, 2] = -1
    sch = schedule(bb, bad, 2)
    assert violations(sch, bad, 2) == []
