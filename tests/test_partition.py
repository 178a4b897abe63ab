"""Element partition and face-trace halo exchange (bbdg/partition.py), as two gloo ranks on
the CPU: each rank computes the face traces of its own elements, the exchange delivers the
neighbour traces its faces need, and every delivered trace equals the neighbour's face values
computed from the whole state. The solvers run on one GPU and do not use this path."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _face_nodes(N):
    from oracle import meshdata
    return meshdata.fmask(N).reshape(4, -1)


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    for p in (ROOT, os.path.join(ROOT, "bernsteinbasis.jl_gb300")):
        sys.path.insert(0, p)
    import bbdg
    from bbdg import partition
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        N, nf = 3, 4
        mesh = bbdg.uniform_tet_mesh(4)
        q = np.random.default_rng(5).standard_normal((nf, mesh.K, bbdg.np3(N)))
        fm = _face_nodes(N)
        plan = partition.halo_plan(mesh, world, rank)
        own = np.arange(plan.start, plan.stop)
        tr = np.stack([q[:, own][:, :, fm[f]] for f in range(4)], axis=0)   # [4, nf, n, Nfp]
        tr = torch.tensor(np.transpose(tr, (2, 0, 1, 3)).copy())             # [n, 4, nf, Nfp]
        ghost, index = partition.exchange(plan, tr, dist)
        bad = 0
        for (e, f), row in index.items():
            bad += not np.array_equal(ghost[row].numpy(), q[:, e][:, fm[f]])
        need = {(int(mesh.nbr[e, f]), int(mesh.nbr_face[e, f]))
                for e in own for f in range(4)
                if not plan.start <= mesh.nbr[e, f] < plan.stop}
        out[rank] = (bad, set(index) == need, plan.n_send(), plan.n_recv(), len(need))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_halo_exchange_two_gloo_ranks(world):
    port = _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
        assert p.exitcode == 0
    sends = recvs = 0
    for r in range(world):
        bad, complete, n_send, n_recv, n_need = out[r]
        assert bad == 0 and complete and n_recv == n_need > 0
        sends += n_send
        recvs += n_recv
    assert sends == recvs


def test_halo_plan_is_symmetric_and_small(bb):
    """What rank a sends to rank b is exactly what b receives from a, for 2..5 ranks; for
    z-slab ranges the halo is a thin layer of the mesh's faces."""
    from bbdg import partition
    mesh = bb.uniform_tet_mesh(6)
    for world in range(2, 6):
        plans = [partition.halo_plan(mesh, world, r) for r in range(world)]
        for a in range(world):
            for b in range(world):
                if a == b:
                    continue
                s = plans[a].send.get(b, np.zeros((0, 2), np.int64))
                r = plans[b].recv.get(a, np.zeros((0, 2), np.int64))
                assert np.array_equal(s, r)
        total = sum(p.n_recv() for p in plans)
        assert 0 < total < 0.25 * 4 * mesh.K
    with pytest.raises(ValueError):
        partition.partition(3, 4)
