"""Element partition over ranks and the face-trace halo it needs (host side).

The stage kernels already exchange information between element tiles only through face
traces: a tile reads the traces of neighbours outside it from a trace buffer and writes its
own outgoing ones. Split the elements over ranks in contiguous ranges (z-slabs of the hex
ordering of `uniform_tet_mesh`, so the cut surfaces stay small) and the same holds between
ranks: per stage each rank sends the traces of its faces whose neighbour lives on another
rank, and receives the neighbour traces its own faces need. This module builds that plan and
does the exchange with point-to-point torch.distributed calls (gloo on CPU; the same calls
take CUDA tensors under NCCL). A trace travels in its owner's face-node order, as the kernels
read a neighbour's block (`trace[(nbr * 4 + nbr_face)][field][node]`) and permute by
orientation themselves.

It is bookkeeping only: the solvers here run on one GPU and do not call it.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def partition(K: int, world: int) -> np.ndarray:
    """Range starts (world + 1 entries): rank r owns elements [starts[r], starts[r+1])."""
    if world < 1 or K < world:
        raise ValueError("need 1 <= world <= K")
    return np.array([K * r // world for r in range(world + 1)], dtype=np.int64)


def owner(starts: np.ndarray, elements: np.ndarray) -> np.ndarray:
    return np.searchsorted(starts, elements, side="right") - 1


@dataclass
class HaloPlan:
    rank: int
    world: int
    start: int
    stop: int
    # peer -> (n, 2) int64 (element, face) pairs, sorted; send: my faces a peer needs;
    # recv: the peer's faces my elements need, in the peer's send order
    send: dict = field(default_factory=dict)
    recv: dict = field(default_factory=dict)

    def n_send(self) -> int:
        return int(sum(len(v) for v in self.send.values()))

    def n_recv(self) -> int:
        return int(sum(len(v) for v in self.recv.values()))


def halo_plan(mesh, world: int, rank: int) -> HaloPlan:
    """Which face traces rank `rank` sends to and receives from every other rank."""
    starts = partition(mesh.K, world)
    lo, hi = int(starts[rank]), int(starts[rank + 1])
    nbr = np.asarray(mesh.nbr, dtype=np.int64)
    nfc = np.asarray(mesh.nbr_face, dtype=np.int64)
    e_all = np.repeat(np.arange(mesh.K, dtype=np.int64), 4)
    f_all = np.tile(np.arange(4, dtype=np.int64), mesh.K)
    n_all, g_all = nbr.reshape(-1), nfc.reshape(-1)
    own_e, own_n = owner(starts, e_all), owner(starts, n_all)
    plan = HaloPlan(rank=rank, world=world, start=lo, stop=hi)
    for peer in range(world):
        if peer == rank:
            continue
        # faces of the peer's elements whose neighbour is mine: I send the neighbour side
        m = (own_e == peer) & (own_n == rank)
        send = np.unique(np.stack([n_all[m], g_all[m]], axis=1), axis=0)
        # faces of my elements whose neighbour is the peer's: I receive the neighbour side
        m = (own_e == rank) & (own_n == peer)
        recv = np.unique(np.stack([n_all[m], g_all[m]], axis=1), axis=0)
        if len(send):
            plan.send[peer] = send
        if len(recv):
            plan.recv[peer] = recv
    return plan


def exchange(plan: HaloPlan, traces_own, dist):
    """Sends the planned face traces and receives the neighbours'. traces_own: tensor
    [stop - start, 4, nf, Nfp] of this rank's face traces. Returns (ghost, index): ghost is a
    tensor [n_recv, nf, Nfp] and index maps (element, face) of a received trace to its row."""
    import torch
    shape = tuple(traces_own.shape[2:])
    ghost = torch.empty((plan.n_recv(),) + shape, dtype=traces_own.dtype,
                        device=traces_own.device)
    index, reqs, row, bufs = {}, [], 0, []
    for peer in sorted(plan.recv):
        keys = plan.recv[peer]
        view = ghost[row:row + len(keys)]
        for i, (e, f) in enumerate(keys):
            index[(int(e), int(f))] = row + i
        reqs.append(dist.irecv(view, src=peer))
        row += len(keys)
    for peer in sorted(plan.send):
        keys = plan.send[peer]
        buf = traces_own[keys[:, 0] - plan.start, keys[:, 1]].contiguous()
        bufs.append(buf)
        reqs.append(dist.isend(buf, dst=peer))
    for r in reqs:
        r.wait()
    return ghost, index
