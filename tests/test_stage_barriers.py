"""The stage kernel's named-barrier hand-offs, simulated on the CPU for every compiled variant.

Each warp's barrier sequence is the kernel's (bbdg_stage_fast_impl.cuh): per tile, element
warps of group g `bar.sync` the group's B->A barrier (tiles after the first), then its A->B
barrier; chain warps `bar.sync` every group's B->A barrier (tiles after the first), then
`bar.arrive` on every group's A->B barrier. Hardware semantics: a barrier phase completes
when `count` threads have arrived; bar.sync blocks until then. Every interleaving must
finish; here a round-robin schedule is run, and any over-arrival (threads of two phases
mixing) or blocked warp fails the test.
"""
import os
import re

import pytest

HDR = os.path.join(os.path.dirname(__file__), "..", "bernsteinbasis.jl_gb300", "csrc",
                   "bbdg_stage_fast_variants.h")


def variants():
    with open(HDR) as fh:
        txt = fh.read()
    return [(int(n), p, int(e), int(t))
            for n, p, e, t in re.findall(r"X\((\d+), (BB_WAVE|BB_MAXWELL), (\d+), (\d+)\)", txt)]


def simulate(EPB, TPE, NCH, T):
    NCHAIN = EPB * 4 * NCH
    CHT = (NCHAIN + 31) // 32 * 32
    GS = 1 if EPB <= 7 else (EPB + 6) // 7
    NG = EPB // GS
    GC = GS * TPE + CHT
    assert EPB % GS == 0 and 2 * NG <= 15 and GC % 32 == 0
    warps = []
    for w in range(EPB * TPE // 32):
        g = (w * 32 // TPE) // GS
        ops = []
        for it in range(T):
            if it > 0:
                ops.append(("sync", 1 + NG + g))
            ops.append(("sync", 1 + g))
        warps.append(ops)
    for _ in range(CHT // 32):
        ops = []
        for it in range(T):
            if it > 0:
                ops += [("sync", 1 + NG + g) for g in range(NG)]
            ops += [("arrive", 1 + g) for g in range(NG)]
        warps.append(ops)
    pc = [0] * len(warps)
    count, blocked = {}, {}
    moved = True
    while moved:
        moved = False
        for w, ops in enumerate(warps):
            if pc[w] >= len(ops) or any(w in v for v in blocked.values()):
                continue
            kind, b = ops[pc[w]]
            count[b] = count.get(b, 0) + 32
            assert count[b] <= GC, f"over-arrival on barrier {b}"
            if count[b] == GC:
                for ww in blocked.get(b, []):
                    pc[ww] += 1
                blocked[b], count[b] = [], 0
                pc[w] += 1
            elif kind == "arrive":
                pc[w] += 1
            else:
                blocked.setdefault(b, []).append(w)
            moved = True
    return all(pc[w] >= len(ops) for w, ops in enumerate(warps))


@pytest.mark.parametrize("tiles", [1, 2, 3, 7])
def test_every_variant_finishes(tiles):
    vs = variants()
    assert len(vs) >= 20
    for N, phys, EPB, TPE in vs:
        NCH = 2 if phys == "BB_WAVE" else 6
        assert simulate(EPB, TPE, NCH, tiles), (N, phys, EPB, TPE, tiles)
