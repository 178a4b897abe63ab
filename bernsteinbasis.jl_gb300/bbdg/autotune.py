"""Per-degree tile autotuner for the stage kernels.

For a solver it times every compiled tile variant (elements per block x threads per
block; every degree-specialised FP32 variant of its physics and degree in the library's
registry, and the generic kernel's tiles) over a few LSRK steps on the solver's own mesh with
CUDA events, keeps the fastest, and caches the choice per (physics, N, dtype, element count,
device name, library content hash) in a JSON file next to the built library (the element
count decides which tiles divide the mesh; a rebuilt library invalidates the entries). The
field vector width is not a tuning dimension: it is fixed by the physics in the specialised
kernels (wave: one 16-byte w entry per point; Maxwell: three 8-byte pieces).
"""
from __future__ import annotations

import json
import os

import torch

from . import _build

CACHE = os.path.join(_build.BUILD, "autotune.json")

# Generic-kernel candidates (kernel, elements per block, threads per block); the
# degree-specialised ones come from the library's registry of compiled variants.
GENERIC = [("generic", e, 256) for e in (1, 2, 4, 6, 8, 12)]


def compiled_variants():
    """Every compiled degree-specialised variant: [(N, physics, elems_per_block, threads)]."""
    import ctypes
    from . import _lib
    from .solver import PHYSICS
    names = {code: name for name, (code, _) in PHYSICS.items()}
    L = _lib.load()
    out, idx = [], 0
    vals = [ctypes.c_int() for _ in range(4)]
    while L.bb_fast_variant(idx, *(ctypes.byref(v) for v in vals)) == 0:
        N, phys, epb, nt = (v.value for v in vals)
        out.append((N, names.get(phys, str(phys)), epb, nt))
        idx += 1
    return out


_LIB_HASH = None


def _lib_hash() -> str:
    """Content hash of the loaded libbbdg.so: a rebuilt library invalidates cached choices."""
    global _LIB_HASH
    if _LIB_HASH is None:
        import hashlib
        h = hashlib.sha1()
        with open(_build.LIB, "rb") as fh:
            for chunk in iter(lambda: fh.read(1 << 20), b""):
                h.update(chunk)
        _LIB_HASH = h.hexdigest()[:16]
    return _LIB_HASH


def _key(solver) -> str:
    name = torch.cuda.get_device_name(solver.device)
    return f"{solver.physics}|{solver.N}|{str(solver.dtype)}|K={solver.K}|{name}|lib={_lib_hash()}"


def _load():
    try:
        with open(CACHE) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def candidates(solver):
    """Every compiled specialised variant for the solver's (physics, N) whose tile divides
    its element count (FP32 only), then the generic tiles; each is timed, the fastest kept."""
    spec = []
    if solver.dtype == torch.float32:
        spec = [("specialised", epb, nt) for (N, phys, epb, nt) in compiled_variants()
                if N == solver.N and phys == solver.physics and solver.K % epb == 0]
    return spec + GENERIC


def tune(solver, steps: int = 3, use_cache: bool = True, verbose: bool = False):
    """Selects the fastest tile for `solver` (in place) and returns (epb, threads, table)."""
    key = _key(solver)
    cache = _load() if use_cache else {}
    if key in cache:
        kind, epb, nt = cache[key]["choice"]
        try:
            solver.set_kernel(kind)
            solver.set_tile(epb, nt)
            if solver.kernel == kind:
                return (kind, epb, nt), cache[key]["ms_per_step"]
        except Exception:  # a stale entry: tune again
            pass
    q = (torch.rand((solver.nf, solver.K, solver.Np), dtype=solver.dtype,
                    device=solver.device) - 0.5) * 1e-3
    r = torch.zeros_like(q)
    dt = solver.dt_cfl()
    table = {}
    for kind, epb, nt in candidates(solver):
        try:
            solver.set_kernel(kind)
            solver.set_tile(epb, nt)
        except Exception:
            continue
        if solver.kernel != kind:
            continue
        solver.run(q, r, dt, 1)
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        s0.record()
        solver.run(q, r, dt, steps)
        s1.record()
        torch.cuda.synchronize()
        name = f"{kind}:{epb}x{nt}"
        table[name] = s0.elapsed_time(s1) / steps
        if verbose:
            print(f"autotune {solver.physics} N={solver.N} {name}: {table[name]:.3f} ms/step")
    if not table:
        raise RuntimeError("no tile variant could run")
    best = min(table, key=table.get)
    kind, tile = best.split(":")
    epb, nt = (int(v) for v in tile.split("x"))
    solver.set_kernel(kind)
    solver.set_tile(epb, nt)
    cache[key] = {"choice": [kind, epb, nt], "ms_per_step": table}
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        with open(CACHE, "w") as fh:
            json.dump(cache, fh, indent=1)
    except OSError:
        pass
    return (kind, epb, nt), table


BATCH_TILES = (1, 2, 4, 6, 8)
# The batched kernel runs every tile with the largest tile's shared memory; keeping tiles at
# or below this leaves three resident blocks per SM for all problems.
BATCH_TILE_BYTES = 72 * 1024


def tile_bytes(physics: str, N: int, dtype, epb: int) -> int:
    """Shared memory of one generic-kernel tile (bb_stage_tile_bytes)."""
    import ctypes
    from . import _lib
    from .solver import PHYSICS
    from .context import dtype_code
    b, c = ctypes.c_int64(), ctypes.c_int()
    rc = _lib.load().bb_stage_tile_bytes(PHYSICS[physics][0], int(N), dtype_code(dtype),
                                         int(epb), ctypes.byref(b), ctypes.byref(c))
    if rc != 0:
        raise ValueError("bad tile description")
    return int(b.value)


def tune_batch(batch, steps: int = 2, verbose: bool = False):
    """Per (physics, N) of a BatchSolver: time the generic stage tile sizes on the largest
    problem of that kind and set the fastest for the batch. Returns {"physics N": {...}}."""
    from .solver import DGSolver
    table = {}
    kinds = {}
    for i, s in enumerate(batch.specs):
        key = (s.physics, s.N)
        if key not in kinds or batch.meshes[i].K > batch.meshes[kinds[key]].K:
            kinds[key] = i
    for (physics, N), i in sorted(kinds.items()):
        spec = batch.specs[i]
        solver = DGSolver(batch.meshes[i], N, physics, dtype=batch.dtype, tau=spec.tau,
                          device=batch.device)
        solver.set_kernel("generic")
        q = torch.rand((solver.nf, solver.K, solver.Np), dtype=batch.dtype,
                       device=batch.device) * 1e-3
        r = torch.zeros_like(q)
        times = {}
        fits = [e for e in BATCH_TILES
                if tile_bytes(physics, N, batch.dtype, e) <= BATCH_TILE_BYTES] or [1]
        for epb in fits:
            try:
                solver.set_tile(epb, 256)
            except Exception:
                continue
            solver.run(q, r, solver.dt_cfl(), 1, graph=False)
            s0 = torch.cuda.Event(enable_timing=True)
            s1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            s0.record()
            solver.run(q, r, solver.dt_cfl(), steps, graph=False)
            s1.record()
            torch.cuda.synchronize()
            times[epb] = s0.elapsed_time(s1) / steps
        best = min(times, key=times.get)
        batch.set_tile(physics, N, best)
        table[f"{physics} N={N}"] = {"elems_per_block": best, "threads": 256,
                                     "ms_per_step": times, "tuned_on_K": solver.K}
        if verbose:
            print(f"batch tile {physics} N={N}: {best} elements/block ({times})")
        solver.close()
    return table
