"""Measurement runs of the benchmark configurations other than the headline.

  python -m bbdg.configs --config 2    operator sweep N=3..15 (Dr, Ds, Dt, lift, separate and
                                       fused, FP32 and FP64) vs a dense Np x Np nodal matmul
  python -m bbdg.configs --config 3    N=9 wave, 32^3 x 6 elements, 200 LSRK45 steps in FP32
                                       vs FP64: per-field relative L2, energy drift, time
  python -m bbdg.configs --config 4    48 uneven wave/Maxwell problems in one persistent
                                       launch per stage (CUDA graph), autotuned tiles per N
  python -m bbdg.configs --config 5    learned closure: degree-10 Maxwell data reduced to
                                       degree 5, MLP trained on the GPU, held-out evaluation

Each run prints one JSON object per line. All inputs are synthetic and seeded: no dataset
is involved. Timings are CUDA events on the launching stream after warm-up; every input
below is larger than the 129 MB L2 unless stated.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import autotune
from .batch import BatchSolver, config4_problems
from .mesh import uniform_tet_mesh
from .operators import (BernsteinDerivativeMatrix_3D_r, BernsteinDerivativeMatrix_3D_s,
                        BernsteinDerivativeMatrix_3D_t, BernsteinLift, fused_apply_, grad_,
                        mul_)
from .ordering import np2, np3
from .solver import DGSolver, relative_l2


def _time(fn, reps: int = 5, warmup: int = 2) -> float:
    for _ in range(warmup):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _peak() -> float:
    import os
    root = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    try:
        with open(os.path.join(root, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0


def config2(degrees=range(3, 16), dtypes=("f32", "f64"), state_bytes=2e9, reps=5):
    """Operator sweep. K is chosen so that 4 fields of FP32 state total about 2 GB; the
    4 fields are applied as 4K element columns (Np x 4K in the reference's layout)."""
    peak = _peak()
    out = []
    gen = torch.Generator(device="cuda").manual_seed(0)
    for N in degrees:
        Np, Nfp = np3(N), np2(N)
        K = int(state_bytes / (4 * 4 * Np))
        cols = 4 * K
        for dt in dtypes:
            t = torch.float32 if dt == "f32" else torch.float64
            s = 4 if dt == "f32" else 8
            x = torch.rand((cols, Np), generator=gen, device="cuda", dtype=t) * 2 - 1
            f = torch.rand((cols, 4 * Nfp), generator=gen, device="cuda", dtype=t) * 2 - 1
            o = [torch.empty_like(x) for _ in range(4)]
            ops = {
                "Dr": lambda: mul_(o[0], BernsteinDerivativeMatrix_3D_r(N), x),
                "Ds": lambda: mul_(o[1], BernsteinDerivativeMatrix_3D_s(N), x),
                "Dt": lambda: mul_(o[2], BernsteinDerivativeMatrix_3D_t(N), x),
                "lift": lambda: mul_(o[3], BernsteinLift(N), f),
                "grad (Dr,Ds,Dt fused)": lambda: grad_(o[0], o[1], o[2], N, x),
                "fused (Dr,Ds,Dt,lift)": lambda: fused_apply_(o[0], o[1], o[2], o[3], N, x, f),
            }
            nbytes = {"Dr": 2 * Np, "Ds": 2 * Np, "Dt": 2 * Np, "lift": 4 * Nfp + Np,
                      "grad (Dr,Ds,Dt fused)": 4 * Np, "fused (Dr,Ds,Dt,lift)": 5 * Np + 4 * Nfp}
            row = {"config": 2, "N": N, "Np": Np, "K_columns": cols, "dtype": dt, "ops": {}}
            for name, fn in ops.items():
                ms = _time(fn, reps)
                gbs = nbytes[name] * s * cols / (ms * 1e-3) / 1e9
                row["ops"][name] = {"ms": ms, "GB/s": gbs, "frac_hbm": gbs / peak}
            # dense nodal comparator: an Np x Np matrix applied to the same columns (cuBLAS)
            A = torch.rand((Np, Np), generator=gen, device="cuda", dtype=t)
            y = torch.empty_like(x)
            ms = _time(lambda: torch.matmul(x, A.t(), out=y), reps)
            row["ops"]["dense Np x Np matmul (cuBLAS)"] = {
                "ms": ms, "GB/s": 2 * Np * s * cols / (ms * 1e-3) / 1e9,
                "GFLOP/s": 2.0 * Np * Np * cols / (ms * 1e-3) / 1e9}
            row["speedup_Dr_vs_dense"] = ms / row["ops"]["Dr"]["ms"]
            out.append(row)
            print(json.dumps(row), flush=True)
            del x, f, o, A, y
            torch.cuda.empty_cache()
    return out


def config3(steps: int = 200, n: int = 32, N: int = 9):
    """FP32 vs FP64 on the N=9 wave workload: accuracy, energy drift and time."""
    from .basis import gaussian_pulses
    mesh = uniform_tet_mesh(n)
    zero = lambda x, y, z: 0 * x  # noqa: E731
    res = {"config": 3, "N": N, "K": mesh.K, "steps": steps}
    states = {}
    for name, t in (("f64", torch.float64), ("f32", torch.float32)):
        s = DGSolver(mesh, N, "wave", dtype=t, tau=1.0)
        if t == torch.float32:
            (kind, epb, nt), _ = autotune.tune(s)
            res["f32_tile"] = [kind, epb, nt]
        q = s.project([gaussian_pulses(1), zero, zero, zero])
        r = torch.zeros_like(q)
        e_start = s.energy(q)
        dt = s.dt_cfl()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.run(q, r, dt, steps)
        torch.cuda.synchronize()
        res[f"{name}_seconds"] = time.perf_counter() - t0
        e_end = s.energy(q)
        res[f"{name}_energy_start"] = e_start
        res[f"{name}_energy_end"] = e_end
        res[f"{name}_energy_drift"] = (e_end - e_start) / e_start
        states[name] = (q, s)
        res["dt"] = dt
        res["t_final"] = dt * steps
    q64, s64 = states["f64"]
    q32, _ = states["f32"]
    res["rel_l2_coeff_per_field"] = relative_l2(q32.double(), q64, N).tolist()
    m_err = s64.mass_norms(q32.double(), q64)
    m_ref = s64.mass_norms(q64)
    res["rel_l2_mass_per_field"] = np.sqrt(m_err / np.maximum(m_ref, 1e-300)).tolist()
    print(json.dumps(res), flush=True)
    return res


def config4(steps: int = 100, dtype=torch.float32, compare_single: bool = True):
    specs = config4_problems()
    B = BatchSolver(specs, dtype=dtype)
    tiles = autotune.tune_batch(B)
    B.run(2)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    B.run(steps, graph=True)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    dofs = B.dofs()
    res = {"config": 4, "problems": len(specs), "steps": steps,
           "total_dofs": dofs, "elements": int(sum(m.K for m in B.meshes)),
           "batched_ms_per_step": ms / steps, "batched_dof_steps_per_s": dofs * steps / (ms * 1e-3),
           "tiles_per_N": tiles,
           "problems_list": [[s.physics, s.N, s.n, m.K] for s, m in zip(specs, B.meshes)]}
    if compare_single:
        # the same problems advanced one solver at a time (5 launches per problem per step),
        # each with the kernel the batch runs it on: the degree-specialised kernel where one
        # exists for (N, physics, K), else the generic kernel with the batch's tile
        solvers = []
        fast = 0
        for p, s in enumerate(specs):
            sv = DGSolver(B.meshes[p], s.N, s.physics, dtype=dtype, tau=s.tau)
            if sv.kernel == "generic":
                sv.set_tile(B.tile(s.physics, s.N), 256)
            else:
                fast += 1
            solvers.append((sv, B.q[p].clone(), torch.zeros_like(B.q[p]), B.dt(p)))
        res["fast_lanes"] = fast
        for sv, q, r, dt in solvers:
            sv.run(q, r, dt, 1)
        torch.cuda.synchronize()
        nstep_single = max(5, steps // 10)
        e0.record()
        for _ in range(nstep_single):
            for sv, q, r, dt in solvers:
                sv.run(q, r, dt, 1, graph=True)
        e1.record()
        torch.cuda.synchronize()
        ms1 = e0.elapsed_time(e1) / nstep_single
        res["one_at_a_time_ms_per_step"] = ms1
        res["batched_speedup"] = ms1 / (ms / steps)
    print(json.dumps(res), flush=True)
    return res


def config5(n: int = 16, n_train: int = 16, nmacro_train: int = 40, epochs: int = 20,
            n_eval: int = 2, nmacro_eval: int = 40, seed: int = 3, lr: float = 1e-3,
            hidden=(512, 512), N_hi: int = 10, N_lo: int = 5, rollout_epochs: int = 0,
            noise: float = 0.0, store_gb: float = 40.0, keep_every: int = 1,
            fp64_ref_seeds: int = 2, truth_seeds: int = 0, truth_points: int = 200_000):
    """Closure training and held-out evaluation. Training initial conditions are drawn from
    `seed`, the held-out ones from seed + 1000; every number is measured on the GPU. The
    first fp64_ref_seeds held-out seeds are scored against the FP64 degree-N_hi run, the rest
    against the FP32 one (the two differ by rounding, about 1e-6, far below the degree-N_lo
    errors); the first truth_seeds are also scored against the refined-mesh truth."""
    from .closure import Closure, ClosureConfig
    mesh = uniform_tet_mesh(n)
    cl = Closure(mesh, ClosureConfig(N_hi=N_hi, N_lo=N_lo, hidden=tuple(hidden)), seed=seed)
    rng = np.random.default_rng(seed)
    train_seeds = [int(s) for s in rng.integers(0, 2**31 - 1, n_train)]
    eval_seeds = [int(s) for s in np.random.default_rng(seed + 1000).integers(0, 2**31 - 1,
                                                                              n_eval)]
    head = {"config": 5, "K": mesh.K, "N_hi": N_hi, "N_lo": N_lo, "dt_hi": cl.dt_hi,
            "macro": cl.macro, "lo_steps_per_macro": cl.lo_steps, "n_train": n_train,
            "nmacro_train": nmacro_train, "t_train": nmacro_train * cl.macro, "epochs": epochs,
            "n_eval": n_eval, "nmacro_eval": nmacro_eval, "t_eval": nmacro_eval * cl.macro,
            "mlp": list(cl.net.dims), "params": cl.net.num_params,
            "rollout_epochs": rollout_epochs, "noise": noise, "keep_every": keep_every,
            "fp64_ref_seeds": fp64_ref_seeds, "truth_seeds": truth_seeds}
    print(json.dumps(head), flush=True)
    cl.fit_scales(train_seeds[0], 3)
    info = cl.train(train_seeds, nmacro_train, epochs=epochs, lr=lr, lr_final=lr / 100,
                    rollout_epochs=rollout_epochs, noise=noise,
                    store_limit_bytes=store_gb * 1e9,
                    log=lambda s: print(s, flush=True), keep_every=keep_every)
    info.update({"s_in": cl.s_in, "s_out": cl.s_out})
    print(json.dumps({"train": info}), flush=True)
    val_seeds = [int(s) for s in np.random.default_rng(seed + 500).integers(0, 2**31 - 1, 2)]
    sel = cl.select_weight(val_seeds, nmacro_eval)
    print(json.dumps({"model_selection": sel}), flush=True)
    rows = []
    for i, s in enumerate(eval_seeds):
        ref = torch.float64 if i < fp64_ref_seeds else torch.float32
        r = cl.evaluate(s, nmacro_eval, reference_dtype=ref, weights=(1.0, 0.5, 0.25))
        r["weight"] = cl.weight
        r["reference"] = "fp64" if ref == torch.float64 else "fp32"
        r.update(cl.apriori(s, nmacro_eval))
        if i < truth_seeds:
            r.update(cl.truth_errors(s, nmacro_eval, npoints=truth_points))
        rows.append(r)
        print(json.dumps(r), flush=True)
    summ = {"config": 5, "summary": True,
            "err_plain_lo_mean": float(np.mean([r["err_plain_lo"] for r in rows])),
            "err_closure_lo_mean": float(np.mean([r["err_closure_lo"] for r in rows])),
            "err_hi_vs_fp64_hi_mean": float(np.mean([r["err_hi_vs_fp64_hi"] for r in rows
                                                     if r["reference"] == "fp64"] or [np.nan])),
            "closure_gain_mean": float(np.mean([r["closure_gain"] for r in rows])),
            "closure_gain_min": float(np.min([r["closure_gain"] for r in rows])),
            "weight": cl.weight,
            "apriori_gain_mean": float(np.mean([r["apriori_gain"] for r in rows])),
            "speedup_closure_vs_hi_mean": float(np.mean([r["speedup_closure_vs_hi"]
                                                         for r in rows]))}
    print(json.dumps(summ), flush=True)
    return cl, info, rows, summ


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, required=True, choices=[2, 3, 4, 5])
    ap.add_argument("--n", type=int, default=16)
    ap.add_argument("--n-train", type=int, default=16)
    ap.add_argument("--nmacro-train", type=int, default=40)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--n-eval", type=int, default=2)
    ap.add_argument("--nmacro-eval", type=int, default=40)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--hidden", type=str, default="512,512")
    ap.add_argument("--N-hi", type=int, default=10)
    ap.add_argument("--N-lo", type=int, default=5)
    ap.add_argument("--rollout-epochs", type=int, default=0)
    ap.add_argument("--noise", type=float, default=0.0)
    ap.add_argument("--keep-every", type=int, default=1,
                    help="config 5: keep every k-th snapshot pair of a training trajectory")
    ap.add_argument("--fp64-ref-seeds", type=int, default=2)
    ap.add_argument("--truth-seeds", type=int, default=0,
                    help="config 5: held-out seeds also scored against the refined-mesh truth")
    ap.add_argument("--truth-points", type=int, default=200_000)
    ap.add_argument("--store-gb", type=float, default=40.0,
                    help="device memory for the training snapshot store (per phase)")
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--degrees", type=str, default="3-15")
    ap.add_argument("--state-gb", type=float, default=2.0,
                    help="config 2: bytes of operator input state per operator, in GB")
    ap.add_argument("--dtypes", type=str, default="f32,f64", help="config 2: f32, f64 or both")
    ap.add_argument("--mesh-n", type=int, default=32,
                    help="config 3: hexes per side (32: the K = 196,608 workload; smaller for profiling)")
    a = ap.parse_args()
    if a.config == 2:
        lo, hi = (int(v) for v in a.degrees.split("-"))
        config2(range(lo, hi + 1), dtypes=tuple(a.dtypes.split(",")), state_bytes=a.state_gb * 1e9)
    elif a.config == 3:
        config3(steps=a.steps or 200, n=a.mesh_n)
    elif a.config == 4:
        config4(steps=a.steps or 100)
    else:
        config5(n=a.n, n_train=a.n_train, nmacro_train=a.nmacro_train, epochs=a.epochs,
                n_eval=a.n_eval, nmacro_eval=a.nmacro_eval, lr=a.lr,
                hidden=tuple(int(v) for v in a.hidden.split(",")), N_hi=a.N_hi, N_lo=a.N_lo,
                rollout_epochs=a.rollout_epochs, noise=a.noise, store_gb=a.store_gb,
                keep_every=a.keep_every, fp64_ref_seeds=a.fp64_ref_seeds,
                truth_seeds=a.truth_seeds, truth_points=a.truth_points)


if __name__ == "__main__":
    main()
