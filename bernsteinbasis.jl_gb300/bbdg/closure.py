"""Learned per-element closure for degree-5 Maxwell (no counterpart in the reference).

A degree-N_lo solve advances in macro steps of length D = hi_steps * dt_hi (the degree-N_hi
time step) made of lo_steps LSRK45 steps; after each macro step a per-element MLP reads the
element's own coefficients and its four neighbours' face traces (bb_closure_features) and its
output is added to the element's coefficients (bb_closure_apply).

Training data come from this same solver: degree-N_hi runs from seeded Gaussian-pulse initial
conditions, their states every hi_steps steps reduced to degree N_lo by the FP64 L2 projection
(bb_project). For consecutive reduced states c_j, c_{j+1}, the network learns
    target = c_{j+1} - S(c_j),      input = features(S(c_j)),
with S the macro step of the plain degree-N_lo solver, i.e. the error the plain solver makes
over one macro step. Snapshot pairs are generated on the GPU and streamed into a bounded
device store; the training batches are whole snapshots (all elements at one time).

Everything here runs on the GPU through the library: the N_hi and N_lo LSRK kernels, the
projection, the feature gather, the tcgen05 GEMM forward/backward, Adam and the apply.
"""
from __future__ import annotations

import dataclasses
import json
import math
import time

import numpy as np
import torch

from .basis import gaussian_pulses
from .mesh import TetMesh
from .mlp import MLP, closure_apply, closure_features, transpose_bf16
from .ordering import np2, np3
from .solver import DGSolver
from . import _lib, autotune
from .context import get_context, ptr, stream_handle

NF = 6  # Maxwell fields


def maxwell_ic(seed: int, count: int = 4):
    """Six fields, each a sum of `count` Gaussian pulses from its own sub-seed."""
    return [gaussian_pulses(seed * 16 + f, count) for f in range(NF)]


def project(q_hi: torch.Tensor, N_hi: int, N_lo: int, out: torch.Tensor | None = None,
            stream=None) -> torch.Tensor:
    """FP64 L2 degree reduction of [nf, K, Np(N_hi)] to [nf, K, Np(N_lo)] (bb_project)."""
    nf, K, _ = q_hi.shape
    if out is None:
        out = torch.empty((nf, K, np3(N_lo)), dtype=q_hi.dtype, device=q_hi.device)
    ctx = get_context(q_hi.device)
    code = _lib.BB_F64 if q_hi.dtype == torch.float64 else _lib.BB_F32
    oc = _lib.BB_F64 if out.dtype == torch.float64 else _lib.BB_F32
    ctx.check(_lib.load().bb_project(ctx.handle, N_hi, N_lo, K, nf, code, ptr(q_hi), oc,
                                     ptr(out), stream_handle(stream)), "bb_project")
    return out


@dataclasses.dataclass
class ClosureConfig:
    N_hi: int = 10
    N_lo: int = 5
    hi_steps: int = 10         # degree-N_hi steps per macro step (snapshot spacing)
    hidden: tuple = (512, 512)
    tau: float = 1.0
    pulses: int = 4


class Closure:
    """The degree-N_lo solver, its closure MLP and the degree-N_hi data generator."""

    def __init__(self, mesh: TetMesh, cfg: ClosureConfig = ClosureConfig(), seed: int = 0,
                 device=None):
        self.mesh, self.cfg = mesh, cfg
        self.K = mesh.K
        if self.K % 8:
            raise ValueError("the closure trains on whole snapshots: K must be a multiple of 8 "
                             "(an even number of hexahedra per side)")
        self.lo = DGSolver(mesh, cfg.N_lo, "maxwell", torch.float32, cfg.tau, device)
        autotune.tune(self.lo)
        self.hi = None
        self.device = self.lo.device
        self.dt_hi = 0.25 * mesh.h / (cfg.N_hi + 1) ** 2
        self.macro = cfg.hi_steps * self.dt_hi
        self.lo_steps = max(1, math.ceil(self.macro / self.lo.dt_cfl() - 1e-9))
        self.dt_lo = self.macro / self.lo_steps
        self.nin = NF * np3(cfg.N_lo) + 4 * NF * np2(cfg.N_lo)
        self.nout = NF * np3(cfg.N_lo)
        self.net = MLP((self.nin, cfg.hidden[0], cfg.hidden[1], self.nout), max_batch=self.K,
                       seed=seed, device=self.device)
        # the output layer starts at zero: the untrained closure is the plain solver
        p = self.net.params()
        p[self.nout_weight_slice()] = 0.0
        self.net.set_params(p)
        self.s_in = 1.0
        self.s_out = 1.0
        self.weight = 1.0  # fraction of the network's correction applied per macro step
        self._X = torch.empty((self.K, self.nin), dtype=torch.bfloat16, device=self.device)
        self._Y = torch.empty((self.K, self.nout), dtype=torch.float32, device=self.device)
        self._res = self.lo.zeros()

    def nout_weight_slice(self) -> slice:
        d = self.net.dims
        off = d[1] * d[0] + d[1] + d[2] * d[1] + d[2]
        return slice(off, off + d[3] * d[2])

    # ---- solver pieces ---------------------------------------------------------------
    def hi_solver(self, dtype=torch.float32) -> DGSolver:
        """The degree-N_hi solver (FP32 one cached; others built per call)."""
        if dtype != torch.float32:
            return DGSolver(self.mesh, self.cfg.N_hi, "maxwell", dtype, self.cfg.tau, self.device)
        if self.hi is None:
            self.hi = DGSolver(self.mesh, self.cfg.N_hi, "maxwell", torch.float32, self.cfg.tau,
                               self.device)
            autotune.tune(self.hi)
        return self.hi

    def initial_state(self, seed: int, solver: DGSolver | None = None) -> torch.Tensor:
        """Degree-N_hi coefficients of the seeded initial condition."""
        s = self.hi_solver() if solver is None else solver
        return s.project(maxwell_ic(seed, self.cfg.pulses))

    def plain_macro(self, q: torch.Tensor, res: torch.Tensor | None = None) -> None:
        res = self._res if res is None else res
        res.zero_()
        self.lo.run(q, res, self.dt_lo, self.lo_steps)

    def correct(self, q: torch.Tensor, weight: float | None = None) -> None:
        """q += weight * MLP(features(q)) / s_out (weight: self.weight by default)."""
        weight = self.weight if weight is None else weight
        closure_features(self.cfg.N_lo, NF, self.lo.conn, q, self.s_in, X=self._X)
        self.net.forward(self._X, out=self._Y)
        closure_apply(self.cfg.N_lo, NF, weight / self.s_out, self._Y, q)

    def run_lo(self, q: torch.Tensor, nmacro: int, closure: bool,
               weight: float | None = None) -> None:
        w = self.weight if weight is None else weight
        for _ in range(nmacro):
            self.plain_macro(q)
            if closure and w != 0.0:
                self.correct(q, w)

    # ---- data ----------------------------------------------------------------------------
    def snapshots(self, seed: int, nmacro: int, rollout: bool = False, noise: float = 0.0):
        """Yields (features BF16 [K, nin], target FP32 [K, nout]) for nmacro macro steps of
        one initial condition, scaled by the current s_in and s_out.

        rollout=False: every input starts from the reduced degree-N_hi state (teacher forced).
        rollout=True: inputs follow the closure-corrected degree-N_lo trajectory of the
        current network, so the targets also carry the error it has accumulated.
        noise > 0: the teacher-forced input state is perturbed by Gaussian noise of that
        relative size (per field RMS) before the plain macro step, and the target still
        points at the reduced degree-N_hi state, so the network also learns to remove
        perturbations like the ones a corrected run accumulates."""
        hi = self.hi_solver()
        q = self.initial_state(seed)
        res = torch.zeros_like(q)
        c = project(q, self.cfg.N_hi, self.cfg.N_lo)
        traj = c.clone()
        gen = torch.Generator(device=self.device).manual_seed(seed ^ 0x5DEECE66D)
        for _ in range(nmacro):
            s = (traj if rollout else c).clone()
            if noise > 0 and not rollout:
                rms = s.pow(2).mean(dim=(1, 2), keepdim=True).sqrt()
                s += noise * rms * torch.randn(s.shape, generator=gen, device=self.device)
            self.plain_macro(s)
            hi.run(q, res, self.dt_hi, self.cfg.hi_steps)
            c = project(q, self.cfg.N_hi, self.cfg.N_lo, out=c)
            X, _ = closure_features(self.cfg.N_lo, NF, self.lo.conn, s, self.s_in)
            T = (c - s).permute(1, 0, 2).reshape(self.K, self.nout) * self.s_out
            if rollout:
                traj.copy_(s)
                self.net.forward(X, out=self._Y)
                closure_apply(self.cfg.N_lo, NF, 1.0 / self.s_out, self._Y, traj)
            yield X, T.contiguous()

    def fit_scales(self, seed: int, nmacro: int = 3) -> None:
        """s_in, s_out = 1 / RMS of the raw features and targets over a few snapshots."""
        self.s_in, self.s_out = 1.0, 1.0
        fx, ft, n = 0.0, 0.0, 0
        for X, T in self.snapshots(seed, nmacro):
            fx += float(X.float().pow(2).mean())
            ft += float(T.pow(2).mean())
            n += 1
        self.s_in = 1.0 / math.sqrt(max(fx / n, 1e-30))
        self.s_out = 1.0 / math.sqrt(max(ft / n, 1e-30))

    def train(self, seeds, nmacro: int, epochs: int = 20, lr: float = 1e-3,
              lr_final: float = 1e-5, rollout_epochs: int = 0, noise: float = 0.0,
              store_limit_bytes: float = 40e9, log=None, keep_every: int = 1) -> dict:
        """Teacher-forced phase: generates the snapshot pairs of every seed (kept on the GPU
        up to the store limit) and runs `epochs` passes of Adam over them in shuffled order,
        one snapshot per step. Rollout phase (rollout_epochs > 0): adds the pairs of the
        current network's own corrected trajectories and trains `rollout_epochs` more passes
        over both sets. keep_every > 1 keeps every keep_every-th snapshot pair of each
        trajectory (more initial conditions in the same device store)."""
        t0 = time.perf_counter()
        per = self.K * (self.nin * 2 + self.nout * 4)
        cap = max(1, int(store_limit_bytes // per))
        store = self._generate(seeds, nmacro, False, cap, noise, keep_every)
        torch.cuda.synchronize()
        info = {"snapshots": len(store), "generate_s": time.perf_counter() - t0}
        losses = self._fit(store, epochs, lr, lr_final, log)
        info.update({"train_s": time.perf_counter() - t0 - info["generate_s"],
                     "epoch_loss": losses})
        if rollout_epochs > 0:
            t1 = time.perf_counter()
            store += self._generate(seeds, nmacro, True, cap, 0.0, keep_every)
            losses2 = self._fit(store, rollout_epochs, lr / 10, lr_final, log)
            torch.cuda.synchronize()
            info.update({"rollout_snapshots": len(store), "rollout_s": time.perf_counter() - t1,
                         "rollout_epoch_loss": losses2})
        return info

    def _generate(self, seeds, nmacro, rollout, cap, noise=0.0, keep_every=1):
        store = []
        for s in seeds:
            for j, (X, T) in enumerate(self.snapshots(s, nmacro, rollout, noise)):
                if len(store) < cap and j % max(1, keep_every) == keep_every // 2:
                    store.append((X, T))
        return store

    def _fit(self, store, epochs, lr, lr_final, log):
        rng = np.random.default_rng(len(store))
        XT = torch.empty((self.nin, self.K), dtype=torch.bfloat16, device=self.device)
        nsteps = max(1, epochs * len(store))
        losses = []
        it = 0
        for ep in range(epochs):
            acc = torch.zeros((), dtype=torch.float64, device=self.device)
            for i in rng.permutation(len(store)):
                X, T = store[i]
                transpose_bf16(X, out=XT)
                Y = self.net.forward(X, XT, train=True)
                acc += self.net.backward(Y, T)[0]
                # cosine decay from lr to lr_final
                lr_t = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * it / nsteps))
                self.net.step(lr_t)
                it += 1
            losses.append(float(acc) / len(store))
            if log:
                log(json.dumps({"epoch": ep, "mean_loss": losses[-1]}))
        return losses

    # ---- evaluation ----------------------------------------------------------------------
    def select_weight(self, seeds, nmacro: int,
                      weights=(1.0, 0.75, 0.5, 0.35, 0.25, 0.15, 0.1)) -> dict:
        """Model selection on validation initial conditions (seeds: one or several, not used
        for training): the correction weight whose free-running corrected runs end closest,
        summed over the seeds, to the (FP32) degree-10 runs; sets self.weight. Weight 0 (the
        plain solver) competes too: when no weight beats it, the closure is switched off
        rather than shipped with a loss."""
        seeds = [seeds] if isinstance(seeds, int) else list(seeds)
        hi = self.hi_solver()
        errs = {"plain": 0.0, **{f"w{w:g}": 0.0 for w in weights}}
        for seed in seeds:
            q = self.initial_state(seed)
            c0 = project(q, self.cfg.N_hi, self.cfg.N_lo)
            res = torch.zeros_like(q)
            hi.run(q, res, self.dt_hi, self.cfg.hi_steps * nmacro)
            ref = project(q, self.cfg.N_hi, self.cfg.N_lo)
            q5 = c0.clone()
            self.run_lo(q5, nmacro, False)
            errs["plain"] += self.rel_l2(q5, ref)
            for w in weights:
                q5 = c0.clone()
                self.run_lo(q5, nmacro, True, float(w))
                e = self.rel_l2(q5, ref)
                errs[f"w{w:g}"] += e if math.isfinite(e) else float("inf")
        best = min(weights, key=lambda w: errs[f"w{w:g}"])
        self.weight = float(best) if errs[f"w{best:g}"] < errs["plain"] else 0.0
        return {"selected_weight": self.weight, "selection_seeds": seeds,
                "selection_errors_summed": errs}

    def apriori(self, seed: int, nmacro: int) -> dict:
        """Teacher-forced one-macro-step error on one trajectory: sum over snapshots of
        |target - MLP| ^2 against |target|^2 (the plain solver's error), in scaled units."""
        num = torch.zeros((), dtype=torch.float64, device=self.device)
        den = torch.zeros((), dtype=torch.float64, device=self.device)
        for X, T in self.snapshots(seed, nmacro):
            Y = self.net.forward(X, out=self._Y)
            num += (T - Y).double().pow(2).sum()
            den += T.double().pow(2).sum()
        ratio = float(num / den)
        return {"apriori_mse_ratio": ratio, "apriori_gain": 1.0 / math.sqrt(max(ratio, 1e-300))}

    def rel_l2(self, a: torch.Tensor, b: torch.Tensor) -> float:
        """Mass-matrix relative L2 of a - b over all fields (degree N_lo)."""
        e = self.lo.mass_norms(a, b)
        r = self.lo.mass_norms(b)
        return float(math.sqrt(np.sum(e) / max(np.sum(r), 1e-300)))

    def evaluate(self, seed: int, nmacro: int, reference_dtype=torch.float64,
                 weights=(1.0,)) -> dict:
        """Errors at t = nmacro * macro against the FP64 degree-N_hi run reduced to N_lo, and
        wall times (CUDA events) of the plain N_hi, plain N_lo and closure N_lo runs."""
        ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
        N_hi, N_lo = self.cfg.N_hi, self.cfg.N_lo
        # reference: FP64 degree N_hi
        ref_s = self.hi_solver(reference_dtype)
        q64 = self.initial_state(seed, ref_s)
        r64 = torch.zeros_like(q64)
        ref_s.run(q64, r64, self.dt_hi, self.cfg.hi_steps * nmacro)
        c_ref = project(q64, N_hi, N_lo).float()
        q_ref = q64.float()
        del r64, q64, ref_s
        # plain FP32 degree N_hi (timed)
        hi = self.hi_solver()
        q = self.initial_state(seed)
        c0 = project(q, N_hi, N_lo)
        res = torch.zeros_like(q)
        hi.run(q.clone(), res, self.dt_hi, 1)  # builds the step graph
        res.zero_()
        e0, e1 = ev(), ev()
        torch.cuda.synchronize()
        e0.record()
        hi.run(q, res, self.dt_hi, self.cfg.hi_steps * nmacro)
        e1.record()
        torch.cuda.synchronize()
        t_hi = e0.elapsed_time(e1) / 1e3
        err_hi = self.rel_l2(project(q, N_hi, N_lo), c_ref)
        err_hi_full = float(math.sqrt(np.sum(hi.mass_norms(q, q_ref)) /
                                      np.sum(hi.mass_norms(q_ref))))
        del q, res, q_ref
        out = {"seed": seed, "t_final": nmacro * self.macro, "hi_steps": self.cfg.hi_steps * nmacro,
               "lo_steps": self.lo_steps * nmacro, "hi_seconds": t_hi,
               "err_hi_vs_fp64_hi": err_hi_full, "err_hi_reduced": err_hi}
        runs = [("plain", False, 1.0), ("closure", True, self.weight)]
        runs += [(f"closure_w{w:g}", True, float(w)) for w in weights if w != self.weight]
        for name, cl, w in runs:
            q5 = c0.clone()
            self.run_lo(q5.clone(), 1, cl, w)  # warm
            e0.record()
            self.run_lo(q5, nmacro, cl, w)
            e1.record()
            torch.cuda.synchronize()
            out[f"{name}_lo_seconds"] = e0.elapsed_time(e1) / 1e3
            out[f"err_{name}_lo"] = self.rel_l2(q5, c_ref)
            out[f"{name}_lo_finite"] = bool(torch.isfinite(q5).all())
        out["closure_gain"] = out["err_plain_lo"] / max(out["err_closure_lo"], 1e-300)
        out["speedup_closure_vs_hi"] = t_hi / max(out["closure_lo_seconds"], 1e-12)
        return out

    def truth_errors(self, seed: int, nmacro: int, npoints: int = 200_000,
                     point_seed: int = 7) -> dict:
        """Errors against an independent truth: the degree-N_hi FP32 run on the mesh refined
        twice in each direction (8 times the elements, half the time step), over the same
        time. The plain degree-N_hi, plain degree-N_lo and closure degree-N_lo runs on this
        mesh and the truth are evaluated at npoints uniform random points of the cube;
        relative L2 = RMS of the difference / RMS of the truth (all fields together). The
        uniform points make the RMS a Monte-Carlo estimate of the L2 norm over the cube."""
        from .basis import evaluate_at_points
        from .mesh import uniform_tet_mesh
        if self.mesh.n < 1:
            raise ValueError("truth_errors needs a uniform_tet_mesh")
        N_hi, N_lo = self.cfg.N_hi, self.cfg.N_lo
        fine = uniform_tet_mesh(2 * self.mesh.n)
        sf = DGSolver(fine, N_hi, "maxwell", torch.float32, self.cfg.tau, self.device)
        autotune.tune(sf)
        qf = sf.project(maxwell_ic(seed, self.cfg.pulses))
        rf = torch.zeros_like(qf)
        sf.run(qf, rf, self.dt_hi / 2, 2 * self.cfg.hi_steps * nmacro)
        pts = np.random.default_rng(point_seed).uniform(-1.0, 1.0, (npoints, 3))
        truth = evaluate_at_points(fine, N_hi, qf.double().cpu().numpy(), pts)
        del qf, rf, sf
        hi = self.hi_solver()
        q = self.initial_state(seed)
        c0 = project(q, N_hi, N_lo)
        res = torch.zeros_like(q)
        hi.run(q, res, self.dt_hi, self.cfg.hi_steps * nmacro)
        vals = {"hi": evaluate_at_points(self.mesh, N_hi, q.double().cpu().numpy(), pts)}
        for name, cl in (("plain_lo", False), ("closure_lo", True)):
            q5 = c0.clone()
            self.run_lo(q5, nmacro, cl)
            vals[name] = evaluate_at_points(self.mesh, N_lo, q5.double().cpu().numpy(), pts)
        scale = math.sqrt(float(np.mean(truth ** 2)))
        out = {"seed": seed, "t_final": nmacro * self.macro, "truth": f"degree {N_hi} FP32 on "
               f"{2 * self.mesh.n}^3 x 6 elements", "points": npoints, "weight": self.weight}
        for k, v in vals.items():
            out[f"truth_err_{k}"] = math.sqrt(float(np.mean((v - truth) ** 2))) / scale
        return out

    def solve(self, seed: int, nmacro: int, growth_tol: float = 1e-2):
        """Closure-corrected degree-N_lo solve of one initial condition. The plain degree-N_hi
        solver is the fallback: when the closure run's energy is not finite or has grown by
        more than growth_tol (the upwind scheme does not create energy), the degree-N_hi run
        is made instead. Returns (state, 'closure' | 'fallback', energies)."""
        hi = self.hi_solver()
        q_hi = self.initial_state(seed)
        q = project(q_hi, self.cfg.N_hi, self.cfg.N_lo)
        e_start = float(np.sum(self.lo.mass_norms(q)))
        self.run_lo(q, nmacro, closure=True)
        e_end = float(np.sum(self.lo.mass_norms(q)))
        if math.isfinite(e_end) and e_end <= e_start * (1.0 + growth_tol):
            return q, "closure", (e_start, e_end)
        res = torch.zeros_like(q_hi)
        hi.run(q_hi, res, self.dt_hi, self.cfg.hi_steps * nmacro)
        return project(q_hi, self.cfg.N_hi, self.cfg.N_lo), "fallback", (e_start, e_end)

    def save(self, path: str) -> None:
        np.savez(path, params=self.net.params(), s_in=self.s_in, s_out=self.s_out,
                 weight=self.weight,
                 dims=np.array(self.net.dims), cfg=json.dumps(dataclasses.asdict(self.cfg)))

    def load(self, path: str) -> None:
        z = np.load(path)
        self.net.set_params(z["params"])
        self.s_in, self.s_out = float(z["s_in"]), float(z["s_out"])
        self.weight = float(z["weight"]) if "weight" in z else 1.0

