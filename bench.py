"""Benchmark: wave DOF-steps/s at N=9, with the stage kernel's fraction of the HBM roofline.

Workload (one "step" = one 5-stage LSRK45 time step over the whole mesh): the 3D acoustic
wave of examples/3d_wave.jl at degree N=9 (Np=220) in FP32 on the cube [-1,1]^3 cut into
32^3 hexahedra x 6 tetrahedra (K=196,608), affine geometry, periodic, face-Jacobian-scaled
upwind penalty (tau=1), dt = 0.25 h/(N+1)^2; initial p = sum of 8 Gaussian pulses (seed 1),
u = v = w = 0 (synthetic data; the reference publishes no dataset).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). value = DOF-steps/s = 4 * Np * K * steps / time over all
ranks (independent replicas on N GPUs). The e2e block runs the same steps through the C ABI
with host buffers (host->device copy of q, one step, device->host copy of q). The reference
arm times the CPU restatement of the reference's path (the oracle port) on all host cores,
on the same mesh.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "bernsteinbasis.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

N_DEG = 9
N_HEX = 32
NF = 4
# algorithmic bytes per element per RK stage (FP32): read q, read res, write res, write q
# (4 nf Np s) + neighbour traces (4 nf Nfp s) + geometry (22 scalars) + connectivity (4 int32)
def stage_bytes_per_element(N=N_DEG, s=4):
    Np = (N + 1) * (N + 2) * (N + 3) // 6
    Nfp = (N + 1) * (N + 2) // 2
    return 4 * NF * Np * s + 4 * NF * Nfp * s + 22 * s + 16


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ("pci.bus_id,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, pci):
        self.pci = pci  # (domain, bus, device) of the CUDA device, or None
        self.lines = []
        self.proc = None

    def start(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
               "-lms", "200"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def _mine(self, bus_field: str) -> bool:
        if self.pci is None:
            return True
        try:
            dom, rest = bus_field.split(":", 1)
            bus, devfn = rest.split(":", 1)
            dev = devfn.split(".")[0]
            return (int(dom, 16), int(bus, 16), int(dev, 16)) == self.pci
        except ValueError:
            return True

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9 or not self._mine(parts[0]):
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_port_rate(N: int, n_hex: int, steps: int, dtype=np.float32, nthreads: int = 0):
    """Times the oracle port (OpenMP over elements) on a mesh sample; DOF-steps/s."""
    import bbdg
    from oracle import cpu, meshdata
    mesh = bbdg.uniform_tet_mesh(n_hex)
    md = meshdata.build(mesh, N)
    zero = lambda x, y, z: 0 * x  # noqa: E731
    q0 = bbdg.project_fields(mesh, N, [bbdg.gaussian_pulses(1), zero, zero, zero]).astype(dtype)
    dt = 0.25 * mesh.h / (N + 1) ** 2
    nthreads = nthreads or cpu.max_threads()
    cpu.lsrk(0, N, q0, md, dt, 1, tau=1.0, nthreads=nthreads)      # warm-up
    t0 = time.perf_counter()
    cpu.lsrk(0, N, q0, md, dt, steps, tau=1.0, nthreads=nthreads)
    el = time.perf_counter() - t0
    Np = (N + 1) * (N + 2) * (N + 3) // 6
    return NF * Np * mesh.K * steps / el, nthreads, mesh.K, el


METRIC = "wave DOF-steps/s at N=9"
REF_MAX_STEPS = 30  # bound on the reference arm's timed steps (about 1.3 s each on 16 cores)


def reference_arm(args, rank):
    """Times the oracle port (the C++ restatement of the reference's CPU loops, OpenMP over
    elements on every host thread) on the same workload as the GPU arm: the full 32^3 x 6
    mesh, N=9, FP32, one LSRK45 step per step. Warm-up is one step (a CPU loop has nothing to
    warm beyond first touch); at most REF_MAX_STEPS steps are timed."""
    if rank != 0:
        return 0
    import bbdg
    from oracle import cpu, meshdata
    mesh = bbdg.uniform_tet_mesh(args.mesh_n)
    md = meshdata.build(mesh, N_DEG)
    zero = lambda x, y, z: 0 * x  # noqa: E731
    q0 = bbdg.project_fields(mesh, N_DEG, [bbdg.gaussian_pulses(1), zero, zero, zero])
    q0 = q0.astype(np.float32)
    dt = 0.25 * mesh.h / (N_DEG + 1) ** 2
    threads = cpu.max_threads()
    q, res = cpu.lsrk(0, N_DEG, q0, md, dt, 1, tau=1.0, nthreads=threads)   # warm-up
    steps = min(args.steps, REF_MAX_STEPS)
    t0 = time.perf_counter()
    cpu.lsrk(0, N_DEG, q, md, dt, steps, tau=1.0, nthreads=threads, res_soa=res)
    el = time.perf_counter() - t0
    Np = (N_DEG + 1) * (N_DEG + 2) * (N_DEG + 3) // 6
    rate = NF * Np * mesh.K * steps / el
    sample = (f"{args.mesh_n}^3 hexes x 6 tets (K={mesh.K}, the whole mesh), N=9 FP32, "
              f"{steps} LSRK45 steps in {el:.1f} s after 1 warm-up step, oracle port, "
              f"{threads} OpenMP threads")
    line = {"impl": "reference", "metric": METRIC, "value": rate,
            "unit": "DOF-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "timed_steps": steps, "ms_per_step": 1e3 * el / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: 8 Gaussian pulses in p (seed 1, centres U[-0.8,0.8]^3, widths "
                    "U[0.1,0.3], amplitudes N(0,1)), u=v=w=0",
            "config": {"workload": f"wave N=9 K={mesh.K} ({args.mesh_n}^3 hexes x 6 tets) FP32 "
                                   "LSRK45, tau=1, dt=0.25h/(N+1)^2",
                       "N": N_DEG, "K": mesh.K, "Np": Np, "fields": NF},
            "cpu_baseline": {"value": rate, "unit": "DOF-steps/s", "cores": threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": "DOF-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "Julia (the reference's language) is not installed on this host; the "
                    "reference arm runs the C++ restatement of its CPU path"}
    print(json.dumps(line), flush=True)
    return 0


def replica_rate(ms_local: float, units_per_rank: float, dist=None, device=None):
    """Whole-job rate of N independent replicas: every rank processed `units_per_rank` units
    in its own `ms_local` milliseconds; the job took the slowest rank's time (all-reduce MAX
    over the process group, when there is one), so the rate is world * units / max time.
    Returns (max milliseconds, units per second)."""
    import torch
    world = dist.get_world_size() if dist else 1
    t = torch.tensor([ms_local], dtype=torch.float64, device=device)
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    return ms_max, world * units_per_rank / (ms_max * 1e-3)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-hex", type=int, default=16, help="hexes per side of the CPU sample")
    ap.add_argument("--cpu-steps", type=int, default=60)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--mesh-n", type=int, default=N_HEX,
                    help="hexes per side (default: the 32^3 workload; smaller only for profiling)")
    ap.add_argument("--tile", type=str, default=None,
                    help="kind,elems_per_block,threads: skip the autotuner (profiling runs)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return reference_arm(args, rank)

    import torch
    import bbdg
    from bbdg import autotune

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    mesh = bbdg.uniform_tet_mesh(args.mesh_n)
    solver = bbdg.DGSolver(mesh, N_DEG, "wave", dtype=torch.float32, tau=1.0)
    zero = lambda x, y, z: 0 * x  # noqa: E731
    q = solver.project([bbdg.gaussian_pulses(1), zero, zero, zero])
    res = torch.zeros_like(q)
    dt = solver.dt_cfl()
    if args.tile:
        kind, epb, nt = args.tile.split(",")
        epb, nt = int(epb), int(nt)
        solver.set_kernel(kind)
        solver.set_tile(epb, nt)
        tune_table = None
    else:
        (kind, epb, nt), tune_table = autotune.tune(solver)
    stream = torch.cuda.current_stream()

    solver.run(q, res, dt, args.warmup)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    props = torch.cuda.get_device_properties(local)
    pci = None
    if all(hasattr(props, a) for a in ("pci_domain_id", "pci_bus_id", "pci_device_id")):
        pci = (int(props.pci_domain_id), int(props.pci_bus_id), int(props.pci_device_id))
    sampler = ClockSampler(pci)
    sampler.start()
    time.sleep(0.3)
    launches0 = solver.ctx.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e0.record(stream)
    solver.run(q, res, dt, args.steps, graph=True, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    launches = solver.ctx.launch_count() - launches0
    ms = e0.elapsed_time(e1)
    K = mesh.K
    Np = solver.Np
    dof = NF * Np * K
    ms_max, value = replica_rate(ms, dof * args.steps, dist, device="cuda")
    stage_ms = ms / (5 * args.steps)
    bpe = stage_bytes_per_element()
    peak, peak_kind = peaks()
    achieved = bpe * K / (stage_ms * 1e-3) / 1e9

    # end to end through the C ABI with host buffers: h2d of q, one step, d2h of q
    hin = q.detach().cpu().pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    qd, rd = torch.empty_like(q), torch.zeros_like(q)
    solver.run_host(hin, hout, qd, rd, dt, 1)
    torch.cuda.synchronize()
    c0 = torch.cuda.Event(enable_timing=True)
    c1 = torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    for _ in range(args.e2e_steps):
        solver.run_host(hout, hout, qd, rd, dt, 1, stream=stream)
    c1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = c0.elapsed_time(c1) / args.e2e_steps
    _, e2e_value = replica_rate(e2e_ms, dof, dist, device="cuda")
    state_bytes = q.numel() * q.element_size()

    # traffic per launch from the committed ncu summary (scaled from the captured case)
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "stage_kernel_traffic.json")) as fh:
            tr = json.load(fh)
        key = f"wave_N9_f32_{kind}_{epb}x{nt}"
        if key in tr:
            traffic = tr[key]["bytes_per_element"] * K
    except (OSError, ValueError, KeyError):
        traffic = None

    cpu_base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            rate, threads, Ks, el = cpu_port_rate(N_DEG, args.cpu_hex, args.cpu_steps)
            cpu_base = {"value": rate, "unit": "DOF-steps/s", "cores": threads, "kind": "port",
                        "sample": f"{args.cpu_hex}^3 hexes x 6 tets (K={Ks}), N=9 FP32, "
                                  f"{args.cpu_steps} LSRK45 steps in {el:.1f} s, oracle port "
                                  f"(C++ restatement of the reference loops), OpenMP"}
            # the same port on one thread (the reference itself is single-threaded)
            r1, _, K1, el1 = cpu_port_rate(N_DEG, 8, 8, nthreads=1)
            cpu_base["single_thread"] = {
                "value": r1, "unit": "DOF-steps/s", "cores": 1,
                "sample": f"8^3 hexes x 6 tets (K={K1}), N=9 FP32, 8 LSRK45 steps in {el1:.1f} s"}
        except Exception as exc:  # the baseline is reported, never required
            cpu_base = {"value": None, "unit": "DOF-steps/s", "cores": None, "kind": "port",
                        "sample": f"failed: {exc}"}

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value, "unit": "DOF-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: 8 Gaussian pulses in p (seed 1, centres U[-0.8,0.8]^3, widths "
                    "U[0.1,0.3], amplitudes N(0,1)), u=v=w=0",
            "config": {"workload": f"wave N=9 K={K} ({args.mesh_n}^3 hexes x 6 tets) FP32 "
                                   "LSRK45, tau=1, dt=0.25h/(N+1)^2",
                       "N": N_DEG, "K": K, "Np": Np, "fields": NF,
                       "parallelism": f"replicas x{world}",
                       "tile": {"kernel": kind, "elems_per_block": epb, "threads": nt},
                       "autotune_ms_per_step": tune_table,
                       "l2": f"inputs larger than L2 (q {state_bytes / 1e9:.2f} GB + res "
                             f"{state_bytes / 1e9:.2f} GB + traces per GPU, L2 129 MB)"
                             if 2 * state_bytes > 129e6 else "inputs fit in L2 (profiling case)"},
            "e2e": {"value": e2e_value, "unit": "DOF-steps/s",
                    "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_source": peak_kind,
                         "kernel": "stage kernel (fused RHS + LSRK stage)",
                         "bytes_per_element": bpe, "stage_ms": stage_ms},
            "cpu_baseline": cpu_base,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
