"""Measurement of the tcgen05 BF16 GEMM on the closure MLP's shapes and a large square shape.

  python bench_gemm.py [--reps R] [--shapes M,N,K;M,N,K...] [--no-cublas]

Prints one JSON line per shape: our kernel's time and TFLOP/s with an FP32 and with a BF16
output, cuBLAS (torch.matmul, BF16 output) on the same operands for comparison, and the
fraction of the measured dense BF16 peak (MEASURED_PEAKS.json, burst figure). Then one line
for a whole closure-MLP training step (forward, backward, Adam) and one for inference at
24,576 rows. Inputs are seeded random; timings are CUDA events after warm-up, around a
CUDA graph of `reps` calls (device time) except for the training step (host loop).
"""
from __future__ import annotations

import argparse
import json
import os

import sys

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "bernsteinbasis.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import torch  # noqa: E402

from bbdg import mlp  # noqa: E402

CLOSURE_SHAPES = [(24576, 512, 840), (24576, 512, 512), (24576, 336, 512), (512, 840, 24576),
                  (512, 512, 24576), (336, 512, 24576)]
SQUARE_SHAPES = [(8192, 8192, 8192)]


def _peak_tflops():
    root = ROOT
    try:
        with open(os.path.join(root, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["bf16_tflops"]), "measured"
    except (OSError, ValueError, KeyError):
        return 1900.0, "fallback"


def _time(fn, reps, graph=True):
    """Milliseconds per call. With graph=True the calls are captured once into a CUDA graph
    and replayed, so the figure is device time without the host's per-call overhead."""
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if graph:
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                for _ in range(reps):
                    fn()
        torch.cuda.current_stream().wait_stream(s)
        g.replay()
        torch.cuda.synchronize()
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def run(shapes, reps=20, cublas=True):
    peak, kind = _peak_tflops()
    g = torch.Generator(device="cuda").manual_seed(0)
    rows = []
    for (M, N, K) in shapes:
        A = torch.randn((M, K), generator=g, device="cuda").bfloat16()
        B = torch.randn((N, K), generator=g, device="cuda").bfloat16()
        C = torch.zeros((M, N), device="cuda")
        Cb = torch.empty((M, N), device="cuda", dtype=torch.bfloat16)
        split = K >= 8192 and M <= 1024  # the weight-gradient shapes (K = batch) split K
        kt = 16 if split else 0
        f = 2.0 * M * N * K
        ms = _time(lambda: mlp.gemm_bf16(A, B, out_f32=C, kt_per=kt), reps)
        row = {"M": M, "N": N, "K": K, "split_k": split, "ms_f32_out": ms,
               "tflops_f32_out": f / ms / 1e9}
        if not split:
            msb = _time(lambda: mlp.gemm_bf16(A, B, out_bf16=Cb), reps)
            row.update({"ms_bf16_out": msb, "tflops_bf16_out": f / msb / 1e9})
        best = max(row.get("tflops_bf16_out", 0.0), row["tflops_f32_out"])
        row.update({"peak_tflops": peak, "peak_source": kind, "frac_of_peak": best / peak})
        if cublas:
            msc = _time(lambda: torch.matmul(A, B.T), reps)
            row.update({"cublas_ms": msc, "cublas_tflops": f / msc / 1e9})
        rows.append(row)
        print(json.dumps(row), flush=True)
        del A, B, C, Cb
    return rows


def mlp_step(batch=24576, dims=(840, 512, 512, 336), reps=10):
    net = mlp.MLP(dims, max_batch=batch)
    g = torch.Generator(device="cuda").manual_seed(1)
    X = torch.randn((batch, dims[0]), generator=g, device="cuda").bfloat16()
    XT = mlp.transpose_bf16(X)
    T = torch.randn((batch, dims[3]), generator=g, device="cuda")
    flops = 2.0 * batch * sum(dims[i] * dims[i + 1] for i in range(3))

    def step():
        Y = net.forward(X, XT, train=True)
        net.backward(Y, T)
        net.step(1e-4)
    ms = _time(step, reps, graph=False)
    msi = _time(lambda: net.forward(X), reps)
    out = {"mlp": list(dims), "batch": batch, "train_step_ms": ms,
           "train_tflops": 3 * flops / ms / 1e9, "infer_ms": msi, "infer_tflops": flops / msi / 1e9}
    print(json.dumps(out), flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--shapes", type=str, default=None)
    ap.add_argument("--no-cublas", action="store_true")
    ap.add_argument("--no-mlp", action="store_true")
    a = ap.parse_args()
    shapes = CLOSURE_SHAPES + SQUARE_SHAPES
    if a.shapes:
        shapes = [tuple(int(v) for v in s.split(",")) for s in a.shapes.split(";")]
    run(shapes, a.reps, not a.no_cublas)
    if not a.no_mlp:
        mlp_step()


if __name__ == "__main__":
    main()
