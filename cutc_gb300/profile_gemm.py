"""Micro-benchmark of the split-precision contraction (cutc_split_gemm_dev).

    python -m cutc_gb300.profile_gemm --m 7260 --n 2048 --k 16384 --slices 5 --reps 3

Runs C = A B^T on seeded FP64 operands shaped like the X build of cutc_int
(m packed AO pairs, n = 4 x r1 points, k = r2 points) and prints the time per
launch and the rates.  Also the command the committed ncu summaries of the
kernel were captured with.
"""
import argparse
import json

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--m", type=int, default=7260)
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--k", type=int, default=16384)
    ap.add_argument("--slices", type=int, default=5)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    import torch
    import cutc_gb300 as cg
    g = torch.Generator(device="cuda").manual_seed(1234)
    A = torch.randn((a.m, a.k), dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn((a.n, a.k), dtype=torch.float64, device="cuda", generator=g)
    C = torch.empty((a.n, a.m), dtype=torch.float64, device="cuda")
    times = []
    for _ in range(a.reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        cg.split_gemm_device(A, B, C, n_slices=a.slices)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    S = a.slices
    alg = 2.0 * a.m * a.n * a.k
    ms = min(times)
    print(json.dumps({"m": a.m, "n": a.n, "k": a.k, "slices": S, "ms_call": ms,
                      "fp64_equiv_tflops": alg / ms / 1e9,
                      "bf16_tflops_executed": alg * S * (S + 1) / 2 / ms / 1e9,
                      "note": "call time includes slicing both operands"}))


if __name__ == "__main__":
    main()
