"""The plain FP64 form on a medium-workload r1 sample, for profiling its DGEMMs.

    python -m cutc_gb300.profile_plain --rows 256 --reps 2

Builds the medium molecule (10 nuclei, 120 AOs, 80 000 r2 points) on `rows` r1
points spread over its grid in the plain FP64 form and prints the per-phase times
from the library's CUDA events.  The X contraction is one cuBLAS strided-batched
DGEMM (M = 7260 packed AO pairs, N = rows, K = 80 000, 4 batches); the device
holds about 6 GB.  Also the command the committed ncu summary of that DGEMM was
captured with.
"""
import argparse
import json

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rows", type=int, default=256)
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args()
    import dataclasses
    import cutc_gb300 as cg
    from cutc_gb300 import synth
    p = synth.make_config("medium")
    idx = np.unique(np.linspace(0, p.n_grid1 - 1, a.rows).round().astype(np.int64))
    sub = dataclasses.replace(p, r1=np.ascontiguousarray(p.r1[idx]),
                              wr1=np.ascontiguousarray(p.wr1[idx]),
                              aos1=np.ascontiguousarray(p.aos1[:, :, idx]))
    for _ in range(a.reps):
        _, _, st = cg.build_integrals(sub, cg.PLAIN_FP64, with_stats=True)
    n = len(idx)
    np_ = p.n_ao * (p.n_ao + 1) // 2
    flops_x = 2.0 * np_ * 4 * n * p.n_grid2
    print(json.dumps({"rows": n, "ms_total": st["ms_total"], "ms_x_gemm": st["ms_x_gemm"],
                      "ms_int2e": st["ms_int2e"], "ms_pair": st["ms_pair"],
                      "x_dgemm_tflops": flops_x / st["ms_x_gemm"] / 1e9}))


if __name__ == "__main__":
    main()
