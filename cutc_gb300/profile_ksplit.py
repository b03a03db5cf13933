"""Split-form builds with different caps on K per tensor-core launch.

    python -m cutc_gb300.profile_ksplit --config large --rows 1500 --k-split 0 40000 200000

Builds a device-resident r1 sample of a named workload (rows spread over its r1
grid, full n_ao and n_grid2) once per `k_split` value, repeated, and prints the
library's per-phase times (CUDA events).  k_split 0 is the automatic choice;
a value >= n_grid2 forces one launch.  The large workload holds about 220 GB on
the device for a 1500-row sample.
"""
import argparse
import json
import os
import sys


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="large")
    ap.add_argument("--rows", type=int, default=1500)
    ap.add_argument("--k-split", type=int, nargs="+", default=[0, 40000])
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args()
    import numpy as np
    import torch
    import cutc_gb300 as cg
    from cutc_gb300 import synth
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    p = synth.make_config(a.config)
    ns = min(a.rows, p.n_grid1)
    sub = bench.strided_rows(p, ns) if ns < p.n_grid1 else p
    dev = torch.device("cuda", 0)
    dr = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in sub.arrays().items()}
    nA2 = p.n_ao ** 2
    X = torch.empty((3, ns, nA2), dtype=torch.float64, device=dev)
    I = torch.empty((nA2, nA2), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def build(ks):
        opt = cg.options(cg.SPLIT_BF16, 5, p.a_en, p.a_ee, 3, True, 0, stream.cuda_stream,
                         k_split=ks)
        st = cg.Stats()
        s = cg.cutc_int_ex(opt, ns, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh, dr["r1"], dr["wr1"],
                           dr["r2"], dr["wr2"], dr["rn"], dr["aos1"], dr["aos2"], dr["c_bh"],
                           dr["m_bh"], dr["n_bh"], dr["o_bh"], X, I, st)
        if s != cg.CUTC_OK:
            raise cg.CutcError(s, cg.last_error())
        return st.as_dict()

    build(a.k_split[0])  # warm-up: workspace
    for _ in range(a.reps):
        for ks in a.k_split:
            d = build(ks)
            print(json.dumps({"config": a.config, "r1_rows": ns, "k_split": ks,
                              "ms_total": round(d["ms_total"], 1),
                              "ms_x_gemm": round(d["ms_x_gemm"], 1),
                              "ms_int2e": round(d["ms_int2e"], 1),
                              "x_launch_tiles": d["n_x_gemm"]}), flush=True)


if __name__ == "__main__":
    main()
