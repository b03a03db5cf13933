"""Micro-benchmark of the double-float pair kernel inside a split-form build.

    python -m cutc_gb300.profile_pair --n-nuc 10 --terms 13 --n1 1024 --n2 80000 --reps 3

Builds a molecule with the medium workload's nuclei and Jastrow terms but few
AOs (the pair terms do not depend on n_ao), so the device holds a few GB, and
prints the pair-kernel time per build from the library's own CUDA events and
the rate in (r1, r2, nucleus) evaluations per second.  Also the command the
committed ncu summary of pair_df_kernel was captured with.
"""
import argparse
import json


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-nuc", type=int, default=10)
    ap.add_argument("--terms", type=int, default=13)
    ap.add_argument("--n-ao", type=int, default=40)
    ap.add_argument("--n1", type=int, default=1024)
    ap.add_argument("--n2", type=int, default=80000)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    import cutc_gb300 as cg
    from cutc_gb300 import synth
    p = synth.make_problem(n_nuc=a.n_nuc, n_ao=a.n_ao, n_grid1=a.n1, n_grid2=a.n2,
                           size_bh=a.terms, seed=2002, box=6.0)
    pair_ms = []
    for _ in range(a.reps):
        _, _, st = cg.build_integrals(p, cg.SPLIT_BF16, with_stats=True)
        pair_ms.append(st["ms_pair"])
    ms = min(pair_ms)
    evals = float(a.n1) * a.n2 * a.n_nuc
    print(json.dumps({"n_nuc": a.n_nuc, "terms_per_nucleus": a.terms, "n1": a.n1, "n2": a.n2,
                      "pair_ms": ms, "pairs_per_s": a.n1 * a.n2 / ms * 1e3,
                      "pair_nucleus_evals_per_s": evals / ms * 1e3}))


if __name__ == "__main__":
    main()
