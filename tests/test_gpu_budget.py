"""The default work budget: min(24 GiB, free device memory / 4).  The free memory a
build sees excludes the working buffers the engine keeps from its previous build, so
a build of the same shape as the last one takes that build's plan (and buffers)
again.  Under memory pressure (a filler tensor leaves 48 GB free) the budget binds:
the second of two identical builds must tile r1 like the first and give the same
bits, and cutc_plan must report that plan beside the first build's buffers.
"""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth

pytestmark = pytest.mark.gpu


def test_default_budget_counts_the_engines_working_buffers():
    import torch
    cg.load().cutc_release()
    torch.cuda.empty_cache()
    free, _ = torch.cuda.mem_get_info()
    keep = 48 << 30
    if free < keep + (8 << 30):
        pytest.skip("needs more than 56 GB of free device memory")
    filler = torch.empty(free - keep, dtype=torch.uint8, device="cuda")
    try:
        # 2.97 MB per r1 row in a tile: a 12 GiB budget takes two tiles of 4300 rows; a
        # budget from the free memory beside the first build's 14 GB of buffers, three
        p = synth.make_problem(n_nuc=4, n_ao=40, n_grid1=8600, n_grid2=40000, size_bh=6, seed=5)
        args = (p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, cg.SPLIT_BF16, 5)
        lone = cg.plan(*args)
        assert lone["n_tiles"] == 2, lone  # the budget binds
        X1, I1, st1 = cg.build_integrals(p, cg.SPLIT_BF16, with_stats=True)
        beside = cg.plan(*args)  # the engine now holds the first build's working buffers
        X2, I2, st2 = cg.build_integrals(p, cg.SPLIT_BF16, with_stats=True)
        assert beside["n_tiles"] == lone["n_tiles"], (lone, beside)
        assert st1["n_r1_tiles"] == st2["n_r1_tiles"] == lone["n_tiles"], (st1, st2, lone)
        assert np.array_equal(X1, X2) and np.array_equal(I1, I2)
    finally:
        del filler
        cg.load().cutc_release()
        torch.cuda.empty_cache()
