"""Both precision forms against the FP64 oracle at the full n_ao and n_grid2 of
every measured configuration, on r1 samples.

The configurations: medium (10 nuclei, n_ao 120, n_grid2 80 000), large
(20 nuclei, n_ao 300, n_grid2 200 000), the scan molecule (8 nuclei, n_ao 80,
n_grid2 50 000) at both ends of its a_en / a_ee range (0.5 and 2.0), and a
serving-stream molecule at the top of its n_ao range (20 nuclei, n_ao 250,
n_grid2 80 000).  Each runs on 32 r1 points spread over its whole r1 grid.

The oracle forms X from the C restatement of the reference's pair and product
kernels (src/jast_bh.cu:115-254, src/long_range_integ.cu:21-45) with r2
windows summed in FP64 (oracle.x_rows), and int_2e's rows and its product with
a random vector from the short-range products
(src/short_range_integ_herm.cu:20-44, src/short_range_integ_nonherm.cu:23-63)
without forming the n_ao^4 matrix.  The library's outputs stay on the device;
the test reads X, the same int_2e rows and int_2e v.

Tolerances (relative, normwise and max-abs/max): 1e-12 for the plain FP64
form (the drop-in), 1e-10 for the split form at its default 5 slices, and
1e-12 for the split form at 6 slices, which reaches the plain form's error
class.
"""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu

ROWS = 32
FORMS = ((cg.SPLIT_BF16, 5, 1e-10), (cg.SPLIT_BF16, 6, 1e-12), (cg.PLAIN_FP64, None, 1e-12))

CASES = {
    "medium": lambda: synth.make_config("medium"),
    "large": lambda: synth.make_config("large"),
    "scan_a0.5_2.0": lambda: synth.make_config("scan", a_en=0.5, a_ee=2.0),
    "scan_a2.0_0.5": lambda: synth.make_config("scan", a_en=2.0, a_ee=0.5),
    "serving_nao250": lambda: synth.serving_molecule(n_nuc=20, n_ao=250),
}


def _release():
    import torch
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    cg.load().cutc_release()


@pytest.mark.parametrize("name", list(CASES))
def test_both_forms_vs_oracle_at_full_size(name):
    import torch
    p = CASES[name]()
    sub = synth.r1_sample(p, ROWS)
    nA2 = sub.n_ao ** 2
    rng = np.random.default_rng(2024)
    rows = np.sort(rng.choice(nA2, min(nA2, 48), replace=False))
    v = rng.standard_normal(nA2)

    X4 = oracle.x_rows(sub)
    S0, S = oracle.short_herm(sub), oracle.short_nonherm(sub)
    I_rows = oracle.int2e_rows(sub, X4, rows, S0, S)
    I_v = oracle.int2e_matvec(sub, X4, v, S0, S)

    _release()
    out = None
    try:
        for prec, n_slices, tol in FORMS:
            X, I = cg.build_integrals_device(sub, prec, n_slices=n_slices, out=out)
            out = (X, I)
            got_x = X.cpu().numpy()
            got_rows = I[torch.from_numpy(rows).to(I.device)].cpu().numpy()
            got_v = (I @ torch.from_numpy(v).to(I.device)).cpu().numpy()
            _release()
            for what, a, b in (("X", got_x, X4[:3]), ("int_2e rows", got_rows, I_rows),
                               ("int_2e v", got_v, I_v)):
                e = oracle.rel_err(a, b)
                assert e["norm"] < tol and e["max"] < tol, (name, prec, n_slices, what, e)
    finally:
        del out
        _release()
