"""The allocation-free pair-terms entry point (cutc_jast_bh_dev_noalloc).

Callers that cannot let a library allocate device memory -- code being
captured into a CUDA graph, latency-critical serving loops where cudaMalloc
would synchronise the device, programs whose own memory manager owns the
device -- use this entry point: its scratch is a fixed 32 MiB array inside the
library.  These tests call it through the C-ABI and check it against the
allocating entry point cutc_jast_bh_dev on two calls in a row (the second call
reuses the scratch the first one left behind), within the 1e-13 tolerance of
the other pair-kernel tests, and check that an oversized request is refused.
This file is collected last on purpose.
"""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth

pytestmark = pytest.mark.gpu


def _dev(p):
    import torch
    return {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in p.arrays().items()}


def _run(fn, d, n1b, n2, i0=0, a_en=1.0, a_ee=1.0):
    import torch
    G = torch.full((4, n1b, n2), float("nan"), dtype=torch.float64, device="cuda")
    s = fn(d["r1"], d["r2"], d["rn"], d["c_bh"], d["m_bh"], d["n_bh"], d["o_bh"], G,
           i0=i0, n1b=n1b, a_en=a_en, a_ee=a_ee)
    assert s == cg.CUTC_OK, cg.last_error()
    return G.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    cases = [
        (synth.add_coalescence(synth.make_problem(n_nuc=3, n_ao=4, n_grid1=200, n_grid2=3000,
                                                  size_bh=9, seed=31)), 40, 120, 1.0, 1.0),
        (synth.make_problem(n_nuc=5, n_ao=4, n_grid1=150, n_grid2=2000, size_bh=6, seed=32),
         0, 150, 0.8, 1.3),
    ]
    for p, i0, n1b, a_en, a_ee in cases:  # two calls in a row, different shapes
        d = _dev(p)
        ref = _run(cg.jast_bh_device, d, n1b, p.n_grid2, i0, a_en, a_ee)
        got = _run(cg.jast_bh_device_noalloc, d, n1b, p.n_grid2, i0, a_en, a_ee)
        torch.cuda.synchronize()
        scale = np.abs(ref).reshape(4, -1).max(axis=1)[:, None, None]
        assert np.all(np.isfinite(got))
        assert np.all(np.abs(got - ref) <= 1e-13 * scale)


def test_noalloc_rejects_requests_beyond_its_scratch():
    import torch
    n2 = 700000  # 8 * n2 * n_nuc bytes of r2 terms alone exceed 32 MiB
    p = synth.make_problem(n_nuc=6, n_ao=2, n_grid1=8, n_grid2=64, size_bh=3, seed=33)
    d = _dev(p)
    d["r2"] = torch.zeros((n2, 3), dtype=torch.float64, device="cuda")
    G = torch.zeros((4, 1, n2), dtype=torch.float64, device="cuda")
    s = cg.jast_bh_device_noalloc(d["r1"], d["r2"], d["rn"], d["c_bh"], d["m_bh"], d["n_bh"],
                                  d["o_bh"], G, i0=0, n1b=1)
    assert s == cg.CUTC_ERR_INVALID
    assert "static scratch" in cg.last_error()
