"""The allocation-free pair-terms entry point (cutc_jast_bh_dev_noalloc).

Some callers cannot let a library allocate device memory: programs whose own
memory manager has reserved the whole device, and serving loops that must not
stall on cudaMalloc / cudaFree.  This entry point serves them with a fixed
32 MiB scratch array inside the library.  These tests call it through the
C-ABI and check
  * its output against the allocating entry point cutc_jast_bh_dev, within the
    1e-13 tolerance of the other pair-kernel tests, on two calls in a row (the
    second reuses the scratch the first one left behind), and on a side stream;
  * its output against the reference's own pair planes (tests/golden), which
    pins its device-side term table independently of cutc_jast_bh_dev;
  * that a warm call allocates nothing (device free memory and torch's
    allocator unchanged);
  * the refusals: a request beyond the scratch, an exponent outside [0, 6],
    more than 4096 kept terms.
This file is collected last on purpose.
"""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth
from golden_util import CASE_NAMES, load_case

pytestmark = pytest.mark.gpu


def _dev(p):
    import torch
    return {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in p.arrays().items()}


def _run(fn, d, n1b, n2, i0=0, a_en=1.0, a_ee=1.0, **kw):
    import torch
    G = torch.full((4, n1b, n2), float("nan"), dtype=torch.float64, device="cuda")
    s = fn(d["r1"], d["r2"], d["rn"], d["c_bh"], d["m_bh"], d["n_bh"], d["o_bh"], G,
           i0=i0, n1b=n1b, a_en=a_en, a_ee=a_ee, **kw)
    assert s == cg.CUTC_OK, cg.last_error()
    torch.cuda.synchronize()
    return G.cpu().numpy()


def _close(got, ref, tol=1e-13):
    scale = np.abs(ref).reshape(4, -1).max(axis=1)[:, None, None]
    assert np.all(np.isfinite(got))
    assert np.all(np.abs(got - ref) <= tol * scale)


def test_noalloc_matches_allocating_entry_point_twice():
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
        _close(got, ref)


def test_noalloc_matches_reference_golden_planes():
    for name in CASE_NAMES:
        p, ref = load_case(name)
        got = _run(cg.jast_bh_device_noalloc, _dev(p), p.n_grid1, p.n_grid2, 0, p.a_en, p.a_ee)
        _close(got, ref["G"])


def test_noalloc_on_a_side_stream_allocates_nothing():
    import torch
    p = synth.make_problem(n_nuc=4, n_ao=3, n_grid1=96, n_grid2=2500, size_bh=9, seed=34)
    d = _dev(p)
    ref = _run(cg.jast_bh_device, d, p.n_grid1, p.n_grid2)
    side = torch.cuda.Stream()
    G = torch.full((4, p.n_grid1, p.n_grid2), float("nan"), dtype=torch.float64, device="cuda")
    call = lambda: cg.jast_bh_device_noalloc(d["r1"], d["r2"], d["rn"], d["c_bh"], d["m_bh"],
                                             d["n_bh"], d["o_bh"], G, stream=side.cuda_stream)
    assert call() == cg.CUTC_OK, cg.last_error()  # warm: set-up done, kernels loaded
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    G.fill_(float("nan"))
    torch.cuda.synchronize()
    assert call() == cg.CUTC_OK, cg.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == alloc0
    _close(G.cpu().numpy(), ref)


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


def test_noalloc_reports_bad_exponents_and_too_many_terms():
    import dataclasses
    import torch
    p = synth.make_problem(n_nuc=2, n_ao=2, n_grid1=16, n_grid2=300, size_bh=4, seed=35)
    m = p.m_bh.copy()
    m[1, 2] = 7
    bad = [dataclasses.replace(p, m_bh=m)]
    # 2 nuclei x 2100 terms with |c| >= 1e-10: 4200 kept terms, over the 4096 limit
    rng = np.random.default_rng(36)
    big = (2, 2100)
    bad.append(dataclasses.replace(
        p, c_bh=rng.uniform(0.5, 1.0, big), m_bh=np.full(big, 2, np.int32),
        n_bh=np.full(big, 3, np.int32), o_bh=np.full(big, 2, np.int32)))
    for q in bad:
        d = _dev(q)
        G = torch.zeros((4, q.n_grid1, q.n_grid2), dtype=torch.float64, device="cuda")
        s = cg.jast_bh_device_noalloc(d["r1"], d["r2"], d["rn"], d["c_bh"], d["m_bh"], d["n_bh"],
                                      d["o_bh"], G)
        assert s == cg.CUTC_ERR_INVALID
        assert "exponent" in cg.last_error()
    # the entry point is usable afterwards: the status word is cleared per call
    got = _run(cg.jast_bh_device_noalloc, _dev(p), p.n_grid1, p.n_grid2)
    ref = _run(cg.jast_bh_device, _dev(p), p.n_grid1, p.n_grid2)
    _close(got, ref)
