"""GPU parity of the plain FP64 form against the oracle and the reference's golden vectors.

Tolerances: the plain form differs from the reference only in summation order
(packed contractions, per-nucleus term grouping), so X and int_2e must agree to
1e-12 relative (normwise and max-abs/max) -- well inside the 1e-10 drop-in
tolerance -- and the pair planes to 1e-13.
"""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth
from golden_util import CASE_NAMES, load_case
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL_PLAIN = 1e-12


def _dims(ref):
    return tuple(int(v) for v in ref["dims"])


@pytest.mark.parametrize("name", CASE_NAMES)
def test_drop_in_cutc_int_matches_reference(name):
    p, ref = load_case(name)
    X = np.full((3, p.n_grid1, p.n_ao ** 2), np.nan)
    I = np.full((p.n_ao ** 2, p.n_ao ** 2), np.nan)
    s = cg.cutc_int(*_dims(ref), p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                    p.r1, p.wr1, p.r2, p.wr2, p.rn, p.aos1, p.aos2,
                    p.c_bh, p.m_bh, p.n_bh, p.o_bh, X, I)
    assert s == 0, cg.last_error()
    ex, ei = oracle.rel_err(X, ref["X"]), oracle.rel_err(I, ref["int2e"])
    assert ex["norm"] < TOL_PLAIN and ex["max"] < TOL_PLAIN, ex
    assert ei["norm"] < TOL_PLAIN and ei["max"] < TOL_PLAIN, ei


@pytest.mark.parametrize("name", CASE_NAMES)
def test_pair_kernel_matches_reference(name):
    import torch
    p, ref = load_case(name)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    G = torch.full((4, p.n_grid1, p.n_grid2), float("nan"), dtype=torch.float64, device="cuda")
    s = cg.jast_bh_device(d(p.r1), d(p.r2), d(p.rn), d(p.c_bh), d(p.m_bh), d(p.n_bh),
                          d(p.o_bh), G)
    assert s == 0, cg.last_error()
    Gh = G.cpu().numpy()
    scale = np.abs(ref["G"]).reshape(4, -1).max(axis=1)[:, None, None]
    assert np.all(np.abs(Gh - ref["G"]) <= 1e-13 * scale)


def test_pair_kernel_row_block():
    """A block of r1 rows [i0, i0+n1b) lands at block-local rows, like cutc_int_bh's ii0."""
    import torch
    p, ref = load_case("tiny_spd")
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    G = torch.zeros((4, 20, p.n_grid2), dtype=torch.float64, device="cuda")
    s = cg.jast_bh_device(d(p.r1), d(p.r2), d(p.rn), d(p.c_bh), d(p.m_bh), d(p.n_bh),
                          d(p.o_bh), G, i0=30, n1b=20)
    assert s == 0, cg.last_error()
    np.testing.assert_allclose(G.cpu().numpy(), ref["G"][:, 30:50], rtol=0, atol=1e-13 * np.abs(ref["G"]).max())


def test_small_workload_plain_vs_oracle():
    p = synth.make_config("small")
    X, I = cg.build_integrals(p, cg.PLAIN_FP64)
    Xo, Io = oracle.cutc_int(p)
    ex, ei = oracle.rel_err(X, Xo), oracle.rel_err(I, Io)
    assert ex["norm"] < TOL_PLAIN and ex["max"] < TOL_PLAIN, ex
    assert ei["norm"] < TOL_PLAIN and ei["max"] < TOL_PLAIN, ei


def test_r1_tiling_is_exact():
    """Forcing many r1 tiles must not change X or int_2e (the reference accumulates
    onto uninitialised memory when it splits r1, src/build_int2_grad1_u12_ao.cu:166)."""
    p = synth.make_problem(n_nuc=3, n_ao=9, n_grid1=300, n_grid2=700, size_bh=6, seed=21)
    X1, I1 = cg.build_integrals(p, cg.PLAIN_FP64)
    row_bytes = 4 * p.n_grid2 * 8
    X2, I2, st = cg.build_integrals(p, cg.PLAIN_FP64, max_work_bytes=37 * row_bytes, with_stats=True)
    assert st["n_r1_tiles"] >= 3
    assert oracle.rel_err(X2, X1)["max"] < 1e-14
    assert oracle.rel_err(I2, I1)["max"] < 1e-13


def test_jastrow_scale_factors_vs_oracle():
    p = synth.make_problem(n_nuc=2, n_ao=6, n_grid1=120, n_grid2=400, size_bh=5, seed=5,
                           a_en=0.7, a_ee=1.6)
    X, I = cg.build_integrals(p, cg.PLAIN_FP64, x_components=4)
    Xo, Io = oracle.cutc_int(p)
    ex, ei = oracle.rel_err(X[:3], Xo), oracle.rel_err(I, Io)
    assert ex["max"] < TOL_PLAIN and ei["max"] < TOL_PLAIN, (ex, ei)


def test_launch_dims_rejected_like_reference():
    p, ref = load_case("tiny_coalesce")
    X = np.zeros((3, p.n_grid1, p.n_ao ** 2))
    I = np.zeros((p.n_ao ** 2, p.n_ao ** 2))
    args = (p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh, p.r1, p.wr1, p.r2, p.wr2, p.rn,
            p.aos1, p.aos2, p.c_bh, p.m_bh, p.n_bh, p.o_bh, X, I)
    assert cg.cutc_int(1, 1, 1, 64, 32, 1, *args) == cg.CUTC_ERR_LAUNCH_DIMS  # 2048 threads
    assert cg.cutc_int(1, 70000, 1, 32, 1, 1, *args) == cg.CUTC_ERR_LAUNCH_DIMS  # grid.y
    assert cg.cutc_int(1, 1, 1, 32, 32, 1, *args) == 0


def test_bad_exponent_is_rejected():
    p, ref = load_case("tiny_coalesce")
    p.o_bh = p.o_bh.copy()
    p.o_bh[0, 0] = 7
    with pytest.raises(cg.CutcError) as e:
        cg.build_integrals(p)
    assert e.value.status == cg.CUTC_ERR_INVALID
