"""The split-precision form (BF16 slices on tcgen05) of the whole build.

Tolerance: 1e-10 relative (normwise and max-abs/max) against the FP64 oracle
for X and int_2e at the default 5 slices -- the accuracy target of the split
form.  The plain FP64 form is the drop-in; this form trades the last ~2
decimal digits for tensor-core speed.
"""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth
from golden_util import CASE_NAMES, load_case
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL_SPLIT = 1e-10


def _check(X, I, Xr, Ir, tol=TOL_SPLIT):
    ex, ei = oracle.rel_err(X, Xr), oracle.rel_err(I, Ir)
    assert ex["norm"] < tol and ex["max"] < tol, ex
    assert ei["norm"] < tol and ei["max"] < tol, ei
    return ex, ei


@pytest.mark.parametrize("name", CASE_NAMES)
def test_split_matches_reference_golden(name):
    p, ref = load_case(name)
    X, I = cg.build_integrals(p, cg.SPLIT_BF16)
    _check(X, I, ref["X"], ref["int2e"])


def test_split_small_workload_vs_oracle():
    p = synth.make_config("small")
    X, I = cg.build_integrals(p, cg.SPLIT_BF16)
    Xo, Io = oracle.cutc_int(p)
    _check(X, I, Xo, Io)


def test_split_r1_tiling_is_exact():
    p = synth.make_problem(n_nuc=3, n_ao=9, n_grid1=300, n_grid2=700, size_bh=6, seed=21)
    X1, I1 = cg.build_integrals(p, cg.SPLIT_BF16)
    X2, I2, st = cg.build_integrals(p, cg.SPLIT_BF16, max_work_bytes=2 << 20, with_stats=True)
    assert st["n_r1_tiles"] > 1
    # the slices of each G row do not depend on the tile, so X is the same bits;
    # int_2e is sliced per r1 tile (per-tile row scales), so its split rounding
    # differs by up to the split tolerance
    assert np.array_equal(X1, X2)
    assert oracle.rel_err(I2, I1)["max"] < 1e-12


def test_split_k_launches():
    """k_split cuts each contraction into K launches whose results are summed in FP64
    (the path every X contraction longer than K = 65536 takes): the oracle's results at
    the split tolerance, the one-launch build's within 1e-12, and the stats count every
    X-contraction launch."""
    p = synth.make_problem(n_nuc=3, n_ao=10, n_grid1=260, n_grid2=1500, size_bh=6, seed=31)
    X1, I1, st1 = cg.build_integrals(p, cg.SPLIT_BF16, with_stats=True)
    X2, I2, st2 = cg.build_integrals(p, cg.SPLIT_BF16, k_split=256, with_stats=True)
    Xo, Io = oracle.cutc_int(p)
    _check(X2, I2, Xo, Io)
    assert oracle.rel_err(X2, X1)["max"] < 1e-12
    assert oracle.rel_err(I2, I1)["max"] < 1e-12
    # K = 1500 padded to 1504: 47 blocks of 32, 8 per launch
    assert st1["n_x_gemm"] == st1["n_r1_tiles"]
    assert st2["n_x_gemm"] == 6 * st2["n_r1_tiles"]
    info = cg.plan(p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, cg.SPLIT_BF16, 5, k_split=256)
    assert info["x_launches_per_tile"] == 6


def test_split_four_components_and_scale_factors():
    p = synth.make_problem(n_nuc=2, n_ao=7, n_grid1=150, n_grid2=500, size_bh=5, seed=9,
                           a_en=1.3, a_ee=0.6)
    X, I = cg.build_integrals(p, cg.SPLIT_BF16, x_components=4)
    Xo, Io = oracle.cutc_int(p)
    _check(X[:3], I, Xo, Io)


def test_split_slice_count_controls_accuracy():
    p = synth.make_problem(n_nuc=3, n_ao=10, n_grid1=400, n_grid2=1600, size_bh=9, seed=4)
    Xo, Io = oracle.cutc_int(p)
    errs = []
    for S in (3, 4, 5):
        X, I = cg.build_integrals(p, cg.SPLIT_BF16, n_slices=S)
        errs.append(oracle.rel_err(I, Io)["norm"])
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < TOL_SPLIT


def test_drop_in_env_selects_split(monkeypatch):
    """CUTC_PRECISION=split switches the unmodified cutc_int entry point."""
    p, ref = load_case("tiny_spd")
    monkeypatch.setenv("CUTC_PRECISION", "split")
    X = np.zeros((3, p.n_grid1, p.n_ao ** 2))
    I = np.zeros((p.n_ao ** 2, p.n_ao ** 2))
    s = cg.cutc_int(*[int(v) for v in ref["dims"]], p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc,
                    p.size_bh, p.r1, p.wr1, p.r2, p.wr2, p.rn, p.aos1, p.aos2,
                    p.c_bh, p.m_bh, p.n_bh, p.o_bh, X, I)
    assert s == 0, cg.last_error()
    _check(X, I, ref["X"], ref["int2e"])


def test_drop_in_env_sets_slice_count(monkeypatch):
    """CUTC_SLICES sets the split form's slice count for the drop-in; 6 slices bring it
    within the plain form's 1e-12 of the reference's own outputs; a count outside 3..7
    is refused."""
    p, ref = load_case("tiny_spd")
    monkeypatch.setenv("CUTC_PRECISION", "split")
    dims = [int(v) for v in ref["dims"]]

    def call():
        X = np.zeros((3, p.n_grid1, p.n_ao ** 2))
        I = np.zeros((p.n_ao ** 2, p.n_ao ** 2))
        s = cg.cutc_int(*dims, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh, p.r1, p.wr1,
                        p.r2, p.wr2, p.rn, p.aos1, p.aos2, p.c_bh, p.m_bh, p.n_bh, p.o_bh, X, I)
        return s, X, I

    monkeypatch.setenv("CUTC_SLICES", "6")
    s, X, I = call()
    assert s == 0, cg.last_error()
    _check(X, I, ref["X"], ref["int2e"], tol=1e-12)
    for bad in ("8", "2", "five", "6x"):
        monkeypatch.setenv("CUTC_SLICES", bad)
        s, _, _ = call()
        assert s == cg.CUTC_ERR_INVALID, bad
        assert "n_slices" in cg.last_error()


@pytest.mark.parametrize("n_slices", [6, 7])
def test_six_and_seven_slices_reach_fp64_class_errors(monkeypatch, n_slices):
    """Builds of 6 and 7 slices: the pair contraction on the tensor cores with 6 slices
    against the double-float pair kernel, and both against the oracle at 1e-12 (the
    plain FP64 form's tolerance), with e-e coalescence and 20 nuclei (K = 80)."""
    for n_nuc, coalesce in ((5, True), (20, False)):
        p = synth.make_problem(n_nuc=n_nuc, n_ao=8, n_grid1=260, n_grid2=900, size_bh=9,
                               seed=90 + n_nuc, a_en=1.1, a_ee=0.8, box=1.5 + 0.4 * n_nuc)
        if coalesce:
            p = synth.add_coalescence(p)
        monkeypatch.delenv("CUTC_PAIR_DF", raising=False)
        X1, I1 = cg.build_integrals(p, cg.SPLIT_BF16, n_slices=n_slices, x_components=4)
        monkeypatch.setenv("CUTC_PAIR_DF", "1")
        X2, I2 = cg.build_integrals(p, cg.SPLIT_BF16, n_slices=n_slices, x_components=4)
        assert oracle.rel_err(X1, X2)["max"] < 1e-13
        assert oracle.rel_err(I1, I2)["max"] < 1e-13
        Xo, Io = oracle.cutc_int(p)
        _check(X1[:3], I1, Xo, Io, tol=1e-12)
        _check(X2[:3], I2, Xo, Io, tol=1e-12)


def test_sparse_power_pair_kernel_matches_general(monkeypatch):
    """Exponents in {0, 2, 3, 4} select the sparse-power df pair kernel; the general
    kernel (CUTC_PAIR_DENSE) evaluates the same polynomials in another order."""
    p = synth.make_problem(n_nuc=4, n_ao=9, n_grid1=300, n_grid2=1200, size_bh=9, seed=17,
                           a_en=0.8, a_ee=1.3)
    assert set(np.unique(np.concatenate([p.m_bh.ravel(), p.n_bh.ravel(), p.o_bh.ravel()]))) <= {0, 2, 3, 4}
    X1, I1 = cg.build_integrals(p, cg.SPLIT_BF16, x_components=4)
    monkeypatch.setenv("CUTC_PAIR_DENSE", "1")
    X2, I2 = cg.build_integrals(p, cg.SPLIT_BF16, x_components=4)
    assert oracle.rel_err(X1, X2)["max"] < 1e-12
    assert oracle.rel_err(I1, I2)["max"] < 1e-12
    Xo, Io = oracle.cutc_int(p)
    _check(X1[:3], I1, Xo, Io)


@pytest.mark.parametrize("n_nuc,coalesce", [(6, False), (3, True), (20, False), (1, False)])
def test_tensor_core_pair_terms_match_double_float_kernel(monkeypatch, n_nuc, coalesce):
    """With exponents in {0, 2, 3, 4} and up to 20 nuclei the split form's pair terms
    run on the tensor cores (a contraction over nucleus and power of f2, K = 4 n_nuc);
    CUTC_PAIR_DF selects the double-float kernel.  Both against each other and the
    oracle, including e-e and e-n coalescence (the FP64 path of the epilogue) and
    K = 80 (20 nuclei), the largest contraction whose leading diagonals stay exact."""
    p = synth.make_problem(n_nuc=n_nuc, n_ao=8, n_grid1=260, n_grid2=900, size_bh=9,
                           seed=70 + n_nuc, a_en=0.9, a_ee=1.2, box=1.5 + 0.4 * n_nuc)
    if coalesce:
        p = synth.add_coalescence(p)
    X1, I1 = cg.build_integrals(p, cg.SPLIT_BF16, x_components=4)
    monkeypatch.setenv("CUTC_PAIR_DF", "1")
    X2, I2 = cg.build_integrals(p, cg.SPLIT_BF16, x_components=4)
    assert oracle.rel_err(X1, X2)["max"] < 1e-12
    assert oracle.rel_err(I1, I2)["max"] < 1e-12
    Xo, Io = oracle.cutc_int(p)
    _check(X1[:3], I1, Xo, Io)
