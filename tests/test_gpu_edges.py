"""Edge cases of the sizes against the oracle, both forms: one AO (no strict pairs,
so no antisymmetric part), two AOs, no Jastrow terms (everything exactly zero,
including the split slicer's all-zero rows), single-point grids, and exponents at
their upper limit of 6."""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL = {cg.PLAIN_FP64: 1e-12, cg.SPLIT_BF16: 1e-10}
CASES = {
    "one_ao": dict(n_nuc=1, n_ao=1, n_grid1=50, n_grid2=70, size_bh=3, seed=1),
    "two_ao": dict(n_nuc=1, n_ao=2, n_grid1=40, n_grid2=60, size_bh=3, seed=2),
    "single_points": dict(n_nuc=1, n_ao=3, n_grid1=1, n_grid2=1, size_bh=2, seed=4),
    "one_r1_point": dict(n_nuc=2, n_ao=6, n_grid1=1, n_grid2=500, size_bh=4, seed=5),
}


def _check(X, I, Xo, Io, prec):
    ex, ei = oracle.rel_err(X, Xo), oracle.rel_err(I, Io)
    assert ex["max"] < TOL[prec] and ei["max"] < TOL[prec], (ex, ei)


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
@pytest.mark.parametrize("name", sorted(CASES))
def test_small_sizes(name, prec):
    p = synth.make_problem(**CASES[name])
    X, I = cg.build_integrals(p, prec)
    assert np.all(np.isfinite(X)) and np.all(np.isfinite(I))
    _check(X, I, *oracle.cutc_int(p), prec)


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
def test_no_jastrow_terms_gives_zeros(prec):
    p = synth.make_problem(n_nuc=2, n_ao=5, n_grid1=30, n_grid2=40, size_bh=0, seed=3)
    X, I = cg.build_integrals(p, prec)
    assert not np.any(X) and not np.any(I)


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
def test_highest_exponents(prec):
    """Exponents 5 and 6 (the reference's powd_int limit) and 1 in every slot."""
    p = synth.make_problem(n_nuc=2, n_ao=6, n_grid1=120, n_grid2=400, size_bh=4, seed=6)
    p.m_bh = np.ascontiguousarray(np.array([[6, 5, 1, 0], [0, 6, 2, 1]], dtype=np.int32))
    p.n_bh = np.ascontiguousarray(np.array([[1, 6, 5, 2], [6, 0, 1, 5]], dtype=np.int32))
    p.o_bh = np.ascontiguousarray(np.array([[5, 1, 6, 3], [1, 6, 0, 6]], dtype=np.int32))
    X, I = cg.build_integrals(p, prec)
    _check(X, I, *oracle.cutc_int(p), prec)


def test_split_tile_with_more_than_65535_g_rows():
    """One split-form r1 tile of 20 000 rows: its G operand has 4 x 20 000 = 80 000
    rows, past the 65 535 blocks a grid dimension holds (the slicer takes rows
    grid-stride).  The reference tiles any n_grid1 (src/build_int2_grad1_u12_ao.cu:63-99)."""
    p = synth.make_problem(n_nuc=3, n_ao=6, n_grid1=20000, n_grid2=2000, size_bh=6, seed=41)
    plan = cg.plan(p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, cg.SPLIT_BF16, max_work_bytes=24 << 30)
    assert plan["n_tiles"] == 1 and 4 * plan["tile_rows"] > 65535
    X, I, st = cg.build_integrals(p, cg.SPLIT_BF16, max_work_bytes=24 << 30, with_stats=True)
    assert st["n_r1_tiles"] == 1
    Xo, Io = oracle.cutc_int(p)
    _check(X, I, Xo, Io, cg.SPLIT_BF16)


def test_split_x_with_more_than_65535_packed_pairs():
    """n_ao = 370: 68 635 packed AO pairs, so the X contraction's A operand has more rows
    than a grid dimension holds (the slicer takes rows grid-stride).  X alone (int_2e
    would be 150 GB), against the oracle's windowed X."""
    import torch
    p = synth.make_problem(n_nuc=2, n_ao=370, n_grid1=24, n_grid2=400, size_bh=4, seed=42)
    nA2 = p.n_ao ** 2
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in p.arrays().items()}
    X = torch.empty((3, p.n_grid1, nA2), dtype=torch.float64, device="cuda")
    opt = cg.options(cg.SPLIT_BF16, None, p.a_en, p.a_ee, 3, True)
    s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh, d["r1"], d["wr1"],
                       d["r2"], d["wr2"], d["rn"], d["aos1"], d["aos2"], d["c_bh"], d["m_bh"],
                       d["n_bh"], d["o_bh"], X, None)
    torch.cuda.synchronize()
    assert s == cg.CUTC_OK, cg.last_error()
    Xo = oracle.x_rows(p)[:3]
    e = oracle.rel_err(X.cpu().numpy(), Xo)
    assert e["norm"] < TOL[cg.SPLIT_BF16] and e["max"] < TOL[cg.SPLIT_BF16], e
    del X, d
    torch.cuda.empty_cache()
    cg.load().cutc_release()
