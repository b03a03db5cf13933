"""Sizes past 32-bit indexing: one r1 tile whose G holds 4 x 7000 x 80 000 =
2.24e9 elements (> 2^31), the size at which the reference's int indices overflow
(its G is 4 n1 n2 doubles).  The build must equal the same build cut into small
tiles (r1 tiling is exact up to cuBLAS's blocking of the plain form), and its first
and last rows must match the oracle."""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
def test_tile_past_int32_indices(prec, monkeypatch):
    p = synth.make_problem(n_nuc=2, n_ao=6, n_grid1=7000, n_grid2=80000, size_bh=5, seed=71)
    assert 4 * p.n_grid1 * p.n_grid2 > 2 ** 31
    budget = 64 << 30  # the whole r1 grid in one tile
    X1, I1, st = cg.build_integrals(p, prec, max_work_bytes=budget, with_stats=True)
    assert st["n_r1_tiles"] == 1
    monkeypatch.setenv("CUTC_TILE_ROWS", "1000")
    X2, I2, st2 = cg.build_integrals(p, prec, max_work_bytes=budget, with_stats=True)
    assert st2["n_r1_tiles"] == 7
    assert oracle.rel_err(X2, X1)["max"] < 1e-14  # cuBLAS may block other N differently
    assert oracle.rel_err(I2, I1)["max"] < 1e-13
    # the first and the last r1 rows against the oracle
    tol = 1e-12 if prec == cg.PLAIN_FP64 else 1e-10
    P = oracle.long_range(p)
    for i0 in (0, p.n_grid1 - 16):
        Xo = oracle.x_block(p, P, i0, 16)[:3]
        assert oracle.rel_err(X1[:, i0:i0 + 16], Xo)["max"] < tol
