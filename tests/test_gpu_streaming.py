"""The streamed build: r1 tiles carried through X and int_2e, outputs copied out
tile by tile (X) and slab by slab (int_2e) while the device works on.

Neither the int_2e slab size nor where the outputs live may change a bit; the
r1 tile size may change only the int_2e sum order (tiles are summed in FP64).
"""
import os

import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL = {cg.PLAIN_FP64: 1e-12, cg.SPLIT_BF16: 1e-11}


def _env_setter(name):
    def set_(v):
        if v is None:
            os.environ.pop(name, None)
        else:
            os.environ[name] = str(v)
    return set_


@pytest.fixture
def slab_cols():
    old = os.environ.get("CUTC_INT2E_SLAB_COLS")
    set_ = _env_setter("CUTC_INT2E_SLAB_COLS")
    yield set_
    set_(old)


@pytest.fixture
def tile_rows():
    """Caps the r1 rows per tile (the same tiles whatever else the build holds)."""
    old = os.environ.get("CUTC_TILE_ROWS")
    set_ = _env_setter("CUTC_TILE_ROWS")
    yield set_
    set_(old)


def _problem():
    # 13 AOs: 169 int_2e columns, so 32-column slabs leave a ragged last slab
    return synth.make_problem(n_nuc=3, n_ao=13, n_grid1=517, n_grid2=1900, size_bh=7, seed=31)


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
def test_slabs_and_tiles(prec, slab_cols):
    p = _problem()
    Xo, Io = oracle.cutc_int(p)
    slab_cols(None)
    X1, I1, st1 = cg.build_integrals(p, prec, with_stats=True)
    assert st1["n_r1_tiles"] == 1
    budget = 3 << 20  # a handful of r1 rows per tile
    X2, I2, st2 = cg.build_integrals(p, prec, max_work_bytes=budget, with_stats=True)
    assert st2["n_r1_tiles"] >= 4
    slab_cols(32)
    X3, I3, st3 = cg.build_integrals(p, prec, max_work_bytes=budget, with_stats=True)
    assert st3["n_r1_tiles"] == st2["n_r1_tiles"]
    # the slab size only changes how int_2e leaves the device
    assert np.array_equal(X3, X2) and np.array_equal(I3, I2)
    # X rows do not depend on the tile they were computed in
    if prec == cg.SPLIT_BF16:
        assert np.array_equal(X2, X1)
    else:
        assert oracle.rel_err(X2, X1)["max"] < 1e-14
    # split int_2e is sliced per r1 tile, so tiling moves its rounding (within TOL)
    assert oracle.rel_err(I2, I1)["max"] < (1e-13 if prec == cg.PLAIN_FP64 else 1e-12)
    for X, I in ((X1, I1), (X2, I2)):
        ex, ei = oracle.rel_err(X, Xo), oracle.rel_err(I, Io)
        assert ex["max"] < TOL[prec] and ei["max"] < TOL[prec], (ex, ei)


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
def test_device_outputs_tiled(prec, tile_rows):
    """Device outputs are written tile by tile straight into the caller's arrays."""
    import torch
    p = _problem()
    tile_rows(40)
    budget = 0
    Xh, Ih = cg.build_integrals(p, prec, x_components=4, max_work_bytes=budget)
    dev = torch.device("cuda", 0)
    dr = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in p.arrays().items()}
    Xd = torch.full((4, p.n_grid1, p.n_ao ** 2), float("nan"), dtype=torch.float64, device=dev)
    Id = torch.full((p.n_ao ** 2, p.n_ao ** 2), float("nan"), dtype=torch.float64, device=dev)
    opt = cg.options(prec, None, p.a_en, p.a_ee, 4, True, budget, None)
    st = cg.Stats()
    s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                       dr["r1"], dr["wr1"], dr["r2"], dr["wr2"], dr["rn"], dr["aos1"], dr["aos2"],
                       dr["c_bh"], dr["m_bh"], dr["n_bh"], dr["o_bh"], Xd, Id, st)
    assert s == 0, cg.last_error()
    torch.cuda.synchronize()
    assert st.n_r1_tiles >= 4
    assert np.array_equal(Xd.cpu().numpy(), Xh)
    assert np.array_equal(Id.cpu().numpy(), Ih)


def test_pinned_outputs_match_pageable(tile_rows):
    """Pinned host outputs take the asynchronous copy path; the bits are the same."""
    import torch
    p = _problem()
    tile_rows(40)
    budget = 0
    Xh, Ih = cg.build_integrals(p, cg.SPLIT_BF16, max_work_bytes=budget)
    Xp = torch.empty((3, p.n_grid1, p.n_ao ** 2), dtype=torch.float64).pin_memory()
    Ip = torch.empty((p.n_ao ** 2, p.n_ao ** 2), dtype=torch.float64).pin_memory()
    opt = cg.options(cg.SPLIT_BF16, None, p.a_en, p.a_ee, 3, False, budget, None)
    s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                       p.r1, p.wr1, p.r2, p.wr2, p.rn, p.aos1, p.aos2,
                       p.c_bh, p.m_bh, p.n_bh, p.o_bh, Xp, Ip)
    assert s == 0, cg.last_error()
    assert np.array_equal(Xp.numpy(), Xh)
    assert np.array_equal(Ip.numpy(), Ih)


@pytest.fixture
def int2e_rows():
    """Caps the r1 rows per int_2e block (rounded down to whole X tiles)."""
    old = os.environ.get("CUTC_INT2E_ROWS")
    set_ = _env_setter("CUTC_INT2E_ROWS")
    yield set_
    set_(old)


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
def test_int2e_blocks_span_tiles(prec, tile_rows, int2e_rows):
    """X tiles of 40 rows feed int_2e blocks of 120 rows (517 = 4 x 120 + 37: a ragged
    last block of a ragged last tile); X is the same bits as one tile and int_2e
    differs by the block sum order (and, split form, the per-block slice scales)."""
    p = _problem()
    X1, I1 = cg.build_integrals(p, prec)
    tile_rows(40)
    int2e_rows(120)
    X2, I2, st = cg.build_integrals(p, prec, with_stats=True)
    assert st["n_r1_tiles"] == 13
    if prec == cg.SPLIT_BF16:
        assert np.array_equal(X2, X1)
    else:
        assert oracle.rel_err(X2, X1)["max"] < 1e-14
    assert oracle.rel_err(I2, I1)["max"] < (1e-13 if prec == cg.PLAIN_FP64 else 1e-12)
    Xo, Io = oracle.cutc_int(p)
    ex, ei = oracle.rel_err(X2, Xo), oracle.rel_err(I2, Io)
    assert ex["max"] < TOL[prec] and ei["max"] < TOL[prec], (ex, ei)


def test_registered_outputs_match_pageable(tile_rows):
    """Caller memory page-locked with cutc_pin_host takes the direct copy path."""
    p = _problem()
    tile_rows(40)
    Xh, Ih = cg.build_integrals(p, cg.SPLIT_BF16)
    nX, nI = 3 * p.n_grid1 * p.n_ao ** 2, p.n_ao ** 4
    blk = cg.PinnedArray(8 * (nX + nI))
    try:
        a = blk.array.view(np.float64)
        X = a[:nX].reshape(3, p.n_grid1, p.n_ao ** 2)
        I = a[nX:].reshape(p.n_ao ** 2, p.n_ao ** 2)
        opt = cg.options(cg.SPLIT_BF16, None, p.a_en, p.a_ee, 3, False, 0, None)
        s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                           p.r1, p.wr1, p.r2, p.wr2, p.rn, p.aos1, p.aos2,
                           p.c_bh, p.m_bh, p.n_bh, p.o_bh, X, I)
        assert s == 0, cg.last_error()
        assert np.array_equal(X, Xh) and np.array_equal(I, Ih)
    finally:
        blk.close()


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
def test_int2e_only_builds_match_full_builds(prec, tile_rows):
    """A NULL X output returns int_2e alone (X is formed on the device and not copied
    out): the same int_2e bit for bit as a full build, from host and from device
    arrays, over several tiles; both outputs NULL is refused."""
    import torch
    p = _problem()
    tile_rows(100)
    X, I = cg.build_integrals(p, prec)
    h = {k: np.ascontiguousarray(v) for k, v in p.arrays().items()}
    opt = cg.options(prec, None, p.a_en, p.a_ee, 3, False, 0, None)
    Ih = np.full((p.n_ao ** 2, p.n_ao ** 2), np.nan)
    st = cg.Stats()
    s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                       h["r1"], h["wr1"], h["r2"], h["wr2"], h["rn"], h["aos1"], h["aos2"],
                       h["c_bh"], h["m_bh"], h["n_bh"], h["o_bh"], None, Ih, st)
    assert s == 0, cg.last_error()
    assert st.n_r1_tiles >= 5
    assert np.array_equal(Ih, I)
    dev = torch.device("cuda", 0)
    d = {k: torch.from_numpy(v).to(dev) for k, v in h.items()}
    Id = torch.full((p.n_ao ** 2, p.n_ao ** 2), float("nan"), dtype=torch.float64, device=dev)
    optd = cg.options(prec, None, p.a_en, p.a_ee, 3, True, 0, None)
    s = cg.cutc_int_ex(optd, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                       d["r1"], d["wr1"], d["r2"], d["wr2"], d["rn"], d["aos1"], d["aos2"],
                       d["c_bh"], d["m_bh"], d["n_bh"], d["o_bh"], None, Id)
    assert s == 0, cg.last_error()
    torch.cuda.synchronize()
    assert np.array_equal(Id.cpu().numpy(), I)
    s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                       h["r1"], h["wr1"], h["r2"], h["wr2"], h["rn"], h["aos1"], h["aos2"],
                       h["c_bh"], h["m_bh"], h["n_bh"], h["o_bh"], None, None)
    assert s == cg.CUTC_ERR_INVALID
