"""The engine's device-memory plan (cutc_plan, host arithmetic only): how the r1
grid is cut into X tiles and int_2e blocks, and the bytes each needs.  Runs
without a GPU."""
import itertools
import math

import pytest

import cutc_gb300 as cg

SIZES = [(517, 1900, 13, 3), (25000, 80000, 120, 10), (60000, 200000, 300, 20), (3000, 12000, 24, 3),
         (1, 5, 1, 1), (20000, 80000, 250, 20)]
BUDGETS = [1 << 20, 64 << 20, 4 << 30, 24 << 30]


@pytest.mark.parametrize("size,budget,prec,dev", list(itertools.product(
    SIZES, BUDGETS, [cg.PLAIN_FP64, cg.SPLIT_BF16], [False, True])))
def test_plan_invariants(size, budget, prec, dev):
    n1, n2, nA, nN = size
    p = cg.plan(n1, n2, nA, nN, prec, device_pointers=dev, max_work_bytes=budget)
    t, k = p["tile_rows"], p["block_rows"]
    assert 1 <= t <= k <= n1
    # a block is whole tiles (the last block and tile may be ragged)
    assert k == n1 or k % t == 0
    assert p["n_tiles"] == math.ceil(n1 / t) and p["n_blocks"] == math.ceil(n1 / k)
    # each part within the budget unless a single row already exceeds it
    assert t == 1 or t * p["tile_row_bytes"] <= budget
    assert k <= max(1, budget // p["block_row_bytes"]) or k == t
    # the footprint covers the fixed part, one tile and one block
    assert p["footprint_bytes"] >= p["fixed_bytes"] + t * p["tile_row_bytes"] + k * p["block_row_bytes"]
    # int_2e output slabs: whole t-columns (nA of them) of the nA^2 x nA^2 matrix
    sc = p["slab_cols"]
    assert sc % nA == 0 and nA <= sc <= nA * nA


def test_plan_monotone_in_budget():
    rows = [cg.plan(25000, 80000, 120, 10, cg.SPLIT_BF16, max_work_bytes=b)["tile_rows"]
            for b in (1 << 30, 4 << 30, 16 << 30)]
    assert rows[0] <= rows[1] <= rows[2]
    host = cg.plan(25000, 80000, 120, 10, cg.SPLIT_BF16, max_work_bytes=8 << 30)
    dev = cg.plan(25000, 80000, 120, 10, cg.SPLIT_BF16, device_pointers=True, max_work_bytes=8 << 30)
    # device outputs need no staging, device inputs no molecule copy
    assert dev["tile_row_bytes"] < host["tile_row_bytes"]
    assert dev["footprint_bytes"] < host["footprint_bytes"]


def test_plan_medium_is_one_block():
    p = cg.plan(25000, 80000, 120, 10, cg.SPLIT_BF16, device_pointers=True, max_work_bytes=24 << 30)
    assert p["block_rows"] == 25000 and p["n_blocks"] == 1 and p["n_tiles"] >= 2


def test_plan_tile_rows_fit_the_pair_kernel_grid():
    # the pair kernels put 8 r1 rows per CTA on gridDim.y (<= 65535): a tile never
    # exceeds 2^18 rows, however small n_grid2 makes a row
    for prec in (cg.PLAIN_FP64, cg.SPLIT_BF16):
        p = cg.plan(2_000_000, 4, 2, 1, prec, device_pointers=True, max_work_bytes=64 << 30)
        assert p["tile_rows"] <= 1 << 18
        assert p["n_tiles"] * p["tile_rows"] >= 2_000_000


def test_plan_split_tile_past_the_old_slicer_limit():
    # 20 000 r1 rows x 2 000 r2 points fit one split-form tile: its G operand has
    # 4 x 20 000 = 80 000 rows, which the slicer handles with grid-stride rows
    p = cg.plan(20000, 2000, 6, 3, cg.SPLIT_BF16, device_pointers=True, max_work_bytes=24 << 30)
    assert p["tile_rows"] == 20000 and p["n_tiles"] == 1


def test_plan_env_caps(monkeypatch):
    monkeypatch.setenv("CUTC_TILE_ROWS", "40")
    monkeypatch.setenv("CUTC_INT2E_ROWS", "120")
    p = cg.plan(517, 1900, 13, 3, cg.SPLIT_BF16, max_work_bytes=8 << 30)
    assert (p["tile_rows"], p["block_rows"], p["n_tiles"], p["n_blocks"]) == (40, 120, 13, 5)


def test_plan_rejects_bad_arguments():
    with pytest.raises(cg.CutcError):
        cg.plan(0, 10, 5, 1, max_work_bytes=1 << 20)
    with pytest.raises(cg.CutcError):
        cg.plan(10, 10, 5, 1, cg.SPLIT_BF16, n_slices=9, max_work_bytes=1 << 20)


def test_plan_without_budget_needs_a_device():
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a device is present")
    with pytest.raises(cg.CutcError) as e:
        cg.plan(100, 100, 5, 1)
    assert e.value.status == cg.CUTC_ERR_NO_DEVICE


def test_x_contraction_launches_per_tile():
    """Split form: one tensor-core launch up to K = n_grid2 = 65536, equal launches of
    at most 49152 beyond (FP64 sums between them); with 16384 or more packed AO pairs
    (the A operand's rows) one launch up to 32768 and launches of at most 24576 beyond;
    an explicit k_split caps them."""
    budget = 8 << 30
    for n2, launches in ((12000, 1), (50000, 1), (65536, 1), (65537, 2), (80000, 2),
                         (120000, 3), (200000, 5)):
        info = cg.plan(500, n2, 20, 3, cg.SPLIT_BF16, 5, max_work_bytes=budget)
        assert info["x_launches_per_tile"] == launches, (n2, info)
    # n_ao = 180: 16290 pairs; 181: 16471
    for n_ao, n2, launches in ((180, 80000, 2), (181, 32768, 1), (181, 32769, 2),
                               (181, 80000, 4), (300, 200000, 9)):
        info = cg.plan(500, n2, n_ao, 3, cg.SPLIT_BF16, 5, max_work_bytes=budget)
        assert info["x_launches_per_tile"] == launches, (n_ao, n2, info)
    assert cg.plan(500, 80000, 20, 3, cg.SPLIT_BF16, 5, max_work_bytes=budget,
                   k_split=16384)["x_launches_per_tile"] == 5
    assert cg.plan(500, 200000, 20, 3, cg.SPLIT_BF16, 5, max_work_bytes=budget,
                   k_split=300000)["x_launches_per_tile"] == 1
    assert cg.plan(500, 200000, 20, 3, cg.PLAIN_FP64, max_work_bytes=budget)["x_launches_per_tile"] == 1
