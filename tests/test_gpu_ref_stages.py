"""The reference's device-level stages under its names and signatures
(src/jast_bh.cu:268-303, src/long_range_integ.cu:52-67,
src/short_range_integ_herm.cu:51-64, src/short_range_integ_nonherm.cu:69-82,
src/build_int2_grad1_u12_ao.cu:9-347, src/build_int_2e_ao.cu:11-145),
each against the oracle on device arrays in the reference's layouts.

The pair products are single roundings of the same products in the same order
as the reference, so they must agree bit for bit; the antisymmetric products
differ at most by the contraction of one product into the subtraction.
"""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu


def _problem():
    # a_en = a_ee = 1: the reference fixes them
    return synth.make_problem(n_nuc=3, n_ao=9, n_grid1=230, n_grid2=700, size_bh=7, seed=57)


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _ptrs(tensors):
    """Device addresses of tensors the caller keeps alive (a temporary's memory
    would go back to torch's allocator before the asynchronous call reads it)."""
    return [t.data_ptr() for t in tensors]


def _sync_ok():
    import torch
    torch.cuda.synchronize()


def test_int_long_range_window_bit_exact():
    import torch
    p = _problem()
    nA, n2 = p.n_ao, p.n_grid2
    jj0, eff, tot = 123, 300, 320
    out = torch.full((nA * nA, tot), float("nan"), dtype=torch.float64, device="cuda")
    L = cg.load()
    w2, a2 = _dev(p.wr2), _dev(p.aos2)  # held: the calls run asynchronously
    L.int_long_range(jj0, eff, tot, n2, nA, w2.data_ptr(), a2.data_ptr(), out.data_ptr())
    _sync_ok()
    got = out.cpu().numpy()
    P = oracle.long_range(p)  # row b + nA a, column r2 point
    assert np.array_equal(got[:, :eff], P[:, jj0:jj0 + eff])
    assert np.isnan(got[:, eff:]).all()  # nothing written past n_grid2_eff


def test_int_short_range_products():
    import torch
    p = _problem()
    nA, n1 = p.n_ao, p.n_grid1
    L = cg.load()
    S0 = torch.empty((nA * nA, n1), dtype=torch.float64, device="cuda")
    S = torch.empty((nA * nA, 3, n1), dtype=torch.float64, device="cuda")
    w1, a1 = _dev(p.wr1), _dev(p.aos1)
    L.int_short_range_herm(n1, nA, w1.data_ptr(), a1.data_ptr(), S0.data_ptr())
    L.int_short_range_nonherm(n1, nA, w1.data_ptr(), a1.data_ptr(), S.data_ptr())
    _sync_ok()
    assert np.array_equal(S0.cpu().numpy(), oracle.short_herm(p))
    So = oracle.short_nonherm(p)
    # bound: a few units in the last place of |w| (|chi_b d_m chi_a| + |chi_a d_m chi_b|),
    # indexed [a, b, m, g] and flattened to the oracle's [b + nA a, m, g]
    v, d = p.aos1[0], p.aos1[1:].transpose(1, 0, 2)  # (nA, n1), (nA, 3, n1)
    t1 = np.abs(v[None, :, None, :] * d[:, None, :, :])
    t2 = np.abs(v[:, None, None, :] * d[None, :, :, :])
    mag = (np.abs(p.wr1) * (t1 + t2)).reshape(nA * nA, 3, n1)
    assert np.all(np.abs(S.cpu().numpy() - So) <= 2.0 ** -50 * mag + 1e-300)


def test_cutc_int_bh_window_and_strides():
    import torch
    p = _problem()
    ii0, n1_eff, n1_tot = 40, 70, 75
    jj0, n2_eff, n2_tot = 100, 500, 530
    G = torch.full((4, n1_tot, n2_tot), float("nan"), dtype=torch.float64, device="cuda")
    L = cg.load()
    mol = [_dev(a) for a in (p.r1, p.r2, p.rn, p.c_bh, p.m_bh, p.n_bh, p.o_bh)]
    grid, block = cg.Dim3(4, 4, 1), cg.Dim3(32, 4, 1)
    L.cutc_int_bh(grid, block, ii0, n1_eff, n1_tot, jj0, n2_eff, n2_tot, p.n_nuc, p.size_bh,
                  *_ptrs(mol), G.data_ptr())
    _sync_ok()
    got = G.cpu().numpy()
    ref = oracle.pair(p)[:, ii0:ii0 + n1_eff, jj0:jj0 + n2_eff]
    np.testing.assert_allclose(got[:, :n1_eff, :n2_eff], ref, rtol=0,
                               atol=1e-13 * np.abs(ref).max())
    assert np.isnan(got[:, n1_eff:, :]).all() and np.isnan(got[:, :, n2_eff:]).all()


def test_cutc_int_bh_rejects_launch_dims_like_cutc_int():
    import torch
    p = _problem()
    G = torch.full((4, 8, 8), 7.0, dtype=torch.float64, device="cuda")
    L = cg.load()
    mol = [_dev(a) for a in (p.r1, p.r2, p.rn, p.c_bh, p.m_bh, p.n_bh, p.o_bh)]
    L.cutc_int_bh(cg.Dim3(1, 1, 1), cg.Dim3(2048, 1, 1), 0, 8, 8, 0, 8, 8, p.n_nuc, p.size_bh,
                  *_ptrs(mol), G.data_ptr())
    _sync_ok()
    assert "threads per block" in cg.last_error()
    assert (G.cpu().numpy() == 7.0).all()


@pytest.mark.parametrize("precision", ["plain", "split", "split6"])
def test_get_int2_grad1_u12_ao_all_four_components(precision, monkeypatch):
    """Both forms, and the split form at 6 slices (CUTC_SLICES) at the plain form's
    tolerance."""
    import torch
    if precision != "plain":
        monkeypatch.setenv("CUTC_PRECISION", "split")
    if precision == "split6":
        monkeypatch.setenv("CUTC_SLICES", "6")
    p = _problem()
    nA2, n1 = p.n_ao ** 2, p.n_grid1
    X = torch.full((4, n1, nA2), float("nan"), dtype=torch.float64, device="cuda")
    L = cg.load()
    mol = [_dev(a) for a in (p.r1, p.r2, p.wr2, p.rn, p.aos2, p.c_bh, p.m_bh, p.n_bh, p.o_bh)]
    L.get_int2_grad1_u12_ao(cg.Dim3(8, 8, 1), cg.Dim3(32, 8, 1), n1, p.n_grid2, p.n_ao, p.n_nuc,
                            p.size_bh, *_ptrs(mol), X.data_ptr())
    _sync_ok()
    Xo = oracle.x_block(p, oracle.long_range(p), 0, n1)
    tol = 1e-10 if precision == "split" else 1e-12
    assert oracle.rel_err(X.cpu().numpy(), Xo)["max"] < tol, cg.last_error()


def test_get_int2_grad1_u12_ao_refuses_a_bad_slice_count(monkeypatch):
    import torch
    monkeypatch.setenv("CUTC_PRECISION", "split")
    monkeypatch.setenv("CUTC_SLICES", "9")
    p = _problem()
    X = torch.full((4, p.n_grid1, p.n_ao ** 2), 7.0, dtype=torch.float64, device="cuda")
    L = cg.load()
    mol = [_dev(a) for a in (p.r1, p.r2, p.wr2, p.rn, p.aos2, p.c_bh, p.m_bh, p.n_bh, p.o_bh)]
    # a launch geometry error first, so that the message checked below is this call's
    L.get_int2_grad1_u12_ao(cg.Dim3(8, 8, 1), cg.Dim3(2048, 1, 1), p.n_grid1, p.n_grid2, p.n_ao,
                            p.n_nuc, p.size_bh, *_ptrs(mol), X.data_ptr())
    assert "n_slices" not in cg.last_error()
    L.get_int2_grad1_u12_ao(cg.Dim3(8, 8, 1), cg.Dim3(32, 8, 1), p.n_grid1, p.n_grid2, p.n_ao,
                            p.n_nuc, p.size_bh, *_ptrs(mol), X.data_ptr())
    torch.cuda.synchronize()
    assert "n_slices" in cg.last_error()
    assert (X.cpu().numpy() == 7.0).all()


@pytest.mark.parametrize("rows", [None, 37])
def test_get_int_2e_ao_from_given_x(rows, monkeypatch):
    """From the oracle's X, and from an X that is not symmetric in the AO pair
    (the contraction uses the caller's full array); 37-row blocks for the cap."""
    import torch
    if rows is not None:
        monkeypatch.setenv("CUTC_INT2E_ROWS", str(rows))
    p = _problem()
    nA2, n1 = p.n_ao ** 2, p.n_grid1
    rng = np.random.default_rng(5)
    X_sym = oracle.x_block(p, oracle.long_range(p), 0, n1)
    X_any = rng.standard_normal((4, n1, nA2))
    L = cg.load()
    w1, a1 = _dev(p.wr1), _dev(p.aos1)
    for X4 in (X_sym, X_any):
        I = torch.full((nA2, nA2), float("nan"), dtype=torch.float64, device="cuda")
        Xd = _dev(X4)
        L.get_int_2e_ao(n1, p.n_ao, w1.data_ptr(), a1.data_ptr(), Xd.data_ptr(), I.data_ptr())
        _sync_ok()
        A = oracle.int2e_from_x(p, X4)   # [col, row]
        ref = A + A.T
        assert oracle.rel_err(I.cpu().numpy(), ref)["max"] < 1e-12, cg.last_error()


def test_x_only_build_through_cutc_int_ex():
    """int_2e_ao NULL builds X alone; wr1 and aos_data1 are then not needed."""
    p = _problem()
    X4, _ = cg.build_integrals(p, cg.PLAIN_FP64, x_components=4)
    opt = cg.options(cg.PLAIN_FP64, None, p.a_en, p.a_ee, 4, False, 0, None)
    X = np.full((4, p.n_grid1, p.n_ao ** 2), np.nan)
    s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                       p.r1, None, p.r2, p.wr2, p.rn, None, p.aos2,
                       p.c_bh, p.m_bh, p.n_bh, p.o_bh, X, None, None)
    assert s == cg.CUTC_OK, cg.last_error()
    assert oracle.rel_err(X, X4)["max"] < 1e-14
