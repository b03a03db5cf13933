"""int_2e index order: the fused PSQT layout option and the reference-named helpers
trans_inplace / trans_pqst_psqt_inplace / trans_pqst_psqt_copy
(src/add_trans_inplace.cu, src/trans_pqst_psqt_inplace.cu, src/trans_pqst_psqt_copy.cu).

All of them only move or add FP64 values, so they must agree bit for bit with the
same permutation or sum done by numpy.
"""
import os

import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth

pytestmark = pytest.mark.gpu


def _psqt(I, n):
    """numpy restatement: (p,q,s,t) column-major -> (p,s,q,t); C axes are [t][s][q][p]."""
    return np.ascontiguousarray(I.reshape(n, n, n, n).transpose(0, 2, 1, 3)).reshape(n * n, n * n)


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
@pytest.mark.parametrize("slab", [None, 30])
def test_fused_psqt_layout(prec, slab, monkeypatch):
    p = synth.make_problem(n_nuc=3, n_ao=13, n_grid1=400, n_grid2=1500, size_bh=7, seed=41)
    if slab is not None:
        # 30 columns -> 26 (two t per slab): several slabs, ragged last one
        monkeypatch.setenv("CUTC_INT2E_SLAB_COLS", str(slab))
    X1, I1 = cg.build_integrals(p, prec)
    X2, I2 = cg.build_integrals(p, prec, int2e_layout=cg.INT2E_PSQT)
    assert np.array_equal(X1, X2)
    assert np.array_equal(I2, _psqt(I1, p.n_ao))


def test_fused_psqt_device_outputs():
    import torch
    p = synth.make_problem(n_nuc=2, n_ao=11, n_grid1=300, n_grid2=900, size_bh=5, seed=42)
    _, Ih = cg.build_integrals(p, cg.SPLIT_BF16)
    dev = torch.device("cuda", 0)
    dr = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in p.arrays().items()}
    Xd = torch.empty((3, p.n_grid1, p.n_ao ** 2), dtype=torch.float64, device=dev)
    Id = torch.empty((p.n_ao ** 2, p.n_ao ** 2), dtype=torch.float64, device=dev)
    opt = cg.options(cg.SPLIT_BF16, None, p.a_en, p.a_ee, 3, True, 0, None,
                     int2e_layout=cg.INT2E_PSQT)
    s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                       dr["r1"], dr["wr1"], dr["r2"], dr["wr2"], dr["rn"], dr["aos1"], dr["aos2"],
                       dr["c_bh"], dr["m_bh"], dr["n_bh"], dr["o_bh"], Xd, Id, None)
    assert s == 0, cg.last_error()
    torch.cuda.synchronize()
    assert np.array_equal(Id.cpu().numpy(), _psqt(Ih, p.n_ao))


def test_bad_layout_rejected():
    p = synth.make_problem(n_nuc=2, n_ao=4, n_grid1=40, n_grid2=60, size_bh=3, seed=43)
    with pytest.raises(cg.CutcError) as e:
        cg.build_integrals(p, cg.PLAIN_FP64, int2e_layout=7)
    assert e.value.status == cg.CUTC_ERR_INVALID


@pytest.mark.parametrize("n", [1, 5, 33, 70])
def test_trans_pqst_psqt_inplace_and_copy(n):
    import torch
    L = cg.load()
    rng = np.random.default_rng(n)
    a = rng.standard_normal(n ** 4)
    d = torch.from_numpy(a.copy()).cuda()
    L.trans_pqst_psqt_inplace(n, cg._vp(d))
    torch.cuda.synchronize()
    ref = _psqt(a.reshape(n * n, n * n), n).ravel()
    assert np.array_equal(d.cpu().numpy(), ref)
    src = torch.from_numpy(a.copy()).cuda()
    dst = torch.full((n ** 4,), np.nan, dtype=torch.float64, device="cuda")
    L.trans_pqst_psqt_copy(n, cg._vp(src), cg._vp(dst))
    torch.cuda.synchronize()
    assert np.array_equal(dst.cpu().numpy(), ref)
    assert np.array_equal(src.cpu().numpy(), a)
    # applying the in-place swap twice restores the array
    L.trans_pqst_psqt_inplace(n, cg._vp(d))
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), a)


@pytest.mark.parametrize("n", [1, 31, 32, 100, 257])
def test_trans_inplace(n):
    import torch
    L = cg.load()
    a = np.random.default_rng(n).standard_normal((n, n))
    d = torch.from_numpy(a.copy()).cuda()
    L.trans_inplace(cg._vp(d), n)
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), a + a.T)
