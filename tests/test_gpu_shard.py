"""r1 windows of one build (cutc_options.r1_begin / r1_end), the GPU side of the r1
sharding: on one GPU the shards run one after another.  Their X rows are the whole
build's rows and their int_2e shares sum to the whole int_2e, against the oracle in
both forms (plain 1e-12, split 1e-10), with device and host arrays (a host window
of aos_data1 is strided: it is copied 2-D)."""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth
from cutc_gb300.shard import library_shard, shard_window
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL = {cg.PLAIN_FP64: 1e-12, cg.SPLIT_BF16: 1e-10}


def _check(a, b, tol):
    e = oracle.rel_err(a, b)
    assert e["norm"] < tol and e["max"] < tol, e


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
def test_device_shards_sum_to_the_whole_build(prec):
    p = synth.make_problem(n_nuc=4, n_ao=11, n_grid1=700, n_grid2=1500, size_bh=9, seed=61,
                           a_en=0.9, a_ee=1.2)
    Xo, Io = oracle.cutc_int(p)
    world = 3
    I = 0.0
    for r in range(world):
        b, e = shard_window(p.n_grid1, r, world)
        Xs, Is = library_shard(p, b, e, prec)
        _check(Xs.cpu().numpy(), Xo[:, b:e], TOL[prec])
        I = I + Is.cpu().numpy()
    _check(I, Io, TOL[prec])


def test_host_window_equals_device_window():
    p = synth.make_problem(n_nuc=3, n_ao=7, n_grid1=300, n_grid2=800, size_bh=6, seed=62)
    b, e = 113, 241
    Xd, Id = library_shard(p, b, e, cg.PLAIN_FP64)
    nA2 = p.n_ao ** 2
    X = np.empty((3, e - b, nA2))
    I = np.empty((nA2, nA2))
    opt = cg.options(cg.PLAIN_FP64, None, p.a_en, p.a_ee, 3, r1_window=(b, e))
    s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh, p.r1, p.wr1, p.r2,
                       p.wr2, p.rn, p.aos1, p.aos2, p.c_bh, p.m_bh, p.n_bh, p.o_bh, X, I)
    assert s == cg.CUTC_OK, cg.last_error()
    assert np.array_equal(X, Xd.cpu().numpy())
    assert np.array_equal(I, Id.cpu().numpy())


def test_bad_windows_are_refused():
    p = synth.make_problem(n_nuc=2, n_ao=3, n_grid1=20, n_grid2=40, size_bh=3, seed=63)
    nA2 = p.n_ao ** 2
    for w in ((5, 5), (-1, 4), (10, 21), (12, 3)):
        X = np.empty((3, 20, nA2))
        I = np.empty((nA2, nA2))
        opt = cg.options(cg.PLAIN_FP64, r1_window=w)
        s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh, p.r1, p.wr1,
                           p.r2, p.wr2, p.rn, p.aos1, p.aos2, p.c_bh, p.m_bh, p.n_bh, p.o_bh, X, I)
        assert s == cg.CUTC_ERR_INVALID, w
