"""AO values and gradients evaluated on the GPU from a basis (cutc_eval_aos and the
basis option of builds, scans and server requests) against the generator's numpy
evaluator (cutc_gb300/synth.py: eval_aos)."""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu


def _close(a, b, tol=1e-13):
    # per-AO scale: values and gradients span many decades across the grid
    scale = np.max(np.abs(b), axis=-1, keepdims=True) + 1e-300
    return float(np.max(np.abs(a - b) / scale)) < tol


def test_eval_aos_matches_generator():
    p = synth.make_problem(n_nuc=4, n_ao=30, n_grid1=2000, n_grid2=10, size_bh=3, seed=11)
    got = cg.eval_aos(p.shells, p.r1, components=4)
    assert got.shape == p.aos1.shape
    assert _close(got, p.aos1)
    got1 = cg.eval_aos(p.shells, p.r1, components=1)
    assert np.array_equal(got1[0], got[0])


def test_eval_aos_higher_powers():
    rng = np.random.default_rng(5)
    rn = rng.uniform(0, 3, size=(2, 3))
    shells = [synth.Shell(rn[0].copy(), 3, np.array([0.7, 2.0]), np.array([0.6, 0.4]),
                          [(3, 0, 0), (1, 2, 0), (0, 1, 2), (1, 1, 1)]),
              synth.Shell(rn[1].copy(), 4, np.array([1.3]), np.array([1.0]),
                          [(4, 0, 0), (2, 2, 0), (0, 0, 4)])]
    r = rng.uniform(-1, 4, size=(777, 3))
    assert _close(cg.eval_aos(shells, r), synth.eval_aos(shells, r))


def test_bad_basis_rejected():
    p = synth.make_problem(n_nuc=2, n_ao=4, n_grid1=20, n_grid2=20, size_bh=3, seed=12)
    shells = [synth.Shell(p.rn[0].copy(), 0, np.array([1.0]), np.array([1.0]), [(9, 0, 0)])]
    with pytest.raises(cg.CutcError) as e:
        cg.eval_aos(shells, p.r1)
    assert e.value.status == cg.CUTC_ERR_INVALID


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
def test_build_from_basis(prec):
    p = synth.make_problem(n_nuc=3, n_ao=15, n_grid1=600, n_grid2=2000, size_bh=7, seed=13)
    X1, I1 = cg.build_integrals(p, prec)
    X2, I2 = cg.build_integrals(p, prec, aos_from_basis=True)
    tol = 1e-13 if prec == cg.PLAIN_FP64 else 1e-12
    assert oracle.rel_err(X2, X1)["max"] < tol
    assert oracle.rel_err(I2, I1)["max"] < tol


def test_scan_from_basis():
    p = synth.make_problem(n_nuc=2, n_ao=9, n_grid1=300, n_grid2=900, size_bh=5, seed=14)
    c = np.random.default_rng(1).normal(0, 0.3, size=(3,) + p.c_bh.shape)
    X1, I1 = cg.scan_integrals(p, c, precision=cg.SPLIT_BF16)
    b = cg.make_basis(p.shells)
    import dataclasses
    q = dataclasses.replace(p)
    # the scan binding takes the basis through the options; AO arrays NULL
    X2, I2 = cg.scan_integrals(q, c, precision=cg.SPLIT_BF16, basis=b)
    assert oracle.rel_err(X2, X1)["max"] < 1e-12
    assert oracle.rel_err(I2, I1)["max"] < 1e-12


def test_server_request_from_basis():
    p = synth.make_problem(n_nuc=2, n_ao=10, n_grid1=400, n_grid2=1200, size_bh=5, seed=15)
    X0, I0 = cg.build_integrals(p, cg.SPLIT_BF16)
    with cg.Server(n_slots=2) as srv:
        t1 = srv.submit(p, molecule_key=0, precision=cg.SPLIT_BF16, aos_from_basis=True)
        t2 = srv.submit(p, molecule_key=77, precision=cg.SPLIT_BF16, aos_from_basis=True)
        t3 = srv.submit(p, molecule_key=77, precision=cg.SPLIT_BF16, aos_from_basis=True)
        for t in (t1, t2, t3):
            X, I, _ = srv.wait(t)
            assert oracle.rel_err(X, X0)["max"] < 1e-12
            assert oracle.rel_err(I, I0)["max"] < 1e-12
