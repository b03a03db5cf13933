"""Pin the CPU oracle against vectors produced by the reference's own code.

The fixtures come from tests/golden/make_golden.py, which runs the reference
cutc_int path (src/cutc_int.c and the kernels it launches) compiled for the
CPU.  The pair terms must agree bit for bit; the contracted outputs differ only
by the summation order of the DGEMMs.
"""
import numpy as np
import pytest

from golden_util import CASE_NAMES, load_case, load_small_digest
from oracle import oracle
from cutc_gb300 import synth


@pytest.mark.parametrize("name", CASE_NAMES)
def test_pair_bit_exact(name):
    p, ref = load_case(name)
    G = oracle.pair(p)
    assert np.array_equal(G, ref["G"])


@pytest.mark.parametrize("name", CASE_NAMES)
def test_cutc_int_matches_reference(name):
    p, ref = load_case(name)
    X3, A = oracle.cutc_int(p)
    ex = oracle.rel_err(X3, ref["X"])
    ei = oracle.rel_err(A, ref["int2e"])
    assert ex["norm"] < 1e-13 and ex["max"] < 1e-13, ex
    assert ei["norm"] < 1e-13 and ei["max"] < 1e-13, ei


@pytest.mark.parametrize("name", CASE_NAMES)
def test_blocked_oracle_is_block_invariant(name):
    p, ref = load_case(name)
    X3a, Aa = oracle.cutc_int(p)
    X3b, Ab = oracle.cutc_int(p, block1=7)
    assert oracle.rel_err(X3b, X3a)["max"] < 1e-14
    assert oracle.rel_err(Ab, Aa)["max"] < 1e-13


def test_small_workload_digest():
    d = load_small_digest()
    p = synth.make_config("small")
    from golden_util import GOLDEN  # noqa: F401
    from tests_inputs import input_checksums
    cs = input_checksums(p)
    np.testing.assert_allclose(cs, d["input_checksums"], rtol=1e-12, atol=1e-12)
    X3, A = oracle.cutc_int(p)
    xm, im = float(d["X_max"]), float(d["I_max"])
    assert np.max(np.abs(X3.ravel()[d["X_idx"]] - d["X_val"])) < 1e-12 * xm
    assert np.max(np.abs(A.ravel()[d["I_idx"]] - d["I_val"])) < 1e-12 * im
    assert abs(np.linalg.norm(X3.ravel()) - d["X_norm"]) < 1e-12 * d["X_norm"]
    assert abs(np.linalg.norm(A.ravel()) - d["I_norm"]) < 1e-12 * d["I_norm"]


def test_oracle_pair_term_symmetries():
    """Properties of the Boys-Handy form the oracle restates (src/jast_bh.cu:203-242):
    swapping m and n in every term leaves u, hence G, unchanged, and scaling every
    coefficient by k scales grad u by k and -1/2 |grad u|^2 by k^2."""
    import dataclasses
    from cutc_gb300 import synth
    p = synth.make_problem(n_nuc=2, n_ao=3, n_grid1=40, n_grid2=60, size_bh=5, seed=31)
    G = oracle.pair(p)
    swapped = dataclasses.replace(p, m_bh=p.n_bh.copy(), n_bh=p.m_bh.copy())
    assert np.array_equal(oracle.pair(swapped), G) or \
        np.abs(oracle.pair(swapped) - G).max() <= 1e-15 * np.abs(G).max()
    k = 0.75
    scaled = dataclasses.replace(p, c_bh=p.c_bh * k)
    Gs = oracle.pair(scaled)
    np.testing.assert_allclose(Gs[:3], k * G[:3], rtol=0, atol=1e-14 * np.abs(G[:3]).max())
    np.testing.assert_allclose(Gs[3], k * k * G[3], rtol=0, atol=1e-14 * np.abs(G[3]).max())


@pytest.mark.parametrize("name", CASE_NAMES)
def test_windowed_oracle_matches_reference(name):
    """x_rows (P formed per r2 window, as for molecules whose whole P does not fit),
    int2e_rows and int2e_matvec against the reference's own outputs."""
    p, ref = load_case(name)
    nA2 = p.n_ao ** 2
    X4 = oracle.x_rows(p, window_bytes=8 * nA2 * 5)  # r2 windows of 5 points
    ex = oracle.rel_err(X4[:3], ref["X"])
    assert ex["norm"] < 1e-13 and ex["max"] < 1e-13, ex
    rows = np.arange(0, nA2, 3)
    ei = oracle.rel_err(oracle.int2e_rows(p, X4, rows), ref["int2e"][rows])
    assert ei["max"] < 1e-13, ei
    v = np.random.default_rng(5).standard_normal(nA2)
    ev = oracle.rel_err(oracle.int2e_matvec(p, X4, v), ref["int2e"] @ v)
    assert ev["max"] < 1e-13, ev
