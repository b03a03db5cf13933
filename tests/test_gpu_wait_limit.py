"""The failure path of the tensor-core kernels' pipeline waits, on a GPU, without a
fault: cutc_check_wait_limit runs one CTA whose barrier nothing completes, so its
bounded wait gives up after its limit and the call reports CUTC_ERR_TIMEOUT -- the
status a build returns when one of its pipeline waits gives up.  The device stays
usable: a split build right after it matches the oracle."""
import time

import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_the_device_stays_usable():
    t0 = time.perf_counter()
    s = cg.load().cutc_check_wait_limit()
    elapsed = time.perf_counter() - t0
    assert s == cg.CUTC_ERR_TIMEOUT, cg.last_error()
    assert "gave up" in cg.last_error()
    assert 1.5 < elapsed < 30.0  # the 2 s limit, not an endless spin
    p = synth.make_problem(n_nuc=3, n_ao=6, n_grid1=200, n_grid2=700, size_bh=6, seed=77)
    X, I = cg.build_integrals(p, cg.SPLIT_BF16)
    Xo, Io = oracle.cutc_int(p)
    assert oracle.rel_err(X, Xo[:3])["max"] < 1e-10
    assert oracle.rel_err(I, Io)["max"] < 1e-10
