"""The Jastrow-parameter scan equals independent builds, set by set."""
import dataclasses

import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [cg.SPLIT_BF16, cg.PLAIN_FP64])
def test_scan_equals_independent_builds(prec):
    p = synth.make_problem(n_nuc=3, n_ao=9, n_grid1=240, n_grid2=900, size_bh=6, seed=51)
    rng = np.random.default_rng(52)
    ns = 4
    c_sets = rng.normal(0.0, 0.3, size=(ns,) + p.c_bh.shape)
    a_en = rng.uniform(0.5, 2.0, ns)
    a_ee = rng.uniform(0.5, 2.0, ns)
    X, I, st = cg.scan_integrals(p, c_sets, a_en, a_ee, precision=prec, with_stats=True)
    assert st["gpu_launches"] > 0
    for s in range(ns):
        q = dataclasses.replace(p, c_bh=np.ascontiguousarray(c_sets[s]), a_en=a_en[s], a_ee=a_ee[s])
        Xs, Is = cg.build_integrals(q, prec)
        assert np.array_equal(X[s], Xs) and np.array_equal(I[s], Is), s
