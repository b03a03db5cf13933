"""The continuous-batching server: results are the same alone and in the mix.

Requests of different molecules, basis and grid sizes, some repeating a
molecule with perturbed Jastrow coefficients, are submitted at once to a
4-slot server; every result must equal the one a standalone cutc_int_ex call
with the same options gives (bit for bit: the same kernels run on the same
data in another context), repeated molecules must come from the cache, and a
budget that fits one request at a time must still complete them all.
"""
import dataclasses

import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth

pytestmark = pytest.mark.gpu


def _mix():
    mols = [synth.make_problem(n_nuc=2, n_ao=6, n_grid1=200, n_grid2=800, size_bh=5, seed=41),
            synth.make_problem(n_nuc=3, n_ao=11, n_grid1=300, n_grid2=1500, size_bh=7, seed=42),
            synth.make_problem(n_nuc=4, n_ao=17, n_grid1=500, n_grid2=2000, size_bh=9, seed=43)]
    rng = np.random.default_rng(44)
    reqs = []
    for i in range(9):
        k = i % 3
        p = mols[k]
        if i >= 3:  # a repeat: same molecule, perturbed Jastrow coefficients
            p = dataclasses.replace(p, c_bh=np.ascontiguousarray(
                p.c_bh * (1 + 0.1 * rng.standard_normal(p.c_bh.shape))))
        prec = cg.SPLIT_BF16 if i % 2 == 0 else cg.PLAIN_FP64
        reqs.append((p, k + 1, prec))
    return reqs


def test_results_same_alone_and_in_the_mix():
    reqs = _mix()
    alone = [cg.build_integrals(p, prec) for p, key, prec in reqs]
    with cg.Server(n_slots=4) as srv:
        tickets = [srv.submit(p, key, prec) for p, key, prec in reqs]
        mixed = [srv.wait(t) for t in tickets]
        st = srv.stats()
    for (Xa, Ia), (Xm, Im, lat), (p, key, prec) in zip(alone, mixed, reqs):
        assert np.array_equal(Xa, Xm) and np.array_equal(Ia, Im), (key, prec)
        assert lat > 0
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["cache_misses"] == 3 and st["cache_hits"] == len(reqs) - 3
    assert st["peak_in_flight"] >= 2
    assert st["p99_ms"] >= st["p50_ms"] > 0


def test_memory_admission_serialises_when_only_one_fits():
    reqs = _mix()[:4]
    with cg.Server(n_slots=3, device_budget_bytes=1) as srv:
        tickets = [srv.submit(p, 0, prec) for p, key, prec in reqs]
        outs = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["peak_in_flight"] == 1 and st["completed"] == 4
    for (X, I, _), (p, key, prec) in zip(outs, reqs):
        Xa, Ia = cg.build_integrals(p, prec)
        assert np.array_equal(X, Xa) and np.array_equal(I, Ia)


def test_failed_request_is_isolated():
    """A request that fails validation (a Jastrow exponent of 7) reports its status
    through wait(); the requests around it complete with their standalone results."""
    reqs = _mix()[:4]
    bad = dataclasses.replace(reqs[1][0], m_bh=reqs[1][0].m_bh.copy())
    bad.m_bh[0, 0] = 7
    with cg.Server(n_slots=2) as srv:
        tickets = [srv.submit(p, key, prec) for p, key, prec in reqs[:2]]
        tb = srv.submit(bad, 0, cg.PLAIN_FP64)
        tickets += [srv.submit(p, key, prec) for p, key, prec in reqs[2:]]
        with pytest.raises(cg.CutcError) as e:
            srv.wait(tb)
        assert e.value.status == cg.CUTC_ERR_INVALID
        assert "exponent" in str(e.value)  # the worker's message reaches the waiting thread
        for (p, key, prec), t in zip(reqs, tickets):
            X, I, _ = srv.wait(t)
            Xs, Is = cg.build_integrals(p, prec)
            assert np.array_equal(X, Xs) and np.array_equal(I, Is)
        st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == len(reqs)


def test_cache_evicts_within_its_budget():
    """A cache budget that holds one molecule: repeats of the most recent molecule
    hit, a new molecule evicts the old one, and every result is still right."""
    a = synth.make_problem(n_nuc=2, n_ao=6, n_grid1=200, n_grid2=800, size_bh=5, seed=51)
    b = synth.make_problem(n_nuc=2, n_ao=7, n_grid1=220, n_grid2=900, size_bh=5, seed=52)
    one = 8 * (4 * 220 + 4 * 900 + 6 + 4 * 220 * 7 + 900 * 7) + 4096
    with cg.Server(n_slots=1, cache_budget_bytes=one) as srv:
        order = [(a, 1), (a, 1), (b, 2), (a, 1)]
        for p, key in order:
            X, I, _ = srv.wait(srv.submit(p, key, cg.SPLIT_BF16))
            Xs, Is = cg.build_integrals(p, cg.SPLIT_BF16)
            assert np.array_equal(X, Xs) and np.array_equal(I, Is)
        st = srv.stats()
    assert st["cache_hits"] == 1 and st["cache_misses"] == 3
    assert st["cache_bytes"] <= one
