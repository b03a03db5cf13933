"""The two-electron contraction of the reference's cutc_no (src/cutc_no.c:415-470) on its
intermediates (cutc_no_2e): 1/2 tmpC1^T X + 1/2 tmpC2^T tmpD2, plus its transpose, then
the (p,q,s,t) -> (p,s,q,t) swap, against the same steps in numpy FP64.  Plain form within
1e-12, split form within 1e-10 (relative to the largest element), host and device arrays."""
import numpy as np
import pytest

import cutc_gb300 as cg

pytestmark = pytest.mark.gpu

TOL = {cg.PLAIN_FP64: 1e-12, cg.SPLIT_BF16: 1e-10}


def _inputs(n_mo, n1, seed):
    rng = np.random.default_rng(seed)
    nm2 = n_mo * n_mo
    # Fortran (3 n1, n_mo^2) and (n1, n_mo^2) as C arrays with the axes reversed
    return (rng.standard_normal((nm2, 3 * n1)), rng.standard_normal((nm2, 3 * n1)),
            rng.standard_normal((nm2, n1)), rng.standard_normal((nm2, n1)))


def _reference(C1, X, C2, D2, n_mo):
    A = 0.5 * (C1 @ X.T + C2 @ D2.T)      # A[i, j]: column-major element i + nm2 j
    out = (A + A.T).T                      # C array [j, i] of the Fortran matrix
    four = out.reshape(n_mo, n_mo, n_mo, n_mo)   # [t, s, q, p]
    return np.ascontiguousarray(np.swapaxes(four, 1, 2)).reshape(n_mo * n_mo, n_mo * n_mo)


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
@pytest.mark.parametrize("n_mo,n1", [(7, 60), (12, 300), (1, 5)])
def test_no_2e_host_and_device(prec, n_mo, n1):
    import torch
    C1, X, C2, D2 = _inputs(n_mo, n1, 80 + n_mo)
    ref = _reference(C1, X, C2, D2, n_mo)
    scale = np.abs(ref).max()
    got = cg.no_2e(C1, X, C2, D2, n_mo, n1, prec)
    assert np.abs(got - ref).max() <= TOL[prec] * scale
    dev = [torch.from_numpy(a).cuda() for a in (C1, X, C2, D2)]
    got_d = cg.no_2e(*dev, n_mo, n1, prec).cpu().numpy()
    assert np.array_equal(got_d, got)


def test_no_2e_rejects_bad_arguments():
    C1, X, C2, D2 = _inputs(2, 4, 1)
    with pytest.raises(cg.CutcError) as e:
        cg.no_2e(C1, X, C2, D2, 0, 4)
    assert e.value.status == cg.CUTC_ERR_INVALID
