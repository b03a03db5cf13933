"""X in the MO basis in cutc_no's order (cutc_x_ao_to_mo) against the numpy
restatement of x_mo(g, m, i, j) = sum_ab L(a, i) X_ao(a, b, g, m) R(b, j)."""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth

pytestmark = pytest.mark.gpu


def _ref(X, L, R):
    # X: (comps, n1, nA, nA) = [m][g][b][a]; L, R: (n_mo, nA) = [i][a]
    return np.einsum("ia,mgba,jb->jimg", L, X, R, optimize=True)


@pytest.mark.parametrize("n_mo", [7, 13, 20])
def test_x_ao_to_mo_host(n_mo):
    rng = np.random.default_rng(n_mo)
    comps, n1, nA = 3, 517, 13
    X = rng.standard_normal((comps, n1, nA, nA))
    X = X + X.transpose(0, 1, 3, 2)
    L = rng.standard_normal((n_mo, nA))
    R = rng.standard_normal((n_mo, nA))
    got = cg.x_ao_to_mo(X, L, R)
    ref = _ref(X, L, R)
    assert np.max(np.abs(got - ref)) < 1e-12 * np.max(np.abs(ref))


def test_x_ao_to_mo_device_four_components():
    import torch
    rng = np.random.default_rng(3)
    comps, n1, nA, n_mo = 4, 300, 11, 9
    X = rng.standard_normal((comps, n1, nA, nA))
    L = rng.standard_normal((n_mo, nA))
    R = L.copy()
    d = lambda a: torch.from_numpy(a).cuda()
    got = cg.x_ao_to_mo(d(X), d(L), d(R))
    torch.cuda.synchronize()
    ref = _ref(X, L, R)
    assert np.max(np.abs(got.cpu().numpy() - ref)) < 1e-12 * np.max(np.abs(ref))


def test_build_then_mo():
    """From a build's X: the trace over the orbitals (cutc_no's tmpJ,
    src/no_tmpJ_cs_kernel.cu:27-31) equals the trace computed in numpy."""
    p = synth.make_problem(n_nuc=2, n_ao=10, n_grid1=200, n_grid2=700, size_bh=5, seed=8)
    X, _ = cg.build_integrals(p, cg.SPLIT_BF16)
    rng = np.random.default_rng(9)
    C = rng.standard_normal((6, p.n_ao))
    Xmo = cg.x_ao_to_mo(X, C, C)
    tmpJ = sum(Xmo[i, i] for i in range(3))  # (comps, n1) over 3 occupied orbitals
    X4 = X.reshape(3, p.n_grid1, p.n_ao, p.n_ao)
    ref = np.einsum("ia,mgba,ib->mg", C[:3], X4, C[:3])
    assert np.max(np.abs(tmpJ - ref)) < 1e-12 * np.max(np.abs(ref))


def test_bad_arguments():
    with pytest.raises(cg.CutcError):  # 2 components
        cg.x_ao_to_mo(np.zeros((2, 5, 3, 3)), np.zeros((2, 3)), np.zeros((2, 3)))
    with pytest.raises(ValueError):
        cg.x_ao_to_mo(np.zeros((3, 5, 4, 4)), np.zeros((2, 3)), np.zeros((2, 3)))
