"""The flattened basis (one entry per AO) describes exactly the functions the
generator evaluates (CPU only; the GPU evaluator is checked in test_gpu_aos.py)."""
import numpy as np

from cutc_gb300 import synth


def _eval_flat(b, r):
    """Values from the flattened arrays, by the formula of include/cutc_int.h."""
    n_ao = b["center"].shape[0]
    out = np.empty((n_ao, r.shape[0]))
    for a in range(n_ao):
        d = r - b["center"][a]
        r2 = np.einsum("ij,ij->i", d, d)
        k0, k1 = b["prim_offset"][a], b["prim_offset"][a + 1]
        rad = sum(c * np.exp(-e * r2) for e, c in zip(b["prim_exp"][k0:k1], b["prim_coef"][k0:k1]))
        lx, ly, lz = b["power"][a]
        out[a] = d[:, 0] ** lx * d[:, 1] ** ly * d[:, 2] ** lz * rad
    return out


def test_basis_arrays_match_generator():
    p = synth.make_problem(n_nuc=3, n_ao=17, n_grid1=50, n_grid2=80, size_bh=3, seed=3)
    b = synth.basis_arrays(p.shells)
    assert b["center"].shape == (17, 3) and b["power"].shape == (17, 3)
    assert b["prim_offset"][0] == 0 and b["prim_offset"][-1] == len(b["prim_exp"])
    np.testing.assert_allclose(_eval_flat(b, p.r1), p.aos1[0], rtol=1e-14, atol=1e-300)
