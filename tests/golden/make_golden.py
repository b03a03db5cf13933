"""Generate the golden fixtures in tests/golden/ from the reference itself.

The reference CuTC sources are compiled for the CPU by
oracle/ref_emul/build_ref.py (host emulation of CUDA/cuBLAS) and called through
their own C-ABI entry point ``cutc_int`` (src/cutc_int.c:15-20) on seeded
synthetic inputs.  The pair kernel is also called alone through its wrapper
``cutc_int_bh`` (src/jast_bh.cu:268-303) so its output can be pinned bit for
bit.  Run it in the development container, where the reference is mounted:

    python tests/golden/make_golden.py

Outputs:
  case_<name>.npz   inputs, launch dims, reference X (3, n1, nA^2),
                    int_2e (nA^2, nA^2) and the pair planes G (4, n1, n2)
  small_digest.npz  the "small" workload (3 nuclei, 24 AOs, 3k x 12k grid):
                    input checksums, norms and 4096 sampled output entries
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from cutc_gb300 import synth  # noqa: E402
from oracle.ref_emul import build_ref  # noqa: E402
from tests_inputs import input_checksums  # noqa: E402


class Dim3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint), ("y", ctypes.c_uint), ("z", ctypes.c_uint)]


def _vp(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def ref_lib():
    path = build_ref.build()
    if path is None:
        raise SystemExit("reference sources are not mounted; cannot regenerate fixtures")
    return ctypes.CDLL(path)


def ref_cutc_int(L, p, dims):
    X = np.full((3, p.n_grid1, p.n_ao ** 2), np.nan)
    I = np.full((p.n_ao ** 2, p.n_ao ** 2), np.nan)
    args = [ctypes.c_int(v) for v in dims]
    args += [ctypes.c_int(v) for v in (p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh)]
    args += [_vp(a) for a in (p.r1, p.wr1, p.r2, p.wr2, p.rn, p.aos1, p.aos2,
                              p.c_bh, p.m_bh, p.n_bh, p.o_bh, X, I)]
    rc = L.cutc_int(*args)
    return rc, X, I


def ref_pair(L, p, dims):
    G = np.full((4, p.n_grid1, p.n_grid2), np.nan)
    L.cutc_int_bh(Dim3(*dims[:3]), Dim3(*dims[3:]), 0, p.n_grid1, p.n_grid1,
                  0, p.n_grid2, p.n_grid2, p.n_nuc, p.size_bh,
                  _vp(p.r1), _vp(p.r2), _vp(p.rn), _vp(p.c_bh), _vp(p.m_bh),
                  _vp(p.n_bh), _vp(p.o_bh), _vp(G))
    return G


def tweak_exponents(p):
    """Exercise exponents 1, 5, 6, an o = 1 term and a skipped |c| < 1e-10 term."""
    p.m_bh[0, 0] = 1
    p.n_bh[0, min(1, p.size_bh - 1)] = 5
    p.o_bh[min(1, p.n_nuc - 1), 0] = 6
    p.o_bh[0, min(2, p.size_bh - 1)] = 1
    p.c_bh[min(1, p.n_nuc - 1), min(1, p.size_bh - 1)] = 1e-11
    return p


CASES = {
    # coalescence branches (r12 = 0, r1 = nucleus, r2 = nucleus), odd sizes
    "tiny_coalesce": dict(make=dict(n_nuc=2, n_ao=5, n_grid1=37, n_grid2=101, size_bh=4, seed=7),
                          coalesce=True, tweak=True, dims=(2, 3, 1, 4, 2, 1)),
    # n_grid2 > 5 n_grid1: the reference tiles r2 in two passes (src/build_int2_grad1_u12_ao.cu:85-99)
    "tiny_r2_passes": dict(make=dict(n_nuc=2, n_ao=4, n_grid1=40, n_grid2=256, size_bh=5, seed=8),
                           coalesce=False, tweak=True, dims=(1, 1, 1, 8, 8, 1)),
    # s, p, d shells on 3 nuclei with the measured exponent set {0,2,3,4}
    "tiny_spd": dict(make=dict(n_nuc=3, n_ao=10, n_grid1=64, n_grid2=256, size_bh=9, seed=11),
                     coalesce=True, tweak=False, dims=(4, 4, 1, 16, 8, 1)),
}


def make_case(name):
    spec = CASES[name]
    p = synth.make_problem(**spec["make"])
    if spec["coalesce"]:
        p = synth.add_coalescence(p)
    if spec["tweak"]:
        p = tweak_exponents(p)
    return p, spec["dims"]


def main():
    L = ref_lib()
    for name in CASES:
        p, dims = make_case(name)
        rc, X, I = ref_cutc_int(L, p, dims)
        G = ref_pair(L, p, dims)
        assert rc == 0 and np.all(np.isfinite(X)) and np.all(np.isfinite(I))
        out = os.path.join(HERE, "case_%s.npz" % name)
        np.savez_compressed(out, dims=np.array(dims, dtype=np.int32), a_en=1.0, a_ee=1.0,
                            X=X, int2e=I, G=G, **p.arrays())
        print("wrote", out, os.path.getsize(out), "bytes")

    p = synth.make_config("small")
    rc, X, I = ref_cutc_int(L, p, (64, 64, 1, 16, 16, 1))
    assert rc == 0 and np.all(np.isfinite(X)) and np.all(np.isfinite(I))
    rng = np.random.default_rng(12345)
    ix = rng.integers(0, X.size, size=4096)
    ii = rng.integers(0, I.size, size=4096)
    out = os.path.join(HERE, "small_digest.npz")
    np.savez_compressed(out, input_checksums=input_checksums(p),
                        X_norm=np.linalg.norm(X.ravel()), I_norm=np.linalg.norm(I.ravel()),
                        X_max=np.abs(X).max(), I_max=np.abs(I).max(),
                        X_idx=ix, X_val=X.ravel()[ix], I_idx=ii, I_val=I.ravel()[ii],
                        X_comp_sums=X.reshape(3, -1).sum(axis=1))
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
