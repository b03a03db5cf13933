"""CPU oracle driver for the cutc_int hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker (or as the timed CPU baseline).  The product
library never imports it.

The element-wise kernels are the C restatement in oracle/cutc_oracle.c; the
dense contractions that the reference runs as cuBLAS DGEMM
(src/build_int2_grad1_u12_ao.cu:152-159, src/build_int_2e_ao.cu:60-67,97-104)
are numpy matmuls here.  The sequence follows src/cutc_int.c:15-243:

    X_m[:, r1]  = sum_r2 P[r2, :] G_m[r2, r1]              m = 0..3
    A           = X_3 S0  - 1/2 sum_m X_m S_m               (K = n1, 3 n1)
    int_2e      = A + A^T                                   (add_trans_inplace)

Outputs use the reference layouts: X(nA, nA, n1, 3) and int_2e(nA, nA, nA, nA)
in Fortran order, i.e. numpy C arrays of shape (3, n1, nA*nA) and
(nA*nA, nA*nA) (the latter indexed [col, row]).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile cutc_oracle.c into oracle/_build/liboracle.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "cutc_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           src, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        i = ctypes.c_int
        d = ctypes.c_double
        L.oracle_pair.argtypes = [i, i, i, i, i, dp, dp, dp, dp, ip, ip, ip, d, d, dp]
        L.oracle_long_range.argtypes = [i, i, i, i, dp, dp, dp]
        L.oracle_short_herm.argtypes = [i, i, dp, dp, dp]
        L.oracle_short_nonherm.argtypes = [i, i, dp, dp, dp]
        L.oracle_add_trans.argtypes = [ctypes.c_int64, dp]
        for f in (L.oracle_pair, L.oracle_long_range, L.oracle_short_herm,
                  L.oracle_short_nonherm, L.oracle_add_trans):
            f.restype = None
        _lib = L
    return _lib


def _dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def pair(p, i0: int = 0, n1b: int | None = None) -> np.ndarray:
    """grad1 u for r1 rows [i0, i0+n1b): array (4, n1b, n2)."""
    n1b = p.n_grid1 - i0 if n1b is None else n1b
    G = np.empty((4, n1b, p.n_grid2))
    lib().oracle_pair(i0, n1b, p.n_grid2, p.n_nuc, p.size_bh, _dp(p.r1), _dp(p.r2), _dp(p.rn),
                      _dp(p.c_bh), _ip(p.m_bh), _ip(p.n_bh), _ip(p.o_bh),
                      float(p.a_en), float(p.a_ee), _dp(G))
    return G


def long_range(p) -> np.ndarray:
    """P as a C array (nA*nA, n2): row j + nA i = w2 chi_i chi_j."""
    P = np.empty((p.n_ao * p.n_ao, p.n_grid2))
    lib().oracle_long_range(0, p.n_grid2, p.n_grid2, p.n_ao, _dp(p.wr2), _dp(p.aos2), _dp(P))
    return P


def short_herm(p) -> np.ndarray:
    S0 = np.empty((p.n_ao * p.n_ao, p.n_grid1))
    lib().oracle_short_herm(p.n_grid1, p.n_ao, _dp(p.wr1), _dp(p.aos1), _dp(S0))
    return S0


def short_nonherm(p) -> np.ndarray:
    S = np.empty((p.n_ao * p.n_ao, 3, p.n_grid1))
    lib().oracle_short_nonherm(p.n_grid1, p.n_ao, _dp(p.wr1), _dp(p.aos1), _dp(S))
    return S


def x_block(p, P: np.ndarray, i0: int, n1b: int) -> np.ndarray:
    """X for r1 rows [i0, i0+n1b), all 4 components: array (4, n1b, nA*nA)."""
    G = pair(p, i0, n1b)
    X = np.empty((4, n1b, P.shape[0]))
    for m in range(4):
        np.matmul(G[m], P.T, out=X[m])
    return X


def x_rows(p, i0: int = 0, n1b: int | None = None, window_bytes: int = 1 << 30) -> np.ndarray:
    """X for r1 rows [i0, i0+n1b), all 4 components, without the whole P.

    P is formed by the C restatement one r2 window at a time
    (src/long_range_integ.cu:21-45 on a window, as the reference's r2 passes do,
    src/build_int2_grad1_u12_ao.cu:113-331) and each window's share
    G_m[:, window] P_window^T is added: the same products as x_block, summed in
    r2 windows.  For molecules whose full P (nA^2 x n2 doubles) does not fit."""
    n1b = p.n_grid1 - i0 if n1b is None else n1b
    G = pair(p, i0, n1b).reshape(4 * n1b, p.n_grid2)
    nA2 = p.n_ao * p.n_ao
    n2 = p.n_grid2
    jc = int(max(1, min(n2, window_bytes // (8 * nA2))))
    X = np.zeros((4 * n1b, nA2))
    Pw = np.empty((nA2, jc))
    for j0 in range(0, n2, jc):
        w = min(jc, n2 - j0)
        Pv = Pw[:, :w] if w == jc else np.empty((nA2, w))
        lib().oracle_long_range(j0, w, n2, p.n_ao, _dp(p.wr2), _dp(p.aos2), _dp(Pv))
        X += np.ascontiguousarray(G[:, j0:j0 + w]) @ Pv.T
    return X.reshape(4, n1b, nA2)


def int2e_rows(p, X4: np.ndarray, rows, S0=None, S=None) -> np.ndarray:
    """Rows `rows` of int_2e (C layout, i.e. Fortran columns) for the r1 points
    of p, from their X (4, n1, nA^2): (A + A^T)[rows, :] with A as int2e_from_x
    returns it, without forming the nA^2 x nA^2 matrix."""
    rows = np.asarray(rows)
    if S0 is None:
        S0 = short_herm(p)
    if S is None:
        S = short_nonherm(p)
    out = S0[rows] @ X4[3] + (S0 @ X4[3][:, rows]).T
    for m in range(3):
        out -= 0.5 * (S[rows, m] @ X4[m] + (S[:, m] @ X4[m][:, rows]).T)
    return out


def int2e_matvec(p, X4: np.ndarray, v: np.ndarray, S0=None, S=None) -> np.ndarray:
    """int_2e (C layout) times v, for the r1 points of p, from their X:
    (A + A^T) v = S0 (X_3 v) + X_3^T (S0^T v) - 1/2 sum_m [...], without
    forming the nA^2 x nA^2 matrix."""
    if S0 is None:
        S0 = short_herm(p)
    if S is None:
        S = short_nonherm(p)
    out = S0 @ (X4[3] @ v) + X4[3].T @ (S0.T @ v)
    for m in range(3):
        Sm = S[:, m]
        out -= 0.5 * (Sm @ (X4[m] @ v) + X4[m].T @ (Sm.T @ v))
    return out


def int2e_from_x(p, X4: np.ndarray, i0: int = 0, S0=None, S=None) -> np.ndarray:
    """Contraction of X (4, n1b, nA^2) over its r1 rows, before A + A^T.

    Returns A as a C array indexed [col, row] (Fortran (nA^2, nA^2)).
    """
    n1b = X4.shape[1]
    if S0 is None:
        S0 = short_herm(p)
    if S is None:
        S = short_nonherm(p)
    sl = slice(i0, i0 + n1b)
    A = S0[:, sl] @ X4[3]
    for m in range(3):
        A -= 0.5 * (S[:, m, sl] @ X4[m])
    return A


def cutc_int(p, block1: int | None = None):
    """Full oracle build: returns (X3 (3, n1, nA^2), int_2e (nA^2, nA^2))."""
    n1 = p.n_grid1
    block1 = n1 if block1 is None else block1
    P = long_range(p)
    S0 = short_herm(p)
    S = short_nonherm(p)
    nA2 = p.n_ao * p.n_ao
    X3 = np.empty((3, n1, nA2))
    A = np.zeros((nA2, nA2))
    for i0 in range(0, n1, block1):
        n1b = min(block1, n1 - i0)
        X = x_block(p, P, i0, n1b)
        X3[:, i0:i0 + n1b] = X[:3]
        A += int2e_from_x(p, X, i0, S0, S)
    lib().oracle_add_trans(nA2, _dp(A))
    return X3, A


def rel_err(a: np.ndarray, b: np.ndarray) -> dict:
    """Normwise and max-abs relative errors of a against the reference b."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = float(np.linalg.norm(b.ravel()))
    mb = float(np.max(np.abs(b))) if b.size else 0.0
    d = (a - b).ravel()
    return {
        "norm": float(np.linalg.norm(d)) / nb if nb > 0 else float(np.linalg.norm(d)),
        "max": float(np.max(np.abs(d))) / mb if mb > 0 else float(np.max(np.abs(d)) if d.size else 0.0),
    }
