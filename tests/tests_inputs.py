"""Checksums of a Problem's inputs (same definition as tests/golden/make_golden.py)."""
import numpy as np


def input_checksums(p):
    return np.array([float(np.sum(a, dtype=np.float64)) for a in
                     (p.r1, p.wr1, p.r2, p.wr2, p.rn, p.aos1, p.aos2, p.c_bh)]
                    + [float(np.sum(p.m_bh) + 7 * np.sum(p.n_bh) + 49 * np.sum(p.o_bh))])
