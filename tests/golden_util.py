"""Loading of the golden fixtures generated from the reference (tests/golden)."""
import os

import numpy as np

from cutc_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASE_NAMES = ["tiny_coalesce", "tiny_r2_passes", "tiny_spd"]


def load_case(name):
    z = np.load(os.path.join(GOLDEN, "case_%s.npz" % name))
    p = synth.Problem(r1=z["r1"], wr1=z["wr1"], r2=z["r2"], wr2=z["wr2"], rn=z["rn"],
                      aos1=z["aos1"], aos2=z["aos2"], c_bh=z["c_bh"], m_bh=z["m_bh"],
                      n_bh=z["n_bh"], o_bh=z["o_bh"], a_en=float(z["a_en"]),
                      a_ee=float(z["a_ee"]))
    return p, {k: z[k] for k in ("X", "int2e", "G", "dims")}


def load_small_digest():
    return dict(np.load(os.path.join(GOLDEN, "small_digest.npz")))
