"""Seeded synthetic transcorrelated-integral inputs.

The reference library takes every input from its caller (the TC workflow
evaluates atomic orbitals on grids itself), so there is no public dataset to
load.  This module builds inputs with the shapes, layouts and value
distributions of the workloads the engine is measured on:

* nuclei at seeded positions inside a box,
* integration grids made of radial shells x random unit directions around each
  nucleus, with positive Becke-like (fuzzy Voronoi) partition weights,
* Cartesian contracted Gaussians (s, p, d shells, 3 primitives, exponents
  log-uniform in [0.1, 50]) evaluated in FP64 with their gradients,
* Boys-Handy Jastrow terms (m, n, o) with coefficients drawn from N(0, sigma).

All arrays are returned in the Fortran column-major layouts of the reference
binding (``src/cutc_module.f90:24-35``), expressed as C-contiguous numpy arrays
with the axes reversed:

==============  =====================  =======================
Fortran         numpy shape (C order)  meaning
==============  =====================  =======================
r(3, n)         (n, 3)                 point coordinates
w(n)            (n,)                   quadrature weights
rn(3, n_nuc)    (n_nuc, 3)             nuclear positions
aos(n, nA, 4)   (4, nA, n)             [value, d/dx, d/dy, d/dz]
c_bh(nB, nN)    (nN, nB)               Jastrow coefficients
m/n/o_bh        (nN, nB) int32         Jastrow exponents
==============  =====================  =======================
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

SHELL_COMPONENTS = {
    0: [(0, 0, 0)],
    1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
    2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)],
}


@dataclasses.dataclass
class Problem:
    """One integral-build request in the reference's array layouts."""

    r1: np.ndarray
    wr1: np.ndarray
    r2: np.ndarray
    wr2: np.ndarray
    rn: np.ndarray
    aos1: np.ndarray
    aos2: np.ndarray
    c_bh: np.ndarray
    m_bh: np.ndarray
    n_bh: np.ndarray
    o_bh: np.ndarray
    a_en: float = 1.0
    a_ee: float = 1.0
    shells: list | None = None  # the basis aos1 / aos2 were evaluated from

    @property
    def n_grid1(self) -> int:
        return self.r1.shape[0]

    @property
    def n_grid2(self) -> int:
        return self.r2.shape[0]

    @property
    def n_ao(self) -> int:
        if self.aos1 is not None:
            return self.aos1.shape[1]
        return sum(len(s.comps) for s in self.shells)

    @property
    def n_nuc(self) -> int:
        return self.rn.shape[0]

    @property
    def size_bh(self) -> int:
        return self.c_bh.shape[1]

    def arrays(self):
        return dict(r1=self.r1, wr1=self.wr1, r2=self.r2, wr2=self.wr2, rn=self.rn,
                    aos1=self.aos1, aos2=self.aos2, c_bh=self.c_bh,
                    m_bh=self.m_bh, n_bh=self.n_bh, o_bh=self.o_bh)

    def flops(self) -> float:
        """Dense-formula flop count of one build: 8 nA^2 n1 n2 + 8 nA^4 n1."""
        nA, n1, n2 = self.n_ao, self.n_grid1, self.n_grid2
        return 8.0 * nA * nA * n1 * n2 + 8.0 * nA ** 4 * n1


def make_nuclei(n_nuc: int, box: float, rng: np.random.Generator,
                min_sep: float = 0.7) -> np.ndarray:
    """Uniform positions in [0, box]^3 with a minimum separation (rejection)."""
    pos = []
    tries = 0
    while len(pos) < n_nuc:
        p = rng.uniform(0.0, box, size=3)
        tries += 1
        if all(np.linalg.norm(p - q) >= min_sep for q in pos) or tries > 10000:
            pos.append(p)
    return np.ascontiguousarray(np.array(pos, dtype=np.float64).reshape(n_nuc, 3))


def make_grid(rn: np.ndarray, n_points: int, rng: np.random.Generator,
              r_scale: float = 1.0) -> tuple[np.ndarray, np.ndarray]:
    """Radial shells x random unit directions around each nucleus.

    Radial nodes follow the Becke map r = R (1+x)/(1-x) on Chebyshev nodes of
    the second kind; angular weights are 4 pi / n_dir; each point is
    multiplied by a fuzzy-Voronoi partition P_A(r) = e_A / sum_B e_B with
    e_A = exp(-2 |r - R_A|), so that all weights are positive.
    """
    n_nuc = rn.shape[0]
    counts = [n_points // n_nuc + (1 if a < n_points % n_nuc else 0) for a in range(n_nuc)]
    pts, wts = [], []
    for a in range(n_nuc):
        cnt = counts[a]
        if cnt == 0:
            continue
        n_rad = max(1, int(round(math.sqrt(cnt / 2.0))))
        n_rad = min(n_rad, cnt)
        per_shell = [cnt // n_rad + (1 if k < cnt % n_rad else 0) for k in range(n_rad)]
        for k in range(n_rad):
            nd = per_shell[k]
            if nd == 0:
                continue
            t = (k + 1) * math.pi / (n_rad + 1)
            x = math.cos(t)
            r = r_scale * (1.0 + x) / (1.0 - x)
            # dr/dt for the Becke map, times the Chebyshev-2 weight pi/(n+1) sin^2 t / sin t
            drdx = 2.0 * r_scale / (1.0 - x) ** 2
            w_rad = (math.pi / (n_rad + 1)) * math.sin(t) * drdx * r * r
            v = rng.normal(size=(nd, 3))
            v /= np.linalg.norm(v, axis=1, keepdims=True)
            pts.append(rn[a] + r * v)
            wts.append(np.full(nd, w_rad * 4.0 * math.pi / nd))
    r = np.ascontiguousarray(np.concatenate(pts).astype(np.float64))
    w = np.concatenate(wts)
    # fuzzy Voronoi partition
    d = np.linalg.norm(r[:, None, :] - rn[None, :, :], axis=2)
    e = np.exp(-2.0 * (d - d.min(axis=1, keepdims=True)))
    owner = np.repeat(np.arange(n_nuc), counts)
    part = e[np.arange(r.shape[0]), owner] / e.sum(axis=1)
    w = np.ascontiguousarray(w * part)
    return r, w


@dataclasses.dataclass
class Shell:
    center: np.ndarray
    l: int
    exps: np.ndarray
    coefs: np.ndarray
    comps: list


def make_basis(rn: np.ndarray, n_ao: int, rng: np.random.Generator) -> list[Shell]:
    """Cartesian s/p/d shells, cycled over the nuclei until n_ao functions exist."""
    shells = []
    n = 0
    k = 0
    n_nuc = rn.shape[0]
    while n < n_ao:
        l = k % 3
        center = rn[(k // 3) % n_nuc]
        exps = np.exp(rng.uniform(math.log(0.1), math.log(50.0), size=3))
        coefs = rng.uniform(0.2, 1.0, size=3)
        # normalise so the largest contracted value at the centre scale is O(1)
        coefs = coefs / coefs.sum()
        comps = SHELL_COMPONENTS[l][: n_ao - n]
        shells.append(Shell(center.copy(), l, exps, coefs, comps))
        n += len(comps)
        k += 1
    return shells


def eval_aos(shells: list[Shell], r: np.ndarray) -> np.ndarray:
    """Values and gradients of every AO at every point: C array (4, nA, n)."""
    n = r.shape[0]
    n_ao = sum(len(s.comps) for s in shells)
    out = np.empty((4, n_ao, n), dtype=np.float64)
    i = 0
    for s in shells:
        d = r - s.center[None, :]
        r2 = np.einsum("ij,ij->i", d, d)
        g = np.zeros(n)
        dg = np.zeros(n)  # d/d(r2) of the radial part
        for a, c in zip(s.exps, s.coefs):
            e = c * np.exp(-a * r2)
            g += e
            dg += -a * e
        for (lx, ly, lz) in s.comps:
            ex = (lx, ly, lz)
            ang = np.ones(n)
            for ax in range(3):
                if ex[ax]:
                    ang = ang * d[:, ax] ** ex[ax]
            out[0, i] = ang * g
            for ax in range(3):
                # d/dx_ax [ang * g] = (d ang/dx_ax) g + ang * 2 d_ax dg
                if ex[ax]:
                    dang = np.ones(n) * ex[ax] * d[:, ax] ** (ex[ax] - 1)
                    for bx in range(3):
                        if bx != ax and ex[bx]:
                            dang = dang * d[:, bx] ** ex[bx]
                else:
                    dang = np.zeros(n)
                out[1 + ax, i] = dang * g + ang * 2.0 * d[:, ax] * dg
            i += 1
    return out


def basis_arrays(shells: list[Shell]) -> dict:
    """The basis one entry per AO, as the engine's cutc_basis takes it: C arrays
    center (nA, 3), power (nA, 3) int32, prim_offset (nA + 1,) int32, prim_exp and
    prim_coef (primitives of AO a at prim_offset[a] .. prim_offset[a + 1] - 1)."""
    center, power, off, ex, co = [], [], [0], [], []
    for s in shells:
        for comp in s.comps:
            center.append(s.center)
            power.append(comp)
            ex.extend(s.exps)
            co.extend(s.coefs)
            off.append(len(ex))
    return dict(center=np.ascontiguousarray(np.array(center, dtype=np.float64).reshape(-1, 3)),
                power=np.ascontiguousarray(np.array(power, dtype=np.int32).reshape(-1, 3)),
                prim_offset=np.ascontiguousarray(np.array(off, dtype=np.int32)),
                prim_exp=np.ascontiguousarray(np.array(ex, dtype=np.float64)),
                prim_coef=np.ascontiguousarray(np.array(co, dtype=np.float64)))


EXP_CHOICES = np.array([0, 2, 3, 4], dtype=np.int32)


def make_jastrow(n_nuc: int, size_bh: int, rng: np.random.Generator,
                 sigma: float = 0.3, exps=EXP_CHOICES, o_exps=EXP_CHOICES):
    """Boys-Handy terms per nucleus: C arrays (n_nuc, size_bh)."""
    c = rng.normal(0.0, sigma, size=(n_nuc, size_bh))
    m = rng.choice(exps, size=(n_nuc, size_bh)).astype(np.int32)
    nn = rng.choice(exps, size=(n_nuc, size_bh)).astype(np.int32)
    o = rng.choice(o_exps, size=(n_nuc, size_bh)).astype(np.int32)
    return (np.ascontiguousarray(c), np.ascontiguousarray(m),
            np.ascontiguousarray(nn), np.ascontiguousarray(o))


def make_problem(n_nuc: int, n_ao: int, n_grid1: int, n_grid2: int, size_bh: int,
                 seed: int, box: float = 3.0, a_en: float = 1.0, a_ee: float = 1.0,
                 sigma: float = 0.3, with_aos: bool = True) -> Problem:
    """with_aos=False leaves aos1 / aos2 as None: the basis (shells) is kept for the
    engine to evaluate the AOs on the device."""
    rng = np.random.default_rng(seed)
    rn = make_nuclei(n_nuc, box, rng)
    r1, wr1 = make_grid(rn, n_grid1, rng)
    r2, wr2 = make_grid(rn, n_grid2, rng)
    shells = make_basis(rn, n_ao, rng)
    aos1 = eval_aos(shells, r1) if with_aos else None
    aos2 = eval_aos(shells, r2) if with_aos else None
    c, m, nn, o = make_jastrow(n_nuc, size_bh, rng, sigma)
    return Problem(r1, wr1, r2, wr2, rn, aos1, aos2, c, m, nn, o, a_en, a_ee, shells)


# Named workloads (sizes of the measured configurations).
CONFIGS = {
    # 3 nuclei in a 3-bohr box, 24 AOs, 3k x 12k grid pairs, 9 terms per atom
    "small": dict(n_nuc=3, n_ao=24, n_grid1=3000, n_grid2=12000, size_bh=9, seed=1001, box=3.0),
    # 10 nuclei, 120 AOs, 25k x 80k grid pairs, 13 terms per atom
    "medium": dict(n_nuc=10, n_ao=120, n_grid1=25000, n_grid2=80000, size_bh=13, seed=2002, box=6.0),
    # 20 nuclei, 300 AOs, 60k x 200k grid pairs, 17 terms per atom
    "large": dict(n_nuc=20, n_ao=300, n_grid1=60000, n_grid2=200000, size_bh=17, seed=3003, box=9.0),
    # one molecule for the Jastrow-parameter scan (8 nuclei, 80 AOs, 15k x 50k)
    "scan": dict(n_nuc=8, n_ao=80, n_grid1=15000, n_grid2=50000, size_bh=13, seed=5005, box=5.0),
}


def make_config(name: str, **overrides) -> Problem:
    kw = dict(CONFIGS[name])
    kw.update(overrides)
    return make_problem(**kw)


def scaled_config(name: str, frac1: float = 1.0, frac2: float = 1.0) -> Problem:
    """The named molecule with grids shrunk by the given fractions (same seed)."""
    kw = dict(CONFIGS[name])
    kw["n_grid1"] = max(kw["n_nuc"], int(kw["n_grid1"] * frac1))
    kw["n_grid2"] = max(kw["n_nuc"], int(kw["n_grid2"] * frac2))
    return make_problem(**kw)


def r1_sample(p: Problem, ns: int) -> Problem:
    """The same molecule with ns r1 points spread evenly over its whole r1 grid
    (every nucleus' shells are represented); r2 and the basis are unchanged."""
    idx = np.unique(np.linspace(0, p.n_grid1 - 1, ns).round().astype(np.int64))
    assert len(idx) == ns
    aos1 = None if p.aos1 is None else np.ascontiguousarray(p.aos1[:, :, idx])
    return dataclasses.replace(p, r1=np.ascontiguousarray(p.r1[idx]),
                               wr1=np.ascontiguousarray(p.wr1[idx]), aos1=aos1)


def serving_molecule(n_nuc: int = 20, n_ao: int = 250, seed: int = 4242) -> Problem:
    """A molecule of the serving stream's shape (n_grid1 = 1000 n_nuc,
    n_grid2 = 4000 n_nuc, 9 Jastrow terms per atom)."""
    return make_problem(n_nuc=n_nuc, n_ao=n_ao, n_grid1=1000 * n_nuc, n_grid2=4000 * n_nuc,
                        size_bh=9, seed=seed, box=1.5 + 0.4 * n_nuc)


def add_coalescence(p: Problem, k: int = 4) -> Problem:
    """Copy some r1 points and nuclei into r2 (and nuclei into r1) exactly.

    This drives the r12 = 0 and r1n = 0 / r2n = 0 branches of the pair terms.
    """
    r1 = p.r1.copy()
    r2 = p.r2.copy()
    k = min(k, r1.shape[0], r2.shape[0] // 2)
    r2[:k] = r1[:k]
    for a in range(p.n_nuc):
        if k + a < r2.shape[0]:
            r2[k + a] = p.rn[a]
        if k + a < r1.shape[0]:
            r1[k + a] = p.rn[a]
    return dataclasses.replace(p, r1=np.ascontiguousarray(r1), r2=np.ascontiguousarray(r2))
