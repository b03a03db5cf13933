"""GB300-native transcorrelated-integral engine (drop-in for CuTC's cutc_int).

The compute path is the CUDA library ``cutc_gb300/lib/libcutcint.so`` (sm_103a),
reached through its C-ABI (include/cutc_int.h) with ctypes.  This module
mirrors the reference's entry point -- same name, argument order, array
layouts and return codes as ``cutc_int`` (src/cutc_int.c:15-20) -- and adds
the extended options.  There is no CPU fallback: if the library cannot be
loaded, every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libcutcint.so")

CUTC_OK = 0
CUTC_ERR_LAUNCH_DIMS = -1
CUTC_ERR_INVALID = -2
CUTC_ERR_NO_MEMORY = -3
CUTC_ERR_CUDA = -4
CUTC_ERR_NO_DEVICE = -5
CUTC_ERR_TIMEOUT = -6

PLAIN_FP64 = 0
SPLIT_BF16 = 1

# every symbol include/cutc_int.h declares
EXPORTS = ["cutc_int", "cutc_int_ex", "cutc_int_scan", "cutc_default_options", "cutc_jast_bh_dev",
           "cutc_jast_bh_dev_noalloc", "cutc_split_gemm_dev", "cutc_fp64_gemm_dev",
           "cutc_check_wait_limit",
           "cutc_validate_launch_dims",
           "cutc_last_error", "cutc_release", "cutc_server_default_config", "cutc_server_create",
           "cutc_server_submit", "cutc_server_wait", "cutc_server_get_stats", "cutc_server_destroy",
           "trans_inplace", "trans_pqst_psqt_inplace", "trans_pqst_psqt_copy", "cutc_eval_aos",
           "cutc_x_ao_to_mo", "cutc_no_2e", "cutc_plan", "cutc_pin_host", "cutc_unpin_host",
           "cutc_int_bh", "int_long_range", "int_short_range_herm", "int_short_range_nonherm",
           "get_int2_grad1_u12_ao", "get_int_2e_ao"]

INT2E_PQST = 0
INT2E_PSQT = 1


class Dim3(ctypes.Structure):
    """CUDA's dim3 by value (cutc_dim3): the reference's launch-geometry argument."""
    _fields_ = [("x", ctypes.c_uint), ("y", ctypes.c_uint), ("z", ctypes.c_uint)]


class PlanInfo(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in ("tile_rows", "block_rows", "n_tiles", "n_blocks",
                                            "slab_cols")] + \
               [(k, ctypes.c_size_t) for k in ("budget_bytes", "fixed_bytes", "tile_row_bytes",
                                               "block_row_bytes", "footprint_bytes")] + \
               [("x_launches_per_tile", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Basis(ctypes.Structure):
    _fields_ = [("n_ao", ctypes.c_int), ("center", ctypes.c_void_p), ("power", ctypes.c_void_p),
                ("prim_offset", ctypes.c_void_p), ("prim_exp", ctypes.c_void_p),
                ("prim_coef", ctypes.c_void_p)]


def make_basis(shells):
    """A cutc_basis for synth shells; the returned object keeps its arrays alive."""
    from .synth import basis_arrays
    arrs = basis_arrays(shells)
    b = Basis()
    b.n_ao = arrs["center"].shape[0]
    for k in ("center", "power", "prim_offset", "prim_exp", "prim_coef"):
        setattr(b, k, arrs[k].ctypes.data)
    b._arrays = arrs
    return b


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("n_slices", ctypes.c_int),
                ("a_en", ctypes.c_double), ("a_ee", ctypes.c_double),
                ("x_components", ctypes.c_int), ("device_pointers", ctypes.c_int),
                ("max_work_bytes", ctypes.c_size_t), ("stream", ctypes.c_void_p),
                ("pair_fp64", ctypes.c_int), ("k_split", ctypes.c_int),
                ("int2e_layout", ctypes.c_int), ("basis", ctypes.c_void_p),
                ("r1_begin", ctypes.c_int), ("r1_end", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("ms_total", ctypes.c_double), ("ms_h2d", ctypes.c_double),
                ("ms_pair", ctypes.c_double), ("ms_x", ctypes.c_double),
                ("ms_int2e", ctypes.c_double), ("ms_d2h", ctypes.c_double),
                ("n_r1_tiles", ctypes.c_int), ("gpu_launches", ctypes.c_int),
                ("ms_x_gemm", ctypes.c_double), ("n_x_gemm", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerConfig(ctypes.Structure):
    _fields_ = [("n_slots", ctypes.c_int), ("device_budget_bytes", ctypes.c_size_t),
                ("cache_budget_bytes", ctypes.c_size_t), ("tile_budget_bytes", ctypes.c_size_t)]


class Request(ctypes.Structure):
    _fields_ = [("molecule_key", ctypes.c_ulonglong)] + \
        [(k, ctypes.c_int) for k in ("n_grid1", "n_grid2", "n_ao", "n_nuc", "size_bh")] + \
        [(k, ctypes.c_void_p) for k in ("r1", "wr1", "r2", "wr2", "rn", "aos_data1", "aos_data2",
                                        "c_bh", "m_bh", "n_bh", "o_bh", "int2_grad1_u12_ao",
                                        "int_2e_ao")] + \
        [("options", Options)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_long), ("failed", ctypes.c_long), ("queued", ctypes.c_long),
                ("in_flight", ctypes.c_int), ("peak_in_flight", ctypes.c_int),
                ("cache_hits", ctypes.c_long), ("cache_misses", ctypes.c_long),
                ("cache_bytes", ctypes.c_size_t), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("builds_per_s", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class CutcError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("cutc status %d: %s" % (status, message))
        self.status = status


_lib = None


def load(path: str = LIB_PATH):
    """Load libcutcint.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(path)
    i, vp, dp = ctypes.c_int, ctypes.c_void_p, ctypes.c_double
    L.cutc_int.argtypes = [i] * 11 + [vp] * 13
    L.cutc_int.restype = i
    L.cutc_int_ex.argtypes = [ctypes.POINTER(Options)] + [i] * 5 + [vp] * 13 + [ctypes.POINTER(Stats)]
    L.cutc_int_ex.restype = i
    L.cutc_int_scan.argtypes = [ctypes.POINTER(Options), i] + [i] * 5 + [vp] * 15 + \
        [ctypes.POINTER(Stats)]
    L.cutc_int_scan.restype = i
    L.cutc_default_options.argtypes = [ctypes.POINTER(Options)]
    L.cutc_default_options.restype = None
    L.cutc_jast_bh_dev.argtypes = [i] * 6 + [vp] * 7 + [dp, dp, vp]
    L.cutc_jast_bh_dev.restype = i
    L.cutc_jast_bh_dev_noalloc.argtypes = [i] * 6 + [vp] * 7 + [dp, dp, vp, vp]
    L.cutc_jast_bh_dev_noalloc.restype = i
    L.cutc_split_gemm_dev.argtypes = [i, i, i, ctypes.c_longlong, vp, vp, vp, ctypes.c_longlong]
    L.cutc_split_gemm_dev.restype = i
    ll = ctypes.c_longlong
    L.cutc_fp64_gemm_dev.argtypes = [i, i, i, ll, ctypes.c_double, vp, ll, ll, vp, ll, ll,
                                     ctypes.c_double, vp, ll, ll, i]
    L.cutc_fp64_gemm_dev.restype = i
    L.cutc_no_2e.argtypes = [ctypes.POINTER(Options), i, i, vp, vp, vp, vp, vp]
    L.cutc_no_2e.restype = i
    L.cutc_validate_launch_dims.argtypes = [i] * 6
    L.cutc_validate_launch_dims.restype = i
    L.cutc_last_error.argtypes = []
    L.cutc_last_error.restype = ctypes.c_char_p
    L.cutc_release.argtypes = []
    L.cutc_release.restype = None
    L.cutc_check_wait_limit.argtypes = []
    L.cutc_check_wait_limit.restype = i
    L.trans_inplace.argtypes = [vp, i]
    L.trans_inplace.restype = None
    L.trans_pqst_psqt_inplace.argtypes = [i, vp]
    L.trans_pqst_psqt_inplace.restype = None
    L.trans_pqst_psqt_copy.argtypes = [i, vp, vp]
    L.trans_pqst_psqt_copy.restype = None
    L.cutc_int_bh.argtypes = [Dim3, Dim3] + [i] * 8 + [vp] * 8
    L.cutc_int_bh.restype = None
    L.int_long_range.argtypes = [i] * 5 + [vp] * 3
    L.int_long_range.restype = None
    L.int_short_range_herm.argtypes = [i, i, vp, vp, vp]
    L.int_short_range_herm.restype = None
    L.int_short_range_nonherm.argtypes = [i, i, vp, vp, vp]
    L.int_short_range_nonherm.restype = None
    L.get_int2_grad1_u12_ao.argtypes = [Dim3, Dim3] + [i] * 5 + [vp] * 10
    L.get_int2_grad1_u12_ao.restype = None
    L.get_int_2e_ao.argtypes = [i, i] + [vp] * 4
    L.get_int_2e_ao.restype = None
    L.cutc_eval_aos.argtypes = [ctypes.POINTER(Basis), i, vp, i, vp, i, vp]
    L.cutc_eval_aos.restype = i
    L.cutc_x_ao_to_mo.argtypes = [i, i, i, i, vp, vp, vp, vp, i, vp]
    L.cutc_x_ao_to_mo.restype = i
    L.cutc_plan.argtypes = [ctypes.POINTER(Options), i, i, i, i, ctypes.POINTER(PlanInfo)]
    L.cutc_plan.restype = i
    L.cutc_pin_host.argtypes = [vp, ctypes.c_size_t]
    L.cutc_pin_host.restype = i
    L.cutc_unpin_host.argtypes = [vp]
    L.cutc_unpin_host.restype = i
    L.cutc_server_default_config.argtypes = [ctypes.POINTER(ServerConfig)]
    L.cutc_server_default_config.restype = None
    L.cutc_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]
    L.cutc_server_create.restype = i
    L.cutc_server_submit.argtypes = [vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_ulonglong)]
    L.cutc_server_submit.restype = i
    L.cutc_server_wait.argtypes = [vp, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_double)]
    L.cutc_server_wait.restype = i
    L.cutc_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
    L.cutc_server_get_stats.restype = i
    L.cutc_server_destroy.argtypes = [vp]
    L.cutc_server_destroy.restype = None
    _lib = L
    return L


def last_error() -> str:
    return load().cutc_last_error().decode()


def _vp(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    assert a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.c_void_p)


def cutc_int(nxBlocks, nyBlocks, nzBlocks, blockxSize, blockySize, blockzSize,
             n_grid1, n_grid2, n_ao, n_nuc, size_bh,
             r1, wr1, r2, wr2, rn, aos_data1, aos_data2,
             c_bh, m_bh, n_bh, o_bh, int2_grad1_u12_ao, int_2e_ao) -> int:
    """The reference entry point: host arrays in, host outputs filled, status out."""
    L = load()
    arrs = [r1, wr1, r2, wr2, rn, aos_data1, aos_data2, c_bh, m_bh, n_bh, o_bh,
            int2_grad1_u12_ao, int_2e_ao]
    return L.cutc_int(nxBlocks, nyBlocks, nzBlocks, blockxSize, blockySize, blockzSize,
                      n_grid1, n_grid2, n_ao, n_nuc, size_bh, *[_vp(a) for a in arrs])


def options(precision=PLAIN_FP64, n_slices=None, a_en=1.0, a_ee=1.0, x_components=3,
            device_pointers=False, max_work_bytes=0, stream=None, pair_fp64=False,
            k_split=0, int2e_layout=INT2E_PQST, basis=None, r1_window=None) -> Options:
    o = Options()
    load().cutc_default_options(ctypes.byref(o))
    o.precision = precision
    if n_slices is not None:
        o.n_slices = n_slices
    o.a_en, o.a_ee = a_en, a_ee
    o.x_components = x_components
    o.device_pointers = 1 if device_pointers else 0
    o.max_work_bytes = max_work_bytes
    o.stream = stream
    o.pair_fp64 = 1 if pair_fp64 else 0
    o.k_split = k_split
    o.int2e_layout = int2e_layout
    if basis is not None:
        o.basis = ctypes.addressof(basis)
        o._basis = basis  # keeps the basis alive with the options
    if r1_window is not None:
        o.r1_begin, o.r1_end = int(r1_window[0]), int(r1_window[1])
    return o


def cutc_int_ex(opt: Options, n_grid1, n_grid2, n_ao, n_nuc, size_bh,
                r1, wr1, r2, wr2, rn, aos_data1, aos_data2, c_bh, m_bh, n_bh, o_bh,
                X, I, stats: Stats | None = None) -> int:
    L = load()
    arrs = [r1, wr1, r2, wr2, rn, aos_data1, aos_data2, c_bh, m_bh, n_bh, o_bh, X, I]
    return L.cutc_int_ex(ctypes.byref(opt), n_grid1, n_grid2, n_ao, n_nuc, size_bh,
                         *[_vp(a) for a in arrs], ctypes.byref(stats) if stats is not None else None)


def build_integrals(p, precision=PLAIN_FP64, n_slices=None, x_components=3,
                    max_work_bytes=0, with_stats=False, pair_fp64=False, k_split=0,
                    int2e_layout=INT2E_PQST, aos_from_basis=False):
    """Host-array convenience call on a synth.Problem: returns (X, int_2e[, stats]).

    X is (x_components, n1, nA^2) == Fortran (nA, nA, n1, comps); int_2e is
    (nA^2, nA^2) == Fortran (nA, nA, nA, nA).
    """
    X = np.empty((x_components, p.n_grid1, p.n_ao ** 2))
    I = np.empty((p.n_ao ** 2, p.n_ao ** 2))
    st = Stats()
    basis = make_basis(p.shells) if aos_from_basis else None
    opt = options(precision, n_slices, p.a_en, p.a_ee, x_components, False, max_work_bytes,
                  None, pair_fp64, k_split, int2e_layout, basis)
    aos1, aos2 = (None, None) if aos_from_basis else (p.aos1, p.aos2)
    s = cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                    p.r1, p.wr1, p.r2, p.wr2, p.rn, aos1, aos2,
                    p.c_bh, p.m_bh, p.n_bh, p.o_bh, X, I, st)
    if s != CUTC_OK:
        raise CutcError(s, last_error())
    return (X, I, st.as_dict()) if with_stats else (X, I)


def build_integrals_device(p, precision=PLAIN_FP64, n_slices=None, x_components=3,
                           out=None, with_stats=False):
    """Device-resident build on a synth.Problem: the molecule arrays are copied to
    the current CUDA device (torch tensors) and X, int_2e stay there, for outputs
    too large for the host.  out=(X, I) reuses float64 device tensors of shapes
    (x_components, n1, nA^2) and (nA^2, nA^2).  Returns (X, I[, stats])."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in p.arrays().items()}
    nA2 = p.n_ao ** 2
    if out is None:
        X = torch.empty((x_components, p.n_grid1, nA2), dtype=torch.float64, device=dev)
        I = torch.empty((nA2, nA2), dtype=torch.float64, device=dev)
    else:
        X, I = out
    st = Stats()
    opt = options(precision, n_slices, p.a_en, p.a_ee, x_components, True, 0,
                  torch.cuda.current_stream(dev).cuda_stream)
    s = cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                    d["r1"], d["wr1"], d["r2"], d["wr2"], d["rn"], d["aos1"], d["aos2"],
                    d["c_bh"], d["m_bh"], d["n_bh"], d["o_bh"], X, I, st)
    torch.cuda.synchronize(dev)
    if s != CUTC_OK:
        raise CutcError(s, last_error())
    return (X, I, st.as_dict()) if with_stats else (X, I)


def scan_integrals(p, c_sets, a_en=None, a_ee=None, precision=PLAIN_FP64, n_slices=None,
                   x_components=3, with_stats=False, out=None, basis=None):
    """Jastrow-parameter scan on one molecule (cutc_int_scan).

    c_sets: (n_sets, n_nuc, size_bh) coefficients (the exponents of p are used for
    every set); a_en / a_ee: per-set scale factors or None.  Returns
    X (n_sets, x_components, n1, nA^2) and int_2e (n_sets, nA^2, nA^2); out=(X, I)
    gives C-contiguous float64 arrays of those shapes (pinned memory is copied
    into directly) to fill instead of new ones; basis (make_basis) replaces the AO
    arrays, which are then evaluated on the GPU once for all sets.
    """
    c_sets = np.ascontiguousarray(c_sets, dtype=np.float64)
    ns = c_sets.shape[0]
    rep = lambda a: np.ascontiguousarray(np.broadcast_to(a, (ns,) + a.shape))
    m, n, o = rep(p.m_bh), rep(p.n_bh), rep(p.o_bh)
    ae = None if a_en is None else np.ascontiguousarray(a_en, dtype=np.float64)
    aee = None if a_ee is None else np.ascontiguousarray(a_ee, dtype=np.float64)
    if out is None:
        X = np.empty((ns, x_components, p.n_grid1, p.n_ao ** 2))
        I = np.empty((ns, p.n_ao ** 2, p.n_ao ** 2))
    else:
        X, I = out
        assert X.shape == (ns, x_components, p.n_grid1, p.n_ao ** 2) and X.dtype == np.float64
        assert I.shape == (ns, p.n_ao ** 2, p.n_ao ** 2) and I.dtype == np.float64
        assert X.flags.c_contiguous and I.flags.c_contiguous
    opt = options(precision, n_slices, p.a_en, p.a_ee, x_components, basis=basis)
    st = Stats()
    aos1, aos2 = (None, None) if basis is not None else (p.aos1, p.aos2)
    arrs = [p.r1, p.wr1, p.r2, p.wr2, p.rn, aos1, aos2, c_sets, m, n, o]
    s = load().cutc_int_scan(ctypes.byref(opt), ns, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc,
                             p.size_bh, *[_vp(a) for a in arrs],
                             _vp(ae) if ae is not None else None,
                             _vp(aee) if aee is not None else None, _vp(X), _vp(I),
                             ctypes.byref(st))
    if s != CUTC_OK:
        raise CutcError(s, last_error())
    return (X, I, st.as_dict()) if with_stats else (X, I)


class PinnedArray:
    """A host float64/uint8 numpy buffer page-locked with cutc_pin_host until close()."""

    def __init__(self, nbytes):
        self.array = np.empty(nbytes, dtype=np.uint8)
        s = load().cutc_pin_host(_vp(self.array), nbytes)
        if s != CUTC_OK:
            raise CutcError(s, last_error())
        self.nbytes = nbytes

    def close(self):
        if self.array is not None:
            load().cutc_unpin_host(_vp(self.array))
            self.array = None


def plan(n_grid1, n_grid2, n_ao, n_nuc, precision=PLAIN_FP64, n_slices=None, x_components=3,
         device_pointers=False, max_work_bytes=0, k_split=0) -> dict:
    """The device-memory plan of a build (cutc_plan): tiles, blocks, bytes and the
    tensor-core launches per X contraction."""
    opt = options(precision, n_slices, 1.0, 1.0, x_components, device_pointers, max_work_bytes,
                  k_split=k_split)
    info = PlanInfo()
    s = load().cutc_plan(ctypes.byref(opt), n_grid1, n_grid2, n_ao, n_nuc, ctypes.byref(info))
    if s != CUTC_OK:
        raise CutcError(s, last_error())
    return info.as_dict()


def eval_aos(shells, r, components=4):
    """AO values (components=1) or values and gradients (4) of synth shells at the
    points r (n, 3), on the GPU: C array (components, n_ao, n)."""
    b = make_basis(shells)
    r = np.ascontiguousarray(r, dtype=np.float64)
    out = np.empty((components, b.n_ao, r.shape[0]))
    s = load().cutc_eval_aos(ctypes.byref(b), r.shape[0], _vp(r), components, _vp(out), 0, None)
    if s != CUTC_OK:
        raise CutcError(s, last_error())
    return out


def x_ao_to_mo(X_ao, mo_l, mo_r):
    """X in the MO basis in cutc_no's order: X_ao is the C array (comps, n1, nA, nA)
    that build_integrals returns, mo_l and mo_r the C arrays (n_mo, nA) (Fortran
    (nA, n_mo) coefficients).  Returns the C array (n_mo, n_mo, comps, n1), i.e.
    Fortran x_mo(n1, comps, n_mo, n_mo); works on host arrays or CUDA tensors."""
    comps, n1 = X_ao.shape[0], X_ao.shape[1]
    nA = mo_l.shape[1]  # X_ao may also be (comps, n1, nA^2), as build_integrals returns it
    if X_ao.shape[2:] not in ((nA, nA), (nA * nA,)):
        raise ValueError("X_ao does not match the coefficients' n_ao")
    n_mo = mo_l.shape[0]
    dev = hasattr(X_ao, "data_ptr")
    if dev:
        import torch
        out = torch.empty((n_mo, n_mo, comps, n1), dtype=torch.float64, device=X_ao.device)
    else:
        X_ao, mo_l, mo_r = (np.ascontiguousarray(a, dtype=np.float64) for a in (X_ao, mo_l, mo_r))
        out = np.empty((n_mo, n_mo, comps, n1))
    s = load().cutc_x_ao_to_mo(n1, nA, n_mo, comps, _vp(mo_l), _vp(mo_r), _vp(X_ao), _vp(out),
                               1 if dev else 0, None)
    if s != CUTC_OK:
        raise CutcError(s, last_error())
    return out


def jast_bh_device(r1, r2, rn, c_bh, m_bh, n_bh, o_bh, G, i0=0, n1b=None,
                   a_en=1.0, a_ee=1.0) -> int:
    """Pair terms on device tensors (torch, float64/int32, contiguous)."""
    n1 = r1.shape[0]
    n1b = n1 - i0 if n1b is None else n1b
    L = load()
    return L.cutc_jast_bh_dev(i0, n1b, n1, r2.shape[0], rn.shape[0], c_bh.shape[1],
                              _vp(r1), _vp(r2), _vp(rn), _vp(c_bh), _vp(m_bh), _vp(n_bh),
                              _vp(o_bh), a_en, a_ee, _vp(G))


def jast_bh_device_noalloc(r1, r2, rn, c_bh, m_bh, n_bh, o_bh, G, i0=0, n1b=None,
                           a_en=1.0, a_ee=1.0, stream=None) -> int:
    """Pair terms on device tensors through the allocation-free entry point.

    Same results as jast_bh_device; its scratch is a fixed 32 MiB device array
    inside the library, so the call allocates nothing.  Calls that overlap on
    the GPU share that array and race.
    """
    n1 = r1.shape[0]
    n1b = n1 - i0 if n1b is None else n1b
    L = load()
    return L.cutc_jast_bh_dev_noalloc(i0, n1b, n1, r2.shape[0], rn.shape[0], c_bh.shape[1],
                                      _vp(r1), _vp(r2), _vp(rn), _vp(c_bh), _vp(m_bh), _vp(n_bh),
                                      _vp(o_bh), a_en, a_ee, _vp(G), stream)


def no_2e(tmpC1, x_mo, tmpC2, tmpD2, n_mo, n_grid1, precision=PLAIN_FP64, n_slices=None,
          out=None):
    """The two-electron contraction of cutc_no on its intermediates (cutc_no_2e): numpy
    arrays (host) or torch tensors (device), FP64, in the reference's layouts; returns
    no_2e (n_mo^4, as an (n_mo^2, n_mo^2) array of Fortran order)."""
    dev = hasattr(tmpC1, "data_ptr")
    if out is None:
        if dev:
            import torch
            out = torch.empty((n_mo * n_mo, n_mo * n_mo), dtype=torch.float64,
                              device=tmpC1.device)
        else:
            out = np.empty((n_mo * n_mo, n_mo * n_mo))
    opt = options(precision, n_slices, device_pointers=dev)
    s = load().cutc_no_2e(ctypes.byref(opt), n_mo, n_grid1, _vp(tmpC1), _vp(x_mo), _vp(tmpC2),
                          _vp(tmpD2), _vp(out))
    if s != CUTC_OK:
        raise CutcError(s, last_error())
    return out


def fp64_gemm_device(a_kmajor, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, stride_a=0,
                     stride_b=0, stride_c=0, batch=1):
    """The plain form's FP64 DMMA GEMM on device tensors, with cuBLAS's
    column-major argument meaning (cutc_fp64_gemm_dev); raises on a status."""
    s = load().cutc_fp64_gemm_dev(int(bool(a_kmajor)), M, N, K, alpha, _vp(A), lda, stride_a,
                                  _vp(B), ldb, stride_b, beta, _vp(C), ldc, stride_c, batch)
    if s != CUTC_OK:
        raise CutcError(s, last_error())
    return C


def split_gemm_device(A, B, C=None, n_slices=5):
    """C = A @ B.T through the split form, on device tensors (float64, row-major)."""
    import torch
    M, K = A.shape
    N = B.shape[0]
    if C is None:
        C = torch.empty((N, M), dtype=torch.float64, device=A.device)  # column-major M x N
    s = load().cutc_split_gemm_dev(n_slices, M, N, K, _vp(A), _vp(B), _vp(C), M)
    if s != CUTC_OK:
        raise CutcError(s, last_error())
    return C.T


class Server:
    """Continuous-batching integral-build server on the current GPU (C-ABI cutc_server_*).

    submit() takes a synth.Problem (host arrays), returns a ticket immediately and
    keeps the arrays alive until wait(ticket) returns (X, int_2e, latency_ms).
    """

    def __init__(self, n_slots=4, device_budget_bytes=0, cache_budget_bytes=0,
                 tile_budget_bytes=0):
        L = load()
        cfg = ServerConfig()
        L.cutc_server_default_config(ctypes.byref(cfg))
        cfg.n_slots = n_slots
        cfg.device_budget_bytes = device_budget_bytes
        cfg.cache_budget_bytes = cache_budget_bytes
        if tile_budget_bytes:
            cfg.tile_budget_bytes = tile_budget_bytes
        self._h = ctypes.c_void_p()
        s = L.cutc_server_create(ctypes.byref(cfg), ctypes.byref(self._h))
        if s != CUTC_OK:
            raise CutcError(s, last_error())
        self._live = {}

    def submit(self, p, molecule_key=0, precision=PLAIN_FP64, n_slices=None, x_components=3,
               aos_from_basis=False, out=None):
        """aos_from_basis: send p.shells instead of the AO arrays (evaluated on the GPU).
        out=(X, I): C-contiguous float64 arrays of shapes (x_components, n1, nA^2) and
        (nA^2, nA^2) to fill (pinned memory is copied into directly)."""
        if out is None:
            X = np.empty((x_components, p.n_grid1, p.n_ao ** 2))
            I = np.empty((p.n_ao ** 2, p.n_ao ** 2))
        else:
            X, I = out
            assert X.shape == (x_components, p.n_grid1, p.n_ao ** 2) and X.dtype == np.float64
            assert I.shape == (p.n_ao ** 2, p.n_ao ** 2) and I.dtype == np.float64
            assert X.flags.c_contiguous and I.flags.c_contiguous
        arrs = dict(p.arrays())
        basis = make_basis(p.shells) if aos_from_basis else None
        if aos_from_basis:
            arrs["aos1"] = arrs["aos2"] = None
        q = Request()
        q.molecule_key = molecule_key
        q.n_grid1, q.n_grid2, q.n_ao, q.n_nuc, q.size_bh = (p.n_grid1, p.n_grid2, p.n_ao,
                                                           p.n_nuc, p.size_bh)
        for k, name in (("r1", "r1"), ("wr1", "wr1"), ("r2", "r2"), ("wr2", "wr2"), ("rn", "rn"),
                        ("aos1", "aos_data1"), ("aos2", "aos_data2"), ("c_bh", "c_bh"),
                        ("m_bh", "m_bh"), ("n_bh", "n_bh"), ("o_bh", "o_bh")):
            setattr(q, name, arrs[k].ctypes.data if arrs[k] is not None else None)
        q.int2_grad1_u12_ao = X.ctypes.data
        q.int_2e_ao = I.ctypes.data
        q.options = options(precision, n_slices, p.a_en, p.a_ee, x_components, basis=basis)
        t = ctypes.c_ulonglong()
        s = load().cutc_server_submit(self._h, ctypes.byref(q), ctypes.byref(t))
        if s != CUTC_OK:
            raise CutcError(s, last_error())
        self._live[t.value] = (p, X, I, q, basis)
        return t.value

    def wait(self, ticket):
        lat = ctypes.c_double()
        s = load().cutc_server_wait(self._h, ticket, ctypes.byref(lat))
        p, X, I, q, _ = self._live.pop(ticket)
        if s != CUTC_OK:
            raise CutcError(s, last_error())
        return X, I, lat.value

    def stats(self):
        st = ServerStats()
        load().cutc_server_get_stats(self._h, ctypes.byref(st))
        return st.as_dict()

    def close(self):
        if self._h:
            load().cutc_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
