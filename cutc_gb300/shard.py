"""r1 sharding of one integral build over several processes (one GPU each).

X_{mu nu}(r1) is independent for every r1 point, and int_2e is a sum over the
r1 points (src/build_int_2e_ao.cu:60-67,97-104 contract over r1), so a build
splits over ranks by r1 with a single exchange: every rank builds the X rows
of its own contiguous r1 window and that window's share of int_2e
(cutc_options.r1_begin / r1_end), and one all-reduce (sum) of the n_ao^4
int_2e shares gives every rank the whole int_2e.  r2 data are replicated.  X
stays distributed: rank k holds the rows of its window.

The reduction goes through torch.distributed (NCCL between GPUs, gloo on
CPUs).  The per-rank build is this library's cutc_int_ex unless another
callable is given (the CPU tests pass the FP64 oracle).
"""
from __future__ import annotations

import numpy as np


def shard_window(n_grid1: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous, balanced r1 window [begin, end) of `rank` among `world` ranks:
    the windows partition [0, n_grid1) in rank order, sizes differing by at most
    one point (a rank gets an empty window only when world > n_grid1)."""
    if world < 1 or not 0 <= rank < world or n_grid1 < 0:
        raise ValueError("bad shard arguments (n_grid1=%d rank=%d world=%d)" % (n_grid1, rank, world))
    base, extra = divmod(n_grid1, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def library_shard(p, begin, end, precision, n_slices=None, x_components=3):
    """This library's build of r1 window [begin, end) of p on the current GPU,
    inputs and outputs in device memory: (X rows (comps, end - begin, nA^2),
    int_2e share (nA^2, nA^2)) as torch tensors."""
    import torch
    import cutc_gb300 as cg
    dev = torch.device("cuda", torch.cuda.current_device())
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in p.arrays().items()}
    nA2 = p.n_ao ** 2
    X = torch.empty((x_components, end - begin, nA2), dtype=torch.float64, device=dev)
    I = torch.empty((nA2, nA2), dtype=torch.float64, device=dev)
    opt = cg.options(precision, n_slices, p.a_en, p.a_ee, x_components, True, 0,
                     torch.cuda.current_stream(dev).cuda_stream, r1_window=(begin, end))
    s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                       d["r1"], d["wr1"], d["r2"], d["wr2"], d["rn"], d["aos1"], d["aos2"],
                       d["c_bh"], d["m_bh"], d["n_bh"], d["o_bh"], X, I, None)
    torch.cuda.synchronize(dev)
    if s != cg.CUTC_OK:
        raise cg.CutcError(s, cg.last_error())
    return X, I


def build_sharded(p, dist=None, precision=0, n_slices=None, build=None):
    """One build of p spread over the ranks of `dist` (torch.distributed, already
    initialised; None = a single rank).  Returns (window, X rows of this rank's
    window, whole int_2e), the last two as torch tensors on the build's device.
    `build(p, begin, end)` returns (X rows, int_2e share) of a window; default:
    this library on the current GPU."""
    import torch
    rank, world = (dist.get_rank(), dist.get_world_size()) if dist is not None else (0, 1)
    begin, end = shard_window(p.n_grid1, rank, world)
    if build is None:
        build = lambda q, b, e: library_shard(q, b, e, precision, n_slices)  # noqa: E731
    if end > begin:
        X, I = build(p, begin, end)
        X, I = torch.as_tensor(X), torch.as_tensor(I)
    else:  # more ranks than r1 points: an empty window adds nothing
        nA2 = p.n_ao ** 2
        dev = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else "cpu"
        X = torch.empty((3, 0, nA2), dtype=torch.float64, device=dev)
        I = torch.zeros((nA2, nA2), dtype=torch.float64, device=dev)
    if dist is not None and world > 1:
        dist.all_reduce(I, op=dist.ReduceOp.SUM)
    return (begin, end), X, I
