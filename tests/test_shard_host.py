"""r1 sharding of one build (cutc_gb300/shard.py) on CPU: the windows partition the
r1 grid, and two gloo ranks that each build their window (with the FP64 oracle
standing in for the GPU library) and all-reduce the int_2e shares reproduce the
whole build: every rank holds the whole int_2e and the X rows of its window."""
import json
import os
import socket
import subprocess
import sys

import pytest

from cutc_gb300.shard import shard_window

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("n1,world", [(10, 1), (10, 3), (7, 7), (5, 8), (25000, 6), (1, 2)])
def test_windows_partition_the_grid(n1, world):
    wins = [shard_window(n1, r, world) for r in range(world)]
    assert wins[0][0] == 0 and wins[-1][1] == n1
    for (b0, e0), (b1, e1) in zip(wins, wins[1:]):
        assert e0 == b1  # contiguous, disjoint, in rank order
    sizes = [e - b for b, e in wins]
    assert min(sizes) >= 0 and max(sizes) - min(sizes) <= 1


def test_window_rejects_bad_ranks():
    with pytest.raises(ValueError):
        shard_window(10, 2, 2)


_WORKER = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import torch.distributed as dist
from cutc_gb300 import synth
from cutc_gb300.shard import build_sharded
from oracle import oracle
import bench

def oracle_window(p, b, e):
    X3, A = oracle.cutc_int(bench.sub_problem(p, b, e - b))
    return X3, A

dist.init_process_group("gloo")
p = synth.make_problem(n_nuc=3, n_ao=5, n_grid1=37, n_grid2=90, size_bh=4, seed=55)
(b, e), X, I = build_sharded(p, dist, build=oracle_window)
X3, Iref = oracle.cutc_int(p)
ex = oracle.rel_err(X.numpy(), X3[:, b:e])
ei = oracle.rel_err(I.numpy(), Iref)
print(json.dumps({"rank": dist.get_rank(), "window": [b, e], "x": ex["max"], "i": ei["max"]}))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reproduce_the_whole_build():
    port = _free_port()
    env = {k: v for k, v in os.environ.items()
           if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT")}
    procs = [subprocess.Popen([sys.executable, "-c", _WORKER, ROOT], stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True,
                              env=dict(env, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r),
                                       MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port)))
             for r in range(2)]
    outs = []
    for pr in procs:
        out, err = pr.communicate(timeout=300)
        assert pr.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert sorted(tuple(o["window"]) for o in outs) == [(0, 19), (19, 37)]
    for o in outs:
        assert o["x"] < 1e-14   # the window's X rows are the whole build's rows
        assert o["i"] < 1e-13   # the summed shares are the whole int_2e
