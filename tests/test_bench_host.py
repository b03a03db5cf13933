"""Host side of bench.py, on CPU: the reference arm's contract line, its rank
handling under torchrun, and the max-over-ranks timing with two gloo ranks."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BENCH = os.path.join(ROOT, "bench.py")


def _env(**kw):
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    env.update({k: str(v) for k, v in kw.items()})
    return env


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, BENCH, "--impl", "reference", "--config", "small",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True,
                       env=_env(), timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]


def test_reference_arm_other_ranks_exit_quietly():
    r = subprocess.run([sys.executable, BENCH, "--impl", "reference", "--config", "small",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                       env=_env(RANK=1, WORLD_SIZE=2, LOCAL_RANK=1), timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


_WORKER = r"""
import os, sys, json
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
rank, world = dist.get_rank(), dist.get_world_size()
secs = bench.max_over_ranks(1.5 + rank, dist, "cpu")   # rank 1 is the slow one
print(json.dumps({"rank": rank, "max": secs,
                  "rate": bench.whole_job_rate(world, 4, secs)}))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_two_gloo_ranks():
    port = _free_port()
    procs = [subprocess.Popen([sys.executable, "-c", _WORKER, ROOT], stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True,
                              env=_env(RANK=r, WORLD_SIZE=2, LOCAL_RANK=r,
                                       MASTER_ADDR="127.0.0.1", MASTER_PORT=port))
             for r in range(2)]
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["max"] == 2.5          # every rank sees the slowest rank's time
        assert o["rate"] == 2 * 4 / 2.5  # whole-job builds/s over both ranks
