"""Throughput of the cutc_int hot path on GB300: TC-integral builds per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config medium] [--precision split|plain]

One step is one full integral build (pair terms, X, int_2e) of the named
workload.  ``value`` is builds/s with inputs and outputs resident in HBM
(device pointers through cutc_int_ex); ``e2e`` is the same metric through the
C-ABI with host buffers, host<->device copies inside the timed region.
``--impl reference`` times the CPU restatement of the reference's formulas
(oracle/, OpenMP C + numpy/OpenBLAS DGEMM) on the host cores: the reference
ships no CPU path, so its arithmetic is transcribed and timed on a bounded
sample of r1 rows, scaled to a full build.

Under torchrun (N > 1) every rank runs an independent replica of the workload
(the path is single-GPU; there is no collective on the data path) and the
reported value is the sum over ranks: weak scaling.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from cutc_gb300 import synth  # noqa: E402

METRIC = "TC integral builds/s (split-precision vs FP64 at 1e-10 rel err)"
UNIT = "builds/s"
CPU_SAMPLE_ROWS = 256       # per step of --impl reference: about 6 s of oracle work on 16 cores
CPU_BASELINE_ROWS = 384     # the cpu_baseline leg: about 10 s; smaller samples underrate the
                            # CPU (48 rows gave 0.00096 builds/s, 256 rows 0.00168)


def log(msg):
    print("[bench %.1fs] %s" % (time.perf_counter() - _T0, msg), file=sys.stderr, flush=True)


_T0 = time.perf_counter()


def max_over_ranks(x, dist, device):
    """The largest of every rank's x (the timing rule: the slowest rank sets the
    time); x itself without a process group."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, steps, seconds):
    """Builds per second of the whole job: every rank ran `steps` builds and the
    slowest one took `seconds`."""
    return world * steps / seconds


def workload_desc(name, p):
    return ("%s: %d nuclei, n_ao=%d, n_grid1=%d, n_grid2=%d, %d Jastrow terms/atom"
            % (name, p.n_nuc, p.n_ao, p.n_grid1, p.n_grid2, p.size_bh))


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def sub_problem(p, i0, n):
    """The same molecule with r1 restricted to rows [i0, i0+n)."""
    import dataclasses
    return dataclasses.replace(
        p, r1=np.ascontiguousarray(p.r1[i0:i0 + n]), wr1=np.ascontiguousarray(p.wr1[i0:i0 + n]),
        aos1=np.ascontiguousarray(p.aos1[:, :, i0:i0 + n]))

def plain_rate_estimate(cg, p, sizes):
    """Plain FP64 builds/s of the full grid from device-timed builds on two r1
    samples: T(n) = a + b n fitted through both, evaluated at n_grid1."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    nA2 = p.n_ao ** 2
    stream = torch.cuda.Stream(device=dev)
    opt = cg.options(cg.PLAIN_FP64, None, p.a_en, p.a_ee, 3, True, 0, stream.cuda_stream)
    Id = torch.empty((nA2, nA2), dtype=torch.float64, device=dev)
    times = []
    for k, ns in enumerate(sizes):
        sub = strided_rows(p, ns)
        dr = {key: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for key, v in sub.arrays().items()}
        Xd = torch.empty((3, ns, nA2), dtype=torch.float64, device=dev)
        reps = 2 if k == 0 else 1  # the first build also sets up the workspace
        for r in range(reps):
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s = cg.cutc_int_ex(opt, ns, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                               dr["r1"], dr["wr1"], dr["r2"], dr["wr2"], dr["rn"], dr["aos1"],
                               dr["aos2"], dr["c_bh"], dr["m_bh"], dr["n_bh"], dr["o_bh"], Xd, Id, None)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            if s != cg.CUTC_OK:
                raise cg.CutcError(s, cg.last_error())
        times.append(e0.elapsed_time(e1))
        del dr, Xd
    (n_a, n_b), (t_a, t_b) = sizes, times
    slope = (t_b - t_a) / (n_b - n_a)
    t_full = t_b + slope * (p.n_grid1 - n_b)
    del Id
    torch.cuda.empty_cache()
    cg.load().cutc_release()
    return {"value_est": 1e3 / t_full, "unit": UNIT, "ms_per_build_est": t_full,
            "basis": "plain FP64 form, device-resident, timed on %d and %d r1 rows (%.0f and %.0f ms) "
                     "and extrapolated linearly to n_grid1=%d" % (n_a, n_b, t_a, t_b, p.n_grid1)}


def strided_rows(p, ns):
    """The same molecule with ns r1 points spread evenly over the whole r1 grid
    (every nucleus' shells are represented)."""
    import dataclasses
    idx = np.unique(np.linspace(0, p.n_grid1 - 1, ns).round().astype(np.int64))
    assert len(idx) == ns
    return dataclasses.replace(
        p, r1=np.ascontiguousarray(p.r1[idx]), wr1=np.ascontiguousarray(p.wr1[idx]),
        aos1=np.ascontiguousarray(p.aos1[:, :, idx]))


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id=None):
        self.lines = []
        self.proc = None
        self.gpu_id = gpu_id

    def start(self):
        cmd = ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
               "-lms", "200"]
        if self.gpu_id:
            cmd += ["-i", self.gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU oracle leg (bounded sample)
# ---------------------------------------------------------------------------
def cpu_sample(p, rows=CPU_SAMPLE_ROWS, reps=1, offsets=(0,)):
    """Time the oracle on `rows` r1 rows (pair terms, X, their int_2e share)
    plus the r2-side products once; scale to the full build."""
    from oracle import oracle
    t0 = time.perf_counter()
    P = oracle.long_range(p)
    t_p = time.perf_counter() - t0
    times = []
    for rep in range(reps):
        i0 = offsets[rep % len(offsets)]
        sub = sub_problem(p, i0, rows)
        t0 = time.perf_counter()
        X = oracle.x_block(sub, P, 0, rows)
        oracle.int2e_from_x(sub, X)
        times.append(time.perf_counter() - t0)
    t_rows = float(np.mean(times))
    t_build = t_p + t_rows * p.n_grid1 / rows
    return {
        "value": 1.0 / t_build,
        "unit": UNIT,
        "cores": os.cpu_count(),
        "kind": "port",
        "sample": ("%d of %d r1 rows (pair terms, X rows and their int_2e share, "
                   "%d rep(s)) + the r2 pair products once; scaled by n_grid1/%d"
                   % (rows, p.n_grid1, reps, rows)),
        "seconds_timed": t_p + sum(times),
    }, t_rows, t_p


def run_reference(args):
    """--impl reference: the CPU restatement of the reference path, rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    p = synth.make_config(args.config)
    from oracle import oracle
    oracle.build()
    t0 = time.perf_counter()
    P = oracle.long_range(p)
    t_p = time.perf_counter() - t0
    rows = CPU_SAMPLE_ROWS
    step_times = []
    for step in range(args.warmup + args.steps):
        i0 = (step * 997 * rows) % max(1, p.n_grid1 - rows)
        sub = sub_problem(p, i0, rows)
        t0 = time.perf_counter()
        X = oracle.x_block(sub, P, 0, rows)
        oracle.int2e_from_x(sub, X)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            step_times.append(dt)
    t_rows = float(np.mean(step_times))
    t_build = t_p + t_rows * p.n_grid1 / rows
    value = 1.0 / t_build
    cb = {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
          "sample": ("each step: %d of %d r1 rows (pair terms, X rows, their int_2e share); "
                     "r2 pair products timed once; scaled by n_grid1/%d"
                     % (rows, p.n_grid1, rows))}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_build * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_desc(args.config, p), "precision": "fp64 (CPU)"},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    import cutc_gb300 as cg

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    prec = cg.SPLIT_BF16 if args.precision == "split" else cg.PLAIN_FP64
    p = synth.make_config(args.config)

    # ---- device-resident arrays ------------------------------------------------
    def d(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    dr = {k: d(v) for k, v in p.arrays().items()}
    nA2 = p.n_ao ** 2
    Xd = torch.empty((3, p.n_grid1, nA2), dtype=torch.float64, device=dev)
    Id = torch.empty((nA2, nA2), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    opt = cg.options(prec, args.slices, p.a_en, p.a_ee, 3, True, 0, stream.cuda_stream,
                     k_split=args.k_split)

    def build_device(stats=None):
        s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                           dr["r1"], dr["wr1"], dr["r2"], dr["wr2"], dr["rn"], dr["aos1"], dr["aos2"],
                           dr["c_bh"], dr["m_bh"], dr["n_bh"], dr["o_bh"], Xd, Id, stats)
        if s != cg.CUTC_OK:
            raise cg.CutcError(s, cg.last_error())

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    log("inputs on device; warm-up")
    for _ in range(args.warmup):
        build_device()
    log("timed region")
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        uuid = None
    sampler = ClockSampler(uuid)
    sampler.start()
    time.sleep(0.5)
    barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    gemm_ms, gemm_launches, launches, pair_ms = 0.0, 0, 0, 0.0
    for _ in range(args.steps):
        st = cg.Stats()
        build_device(st)
        gemm_ms += st.ms_x_gemm
        gemm_launches += st.n_x_gemm
        launches += st.gpu_launches
        pair_ms += st.ms_pair
    ev1.record(stream)
    barrier()
    clocks = sampler.stop()
    elapsed_ms = max_over_ranks(ev0.elapsed_time(ev1), dist, dev)
    ms_per_step = elapsed_ms / args.steps
    value = whole_job_rate(world, args.steps, elapsed_ms / 1e3)

    # ---- end to end through the C-ABI with host buffers -------------------------
    def pinned(a):
        t_ = torch.empty(a.shape, dtype=torch.from_numpy(np.empty(0, a.dtype)).dtype, pin_memory=True)
        t_.numpy()[...] = a
        return t_.numpy()

    log("device-resident: %.3f builds/s; end-to-end leg" % value)
    hp = {k: pinned(v) for k, v in p.arrays().items()}
    Xh = torch.empty((3, p.n_grid1, nA2), dtype=torch.float64, pin_memory=True).numpy()
    Ih = torch.empty((nA2, nA2), dtype=torch.float64, pin_memory=True).numpy()
    opt_h = cg.options(prec, args.slices, p.a_en, p.a_ee, 3, False, 0, stream.cuda_stream,
                       k_split=args.k_split)

    def build_host(stats=None):
        s = cg.cutc_int_ex(opt_h, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                           hp["r1"], hp["wr1"], hp["r2"], hp["wr2"], hp["rn"], hp["aos1"], hp["aos2"],
                           hp["c_bh"], hp["m_bh"], hp["n_bh"], hp["o_bh"], Xh, Ih, stats)
        if s != cg.CUTC_OK:
            raise cg.CutcError(s, cg.last_error())

    build_host()
    barrier()
    e2e_steps = max(1, min(args.steps, 3))
    e2e_phases = {}
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        st = cg.Stats()
        build_host(st)
        for k, v in st.as_dict().items():
            e2e_phases[k] = e2e_phases.get(k, 0) + v / e2e_steps
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, dev)
    e2e_value = whole_job_rate(world, e2e_steps, e2e_s)
    h2d = (p.r1.nbytes + p.wr1.nbytes + p.r2.nbytes + p.wr2.nbytes + p.rn.nbytes + p.aos1.nbytes
           + p.aos2.nbytes // 4 + p.c_bh.nbytes + 3 * p.m_bh.nbytes)
    d2h = Xh.nbytes + Ih.nbytes

    # ---- the unmodified drop-in call: cutc_int, pageable arrays, form from the env --------
    drop_in = None
    if p.a_en == 1.0 and p.a_ee == 1.0:  # cutc_int fixes them, like the reference
        prev = os.environ.get("CUTC_PRECISION")
        os.environ["CUTC_PRECISION"] = "split" if prec == cg.SPLIT_BF16 else "plain"
        ha = {k: np.ascontiguousarray(v) for k, v in p.arrays().items()}
        Xp = np.empty((3, p.n_grid1, nA2))
        Ip = np.empty((nA2, nA2))

        def build_drop_in():
            s = cg.cutc_int(100, 32, 1, 32, 1, 1, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc,
                            p.size_bh, ha["r1"], ha["wr1"], ha["r2"], ha["wr2"], ha["rn"],
                            ha["aos1"], ha["aos2"], ha["c_bh"], ha["m_bh"], ha["n_bh"], ha["o_bh"],
                            Xp, Ip)
            if s != cg.CUTC_OK:
                raise cg.CutcError(s, cg.last_error())

        build_drop_in()  # also the first touch of the pageable outputs
        barrier()
        t0 = time.perf_counter()
        drop_steps = 2
        for _ in range(drop_steps):
            build_drop_in()
        barrier()
        drop_s = max_over_ranks(time.perf_counter() - t0, dist, dev)
        drop_in = {"value": whole_job_rate(world, drop_steps, drop_s), "unit": UNIT,
                   "steps": drop_steps,
                   "entry": "cutc_int with its launch integers, pageable numpy arrays in and "
                            "out, CUTC_PRECISION=%s" % os.environ["CUTC_PRECISION"]}
        if prev is None:
            del os.environ["CUTC_PRECISION"]
        else:
            os.environ["CUTC_PRECISION"] = prev
        log("drop-in cutc_int, pageable arrays: %.3f builds/s" % drop_in["value"])

    out = None
    if rank == 0:
        peaks, peak_kind = measured_peaks()
        alg_flops_x = 8.0 * nA2 * p.n_grid1 * p.n_grid2  # per build, dense formula
        per_launch_flops = alg_flops_x * args.steps / max(1, gemm_launches)
        per_launch_ms = gemm_ms / max(1, gemm_launches)
        achieved = per_launch_flops / (per_launch_ms * 1e-3) / 1e12
        peak = float(peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops")))
        S = args.slices
        n_products = S * (S + 1) // 2 if prec == cg.SPLIT_BF16 else 0
        packed = p.n_ao * (p.n_ao + 1) / 2.0 / nA2
        executed = achieved * packed * n_products if n_products else None
        roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak, "traffic": traffic_per_launch(args, p, gemm_launches),
                    "kernel": "split_gemm_kernel (X build, one launch per r1 tile)",
                    "peak_source": "bf16_tflops_sustained of %s" % peak_kind,
                    "alg_flops_per_launch": per_launch_flops, "ms_per_launch": per_launch_ms,
                    "executed_bf16_tflops": executed,
                    "executed_frac": (executed / peak) if executed else None,
                    "note": ("achieved counts the dense FP64 formula 8 nA^2 n1 n2; the kernel "
                             "executes %d BF16 slice products on the packed (a>=b) AO pairs"
                             % n_products)}
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "bf16" if prec == cg.SPLIT_BF16 else "f64", "data": "synthetic",
               "config": {"workload": workload_desc(args.config, p),
                          "precision": args.precision, "n_slices": S if prec else None,
                          "k_split": args.k_split,
                          "l2": "inputs larger than L2: per-build working set of tens of GB",
                          "parallelism": "replicas" if world > 1 else "1 GPU"},
               "gpu_launches": launches,
               "clocks": clocks,
               "roofline": roofline,
               "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                       "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                       "buffers": "pinned host memory through cutc_int_ex",
                       "phases_ms_per_step": e2e_phases},
               "e2e_drop_in": drop_in,
               "phases_ms_per_step": {"pair": pair_ms / args.steps,
                                      "x_gemm": gemm_ms / args.steps}}
    # ---- accuracy and the plain FP64 rate on an r1 sample --------------------------
    log("e2e: %.3f builds/s" % e2e_value)
    if rank == 0 and not args.skip_accuracy:
        log("accuracy / plain sample")
        rows = 256
        sub = sub_problem(p, (p.n_grid1 // 2) // 64 * 64, rows)
        Xs, Is = cg.build_integrals(sub, cg.SPLIT_BF16, n_slices=args.slices)
        Xp, Ip = cg.build_integrals(sub, cg.PLAIN_FP64)
        from oracle.oracle import rel_err
        out["accuracy"] = {"X_vs_fp64": rel_err(Xs, Xp), "int2e_vs_fp64": rel_err(Is, Ip),
                           "sample": "%d of %d r1 rows of the workload; split (%d slices) vs "
                                     "the plain FP64 form (itself 1e-12 from the oracle)"
                                     % (rows, p.n_grid1, args.slices)}
        out["plain_fp64"] = plain_rate_estimate(cg, p, (rows, 2 * rows))
    if rank == 0 and world == 1 and not args.skip_cpu:
        log("cpu baseline sample")
        cb, _, _ = cpu_sample(p, rows=min(CPU_BASELINE_ROWS, p.n_grid1))
        out["cpu_baseline"] = cb
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# the large workload: r1 samples of the full molecule and grids
# ---------------------------------------------------------------------------
def run_large(args):
    """Large workload (n_ao=300, n_grid2=200,000) timed on two r1 samples spread
    over the 60,000-point r1 grid and extrapolated linearly in n_grid1.

    A full build's outputs (X: 130 GB, int_2e: 65 GB) do not fit the GPU host's
    memory beside each other, so the full grid is not built in one call; the
    device-resident cost of a build is exactly linear in the r1 rows it holds
    (every r1 tile does the same work), plus a fixed part (P slices, int_2e
    assembly), which the two samples separate.
    """
    import torch
    import cutc_gb300 as cg

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    prec = cg.SPLIT_BF16 if args.precision == "split" else cg.PLAIN_FP64
    p = synth.make_config(args.config)
    nA2 = p.n_ao ** 2
    sizes = (args.r1_sample // 2, args.r1_sample)
    stream = torch.cuda.Stream(device=dev)
    opt = cg.options(prec, args.slices, p.a_en, p.a_ee, 3, True, 0, stream.cuda_stream,
                     k_split=args.k_split)
    Id = torch.empty((nA2, nA2), dtype=torch.float64, device=dev)
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        pass
    samples = []
    gemm_ms, gemm_launches, launches, pair_ms, flops_x = 0.0, 0, 0, 0.0, 0.0
    sampler = ClockSampler(uuid)
    for ns in sizes:
        sub = strided_rows(p, ns)
        dr = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in sub.arrays().items()}
        Xd = torch.empty((3, ns, nA2), dtype=torch.float64, device=dev)

        def build(stats=None):
            s = cg.cutc_int_ex(opt, ns, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                               dr["r1"], dr["wr1"], dr["r2"], dr["wr2"], dr["rn"], dr["aos1"],
                               dr["aos2"], dr["c_bh"], dr["m_bh"], dr["n_bh"], dr["o_bh"], Xd, Id,
                               stats)
            if s != cg.CUTC_OK:
                raise cg.CutcError(s, cg.last_error())

        log("large: %d r1 rows, warm-up" % ns)
        for _ in range(args.warmup):
            build()
        if ns == sizes[-1]:
            sampler.start()
            time.sleep(0.5)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        tiles = 0
        for _ in range(args.steps):
            st = cg.Stats()
            build(st)
            tiles = st.n_r1_tiles
            if ns == sizes[-1]:
                gemm_ms += st.ms_x_gemm
                gemm_launches += st.n_x_gemm
                launches += st.gpu_launches
                pair_ms += st.ms_pair
                flops_x += 8.0 * nA2 * ns * p.n_grid2
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / args.steps
        samples.append({"r1_rows": ns, "ms_per_build": ms, "r1_tiles": tiles})
        log("large: %d rows: %.1f ms per build" % (ns, ms))
        del dr, Xd
    clocks = sampler.stop()
    del Id
    torch.cuda.empty_cache()
    cg.load().cutc_release()
    (n_a, n_b), (t_a, t_b) = sizes, (samples[0]["ms_per_build"], samples[1]["ms_per_build"])
    slope = (t_b - t_a) / (n_b - n_a)
    t_full = t_b + slope * (p.n_grid1 - n_b)
    value = 1e3 / t_full

    peaks, peak_kind = measured_peaks()
    peak = float(peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops")))
    per_launch_ms = gemm_ms / max(1, gemm_launches)
    achieved = flops_x / max(1, gemm_launches) / (per_launch_ms * 1e-3) / 1e12
    S = args.slices
    n_products = S * (S + 1) // 2 if prec == cg.SPLIT_BF16 else 0
    packed = p.n_ao * (p.n_ao + 1) / 2.0 / nA2
    executed = achieved * packed * n_products if n_products else None
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_full, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": "bf16" if prec == cg.SPLIT_BF16 else "f64", "data": "synthetic",
           "config": {"workload": workload_desc(args.config, p), "precision": args.precision,
                      "n_slices": S if prec else None,
                      "projection": "device-resident builds on %d and %d r1 rows spread over the "
                                    "r1 grid, extrapolated linearly to n_grid1=%d"
                                    % (n_a, n_b, p.n_grid1),
                      "l2": "inputs larger than L2: P slices alone are %.0f GB" %
                            (2 * S * p.n_ao * (p.n_ao + 1) / 2 * p.n_grid2 / 1e9),
                      "parallelism": "1 GPU"},
           "samples": samples, "gpu_launches": launches, "clocks": clocks,
           "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                        "frac": achieved / peak, "traffic": None,
                        "kernel": "split_gemm_kernel (X build, one launch per r1 tile)",
                        "peak_source": "bf16_tflops_sustained of %s" % peak_kind,
                        "ms_per_launch": per_launch_ms, "executed_bf16_tflops": executed,
                        "executed_frac": (executed / peak) if executed else None},
           "phases_ms_per_build_sample": {"pair": pair_ms / args.steps,
                                          "x_gemm": gemm_ms / args.steps},
           "e2e": {"value": None, "unit": UNIT,
                   "reason": "the full build's host outputs (195 GB) exceed the GPU host's memory"}}

    if not args.skip_accuracy:
        rows = 128
        log("large: accuracy on %d rows" % rows)
        sub = strided_rows(p, rows)
        out["accuracy"] = large_accuracy(cg, sub, args.slices)
        out["accuracy"]["sample"] = ("%d of %d r1 rows spread over the grid; split (%d slices) vs "
                                     "the plain FP64 form" % (rows, p.n_grid1, S))
        log("large: plain FP64 rate")
        out["plain_fp64"] = plain_rate_estimate(cg, p, (rows, 2 * rows))
        out["speedup_vs_plain_fp64"] = value / out["plain_fp64"]["value_est"]
    print(json.dumps(out), flush=True)
    return 0


def large_accuracy(cg, sub, n_slices):
    """X and int_2e of the split form against the plain FP64 form on one r1 sample,
    with int_2e compared in row blocks (one copy of it lives on the host)."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    nA2 = sub.n_ao ** 2
    ns = sub.n_grid1
    dr = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in sub.arrays().items()}

    def build(prec, X, I):
        opt = cg.options(prec, n_slices if prec == cg.SPLIT_BF16 else None, sub.a_en, sub.a_ee,
                         3, True, 0, None)
        s = cg.cutc_int_ex(opt, ns, sub.n_grid2, sub.n_ao, sub.n_nuc, sub.size_bh,
                           dr["r1"], dr["wr1"], dr["r2"], dr["wr2"], dr["rn"], dr["aos1"],
                           dr["aos2"], dr["c_bh"], dr["m_bh"], dr["n_bh"], dr["o_bh"], X, I, None)
        torch.cuda.synchronize(dev)
        if s != cg.CUTC_OK:
            raise cg.CutcError(s, cg.last_error())

    X = torch.empty((3, ns, nA2), dtype=torch.float64, device=dev)
    I = torch.empty((nA2, nA2), dtype=torch.float64, device=dev)
    build(cg.SPLIT_BF16, X, I)
    Xs = X.cpu().numpy()
    Is = I.cpu().numpy()
    cg.load().cutc_release()
    build(cg.PLAIN_FP64, X, I)
    from oracle.oracle import rel_err
    ex = rel_err(Xs, X.cpu().numpy())
    d2 = r2 = 0.0
    dmax = rmax = 0.0
    step = max(1, (1 << 30) // (8 * nA2))
    for r0 in range(0, nA2, step):
        ref = I[r0:r0 + step].cpu().numpy()
        d = Is[r0:r0 + step] - ref
        d2 += float(np.sum(d * d))
        r2 += float(np.sum(ref * ref))
        dmax = max(dmax, float(np.max(np.abs(d))))
        rmax = max(rmax, float(np.max(np.abs(ref))))
    del X, I, dr
    torch.cuda.empty_cache()
    cg.load().cutc_release()
    return {"X_vs_fp64": ex, "int2e_vs_fp64": {"norm": (d2 / r2) ** 0.5 if r2 > 0 else d2 ** 0.5,
                                               "max": dmax / rmax if rmax > 0 else dmax}}


def serving_requests(n, max_ao, seed=4004):
    """The serving stream: molecules of 2-20 nuclei, n_ao uniform in [10, max_ao],
    n_grid1 = 1000 n_nuc, n_grid2 = 4000 n_nuc; 30% repeat an earlier molecule with
    Jastrow coefficients perturbed by a 10% Gaussian.  Molecules carry their basis,
    not AO arrays: the server evaluates the AOs on the GPU."""
    import dataclasses
    rng = np.random.default_rng(seed)
    mols, reqs = [], []
    for i in range(n):
        if mols and rng.random() < 0.3:
            k = int(rng.integers(len(mols)))
            p = mols[k]
            p = dataclasses.replace(p, c_bh=np.ascontiguousarray(
                p.c_bh * (1.0 + 0.1 * rng.standard_normal(p.c_bh.shape))))
            reqs.append((k + 1, p))
        else:
            nn = int(rng.integers(2, 21))
            na = int(rng.integers(10, max_ao + 1))
            p = synth.make_problem(n_nuc=nn, n_ao=na, n_grid1=1000 * nn, n_grid2=4000 * nn,
                                   size_bh=9, seed=int(rng.integers(1 << 30)), box=1.5 + 0.4 * nn,
                                   with_aos=False)
            mols.append(p)
            reqs.append((len(mols), p))
    return reqs


def output_bytes(p):
    return 8 * (3 * p.n_grid1 * p.n_ao ** 2 + p.n_ao ** 4)


def run_serving(args):
    """Poisson arrivals into the continuous-batching server; p50/p99 latency and builds/s.

    The host holds at most --host-gb of request outputs at a time (X and int_2e of
    an n_ao = 250 request are 61 GB): past that, the stream waits for the oldest
    request before submitting the next, and the time it waited is reported."""
    import cutc_gb300 as cg
    import torch
    torch.cuda.set_device(0)
    reqs = serving_requests(args.requests, args.max_ao)
    log("serving: %d requests generated" % len(reqs))
    prec = cg.SPLIT_BF16 if args.precision == "split" else cg.PLAIN_FP64
    rng = np.random.default_rng(7)
    gaps = rng.exponential(1.0 / args.rate, size=len(reqs))
    budget = args.host_gb * 1e9
    lat = []
    held = 0.0
    t_blocked = 0.0
    with cg.Server(n_slots=args.slots) as srv:
        t0 = time.perf_counter()
        tickets = []  # (ticket, output bytes)
        t_next = t0
        for (key, p), gap in zip(reqs, gaps):
            t_next += gap
            while time.perf_counter() < t_next:
                time.sleep(min(0.001, max(0.0, t_next - time.perf_counter())))
            need = output_bytes(p)
            tb = time.perf_counter()
            while tickets and held + need > budget:
                t, b = tickets.pop(0)
                lat.append(srv.wait(t)[2])
                held -= b
            t_blocked += time.perf_counter() - tb
            tickets.append((srv.submit(p, key, prec, args.slices, aos_from_basis=True), need))
            held += need
        for t, _ in tickets:
            lat.append(srv.wait(t)[2])
        elapsed = time.perf_counter() - t0
        st = srv.stats()
    flops = sum(p.flops() for _, p in reqs)
    accuracy = None
    if not args.skip_accuracy:
        accuracy = serving_accuracy(cg, reqs, args.slices)
    line = {"metric": "TC integral builds/s and latency, serving stream", "value": len(reqs) / elapsed,
            "unit": "builds/s", "n_gpus": 1, "higher_is_better": True,
            "dtype": "bf16" if prec == cg.SPLIT_BF16 else "f64", "data": "synthetic",
            "config": {"workload": "serving: %d requests, Poisson arrivals at %.1f/s, 2-20 nuclei, "
                                   "n_ao in [10, %d], n_grid1 = 1000 n_nuc, n_grid2 = 4000 n_nuc, "
                                   "30%% repeats with perturbed Jastrow coefficients, AOs evaluated "
                                   "on the GPU from each request's basis"
                                   % (len(reqs), args.rate, args.max_ao),
                       "slots": args.slots, "precision": args.precision,
                       "host_output_budget_gb": args.host_gb},
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "arrivals_held_back_s": t_blocked,
            "server": st, "alg_tflops": flops / elapsed / 1e12, "accuracy": accuracy}
    print(json.dumps(line), flush=True)
    return 0


def serving_accuracy(cg, reqs, n_slices, rows=128, max_ao=200):
    """Split vs plain FP64 for three molecules of the stream (smallest, median and
    largest n_ao up to max_ao, so that int_2e stays a few GB), on `rows` r1 points
    spread over each grid, AOs from the basis as in the stream."""
    import dataclasses
    from oracle.oracle import rel_err
    mols = {}
    for key, p in reqs:
        if p.n_ao <= max_ao and key not in mols:
            mols[key] = p
    ps = sorted(mols.values(), key=lambda q: q.n_ao)
    pick = [ps[0], ps[len(ps) // 2], ps[-1]] if len(ps) >= 3 else ps
    out = []
    for p in pick:
        idx = np.unique(np.linspace(0, p.n_grid1 - 1, min(rows, p.n_grid1)).round().astype(np.int64))
        sub = dataclasses.replace(p, r1=np.ascontiguousarray(p.r1[idx]),
                                  wr1=np.ascontiguousarray(p.wr1[idx]))
        Xs, Is = cg.build_integrals(sub, cg.SPLIT_BF16, n_slices=n_slices, aos_from_basis=True)
        Xp, Ip = cg.build_integrals(sub, cg.PLAIN_FP64, aos_from_basis=True)
        out.append({"n_nuc": p.n_nuc, "n_ao": p.n_ao, "n_grid2": p.n_grid2, "r1_rows": len(idx),
                    "X_vs_fp64": rel_err(Xs, Xp), "int2e_vs_fp64": rel_err(Is, Ip)})
        del Xs, Is, Xp, Ip
    return out


def run_scan(args):
    """Batched Jastrow-parameter scan: one molecule, n_sets parameter sets."""
    import dataclasses
    import cutc_gb300 as cg
    import torch
    from oracle.oracle import rel_err
    torch.cuda.set_device(0)
    p = synth.make_config("scan")
    rng = np.random.default_rng(5050)
    ns = args.sets
    c_sets = rng.normal(0.0, 0.3, size=(ns,) + p.c_bh.shape)
    a_en = rng.uniform(0.5, 2.0, ns)
    a_ee = rng.uniform(0.5, 2.0, ns)
    prec = cg.SPLIT_BF16 if args.precision == "split" else cg.PLAIN_FP64
    batch = min(ns, args.scan_batch)
    # the outputs of one call live in pinned host memory reused by every call, as a
    # scanning caller would keep them
    nA2 = p.n_ao ** 2
    Xo = torch.empty((batch, 3, p.n_grid1, nA2), dtype=torch.float64, pin_memory=True).numpy()
    Io = torch.empty((batch, nA2, nA2), dtype=torch.float64, pin_memory=True).numpy()
    log("scan: warm-up")
    cg.scan_integrals(p, c_sets[:batch], a_en[:batch], a_ee[:batch], prec, args.slices,
                      out=(Xo, Io))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    launches = 0
    for b0 in range(0, ns, batch):
        sl = slice(b0, min(ns, b0 + batch))
        k = sl.stop - sl.start
        X, I, st = cg.scan_integrals(p, c_sets[sl], a_en[sl], a_ee[sl], prec, args.slices,
                                     with_stats=True, out=(Xo[:k], Io[:k]))
        launches += st["gpu_launches"]
    elapsed = time.perf_counter() - t0
    log("scan: %.3f sets/s; accuracy sample" % (ns / elapsed))
    rows = 256
    i0 = (p.n_grid1 // 2) // 64 * 64
    sub = dataclasses.replace(p, r1=np.ascontiguousarray(p.r1[i0:i0 + rows]),
                              wr1=np.ascontiguousarray(p.wr1[i0:i0 + rows]),
                              aos1=np.ascontiguousarray(p.aos1[:, :, i0:i0 + rows]))
    Xs, Is = cg.scan_integrals(sub, c_sets, a_en, a_ee, prec, args.slices)
    Xp, Ip = cg.scan_integrals(sub, c_sets, a_en, a_ee, cg.PLAIN_FP64)
    ex = [rel_err(Xs[k], Xp[k]) for k in range(ns)]
    ei = [rel_err(Is[k], Ip[k]) for k in range(ns)]
    line = {"metric": "TC integral builds/s, Jastrow-parameter scan", "value": ns / elapsed,
            "unit": "builds/s", "n_gpus": 1, "higher_is_better": True,
            "dtype": "bf16" if prec == cg.SPLIT_BF16 else "f64", "data": "synthetic",
            "config": {"workload": "scan: " + workload_desc("scan", p) + ", %d Jastrow parameter "
                                   "sets (c ~ N(0, 0.3), a_en, a_ee ~ U[0.5, 2]), %d sets per "
                                   "cutc_int_scan call, outputs in reused pinned host memory"
                                   % (ns, batch),
                       "precision": args.precision},
            "gpu_launches": launches,
            "alg_tflops": ns * p.flops() / elapsed / 1e12,
            "accuracy": {"X_vs_fp64_max_over_sets": max(e["norm"] for e in ex),
                         "X_vs_fp64_maxabs_max_over_sets": max(e["max"] for e in ex),
                         "int2e_vs_fp64_max_over_sets": max(e["norm"] for e in ei),
                         "int2e_vs_fp64_maxabs_max_over_sets": max(e["max"] for e in ei),
                         "sample": "%d of %d r1 rows, every set; split vs the plain FP64 form"
                                   % (rows, p.n_grid1)}}
    print(json.dumps(line), flush=True)
    return 0


def traffic_per_launch(args, p, launches):
    """DRAM bytes per X-contraction launch from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", "split_gemm_traffic.json")
    if not os.path.exists(path):
        return None
    try:
        with open(path) as f:
            d = json.load(f)
        # bytes per (M x N x K) unit measured on the captured launch, scaled to this launch
        per_unit = float(d["dram_bytes_per_mnk"])
        np_ = p.n_ao * (p.n_ao + 1) // 2
        n_per_launch = 4.0 * p.n_grid1 / max(1, launches / max(1, args.steps))
        return per_unit * np_ * n_per_launch * p.n_grid2
    except Exception:
        return None


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="medium", choices=sorted(synth.CONFIGS))
    ap.add_argument("--precision", choices=["split", "plain"], default="split")
    ap.add_argument("--slices", type=int, default=5)
    ap.add_argument("--k-split", type=int, default=0,
                    help="max K per tensor-core launch (0 = library default)")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-accuracy", action="store_true")
    ap.add_argument("--serving", action="store_true", help="run the serving stream instead")
    ap.add_argument("--requests", type=int, default=256)
    ap.add_argument("--rate", type=float, default=8.0, help="serving arrivals per second")
    ap.add_argument("--max-ao", type=int, default=120)
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--host-gb", type=float, default=48.0,
                    help="serving: host memory for outputs of requests in flight")
    ap.add_argument("--scan", action="store_true", help="run the Jastrow-parameter scan instead")
    ap.add_argument("--sets", type=int, default=64)
    ap.add_argument("--scan-batch", type=int, default=8)
    ap.add_argument("--r1-sample", type=int, default=6000,
                    help="large workload: r1 rows of the bigger of the two timed samples")
    args = ap.parse_args(argv)
    if args.serving:
        return run_serving(args)
    if args.scan:
        return run_scan(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "large":
        return run_large(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
