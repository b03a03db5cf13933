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

On one GPU the line also carries the rest of the metric, each measured in the
same run: the error of both forms against the FP64 oracle (``accuracy``), the
plain FP64 form's rate, the split form at 6 slices (the plain form's error
class, ``split_6_slices``), the large workload as one full build and on r1
samples (``large``), the Jastrow-parameter scan (``scan``), a prefix of the
serving stream with p50/p99 latency (``serving``) and the split contraction
beside cuBLAS's own FP64 emulation on the same operands (``rival``).

Under torchrun (N > 1) every rank runs an independent replica of the workload
(the path is single-GPU; there is no collective on the data path) and the
reported value is the sum over ranks: weak scaling.

Micro-benchmarks of single kernels (the cases the committed ncu summaries were
captured on) and device-resident sample builds: ``--kernel split_gemm|fp64_gemm|pair|plain_build|sample_build|rival``.
"""
from __future__ import annotations

import argparse
import ctypes
import dataclasses
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
FP64_CLASS_SLICES = 6        # the split form's slice count with the plain form's error class
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
    return dataclasses.replace(
        p, r1=np.ascontiguousarray(p.r1[i0:i0 + n]), wr1=np.ascontiguousarray(p.wr1[i0:i0 + n]),
        aos1=np.ascontiguousarray(p.aos1[:, :, i0:i0 + n]))


def release_device():
    import torch
    import cutc_gb300 as cg
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    cg.load().cutc_release()


def cuda_ms(fn, stream=None):
    """Device time of fn() on `stream` (torch's current stream by default)."""
    import torch
    s = stream or torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    fn()
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def fp64_class_leg(cg, p, n_slices, steps=2):
    """The split form at n_slices (6: the plain form's error class) on the full
    workload, device-resident, timed with CUDA events after one warm-up build."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    nA2 = p.n_ao ** 2
    stream = torch.cuda.Stream(device=dev)
    opt = cg.options(cg.SPLIT_BF16, n_slices, p.a_en, p.a_ee, 3, True, 0, stream.cuda_stream)
    dr = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in p.arrays().items()}
    Xd = torch.empty((3, p.n_grid1, nA2), dtype=torch.float64, device=dev)
    Id = torch.empty((nA2, nA2), dtype=torch.float64, device=dev)

    def build():
        s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                           dr["r1"], dr["wr1"], dr["r2"], dr["wr2"], dr["rn"], dr["aos1"],
                           dr["aos2"], dr["c_bh"], dr["m_bh"], dr["n_bh"], dr["o_bh"], Xd, Id, None)
        if s != cg.CUTC_OK:
            raise cg.CutcError(s, cg.last_error())

    build()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        build()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / steps
    del dr, Xd, Id
    release_device()
    return {"value": 1e3 / ms, "unit": UNIT, "ms_per_build": ms, "n_slices": n_slices,
            "steps": steps, "note": "device-resident builds of the full workload in the split "
                                    "form at %d slices; its error against the oracle is the "
                                    "accuracy object's split_%d_slices entry" % (n_slices, n_slices)}


def plain_rate_estimate(cg, p, sizes):
    """Plain FP64 builds/s of the full grid from device-timed builds on two r1
    samples: T(n) = a + b n fitted through both, evaluated at n_grid1."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    nA2 = p.n_ao ** 2
    stream = torch.cuda.Stream(device=dev)
    opt = cg.options(cg.PLAIN_FP64, None, p.a_en, p.a_ee, 3, True, 0, stream.cuda_stream)
    Id = torch.empty((nA2, nA2), dtype=torch.float64, device=dev)
    times, gemm = [], []
    for k, ns in enumerate(sizes):
        sub = synth.r1_sample(p, ns)
        dr = {key: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for key, v in sub.arrays().items()}
        Xd = torch.empty((3, ns, nA2), dtype=torch.float64, device=dev)
        reps = 2 if k == 0 else 1  # the first build also sets up the workspace
        for r in range(reps):
            st = cg.Stats()
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s = cg.cutc_int_ex(opt, ns, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                               dr["r1"], dr["wr1"], dr["r2"], dr["wr2"], dr["rn"], dr["aos1"],
                               dr["aos2"], dr["c_bh"], dr["m_bh"], dr["n_bh"], dr["o_bh"], Xd, Id, st)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            if s != cg.CUTC_OK:
                raise cg.CutcError(s, cg.last_error())
        times.append(e0.elapsed_time(e1))
        np_ = p.n_ao * (p.n_ao + 1) // 2
        gemm.append(2.0 * np_ * 4 * ns * p.n_grid2 / (st.ms_x_gemm * 1e-3) / 1e12)
        del dr, Xd
    (n_a, n_b), (t_a, t_b) = sizes, times
    slope = (t_b - t_a) / (n_b - n_a)
    t_full = t_b + slope * (p.n_grid1 - n_b)
    del Id
    release_device()
    return {"value_est": 1e3 / t_full, "unit": UNIT, "ms_per_build_est": t_full,
            "x_gemm_fp64_tflops": gemm[-1],
            "x_gemm_kernel": "fp64_gemm_kernel (DMMA m8n8k4 tiles, this library)",
            "basis": "plain FP64 form, device-resident, timed on %d and %d r1 rows (%.0f and %.0f ms) "
                     "and extrapolated linearly to n_grid1=%d" % (n_a, n_b, t_a, t_b, p.n_grid1)}


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


def gpu_uuid(dev):
    import torch
    try:
        return "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        return None


# ---------------------------------------------------------------------------
# CPU oracle leg (bounded sample)
# ---------------------------------------------------------------------------
def cpu_sample(p, rows=CPU_SAMPLE_ROWS):
    """Time the oracle on `rows` r1 rows spread over the grid (pair terms, X,
    their int_2e share) plus the r2-side products once; scale to the full build.
    Returns the cpu_baseline record and the oracle's outputs on the sample
    (sub-problem, X (4, rows, nA^2), int_2e (nA^2, nA^2))."""
    from oracle import oracle
    t0 = time.perf_counter()
    P = oracle.long_range(p)
    t_p = time.perf_counter() - t0
    sub = synth.r1_sample(p, rows)
    t0 = time.perf_counter()
    X4 = oracle.x_block(sub, P, 0, rows)
    A = oracle.int2e_from_x(sub, X4)
    t_rows = time.perf_counter() - t0
    del P
    t_build = t_p + t_rows * p.n_grid1 / rows
    cb = {
        "value": 1.0 / t_build,
        "unit": UNIT,
        "cores": os.cpu_count(),
        "kind": "port",
        "sample": ("%d of %d r1 rows spread over the grid (pair terms, X rows and their int_2e "
                   "share) + the r2 pair products once; scaled by n_grid1/%d"
                   % (rows, p.n_grid1, rows)),
        "seconds_timed": t_p + t_rows,
    }
    return cb, sub, X4, A + A.T


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
    rows = min(CPU_SAMPLE_ROWS, p.n_grid1)
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
    sampler = ClockSampler(gpu_uuid(dev))
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
    del hp, Xh, Ih

    # ---- the unmodified drop-in call: cutc_int, pageable arrays, form from the env --------
    drop_in = None
    if p.a_en == 1.0 and p.a_ee == 1.0:  # cutc_int fixes them, like the reference
        prev = os.environ.get("CUTC_PRECISION")
        prev_slices = os.environ.get("CUTC_SLICES")
        os.environ["CUTC_PRECISION"] = "split" if prec == cg.SPLIT_BF16 else "plain"
        os.environ["CUTC_SLICES"] = str(args.slices)
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
                            "out, CUTC_PRECISION=%s, CUTC_SLICES=%s"
                            % (os.environ["CUTC_PRECISION"], os.environ["CUTC_SLICES"])}
        for key, old in (("CUTC_PRECISION", prev), ("CUTC_SLICES", prev_slices)):
            if old is None:
                del os.environ[key]
            else:
                os.environ[key] = old
        del Xp, Ip, ha
        log("drop-in cutc_int, pageable arrays: %.3f builds/s" % drop_in["value"])
    log("e2e: %.3f builds/s" % e2e_value)

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
                    "kernel": "split_gemm_kernel (X build: the K launches of each r1 tile)",
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
    one_gpu = rank == 0 and world == 1
    if one_gpu and not args.skip_rival:
        log("rival: cuBLAS FP64 emulation vs the split contraction")
        out["rival"] = guarded(rival_leg, cg, p, dr, Xd, args.slices)
    del dr, Xd, Id
    release_device()

    # ---- the CPU oracle: baseline timing and the accuracy of both forms -------------
    if one_gpu and not args.skip_cpu:
        log("cpu baseline sample")
        cb, sub, Xo, Io = cpu_sample(p, rows=min(CPU_BASELINE_ROWS, p.n_grid1))
        out["cpu_baseline"] = cb
        if not args.skip_accuracy:
            log("accuracy of both forms vs the oracle")
            acc = {"sample": "%d of %d r1 rows spread over the grid; both forms against the FP64 "
                             "oracle (oracle/, C restatement of the reference's kernels + numpy "
                             "DGEMM)" % (sub.n_grid1, p.n_grid1)}
            forms = [("split", cg.SPLIT_BF16, args.slices), ("plain", cg.PLAIN_FP64, None)]
            if prec == cg.SPLIT_BF16 and args.slices < FP64_CLASS_SLICES:
                forms.append(("split_%d_slices" % FP64_CLASS_SLICES, cg.SPLIT_BF16,
                              FP64_CLASS_SLICES))
            for name, pr, ns in forms:
                X, I = cg.build_integrals(sub, pr, n_slices=ns)
                acc[name] = {"X_vs_oracle": rel(X, Xo[:3]), "int2e_vs_oracle": rel(I, Io)}
                del X, I
            out["accuracy"] = acc
        del Xo, Io
        release_device()
    if one_gpu and not args.skip_accuracy:
        log("plain FP64 rate")
        out["plain_fp64"] = guarded(plain_rate_estimate, cg, p, (256, 512))
        if prec == cg.SPLIT_BF16 and args.slices < FP64_CLASS_SLICES:
            log("split form at %d slices" % FP64_CLASS_SLICES)
            out["split_%d_slices" % FP64_CLASS_SLICES] = guarded(fp64_class_leg, cg, p,
                                                                  FP64_CLASS_SLICES)
    if one_gpu and not args.skip_large:
        log("large workload on r1 samples")
        out["large"] = guarded(large_leg, cg, args, 1, 1, not args.skip_accuracy)
    if one_gpu and not args.skip_scan:
        log("Jastrow-parameter scan")
        out["scan"] = guarded(scan_leg, cg, args, 16, not args.skip_accuracy)
    if one_gpu and not args.skip_serving:
        log("serving stream prefix")
        plain_tf = (out.get("plain_fp64") or {}).get("x_gemm_fp64_tflops")
        out["serving"] = guarded(serving_leg, cg, args, 32, 1.0, 250, not args.skip_accuracy,
                                 plain_tf)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def run_shard(args):
    """--shard under torchrun: ONE build per step spread over the ranks by r1 (each
    rank builds its r1 window's X rows and int_2e share on its GPU, device-resident;
    one NCCL all-reduce sums the int_2e shares): strong scaling of a single build."""
    import torch
    import torch.distributed as dist
    import cutc_gb300 as cg
    from cutc_gb300.shard import build_sharded
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist.init_process_group("nccl" if world > 1 else "gloo")
    prec = cg.SPLIT_BF16 if args.precision == "split" else cg.PLAIN_FP64
    p = synth.make_config(args.config)

    def step():
        return build_sharded(p, dist, prec, args.slices if prec else None)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        (b, e), X, I = step()
    torch.cuda.synchronize(dev)
    dist.barrier()
    secs = max_over_ranks(time.perf_counter() - t0, dist if world > 1 else None, dev)
    if rank == 0:
        v = args.steps / secs
        print(json.dumps({
            "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "bf16" if prec == cg.SPLIT_BF16 else "f64", "data": "synthetic",
            "config": {"workload": workload_desc(args.config, p), "precision": args.precision,
                       "parallelism": "r1 sharded over %d GPUs, one all-reduce of int_2e" % world,
                       "window_rank0": [b, e]},
            "e2e": {"value": None, "reason": "each step copies the molecule's host arrays to "
                                             "every rank's GPU and builds its window there; X "
                                             "stays on the device"}}), flush=True)
    dist.destroy_process_group()
    return 0


def rel(a, b):
    from oracle.oracle import rel_err
    return rel_err(a, b)


def guarded(fn, *a):
    """One extra leg of the line: its record, or the error that stopped it (the
    main measurement stands either way)."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001
        log("leg %s failed: %r" % (fn.__name__, e))
        try:
            release_device()
        except Exception:  # noqa: BLE001
            pass
        return {"error": repr(e)[:400]}


# ---------------------------------------------------------------------------
# the large workload: r1 samples of the full molecule and grids
# ---------------------------------------------------------------------------
def large_leg(cg, args, warmup, steps, with_accuracy, sizes=(3000, 6000), full_build=True):
    """Large workload (n_ao=300, n_grid2=200,000): one full device-resident build of
    the 60,000-point r1 grid with int_2e returned and X formed on the device but not
    copied out, and, as a cross-check, two r1 samples spread over the grid,
    extrapolated linearly in n_grid1.

    A full build's outputs (X: 130 GB, int_2e: 65 GB) do not fit the GPU host's
    memory beside each other, nor the device beside the working set, so the full
    build returns int_2e alone; the samples return X as well.  The device-resident
    cost of a build is linear in the r1 rows it holds (every r1 tile does the same
    work) plus a fixed part (P slices, int_2e assembly), which the two samples
    separate.
    """
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    prec = cg.SPLIT_BF16 if args.precision == "split" else cg.PLAIN_FP64
    p = synth.make_config("large")
    nA2 = p.n_ao ** 2
    stream = torch.cuda.Stream(device=dev)
    opt = cg.options(prec, args.slices, p.a_en, p.a_ee, 3, True, 0, stream.cuda_stream,
                     k_split=args.k_split)
    release_device()
    Id = torch.empty((nA2, nA2), dtype=torch.float64, device=dev)
    samples = []
    gemm_ms, gemm_launches, launches, pair_ms, flops_x = 0.0, 0, 0, 0.0, 0.0
    sampler = ClockSampler(gpu_uuid(dev))
    for ns in sizes:
        sub = synth.r1_sample(p, ns)
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
        for _ in range(warmup):
            build()
        if ns == sizes[-1]:
            sampler.start()
            time.sleep(0.5)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        tiles = 0
        for _ in range(steps):
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
        ms = e0.elapsed_time(e1) / steps
        samples.append({"r1_rows": ns, "ms_per_build": ms, "r1_tiles": tiles})
        log("large: %d rows: %.1f ms per build" % (ns, ms))
        del dr, Xd
    full = None
    if full_build:
        # the whole r1 grid in one call: X (130 GB) is formed on the device in the
        # contractions' packed layout but not returned, int_2e (65 GB) stays on the device
        log("large: one full build, int_2e returned, X not copied out")
        # the samples' workspace would otherwise shrink the free memory the build plans with
        cg.load().cutc_release()
        dr = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in p.arrays().items()}
        torch.cuda.synchronize(dev)
        st = cg.Stats()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                           dr["r1"], dr["wr1"], dr["r2"], dr["wr2"], dr["rn"], dr["aos1"],
                           dr["aos2"], dr["c_bh"], dr["m_bh"], dr["n_bh"], dr["o_bh"], None, Id, st)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        if s != cg.CUTC_OK:
            raise cg.CutcError(s, cg.last_error())
        full = {"ms_per_build": e0.elapsed_time(e1), "r1_tiles": st.n_r1_tiles,
                "ms_x_gemm": st.ms_x_gemm, "ms_pair": st.ms_pair, "ms_int2e": st.ms_int2e,
                "note": "one device-resident build of all %d r1 rows (no warm-up beyond the "
                        "samples'), int_2e returned on the device, X formed but not copied "
                        "out (cutc_int_ex with int2_grad1_u12_ao = NULL)" % p.n_grid1}
        log("large: full build %.0f ms" % full["ms_per_build"])
        del dr
    clocks = sampler.stop()
    del Id
    release_device()
    (n_a, n_b), (t_a, t_b) = sizes, (samples[0]["ms_per_build"], samples[1]["ms_per_build"])
    slope = (t_b - t_a) / (n_b - n_a)
    t_proj = t_b + slope * (p.n_grid1 - n_b)
    t_full = full["ms_per_build"] if full else t_proj
    value = 1e3 / t_full

    peaks, peak_kind = measured_peaks()
    peak = float(peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops")))
    per_launch_ms = gemm_ms / max(1, gemm_launches)
    achieved = flops_x / max(1, gemm_launches) / (per_launch_ms * 1e-3) / 1e12
    S = args.slices
    n_products = S * (S + 1) // 2 if prec == cg.SPLIT_BF16 else 0
    packed = p.n_ao * (p.n_ao + 1) / 2.0 / nA2
    executed = achieved * packed * n_products if n_products else None
    out = {"value": value, "unit": UNIT, "ms_per_build": t_full,
           "workload": workload_desc("large", p), "precision": args.precision,
           "full_build": full,
           "projection": "device-resident builds on %d and %d r1 rows spread over the r1 grid "
                         "(%d warm-up, %d timed each), extrapolated linearly to n_grid1=%d: "
                         "%.0f ms per build" % (n_a, n_b, warmup, steps, p.n_grid1, t_proj),
           "samples": samples, "gpu_launches": launches, "clocks": clocks,
           "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                        "unit": "TFLOP/s", "frac": achieved / peak,
                        "kernel": "split_gemm_kernel (X build)",
                        "peak_source": "bf16_tflops_sustained of %s" % peak_kind,
                        "ms_per_launch": per_launch_ms, "executed_bf16_tflops": executed,
                        "executed_frac": (executed / peak) if executed else None},
           "phases_ms_per_build_sample": {"pair": pair_ms / steps, "x_gemm": gemm_ms / steps},
           "e2e": {"value": None, "reason": "the full build's host outputs (195 GB) exceed the "
                                            "GPU host's memory"}}
    if with_accuracy:
        log("large: accuracy vs the oracle")
        out["accuracy"] = oracle_check(cg, p, 32, S)
    return out


def oracle_check(cg, p, rows, n_slices):
    """Both forms against the FP64 oracle on `rows` r1 points spread over the grid of
    p, at its full n_ao and n_grid2, with the outputs left on the device: X in full,
    48 rows of int_2e and int_2e times a random vector (oracle.x_rows,
    int2e_rows, int2e_matvec form neither the whole P nor the n_ao^4 matrix)."""
    import torch
    from oracle import oracle
    sub = synth.r1_sample(p, rows)
    nA2 = sub.n_ao ** 2
    rng = np.random.default_rng(2024)
    sel = np.sort(rng.choice(nA2, min(nA2, 48), replace=False))
    v = rng.standard_normal(nA2)
    X4 = oracle.x_rows(sub)
    S0, S = oracle.short_herm(sub), oracle.short_nonherm(sub)
    I_sel = oracle.int2e_rows(sub, X4, sel, S0, S)
    I_v = oracle.int2e_matvec(sub, X4, v, S0, S)
    release_device()
    res = {"sample": "%d of %d r1 rows spread over the grid, full n_ao and n_grid2; X in full, "
                     "48 int_2e rows and int_2e v against the FP64 oracle"
                     % (rows, p.n_grid1)}
    buf = None
    for name, prec in (("split", cg.SPLIT_BF16), ("plain", cg.PLAIN_FP64)):
        X, I = cg.build_integrals_device(sub, prec, n_slices=n_slices if prec else None, out=buf)
        buf = (X, I)
        res[name] = {"X_vs_oracle": rel(X.cpu().numpy(), X4[:3]),
                     "int2e_rows_vs_oracle": rel(I[torch.from_numpy(sel).to(I.device)].cpu().numpy(),
                                                 I_sel),
                     "int2e_v_vs_oracle": rel((I @ torch.from_numpy(v).to(I.device)).cpu().numpy(),
                                              I_v)}
        release_device()
    del buf
    release_device()
    return res


# ---------------------------------------------------------------------------
# the Jastrow-parameter scan
# ---------------------------------------------------------------------------
def scan_sets(p, n, seed=5050):
    rng = np.random.default_rng(seed)
    return (rng.normal(0.0, 0.3, size=(n,) + p.c_bh.shape), rng.uniform(0.5, 2.0, n),
            rng.uniform(0.5, 2.0, n))


def scan_leg(cg, args, n_sets, with_accuracy, batch=8):
    """The scan molecule with n_sets Jastrow parameter sets, `batch` sets per
    cutc_int_scan call, outputs in reused pinned host memory."""
    import torch
    from oracle import oracle
    p = synth.make_config("scan")
    c_sets, a_en, a_ee = scan_sets(p, n_sets)
    prec = cg.SPLIT_BF16 if args.precision == "split" else cg.PLAIN_FP64
    batch = min(n_sets, batch)
    nA2 = p.n_ao ** 2
    Xo = torch.empty((batch, 3, p.n_grid1, nA2), dtype=torch.float64, pin_memory=True).numpy()
    Io = torch.empty((batch, nA2, nA2), dtype=torch.float64, pin_memory=True).numpy()
    cg.scan_integrals(p, c_sets[:batch], a_en[:batch], a_ee[:batch], prec, args.slices,
                      out=(Xo, Io))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    launches = 0
    for b0 in range(0, n_sets, batch):
        sl = slice(b0, min(n_sets, b0 + batch))
        k = sl.stop - sl.start
        X, I, st = cg.scan_integrals(p, c_sets[sl], a_en[sl], a_ee[sl], prec, args.slices,
                                     with_stats=True, out=(Xo[:k], Io[:k]))
        launches += st["gpu_launches"]
    elapsed = time.perf_counter() - t0
    del Xo, Io
    out = {"value": n_sets / elapsed, "unit": UNIT,
           "workload": "scan: " + workload_desc("scan", p) + ", %d Jastrow parameter sets "
                       "(c ~ N(0, 0.3), a_en, a_ee ~ U[0.5, 2]), %d sets per cutc_int_scan "
                       "call, outputs in reused pinned host memory" % (n_sets, batch),
           "precision": args.precision, "gpu_launches": launches,
           "alg_tflops": n_sets * p.flops() / elapsed / 1e12}
    release_device()
    if with_accuracy:
        rows, k = 64, 4
        sub = synth.r1_sample(p, rows)
        Xs, Is = cg.scan_integrals(sub, c_sets[:k], a_en[:k], a_ee[:k], cg.SPLIT_BF16, args.slices)
        Xp, Ip = cg.scan_integrals(sub, c_sets[:k], a_en[:k], a_ee[:k], cg.PLAIN_FP64)
        worst = {"split": {"X": 0.0, "int2e": 0.0}, "plain": {"X": 0.0, "int2e": 0.0}}
        for s in range(k):
            q = dataclasses.replace(sub, c_bh=np.ascontiguousarray(c_sets[s]), a_en=float(a_en[s]),
                                    a_ee=float(a_ee[s]))
            Xr, Ir = oracle.cutc_int(q)
            for name, Xg, Ig in (("split", Xs[s], Is[s]), ("plain", Xp[s], Ip[s])):
                ex, ei = rel(Xg, Xr), rel(Ig, Ir)
                worst[name]["X"] = max(worst[name]["X"], ex["norm"], ex["max"])
                worst[name]["int2e"] = max(worst[name]["int2e"], ei["norm"], ei["max"])
        out["accuracy"] = {"worst_vs_oracle": worst,
                           "sample": "%d of %d r1 rows, the first %d sets; the worst of the "
                                     "normwise and max-abs/max relative errors against the "
                                     "FP64 oracle" % (rows, p.n_grid1, k)}
        release_device()
    return out


# ---------------------------------------------------------------------------
# the serving stream
# ---------------------------------------------------------------------------
def serving_requests(n, max_ao, seed=4004):
    """The serving stream: molecules of 2-20 nuclei, n_ao uniform in [10, max_ao],
    n_grid1 = 1000 n_nuc, n_grid2 = 4000 n_nuc; 30% repeat an earlier molecule with
    Jastrow coefficients perturbed by a 10% Gaussian.  Molecules carry their basis,
    not AO arrays: the server evaluates the AOs on the GPU."""
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


def serving_stream(cg, reqs, rate, prec, n_slices, slots, host_gb):
    """Poisson arrivals into the continuous-batching server.  The host holds at most
    host_gb of request outputs at a time (X and int_2e of an n_ao = 250 request are
    61 GB): past that, the stream waits for the oldest request before submitting the
    next, and the time it waited is reported."""
    rng = np.random.default_rng(7)
    gaps = rng.exponential(1.0 / rate, size=len(reqs))
    budget = host_gb * 1e9
    lat = []
    held = 0.0
    t_blocked = 0.0
    with cg.Server(n_slots=slots) as srv:
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
            tickets.append((srv.submit(p, key, prec, n_slices, aos_from_basis=True), need))
            held += need
        for t, _ in tickets:
            lat.append(srv.wait(t)[2])
        elapsed = time.perf_counter() - t0
        st = srv.stats()
    flops = sum(p.flops() for _, p in reqs)
    return {"value": len(reqs) / elapsed, "unit": UNIT,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "max_ms": float(np.max(lat)), "arrivals_held_back_s": t_blocked,
            "server": st, "alg_tflops": flops / elapsed / 1e12}


def serving_leg(cg, args, n, rate, max_ao, with_accuracy, plain_fp64_tflops):
    """The first n requests of the serving stream (BASELINE rate and n_ao range) in
    the split form, p50/p99 latency and builds/s; the plain FP64 form's rate on the
    same requests from its measured FP64 contraction rate; one molecule of the
    prefix against the oracle in both forms."""
    reqs = serving_requests(n, max_ao)
    out = serving_stream(cg, reqs, rate, cg.SPLIT_BF16, args.slices, 4, 48.0)
    out["workload"] = ("serving: the first %d requests of the 256-request stream, Poisson "
                       "arrivals at %.1f/s, 2-20 nuclei, n_ao in [10, %d], n_grid1 = 1000 n_nuc, "
                       "n_grid2 = 4000 n_nuc, 30%% repeats with perturbed Jastrow coefficients, "
                       "AOs evaluated on the GPU from each request's basis, 4 slots"
                       % (n, rate, max_ao))
    out["precision"] = "split"
    if plain_fp64_tflops:
        # the plain form's dominant cost is its FP64 contractions: packed X (4 nA(nA+1) n1 n2
        # flops) and int_2e (about 4 nA^4 n1 with the packed pairs)
        secs = [(4.0 * q.n_ao * (q.n_ao + 1) * q.n_grid1 * q.n_grid2 + 4.0 * q.n_ao ** 4 * q.n_grid1)
                / (plain_fp64_tflops * 1e12) for _, q in reqs]
        out["plain_projection"] = {
            "builds_per_s": len(reqs) / sum(secs), "mean_s_per_request": float(np.mean(secs)),
            "basis": "each request's packed FP64 contraction flops at the plain form's measured "
                     "X-contraction rate (%.3f TF/s); the stream's arrival rate exceeds this "
                     "service rate, so its latency grows without bound" % plain_fp64_tflops}
    if with_accuracy:
        ps = sorted({k: q for k, q in reqs if q.n_ao <= 200}.values(), key=lambda q: q.n_ao)
        if ps:
            q = ps[-1]
            q = dataclasses.replace(q, aos1=synth.eval_aos(q.shells, q.r1),
                                    aos2=synth.eval_aos(q.shells, q.r2))
            out["accuracy"] = oracle_check(cg, q, 32, args.slices)
            out["accuracy"]["molecule"] = {"n_nuc": q.n_nuc, "n_ao": q.n_ao, "n_grid2": q.n_grid2}
    release_device()
    return out


# ---------------------------------------------------------------------------
# the rival: cuBLAS's own FP64 emulation on the split contraction's operands
# ---------------------------------------------------------------------------
class Cublas:
    """The handful of cuBLAS calls the rival leg needs, through ctypes (cuBLAS is
    not linked into this library)."""
    OP_N, OP_T = 0, 1
    FP64_EMULATED_FIXEDPOINT_MATH = 8  # cublasMath_t
    EMULATION_STRATEGY_EAGER = 2       # cublasEmulationStrategy_t
    MANTISSA_DYNAMIC, MANTISSA_FIXED = 0, 1  # cudaEmulationMantissaControl

    def __init__(self):
        self.L = None
        for name in ("libcublas.so.13", "/usr/local/cuda/lib64/libcublas.so.13",
                     "/usr/local/cuda/lib64/libcublas.so"):
            try:
                self.L = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if self.L is None:
            raise RuntimeError("libcublas not found")
        L, vp, i = self.L, ctypes.c_void_p, ctypes.c_int
        dp = ctypes.POINTER(ctypes.c_double)
        L.cublasCreate_v2.argtypes = [ctypes.POINTER(vp)]
        L.cublasDestroy_v2.argtypes = [vp]
        L.cublasSetStream_v2.argtypes = [vp, vp]
        L.cublasSetMathMode.argtypes = [vp, i]
        L.cublasSetWorkspace_v2.argtypes = [vp, vp, ctypes.c_size_t]
        L.cublasDgemm_v2.argtypes = [vp, i, i, i, i, i, dp, vp, i, vp, i, dp, vp, i]
        for f in ("cublasSetEmulationStrategy", "cublasSetFixedPointEmulationMantissaControl",
                  "cublasSetFixedPointEmulationMaxMantissaBitCount"):
            getattr(L, f).argtypes = [vp, i]
        self.h = vp()
        self._check(L.cublasCreate_v2(ctypes.byref(self.h)), "cublasCreate")

    @staticmethod
    def _check(s, what):
        if s != 0:
            raise RuntimeError("%s: cuBLAS status %d" % (what, s))

    def configure(self, stream, workspace, emulated, mantissa_bits=None):
        L = self.L
        self._check(L.cublasSetStream_v2(self.h, stream), "cublasSetStream")
        self._check(L.cublasSetWorkspace_v2(self.h, workspace.data_ptr(), workspace.numel()),
                    "cublasSetWorkspace")
        if not emulated:
            self._check(L.cublasSetMathMode(self.h, 0), "cublasSetMathMode")
            return
        self._check(L.cublasSetMathMode(self.h, self.FP64_EMULATED_FIXEDPOINT_MATH),
                    "cublasSetMathMode(FP64_EMULATED_FIXEDPOINT)")
        self._check(L.cublasSetEmulationStrategy(self.h, self.EMULATION_STRATEGY_EAGER),
                    "cublasSetEmulationStrategy(EAGER)")
        if mantissa_bits is None:
            self._check(L.cublasSetFixedPointEmulationMantissaControl(self.h, self.MANTISSA_DYNAMIC),
                        "mantissa control DYNAMIC")
        else:
            self._check(L.cublasSetFixedPointEmulationMantissaControl(self.h, self.MANTISSA_FIXED),
                        "mantissa control FIXED")
            self._check(L.cublasSetFixedPointEmulationMaxMantissaBitCount(self.h, mantissa_bits),
                        "max mantissa bits")

    def gemm_nt(self, M, N, K, A, B, C):
        """C (M x N, column-major) = A B^T with A (M x K) and B (N x K) row-major."""
        one, zero = ctypes.c_double(1.0), ctypes.c_double(0.0)
        self._check(self.L.cublasDgemm_v2(self.h, self.OP_T, self.OP_N, M, N, K, ctypes.byref(one),
                                          A.data_ptr(), K, B.data_ptr(), K, ctypes.byref(zero),
                                          C.data_ptr(), M), "cublasDgemm")

    def close(self):
        self.L.cublasDestroy_v2(self.h)


def rival_shapes(p, dr, Xd, n_cols):
    """The split contraction's real operands on the medium molecule, as FP64
    row-major device tensors: the X build (A = packed pair products P, B = rows of
    the pair-term planes G of n_cols / 4 r1 points, K = n_grid2) and an int_2e
    contraction (A = packed X_0 over all r1 points, B = n_cols packed S0 rows,
    K = n_grid1)."""
    import torch
    import cutc_gb300 as cg
    dev = Xd.device
    nA = p.n_ao
    a_idx, b_idx = np.tril_indices(nA)  # packed pairs a >= b
    order = np.lexsort((a_idx, b_idx))  # column by column, as the library packs them
    a_t = torch.from_numpy(a_idx[order]).to(dev)
    b_t = torch.from_numpy(b_idx[order]).to(dev)
    chi2 = dr["aos2"][0]  # (nA, n2): value component
    P = (dr["wr2"][None, :] * chi2[a_t]) * chi2[b_t]
    nr1 = n_cols // 4
    G = torch.empty((4, nr1, p.n_grid2), dtype=torch.float64, device=dev)
    s = cg.jast_bh_device(dr["r1"], dr["r2"], dr["rn"], dr["c_bh"], dr["m_bh"], dr["n_bh"],
                          dr["o_bh"], G, i0=0, n1b=nr1, a_en=p.a_en, a_ee=p.a_ee)
    if s != cg.CUTC_OK:
        raise cg.CutcError(s, cg.last_error())
    Bx = G.reshape(4 * nr1, p.n_grid2)
    X0 = Xd[0][:, a_t * nA + b_t].T.contiguous()  # (np, n1)
    chi1 = dr["aos1"][0]  # (nA, n1)
    sel = torch.arange(0, min(n_cols, a_t.numel()), device=dev)
    S0 = (dr["wr1"][None, :] * chi1[a_t[sel]]) * chi1[b_t[sel]]
    return [("X build", P, Bx), ("int_2e (N contraction shape)", X0, S0.contiguous())]


def rival_leg(cg, p, dr, Xd, n_slices, n_cols=2048, bits=(None, 40)):
    """cuBLAS FP64 DGEMM, this library's FP64 DMMA GEMM, cuBLAS with FP64
    fixed-point emulation (dynamic and fixed mantissa bits) and the split
    contraction on the same operands; errors against the cuBLAS FP64 result."""
    import torch
    dev = Xd.device
    out = {"note": "each call's device time (CUDA events) includes the slicing of both operands "
                   "for the emulated and split forms; errors are normwise and max-abs/max "
                   "against cuBLAS FP64 DGEMM on the same operands"}
    cb = Cublas()
    ws = torch.empty(4 << 30, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    try:
        for name, A, B in rival_shapes(p, dr, Xd, n_cols):
            M, K = A.shape
            N = B.shape[0]
            flops = 2.0 * M * N * K
            rec = {"M": M, "N": N, "K": K}
            C_ref = torch.empty((N, M), dtype=torch.float64, device=dev)
            cb.configure(stream, ws, False)
            cb.gemm_nt(M, N, K, A, B, C_ref)  # warm-up
            ms = cuda_ms(lambda: cb.gemm_nt(M, N, K, A, B, C_ref))
            rec["cublas_fp64"] = {"ms": ms, "fp64_tflops": flops / ms / 1e9}
            C = torch.empty_like(C_ref)
            cg.fp64_gemm_device(True, M, N, K, 1.0, A, K, B, K, 0.0, C, M)
            ms = cuda_ms(lambda: cg.fp64_gemm_device(True, M, N, K, 1.0, A, K, B, K, 0.0, C, M))
            rec["ours_fp64_dmma"] = {"ms": ms, "fp64_tflops": flops / ms / 1e9,
                                     "err": rel(C.cpu().numpy(), C_ref.cpu().numpy())}
            ref_h = C_ref.cpu().numpy()
            for b in bits:
                key = "cublas_emulated_%s" % ("dynamic" if b is None else "fixed%d" % b)
                try:
                    cb.configure(stream, ws, True, b)
                    cb.gemm_nt(M, N, K, A, B, C)
                    ms = cuda_ms(lambda: cb.gemm_nt(M, N, K, A, B, C))
                    rec[key] = {"ms": ms, "fp64_equiv_tflops": flops / ms / 1e9,
                                "err": rel(C.cpu().numpy(), ref_h)}
                except Exception as e:  # noqa: BLE001
                    rec[key] = {"error": repr(e)[:200]}
            cg.split_gemm_device(A, B, C, n_slices=n_slices)
            ms = cuda_ms(lambda: cg.split_gemm_device(A, B, C, n_slices=n_slices))
            rec["ours_split_%d" % n_slices] = {"ms": ms, "fp64_equiv_tflops": flops / ms / 1e9,
                                               "err": rel(C.cpu().numpy(), ref_h)}
            out[name] = rec
            log("rival %s: %s" % (name, json.dumps(rec)))
            del C, C_ref, A, B
    finally:
        cb.close()
        del ws
        release_device()
    return out


def traffic_per_launch(args, p, launches):
    """DRAM bytes per X-contraction launch from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", "split_gemm_traffic.json")
    if not os.path.exists(path):
        return None
    try:
        with open(path) as f:
            d = json.load(f)
        # bytes per (M x N x K) unit measured on the captured launches, times the M N K
        # of one launch: a build's X contractions (np x 4 n1 x n2) over its launches
        per_unit = float(d["dram_bytes_per_mnk"])
        np_ = p.n_ao * (p.n_ao + 1) // 2
        launches_per_build = max(1.0, launches / max(1, args.steps))
        return per_unit * np_ * 4.0 * p.n_grid1 * p.n_grid2 / launches_per_build
    except Exception:
        return None


# ---------------------------------------------------------------------------
# single-kernel micro-benchmarks (the cases of the committed ncu summaries)
# ---------------------------------------------------------------------------
def run_kernel(args):
    import torch
    import cutc_gb300 as cg
    torch.cuda.set_device(0)
    k = args.kernel
    if k in ("split_gemm", "fp64_gemm"):
        # C = A B^T on seeded FP64 operands shaped like the X build of cutc_int
        # (m packed AO pairs, n = 4 x r1 points, k = r2 points)
        g = torch.Generator(device="cuda").manual_seed(1234)
        A = torch.randn((args.m, args.k), dtype=torch.float64, device="cuda", generator=g)
        B = torch.randn((args.n, args.k), dtype=torch.float64, device="cuda", generator=g)
        C = torch.empty((args.n, args.m), dtype=torch.float64, device="cuda")
        if k == "split_gemm":
            call = lambda: cg.split_gemm_device(A, B, C, n_slices=args.slices)
        else:
            call = lambda: cg.fp64_gemm_device(True, args.m, args.n, args.k, 1.0, A, args.k, B,
                                               args.k, 0.0, C, args.m)
        times = [cuda_ms(call) for _ in range(args.reps)]
        alg = 2.0 * args.m * args.n * args.k
        ms = min(times)
        rec = {"kernel": k, "m": args.m, "n": args.n, "k": args.k, "ms_call": ms,
               "fp64_equiv_tflops": alg / ms / 1e9}
        if k == "split_gemm":
            S = args.slices
            rec.update(slices=S, bf16_tflops_executed=alg * S * (S + 1) / 2 / ms / 1e9,
                       note="call time includes slicing both operands")
        print(json.dumps(rec))
    elif k == "pair":
        # a molecule with the medium workload's nuclei and Jastrow terms; by default few AOs
        # (the pair terms do not depend on n_ao), so the device holds a few GB
        p = synth.make_problem(n_nuc=args.n_nuc, n_ao=args.n_ao, n_grid1=args.n1,
                               n_grid2=args.n2, size_bh=args.terms, seed=2002, box=6.0)
        pair_ms = []
        for _ in range(args.reps):
            _, _, st = cg.build_integrals(p, cg.SPLIT_BF16, with_stats=True)
            pair_ms.append(st["ms_pair"])
        ms = min(pair_ms)
        print(json.dumps({"kernel": k, "n_nuc": args.n_nuc, "terms_per_nucleus": args.terms,
                          "n1": args.n1, "n2": args.n2, "pair_ms": ms,
                          "pairs_per_s": args.n1 * args.n2 / ms * 1e3,
                          "pair_nucleus_evals_per_s": args.n1 * args.n2 * args.n_nuc / ms * 1e3}))
    elif k == "plain_build":
        # the medium molecule in the plain FP64 form on `rows` r1 points spread over its grid
        p = synth.make_config("medium")
        sub = synth.r1_sample(p, args.rows)
        for _ in range(args.reps):
            _, _, st = cg.build_integrals(sub, cg.PLAIN_FP64, with_stats=True)
        np_ = p.n_ao * (p.n_ao + 1) // 2
        flops_x = 2.0 * np_ * 4 * args.rows * p.n_grid2
        print(json.dumps({"kernel": k, "rows": args.rows, "ms_total": st["ms_total"],
                          "ms_x_gemm": st["ms_x_gemm"], "ms_int2e": st["ms_int2e"],
                          "ms_pair": st["ms_pair"],
                          "x_gemm_fp64_tflops": flops_x / st["ms_x_gemm"] / 1e9}))
    elif k == "sample_build":
        # device-resident builds of `rows` r1 points spread over the grid of --config (the
        # whole grid when rows >= n_grid1), outputs on the device, per-build phase times
        p = synth.make_config(args.config)
        sub = synth.r1_sample(p, args.rows) if args.rows < p.n_grid1 else p
        prec = cg.SPLIT_BF16 if args.precision == "split" else cg.PLAIN_FP64
        dev = torch.device("cuda", 0)
        nA2 = p.n_ao ** 2
        out = (torch.empty((3, sub.n_grid1, nA2), dtype=torch.float64, device=dev),
               torch.empty((nA2, nA2), dtype=torch.float64, device=dev))
        runs = []
        for _ in range(args.reps):
            _, _, st = cg.build_integrals_device(sub, prec, n_slices=args.slices, out=out,
                                                 with_stats=True)
            runs.append({key: st[key] for key in ("ms_total", "ms_x_gemm", "n_x_gemm",
                                                  "n_r1_tiles", "ms_pair", "ms_int2e")})
        print(json.dumps({"kernel": k, "config": args.config, "rows": sub.n_grid1,
                          "precision": args.precision, "builds": runs}))
    elif k == "rival":
        p = synth.make_config("medium")
        dev = torch.device("cuda", 0)
        dr = {kk: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for kk, v in p.arrays().items()}
        Xd = torch.empty((3, p.n_grid1, p.n_ao ** 2), dtype=torch.float64, device=dev)
        cg.build_integrals_device(p, cg.SPLIT_BF16, n_slices=args.slices,
                                  out=(Xd, torch.empty((p.n_ao ** 2,) * 2, dtype=torch.float64,
                                                       device=dev)))
        bits = [None if b == "dynamic" else int(b) for b in args.bits]
        print(json.dumps(rival_leg(cg, p, dr, Xd, args.slices, args.n, bits)))
    return 0


# ---------------------------------------------------------------------------
# stand-alone legs
# ---------------------------------------------------------------------------
def run_large_cli(args):
    import torch
    import cutc_gb300 as cg
    torch.cuda.set_device(0)
    leg = large_leg(cg, args, args.warmup, args.steps, not args.skip_accuracy,
                    (args.r1_sample // 2, args.r1_sample))
    S = args.slices
    out = {"metric": METRIC, "value": leg["value"], "unit": UNIT, "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": leg["ms_per_build"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "bf16" if args.precision == "split" else "f64", "data": "synthetic",
           "config": {"workload": leg["workload"], "precision": args.precision, "n_slices": S,
                      "projection": leg["projection"], "parallelism": "1 GPU",
                      "l2": "inputs larger than L2: P slices alone are %.0f GB"
                            % (2 * S * 300 * 301 / 2 * 200000 / 1e9)}}
    out.update({k: v for k, v in leg.items() if k not in out and k not in ("workload",)})
    print(json.dumps(out), flush=True)
    return 0


def run_serving_cli(args):
    import cutc_gb300 as cg
    import torch
    torch.cuda.set_device(0)
    reqs = serving_requests(args.requests, args.max_ao)
    log("serving: %d requests generated" % len(reqs))
    prec = cg.SPLIT_BF16 if args.precision == "split" else cg.PLAIN_FP64
    line = serving_stream(cg, reqs, args.rate, prec, args.slices, args.slots, args.host_gb)
    line.update({"metric": "TC integral builds/s and latency, serving stream", "n_gpus": 1,
                 "higher_is_better": True,
                 "dtype": "bf16" if prec == cg.SPLIT_BF16 else "f64", "data": "synthetic",
                 "config": {"workload": "serving: %d requests, Poisson arrivals at %.1f/s, 2-20 "
                                        "nuclei, n_ao in [10, %d], n_grid1 = 1000 n_nuc, n_grid2 = "
                                        "4000 n_nuc, 30%% repeats with perturbed Jastrow "
                                        "coefficients, AOs evaluated on the GPU from each "
                                        "request's basis" % (len(reqs), args.rate, args.max_ao),
                            "slots": args.slots, "precision": args.precision,
                            "host_output_budget_gb": args.host_gb}})
    print(json.dumps(line), flush=True)
    return 0


def run_scan_cli(args):
    import cutc_gb300 as cg
    import torch
    torch.cuda.set_device(0)
    leg = scan_leg(cg, args, args.sets, not args.skip_accuracy, args.scan_batch)
    leg.update({"metric": "TC integral builds/s, Jastrow-parameter scan", "n_gpus": 1,
                "higher_is_better": True, "data": "synthetic",
                "dtype": "bf16" if args.precision == "split" else "f64"})
    print(json.dumps(leg), flush=True)
    return 0


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
    ap.add_argument("--skip-rival", action="store_true")
    ap.add_argument("--skip-large", action="store_true")
    ap.add_argument("--skip-scan", action="store_true")
    ap.add_argument("--skip-serving", action="store_true")
    ap.add_argument("--main-only", action="store_true",
                    help="the medium line alone: skip the CPU, accuracy and extra legs")
    ap.add_argument("--shard", action="store_true",
                    help="under torchrun: one build per step, r1 sharded over the ranks")
    ap.add_argument("--serving", action="store_true", help="run the serving stream instead")
    ap.add_argument("--requests", type=int, default=256)
    ap.add_argument("--rate", type=float, default=1.0, help="serving arrivals per second")
    ap.add_argument("--max-ao", type=int, default=250)
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--host-gb", type=float, default=48.0,
                    help="serving: host memory for outputs of requests in flight")
    ap.add_argument("--scan", action="store_true", help="run the Jastrow-parameter scan instead")
    ap.add_argument("--sets", type=int, default=64)
    ap.add_argument("--scan-batch", type=int, default=8)
    ap.add_argument("--r1-sample", type=int, default=6000,
                    help="large workload: r1 rows of the bigger of the two timed samples")
    ap.add_argument("--kernel", choices=["split_gemm", "fp64_gemm", "pair", "plain_build",
                                         "sample_build", "rival"],
                    help="run one kernel's micro-benchmark instead")
    ap.add_argument("--m", type=int, default=7260)
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--k", type=int, default=16384)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--rows", type=int, default=256)
    ap.add_argument("--n-nuc", type=int, default=10)
    ap.add_argument("--n-ao", type=int, default=40, help="pair micro-benchmark: AOs of the molecule")
    ap.add_argument("--terms", type=int, default=13)
    ap.add_argument("--n1", type=int, default=1024)
    ap.add_argument("--n2", type=int, default=80000)
    ap.add_argument("--bits", nargs="+", default=["dynamic", "40"],
                    help="rival: mantissa settings of cuBLAS's FP64 emulation")
    args = ap.parse_args(argv)
    if args.main_only:
        args.skip_cpu = args.skip_accuracy = args.skip_rival = True
        args.skip_large = args.skip_scan = args.skip_serving = True
    if args.kernel:
        return run_kernel(args)
    if args.shard:
        return run_shard(args)
    if args.serving:
        return run_serving_cli(args)
    if args.scan:
        return run_scan_cli(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "large":
        return run_large_cli(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
