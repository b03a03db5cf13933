"""Build libcutcint.so for sm_103a (GB300) in-tree: cutc_gb300/lib/.

    python -m cutc_gb300.build [--force]

nvcc compiles each CUDA translation unit with
``-gencode arch=compute_103a,code=sm_103a -lineinfo``; the drop-in entry point
cutc_int.c is compiled by gcc (the reference builds its driver with gcc too).
Translation units are compiled in parallel; nothing is rebuilt when the
library is newer than every source.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libcutcint.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-Wall,-Wextra", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    c = sorted(glob.glob(os.path.join(CSRC, "*.c")))
    hdr = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INC, "*.h")))
    return cu, c, hdr


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    cu, c, hdr = sources()
    newest = max(os.path.getmtime(p) for p in cu + c + hdr + [__file__])
    return os.path.getmtime(LIB) >= newest


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    os.makedirs(OBJDIR, exist_ok=True)
    cu, c, _ = sources()
    jobs = []
    for src in cu:
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-I", INC, "-I", CSRC, "-c", src, "-o", obj])
    for src in c:
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        jobs.append(["gcc", "-O2", "-fPIC", "-std=c11", "-Wall", "-I", INC, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [j[-1] for j in jobs]
    tmp = LIB + ".tmp%d" % os.getpid()
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs,
          "-Xlinker", "-rpath," + os.path.join(home, "lib64"),
          "-Xlinker", "--no-undefined"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
