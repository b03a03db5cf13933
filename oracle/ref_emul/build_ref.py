"""Build the reference's own cutc_int path for the CPU -- TEST INFRASTRUCTURE.

Compiles the CuTC sources where they lie (under /root/reference/src) against
the host emulation of CUDA/cuBLAS in this directory, producing
oracle/_ref/libcutcint_emul.so.  Nothing of the reference is copied into the
repository: the only intermediate files are launch-syntax rewrites written to
oracle/_ref/build/ (git-ignored), where each ``k<<<g, b[, s]>>>(args);`` becomes
``emu_launch(g, b[, s], [&]{ k(args); });`` so that g++ can parse them.

Files compiled (the whole cutc_int call tree, src/cutc_int.c:15-243):
    src/cutc_int.c                  (as C, like the reference Makefile:57-62)
    src/build_int2_grad1_u12_ao.cu  src/build_int_2e_ao.cu   src/jast_bh.cu
    src/long_range_integ.cu         src/short_range_integ_herm.cu
    src/short_range_integ_nonherm.cu  src/add_trans_inplace.cu  src/utils.cu

The library is used only to generate golden vectors (tests/golden/) that pin
the oracle restatement in oracle/cutc_oracle.c.  /root/reference exists only in
the development container, so this step is skipped elsewhere.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
REF = os.environ.get("CUTC_REFERENCE_DIR", "/root/reference")

CU_FILES = [
    "build_int2_grad1_u12_ao.cu", "build_int_2e_ao.cu", "jast_bh.cu",
    "long_range_integ.cu", "short_range_integ_herm.cu",
    "short_range_integ_nonherm.cu", "add_trans_inplace.cu", "utils.cu",
]
C_FILES = ["cutc_int.c"]

LAUNCH = re.compile(r"(\w+)\s*<<<(.*?)>>>\s*\((.*?)\)\s*;", re.S)


def rewrite_launches(text: str) -> str:
    return LAUNCH.sub(lambda m: "emu_launch(%s, [&]() { %s(%s); });"
                      % (m.group(2), m.group(1), m.group(3)), text)


def available() -> bool:
    return os.path.isdir(os.path.join(REF, "src"))


def build(force: bool = False) -> str | None:
    if not available():
        return None
    lib = os.path.join(OUT, "libcutcint_emul.so")
    srcs = [os.path.join(REF, "src", f) for f in CU_FILES + C_FILES]
    mine = [os.path.join(HERE, f) for f in ("emu_cuda.h", "emu_runtime.cpp", "build_ref.py")]
    if not force and os.path.exists(lib):
        newest = max(os.path.getmtime(p) for p in srcs + mine)
        if os.path.getmtime(lib) >= newest:
            return lib
    bdir = os.path.join(OUT, "build")
    os.makedirs(bdir, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "stub"), "-I", os.path.join(REF, "include"), "-I", HERE]
    flags = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-w"]
    objs = []
    for f in CU_FILES:
        with open(os.path.join(REF, "src", f)) as fh:
            text = rewrite_launches(fh.read())
        cpp = os.path.join(bdir, f + ".cpp")
        with open(cpp, "w") as fh:
            fh.write(text)
        obj = cpp + ".o"
        subprocess.check_call(["g++", "-std=c++17", *flags, "-include", "emu_cuda.h", *inc,
                               "-c", cpp, "-o", obj])
        objs.append(obj)
    for f in C_FILES:
        obj = os.path.join(bdir, f + ".o")
        subprocess.check_call(["gcc", *flags, *inc, "-c", os.path.join(REF, "src", f), "-o", obj])
        objs.append(obj)
    obj = os.path.join(bdir, "emu_runtime.o")
    subprocess.check_call(["g++", "-std=c++17", *flags, *inc, "-c",
                           os.path.join(HERE, "emu_runtime.cpp"), "-o", obj])
    objs.append(obj)
    tmp = lib + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-shared", "-fopenmp", *objs, "-o", tmp])
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    path = build(force="--force" in sys.argv)
    print(path if path else "reference sources not present; skipped")
