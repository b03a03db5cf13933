"""The slicer's digit arithmetic (cutc_gb300/csrc/digits.cuh), built for the host
by g++ from the same header the kernels include and checked against exact
arithmetic: FP64 rounding at the last digit, the integer-only double-float
rounding against it, the digit decomposition, and the FP32 digit cut of
double-float values that the G slicer uses (tests/c_abi/digits_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_digit_rounding_matches_exact_arithmetic(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "digits_check"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-Wextra",
                           "-Werror",
                           "-I", os.path.join(ROOT, "cutc_gb300", "csrc"),
                           os.path.join(HERE, "c_abi", "digits_check.cpp"), "-o", str(exe)])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    words = r.stdout.split()
    assert words[0] == "ok" and int(words[1]) > 2_000_000 and int(words[2]) > 1_000_000
