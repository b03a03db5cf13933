"""The drop-in ABI from plain C: gcc builds a caller linked against libcutcint.so,
which runs cutc_int on a golden case; its outputs must match the reference's
golden vectors to the plain-form tolerance (1e-12 relative)."""
import os
import subprocess

import numpy as np
import pytest

import cutc_gb300 as cg
from golden_util import load_case
from oracle.oracle import rel_err

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_c_program_calls_drop_in_entry_point(tmp_path):
    cg.load()  # builds the library if needed
    exe = tmp_path / "call_cutc_int"
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-I", os.path.join(ROOT, "include"),
                           os.path.join(HERE, "c_abi", "call_cutc_int.c"), "-o", str(exe),
                           "-L", os.path.dirname(cg.LIB_PATH), "-lcutcint",
                           "-Wl,-rpath," + os.path.dirname(cg.LIB_PATH)])
    p, ref = load_case("tiny_spd")
    for k, v in p.arrays().items():
        np.ascontiguousarray(v).tofile(str(tmp_path / (k + ".bin")))
    out = subprocess.run([str(exe), str(tmp_path), str(p.n_grid1), str(p.n_grid2), str(p.n_ao),
                          str(p.n_nuc), str(p.size_bh)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "status 0" in out.stdout
    X = np.fromfile(str(tmp_path / "X.bin")).reshape(ref["X"].shape)
    I = np.fromfile(str(tmp_path / "int2e.bin")).reshape(ref["int2e"].shape)
    assert rel_err(X, ref["X"])["max"] < 1e-12
    assert rel_err(I, ref["int2e"])["max"] < 1e-12


def test_c_program_drives_reference_stages(tmp_path):
    """A C caller with the reference's own prototypes (CUDA dim3 by value) runs
    get_int2_grad1_u12_ao then get_int_2e_ao on device buffers, as the
    reference's driver does, and gets the golden X and int_2e."""
    cg.load()
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = tmp_path / "call_ref_stages"
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-I", os.path.join(cuda, "include"),
                           os.path.join(HERE, "c_abi", "call_ref_stages.c"), "-o", str(exe),
                           "-L", os.path.dirname(cg.LIB_PATH), "-lcutcint",
                           "-L", os.path.join(cuda, "lib64"), "-lcudart",
                           "-Wl,-rpath," + os.path.dirname(cg.LIB_PATH),
                           "-Wl,-rpath," + os.path.join(cuda, "lib64")])
    p, ref = load_case("tiny_spd")
    for k, v in p.arrays().items():
        np.ascontiguousarray(v).tofile(str(tmp_path / (k + ".bin")))
    out = subprocess.run([str(exe), str(tmp_path), str(p.n_grid1), str(p.n_grid2), str(p.n_ao),
                          str(p.n_nuc), str(p.size_bh)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    X4 = np.fromfile(str(tmp_path / "X4.bin")).reshape((4,) + ref["X"].shape[1:])
    I = np.fromfile(str(tmp_path / "int2e.bin")).reshape(ref["int2e"].shape)
    assert rel_err(X4[:3], ref["X"])["max"] < 1e-12, out.stdout
    assert rel_err(I, ref["int2e"])["max"] < 1e-12, out.stdout
