"""The C-ABI library builds, loads without a GPU and exports what the header declares."""
import os
import re

import pytest

import cutc_gb300 as cg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_drop_in_signature():
    names = declared_functions()
    assert "cutc_int" in names
    text = open(os.path.join(ROOT, "include", "cutc_int.h")).read()
    # the argument list of src/cutc_int.c:15-20
    sig = re.search(r"int cutc_int\((.*?)\);", text, flags=re.S).group(1)
    params = [p.strip().split()[-1].lstrip("*") for p in sig.split(",")]
    assert params == ["nxBlocks", "nyBlocks", "nzBlocks", "blockxSize", "blockySize",
                      "blockzSize", "n_grid1", "n_grid2", "n_ao", "n_nuc", "size_bh",
                      "r1", "wr1", "r2", "wr2", "rn", "aos_data1", "aos_data2",
                      "c_bh", "m_bh", "n_bh", "o_bh", "int2_grad1_u12_ao", "int_2e_ao"]


def test_library_exports_every_declared_symbol():
    L = cg.load()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert sorted(declared_functions()) == sorted(cg.EXPORTS)


def test_no_device_is_a_status_not_an_exit():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np
    z = np.zeros(16)
    zi = np.zeros(16, dtype=np.int32)
    s = cg.cutc_int(1, 1, 1, 32, 1, 1, 2, 2, 1, 1, 1, z, z, z, z, z, z, z, z, zi, zi, zi, z, z)
    assert s == cg.CUTC_ERR_NO_DEVICE
    assert "device" in cg.last_error()


# The reference's device-level stages: parameter names in the reference's order
# (src/jast_bh.cu:268-272, src/long_range_integ.cu:52-54,
# src/short_range_integ_herm.cu:51-52, src/short_range_integ_nonherm.cu:69-70,
# src/build_int2_grad1_u12_ao.cu:9-13, src/build_int_2e_ao.cu:11-12).
REFERENCE_STAGES = {
    "cutc_int_bh": ["dimGrid", "dimBlock", "ii0", "n_grid1_eff", "n_grid1_tot", "jj0",
                    "n_grid2_eff", "n_grid2_tot", "n_nuc", "size_bh", "r1", "r2", "rn", "c_bh",
                    "m_bh", "n_bh", "o_bh", "grad1_u12"],
    "int_long_range": ["jj0", "n_grid2_eff", "n_grid2_tot", "n_grid2", "n_ao", "wr2",
                       "aos_data2", "int_fct_long_range"],
    "int_short_range_herm": ["n_grid1", "n_ao", "wr1", "aos_data1", "int_fct_short_range_herm"],
    "int_short_range_nonherm": ["n_grid1", "n_ao", "wr1", "aos_data1",
                                "int_fct_short_range_nonherm"],
    "get_int2_grad1_u12_ao": ["dimGrid", "dimBlock", "n_grid1", "n_grid2", "n_ao", "n_nuc",
                              "size_bh", "r1", "r2", "wr2", "rn", "aos_data2", "c_bh", "m_bh",
                              "n_bh", "o_bh", "int2_grad1_u12_ao"],
    "get_int_2e_ao": ["n_grid1", "n_ao", "wr1", "aos_data1", "int2_grad1_u12", "int_2e_ao"],
}


def test_reference_stage_signatures():
    text = open(os.path.join(ROOT, "include", "cutc_int.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    for name, want in REFERENCE_STAGES.items():
        m = re.search(r"void %s\((.*?)\);" % name, text, flags=re.S)
        assert m, name
        params = [p.strip().split()[-1].lstrip("*") for p in m.group(1).split(",")]
        assert params == want, (name, params)
        # dim3 arguments are passed by value as three unsigned ints
        if "dimGrid" in want:
            assert re.search(r"cutc_dim3 dimGrid, cutc_dim3 dimBlock", m.group(1)), name
    assert re.search(r"typedef struct cutc_dim3 \{\s*unsigned int x, y, z;\s*\} cutc_dim3;", text)


def test_header_compiles_as_c_and_cpp(tmp_path):
    """include/cutc_int.h is a plain C header (the reference's callers are C and
    Fortran) that also compiles as C++, warning-free in both."""
    import shutil
    import subprocess
    src_c = tmp_path / "use.c"
    src_c.write_text('#include "cutc_int.h"\nint main(void) { cutc_options o; '
                     'cutc_default_options(&o); cutc_dim3 g = {1, 1, 1}; (void)g; '
                     'return o.precision; }\n')
    src_cpp = tmp_path / "use.cpp"
    src_cpp.write_text(src_c.read_text())
    inc = os.path.join(ROOT, "include")
    for compiler, src, std in (("gcc", src_c, "-std=c99"), ("g++", src_cpp, "-std=c++17")):
        if shutil.which(compiler) is None:
            pytest.skip(compiler + " not available")
        subprocess.check_call([compiler, std, "-Wall", "-Wextra", "-Werror", "-pedantic",
                               "-fsyntax-only", "-I", inc, str(src)])
