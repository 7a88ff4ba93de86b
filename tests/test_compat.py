"""The reference-compatible C++ layer (include/hsmu_nhc_compat.h): a caller
written against the reference's NHC_spgemm interface compiles against it
(CPU test) and, on a GPU, gets the oracle's product (GPU test)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG_DIR, ROOT


def build_driver(tmp_path):
    from hsmu_gb import build

    lib = build.build()
    exe = str(tmp_path / "compat_driver")
    libdir = os.path.dirname(lib)
    subprocess.check_call([build.nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "native", "compat_driver.cu"),
                           "-o", exe, "-L", libdir, "-lhsmu_gb", "-Xlinker", "-rpath", "-Xlinker", libdir])
    return exe


def test_reference_style_caller_compiles(tmp_path):
    exe = build_driver(tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["lap64", "st10"])
def test_reference_style_caller_gets_the_oracle_product(tmp_path, name):
    import oracle
    from hsmu_gb import gen
    from oracle import ref_run

    A = gen.laplacian2d(64, seed=0) if name == "lap64" else gen.stencil27(10, 3, seed=1)
    exe = build_driver(tmp_path)
    a, c = str(tmp_path / "A.bin"), str(tmp_path / "C.bin")
    ref_run._write(a, A)
    out = subprocess.run([exe, a, c], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    C = ref_run._read(c)
    rp, col, val = oracle.spgemm(A, A)
    np.testing.assert_array_equal(C.row_ptr, rp.astype(np.int32))
    np.testing.assert_array_equal(C.col, col)
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))
