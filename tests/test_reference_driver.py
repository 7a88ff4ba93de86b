"""The reference's own driver as a caller of this engine.

The reference's `src/test.cu` (its `./test matrix.mtx` program) includes
"NHC_spgemm.cuh", loads a Matrix Market file, uploads A and B with
HtD_value_col_ptr and calls NHC_spgemm.  The drop-in swaps that one include:
a one-line NHC_spgemm.cuh that includes include/hsmu_nhc_compat.h sits beside
an unchanged, byte-identical copy of test.cu (a quoted include is looked up in
the including file's directory first), and the reference's Matrix Market
loader and cuSPARSE check file are taken from its source tree.  The driver
links libhsmu_gb.so.

The source tree is the staged copy that oracle/ref_build.py makes for the
reference harness; where it is missing (a machine without the reference)
these tests are skipped.
"""
import filecmp
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

REF_SRC = os.path.join(ROOT, "oracle", "_ref", "src")
needs_ref = pytest.mark.skipif(not os.path.exists(os.path.join(REF_SRC, "test.cu")),
                               reason="reference sources not staged on this machine")


def build_reference_driver(tmp_path):
    from hsmu_gb import build

    lib = build.build()
    libdir = os.path.dirname(lib)
    work = tmp_path / "driver"
    work.mkdir()
    shutil.copyfile(os.path.join(REF_SRC, "test.cu"), work / "test.cu")
    assert filecmp.cmp(os.path.join(REF_SRC, "test.cu"), work / "test.cu", shallow=False)
    (work / "NHC_spgemm.cuh").write_text('#include "hsmu_nhc_compat.h"\n')
    exe = str(work / "test")
    cmd = [build.nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-w",
           "-I", str(work), "-I", REF_SRC, "-I", os.path.join(ROOT, "include"), str(work / "test.cu"),
           "-o", exe, "-L", libdir, "-lhsmu_gb", "-lcusparse", "-Xlinker", "-rpath", "-Xlinker", libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def write_mtx(path, A):
    """general real Matrix Market file, entries in row-major order (so the
    reference loader's CSR comes out with sorted columns)"""
    rows = np.repeat(np.arange(A.M), np.diff(A.row_ptr))
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write("%d %d %d\n" % (A.M, A.N, A.nnz))
        f.writelines("%d %d %.17g\n" % (r + 1, c + 1, v) for r, c, v in zip(rows, A.col, A.val))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    return build_reference_driver(tmp_path_factory.mktemp("refdriver"))


@needs_ref
def test_reference_driver_compiles_unchanged(driver):
    assert os.path.exists(driver)


@needs_ref
@pytest.mark.gpu
@pytest.mark.parametrize("name", ["lap128", "rmat12"])
def test_reference_driver_calls_the_engine(tmp_path, driver, name):
    import oracle
    from hsmu_gb import gen

    A = gen.laplacian2d(128, seed=0) if name == "lap128" else gen.rmat(12, 16, seed=2)
    exe = driver
    mtx = str(tmp_path / (name + ".mtx"))
    write_mtx(mtx, A)
    env = dict(os.environ, HSMU_VERBOSE="1")
    r = subprocess.run([exe, mtx], capture_output=True, text=True, env=env, cwd=str(tmp_path), timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    m = re.search(r"NHC_spgemm \(GB300 engine\).*products (\d+), nnz\(C\) (\d+)", r.stdout)
    assert m, "the driver did not call the engine:\n" + r.stdout
    want = oracle.symbolic(A, A)
    assert int(m.group(2)) == int(want.sum())
    assert int(m.group(1)) == oracle.products(A, A)
