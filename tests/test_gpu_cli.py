"""The command-line product (python -m hsmu_gb.cli, the counterpart of the
reference's `./test matrix.mtx`) on Matrix Market files: its written C equals
the oracle's product of the same file, bit for bit."""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from conftest import PKG_DIR, ROOT
from hsmu_gb import gen, mtx

pytestmark = pytest.mark.gpu


def run_cli(*args):
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([PKG_DIR, ROOT, os.environ.get("PYTHONPATH", "")]))
    r = subprocess.run([sys.executable, "-m", "hsmu_gb.cli", *args, "--repeat", "2"], capture_output=True,
                       text=True, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.parametrize("aat", [False, True])
def test_cli_product_matches_oracle(tmp_path, aat):
    A = gen.rmat(11, 8, seed=5, lo=-1.0, hi=1.0)
    src, out = str(tmp_path / "a.mtx"), str(tmp_path / "c.mtx")
    mtx.write_mtx(src, A)
    text = run_cli(src, "--out", out, *(["--aat"] if aat else []))
    assert "GFLOPS" in text and "input matrix A: ( 2048, 2048 )" in text
    C = mtx.read_mtx(out)
    B = gen.CSR(A.N, A.M, *oracle.transpose(A)) if aat else A
    rp, col, val = oracle.spgemm(A, B)
    np.testing.assert_array_equal(C.row_ptr.astype(np.int64), rp)
    np.testing.assert_array_equal(C.col, col)
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))


def test_cli_symmetric_file(tmp_path):
    # lower triangle of a symmetric matrix: the reader mirrors it like the reference's loader
    L = gen.laplacian2d(20, seed=0)
    D = np.zeros((L.M, L.N))
    for i in range(L.M):
        for p in range(L.row_ptr[i], L.row_ptr[i + 1]):
            D[i, L.col[p]] = L.val[p]
    S = np.tril(D) + np.tril(D, -1).T
    rows, cols = np.nonzero(S)
    A = mtx.coo_to_csr(L.M, L.N, rows, cols, S[rows, cols])
    src, out = str(tmp_path / "s.mtx"), str(tmp_path / "c.mtx")
    mtx.write_mtx(src, A, symmetric=True)
    run_cli(src, "--out", out)
    C = mtx.read_mtx(out)
    rp, col, val = oracle.spgemm(A, A)
    np.testing.assert_array_equal(C.col, col)
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))
