"""CPU tests of the oracle: independent restatements and invariants.

Pins: (1) structure against scipy's SpGEMM (a third implementation),
(2) values bit for bit against a pure-Python restatement of the same
summation order on small inputs, (3) values within 1e-12 of scipy's
(different order), (4) the golden fixtures of the reference's own GPU output
(tests/golden/, produced on a GB300 by tests/golden/make_golden.py).
"""
import numpy as np
import pytest

import oracle
from hsmu_gb import gen


def py_gustavson(A, B):
    """Plain-Python C = A*B: products rounded, then added in A-row order."""
    rp = [0]
    cols, vals = [], []
    for i in range(A.M):
        acc = {}
        for p in range(A.row_ptr[i], A.row_ptr[i + 1]):
            k, a = int(A.col[p]), float(A.val[p])
            for q in range(B.row_ptr[k], B.row_ptr[k + 1]):
                j = int(B.col[q])
                acc[j] = acc.get(j, 0.0) + a * float(B.val[q])
        for j in sorted(acc):
            cols.append(j)
            vals.append(acc[j])
        rp.append(len(cols))
    return np.array(rp, np.int64), np.array(cols, np.int32), np.array(vals, np.float64)


@pytest.mark.parametrize("mk", [
    lambda: (gen.laplacian2d(12, seed=3),) * 2,
    lambda: (gen.stencil27(3, 2, seed=4),) * 2,
    lambda: (lambda A: (A, gen.transpose(A)))(gen.rmat(7, 8, seed=5, lo=-1.0, hi=1.0)),
    lambda: (gen.poisson_random(60, 4, seed=6, ncols=80), gen.poisson_random(80, 5, seed=7, ncols=90)),
])
def test_oracle_bitwise_vs_python(mk):
    A, B = mk()
    rp, col, val = oracle.spgemm(A, B)
    prp, pcol, pval = py_gustavson(A, B)
    np.testing.assert_array_equal(rp, prp)
    np.testing.assert_array_equal(col, pcol)
    assert np.array_equal(val.view(np.int64), pval.view(np.int64))


@pytest.mark.parametrize("mk", [
    lambda: (gen.laplacian2d(64, seed=0),) * 2,
    lambda: (gen.stencil27(8, 3, seed=1),) * 2,
    lambda: (gen.rmat(12, 16, seed=2),) * 2,
    lambda: (lambda A: (A, gen.transpose(A)))(gen.rmat(11, 16, seed=2)),
])
def test_oracle_vs_scipy(mk):
    A, B = mk()
    rp, col, val, absv = oracle.spgemm(A, B, with_abs=True)
    S = (A.to_scipy() @ B.to_scipy()).tocsr()
    S.sort_indices()
    # scipy drops nothing structural here (products of nonzero values) but may
    # hold explicit zeros the same way; compare structure and values
    np.testing.assert_array_equal(rp, S.indptr.astype(np.int64))
    np.testing.assert_array_equal(col, S.indices)
    err = np.abs(val - S.data) / np.maximum(np.abs(val), absv)
    assert err.max() <= 1e-12


def test_row_subset_and_threads():
    A = gen.rmat(11, 16, seed=2, lo=-1.0, hi=1.0)
    full = oracle.spgemm(A, A, nthreads=1)
    rows = np.array([5, 0, 77, 2047, 1000], np.int32)
    sub = oracle.spgemm(A, A, rows=rows, nthreads=3)
    for r_i, r in enumerate(rows):
        a, b = full[0][r], full[0][r + 1]
        c, d = sub[0][r_i], sub[0][r_i + 1]
        np.testing.assert_array_equal(full[1][a:b], sub[1][c:d])
        assert np.array_equal(full[2][a:b].view(np.int64), sub[2][c:d].view(np.int64))
    many = oracle.spgemm(A, A, nthreads=8)
    assert np.array_equal(full[2].view(np.int64), many[2].view(np.int64))


def test_products_and_symbolic():
    A = gen.laplacian2d(256, seed=0)
    assert oracle.products(A, A) == gen.products(A, A) == 1629192
    assert int(oracle.symbolic(A, A).sum()) == 846852


def test_cancellation_kept():
    A = gen.CSR(1, 2, np.array([0, 2], np.int32), np.array([0, 1], np.int32), np.array([1.0, 1.0]))
    B = gen.CSR(2, 1, np.array([0, 1, 2], np.int32), np.array([0, 0], np.int32), np.array([1.0, -1.0]))
    rp, col, val = oracle.spgemm(A, B)
    assert rp.tolist() == [0, 1] and col.tolist() == [0] and val[0] == 0.0


def test_transpose_matches_numpy():
    A = gen.rmat(10, 8, seed=9)
    trp, tcol, tval = oracle.transpose(A)
    T = gen.transpose(A)
    np.testing.assert_array_equal(trp, T.row_ptr)
    np.testing.assert_array_equal(tcol, T.col)
    np.testing.assert_array_equal(tval, T.val)
