"""hsmu_csr_transpose: A^T on the device (stable radix sort by column) against
the oracle's host transpose, bit for bit, and the A*A^T product built on it."""
import numpy as np
import pytest

import oracle
from hsmu_gb import gen

pytestmark = pytest.mark.gpu


def device_transpose(engine, A):
    import hsmu_gb

    return engine.transpose(hsmu_gb.DeviceCSR.from_host(A)).to_host()


def host_transpose(A):
    trp, tcol, tval = oracle.transpose(A)
    return gen.CSR(A.N, A.M, trp, tcol, tval)


CASES = {
    "rmat12": lambda: gen.rmat(12, 16, seed=2, lo=-1.0, hi=1.0),          # 12-bit columns: 2 passes
    "wide": lambda: gen.poisson_random(3000, 40, seed=3, ncols=1_200_000),  # 21 bits: 3 passes
    "narrow": lambda: gen.poisson_random(5000, 3, seed=4, ncols=200),       # 8 bits: 1 pass
    "lap": lambda: gen.laplacian2d(64, seed=0),
    "sparse": lambda: gen.poisson_random(4000, 0.4, seed=5, ncols=9000),    # empty rows and columns
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_transpose_matches_host(engine, name):
    A = CASES[name]()
    T = device_transpose(engine, A)
    W = host_transpose(A)
    assert (T.M, T.N, T.nnz) == (W.M, W.N, W.nnz)
    np.testing.assert_array_equal(T.row_ptr, W.row_ptr)
    np.testing.assert_array_equal(T.col, W.col)
    assert np.array_equal(T.val.view(np.int64), W.val.view(np.int64))


def test_transpose_degenerate(engine):
    Z = gen.CSR(7, 5, np.zeros(8, np.int32), np.zeros(0, np.int32), np.zeros(0))
    T = device_transpose(engine, Z)
    assert (T.M, T.N, T.nnz) == (5, 7, 0) and np.all(T.row_ptr == 0)
    one = gen.CSR(3, 1, np.array([0, 1, 1, 2], np.int32), np.array([0, 0], np.int32), np.array([2.0, 3.0]))
    T = device_transpose(engine, one)
    np.testing.assert_array_equal(T.row_ptr, [0, 2])
    np.testing.assert_array_equal(T.col, [0, 2])
    np.testing.assert_array_equal(T.val, [2.0, 3.0])


def test_aat_with_device_transpose(engine):
    import hsmu_gb

    A = gen.rmat(12, 16, seed=7, lo=-1.0, hi=1.0)
    dA = hsmu_gb.DeviceCSR.from_host(A)
    dAt = engine.transpose(dA)
    C = engine.spgemm(dA, dAt).to_host()
    rp, col, val = oracle.spgemm(A, host_transpose(A))
    np.testing.assert_array_equal(C.col, col)
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))
