"""Workload generators: sizes of the measured workloads, canonical form,
determinism (the same seed gives the same matrix on every machine)."""
import hashlib

import numpy as np

from hsmu_gb import gen


def digest(A):
    h = hashlib.sha256()
    for a in (A.row_ptr, A.col, A.val):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_laplacian_sizes():
    A = gen.laplacian2d(256, seed=0)
    A.check()
    assert (A.M, A.nnz, gen.products(A, A)) == (65536, 326656, 1629192)


def test_stencil27_structure():
    A = gen.stencil27(6, 3, seed=1)
    A.check()
    S = A.to_scipy()
    assert (S != S.T).nnz == 0 or np.array_equal(S.indptr, S.T.tocsr().indptr)
    assert np.diff(A.row_ptr).max() == 81
    # full-size counts (n = 192,000; nnz = 118^3 * 9)
    assert gen.stencil27(40, 3).nnz == 118 ** 3 * 9


def test_rmat_deterministic_and_canonical():
    A = gen.rmat(12, 16, seed=2)
    A.check()
    assert digest(A) == digest(gen.rmat(12, 16, seed=2))
    assert digest(A) != digest(gen.rmat(12, 16, seed=3))
    assert A.val.min() >= 0.0 and A.val.max() < 1.0


def test_transpose_and_products():
    A = gen.rmat(10, 16, seed=2)
    T = gen.transpose(A)
    T.check()
    S = A.to_scipy().T.tocsr()
    S.sort_indices()
    np.testing.assert_array_equal(T.row_ptr, S.indptr)
    np.testing.assert_array_equal(T.col, S.indices)
    assert gen.products(A, T) == int(np.diff(T.row_ptr)[A.col].sum())


def test_amg_operators():
    A = gen.poisson7(9)
    P = gen.aggregation_prolongator(9)
    A.check()
    P.check()
    assert P.N == 125 and np.all(np.diff(P.row_ptr) == 1)
    assert np.diff(A.row_ptr).max() == 7
