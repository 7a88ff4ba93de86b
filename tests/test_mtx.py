"""Matrix Market reader (CPU): the reference loader's value and symmetry rules,
then canonical rows (sorted columns, duplicates summed in file order)."""
import numpy as np
import pytest

from hsmu_gb import gen, mtx


def write(tmp_path, text):
    p = tmp_path / "m.mtx"
    p.write_text(text)
    return str(p)


def dense(A):
    D = np.zeros((A.M, A.N))
    for i in range(A.M):
        for p in range(A.row_ptr[i], A.row_ptr[i + 1]):
            D[i, A.col[p]] += A.val[p]
    return D


def canonical(A):
    for i in range(A.M):
        c = A.col[A.row_ptr[i]:A.row_ptr[i + 1]]
        assert np.all(np.diff(c) > 0)


def test_general_real(tmp_path):
    A = mtx.read_mtx(write(tmp_path, "%%MatrixMarket matrix coordinate real general\n% comment\n"
                                     "3 4 4\n3 4 2.5\n1 2 -1\n1 1 3e0\n2 3 7\n"))
    canonical(A)
    np.testing.assert_array_equal(dense(A), [[3, -1, 0, 0], [0, 0, 7, 0], [0, 0, 0, 2.5]])


def test_symmetric_integer_expands(tmp_path):
    A = mtx.read_mtx(write(tmp_path, "%%MatrixMarket matrix coordinate integer symmetric\n3 3 3\n1 1 4\n3 1 -2\n2 2 5\n"))
    canonical(A)
    np.testing.assert_array_equal(dense(A), [[4, 0, -2], [0, 5, 0], [-2, 0, 0]])


def test_pattern_and_complex_and_hermitian(tmp_path):
    P = mtx.read_mtx(write(tmp_path, "%%MatrixMarket matrix coordinate pattern general\n2 2 2\n2 1\n1 2\n"))
    np.testing.assert_array_equal(dense(P), [[0, 1], [1, 0]])
    C = mtx.read_mtx(write(tmp_path, "%%MatrixMarket matrix coordinate complex hermitian\n2 2 2\n1 1 2 0\n2 1 3 4\n"))
    np.testing.assert_array_equal(dense(C), [[2, 3], [3, 0]])  # real parts, mirrored like the reference


def test_duplicates_summed_in_file_order(tmp_path):
    A = mtx.read_mtx(write(tmp_path, "%%MatrixMarket matrix coordinate real general\n1 2 3\n1 2 1e16\n1 2 1\n1 2 -1e16\n"))
    assert A.nnz == 1 and A.val[0] == (1e16 + 1.0) + -1e16


def test_round_trip_and_errors(tmp_path):
    A = gen.rmat(9, 8, seed=4, lo=-1.0, hi=1.0)
    p = str(tmp_path / "r.mtx")
    mtx.write_mtx(p, A)
    B = mtx.read_mtx(p)
    np.testing.assert_array_equal(B.row_ptr, A.row_ptr)
    np.testing.assert_array_equal(B.col, A.col)
    assert np.array_equal(B.val.view(np.int64), A.val.view(np.int64))
    with pytest.raises(ValueError):
        mtx.read_mtx(write(tmp_path, "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n"))
    with pytest.raises(ValueError):
        mtx.read_mtx(write(tmp_path, "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n"))
