"""hsmu_spgemm_host: host operands in, host CSR out, copies pipelined behind
row panels of the product.  The result must be identical, bit for bit, to the
device-resident call followed by a download (and hence to the oracle)."""
import numpy as np
import pytest

import oracle
from hsmu_gb import gen

pytestmark = pytest.mark.gpu


class Host:
    """a host CSR with the attribute names the wrapper reads"""

    def __init__(self, M, N, row_ptr, col, val):
        self.M, self.N, self.row_ptr, self.col, self.val = M, N, row_ptr, col, val


def pinned(X):
    import torch

    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    return Host(X.M, X.N, t(X.row_ptr.astype(np.int32)), t(X.col), t(X.val))


def numpy_host(X):
    return Host(X.M, X.N, np.ascontiguousarray(X.row_ptr, np.int32), np.ascontiguousarray(X.col),
                np.ascontiguousarray(X.val))


def expect(A, B, fma=False):
    rp, col, val = oracle.spgemm(A, B, fma=fma)
    return rp.astype(np.int32), col, val


def same(got, want):
    rp, col, val = (np.asarray(x) for x in got)
    np.testing.assert_array_equal(rp, want[0])
    np.testing.assert_array_equal(col, want[1])
    assert np.array_equal(val.view(np.int64), want[2].view(np.int64))


CASES = {
    "st27_10": lambda: (gen.stencil27(10, 3, seed=1),) * 2,
    "lap128": lambda: (gen.laplacian2d(128, seed=0),) * 2,
    "rmat12": lambda: (gen.rmat(12, 16, seed=2, lo=-1.0, hi=1.0),) * 2,
    "rmat11T": lambda: (lambda A: (A, gen.transpose(A)))(gen.rmat(11, 16, seed=4)),
    "rect": lambda: (gen.poisson_random(3000, 12, seed=5, ncols=50000),
                     gen.poisson_random(50000, 6, seed=6, ncols=70000)),
    "wide": lambda: (gen.poisson_random(400, 40, seed=7, ncols=2000),
                     gen.poisson_random(2000, 60, seed=8, ncols=1_200_000)),
}


@pytest.mark.parametrize("panels", [0, 1, 7, 32])
@pytest.mark.parametrize("name", sorted(CASES))
def test_host_matches_oracle(engine, name, panels):
    A, B = CASES[name]()
    hA = pinned(A)
    hB = hA if B is A else pinned(B)
    same(engine.spgemm_host(hA, hB, panels=panels), expect(A, B))


def test_host_pageable_and_fma(engine):
    import hsmu_gb

    A = gen.stencil27(8, 3, seed=3)
    B = gen.stencil27(8, 3, seed=4)
    same(engine.spgemm_host(numpy_host(A), numpy_host(B), panels=5), expect(A, B))
    same(engine.spgemm_host(numpy_host(A), numpy_host(B), arith=hsmu_gb.ARITH_FMA), expect(A, B, fma=True))


def test_host_into_caller_buffers_and_capacity(engine):
    import torch

    import hsmu_gb

    A = gen.rmat(11, 16, seed=9, lo=-1.0, hi=1.0)
    want = expect(A, A)
    nnz = want[1].size
    hA = pinned(A)
    rp = torch.empty(A.M + 1, dtype=torch.int32).pin_memory()
    # too small: the size comes back, nothing is written to col/val
    col = torch.full((nnz - 1,), -7, dtype=torch.int32).pin_memory()
    val = torch.zeros(nnz - 1, dtype=torch.float64).pin_memory()
    with pytest.raises(hsmu_gb.HsmuError) as e:
        engine.spgemm_host(hA, hA, out=(rp, col, val))
    assert e.value.status == hsmu_gb.HSMU_ERR_CAPACITY
    np.testing.assert_array_equal(rp.numpy(), want[0])
    assert int(col.min()) == -7 and int(col.max()) == -7
    # large enough (with room to spare): filled in place
    col = torch.empty(nnz + 100, dtype=torch.int32).pin_memory()
    val = torch.empty(nnz + 100, dtype=torch.float64).pin_memory()
    got = engine.spgemm_host(hA, hA, out=(rp, col, val), panels=3, stats=True)
    same((g.numpy() for g in got), want)
    st = engine.last_stats
    assert st["nnz_c"] == nnz and st["products"] == gen.products(A, A)


def test_host_empty_and_degenerate(engine):
    Z = gen.CSR(5, 7, np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0))
    Y = gen.poisson_random(7, 3, seed=1, ncols=9)
    for A, B in ((Z, Y), (gen.poisson_random(4, 2, seed=2, ncols=7), Y)):
        same(engine.spgemm_host(numpy_host(A), numpy_host(B), panels=4), expect(A, B))


def test_host_rejects_bad_arguments(engine):
    import hsmu_gb

    A = gen.laplacian2d(8, seed=0)
    B = gen.laplacian2d(9, seed=0)
    with pytest.raises(hsmu_gb.HsmuError):
        engine.spgemm_host(numpy_host(A), numpy_host(B))  # inner dimensions differ
    with pytest.raises(hsmu_gb.HsmuError):
        engine.spgemm_host(numpy_host(A), numpy_host(A), panels=-1)
