"""hsmu_spgemm64: C with int64 row pointers, computed in row panels.

Panels forced small (max_panel_nnz) must give exactly the single-call
result; a product with more than INT32_MAX entries (which hsmu_spgemm
reports as HSMU_ERR_OVERFLOW) is checked through size-independent
properties: every row pointer, and sampled rows against the exact product.
"""
import numpy as np
import pytest

from hsmu_gb import gen

pytestmark = pytest.mark.gpu


def dev(A):
    import hsmu_gb

    return hsmu_gb.DeviceCSR.from_host(A)


CASES = {
    "rmat12": lambda: (gen.rmat(12, 16, seed=2, lo=-1.0, hi=1.0),) * 2,
    "stencil6": lambda: (gen.stencil27(6, 3, seed=1),) * 2,
    "rect": lambda: (gen.poisson_random(700, 9, seed=21, ncols=3000),
                     gen.poisson_random(3000, 30, seed=22, ncols=90000)),
    "empty_rows": lambda: (gen.poisson_random(500, 0.6, seed=23, ncols=400),
                           gen.poisson_random(400, 2.0, seed=24, ncols=800)),
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("cap_div", [0, 5, 40])
def test_panels_match_single_call(engine, name, cap_div):
    A, B = CASES[name]()
    dA = dev(A)
    dB = dA if B is A else dev(B)
    ref = engine.spgemm(dA, dB).to_host()
    # cap 0: one panel (INT32_MAX); otherwise about cap_div panels, rows above the cap alone
    cap = 0 if cap_div == 0 else max(1, ref.nnz // cap_div)
    C = engine.spgemm64(dA, dB, max_panel_nnz=cap)
    rp, col, val = C.to_host()
    C.free()
    assert rp.dtype == np.int64 and rp[-1] == ref.nnz
    np.testing.assert_array_equal(rp, ref.row_ptr.astype(np.int64))
    np.testing.assert_array_equal(col, ref.col)
    assert np.array_equal(val.view(np.int64), ref.val.view(np.int64))


def test_one_row_per_panel(engine):
    A = gen.laplacian2d(12, seed=3)
    dA = dev(A)
    ref = engine.spgemm(dA, dA).to_host()
    C = engine.spgemm64(dA, dA, max_panel_nnz=1, validate=True)
    rp, col, val = C.to_host()
    np.testing.assert_array_equal(rp, ref.row_ptr.astype(np.int64))
    np.testing.assert_array_equal(col, ref.col)
    assert np.array_equal(val.view(np.int64), ref.val.view(np.int64))


def test_beyond_int32(engine):
    # a 50,000 x 1 column times a 1 x 50,000 row: 2.5e9 entries (30 GB), C[i, j] = a_i * b_j
    import ctypes

    import hsmu_gb

    n = 50_000
    rng = np.random.default_rng(31)
    a = rng.uniform(-1.0, 1.0, n)
    b = rng.uniform(-1.0, 1.0, n)
    colA = gen.CSR(n, 1, np.arange(n + 1, dtype=np.int32), np.zeros(n, np.int32), a)
    rowB = gen.CSR(1, n, np.array([0, n], np.int32), np.arange(n, dtype=np.int32), b)
    dA, dB = dev(colA), dev(rowB)
    with pytest.raises(hsmu_gb.HsmuError) as e:
        engine.spgemm(dA, dB)
    assert e.value.status == 4  # HSMU_ERR_OVERFLOW: an int32 CSR cannot hold it
    C = engine.spgemm64(dA, dB)
    try:
        assert C.nnz == n * n and C.nnz > 2**31 - 1
        # sampled rows: download a view of them (row pointers stay absolute)
        rows = np.unique(np.concatenate([[0, 1, n // 2, n - 1], rng.integers(0, n, 12)]))
        for i in rows:
            view = hsmu_gb.c_csr64()
            view.M, view.N = 1, n
            lo = int(i) * n
            view.nnz = n
            view.row_ptr = C.desc.row_ptr + 8 * int(i)
            view.col = C.desc.col + 4 * lo
            view.val = C.desc.val + 8 * lo
            rp = np.empty(2, np.int64)
            col = np.empty(n, np.int32)
            val = np.empty(n, np.float64)
            rc = hsmu_gb.load_library().hsmu_csr64_download(ctypes.byref(view), rp.ctypes.data,
                                                           col.ctypes.data, val.ctypes.data, None)
            assert rc == 0
            assert rp[0] == lo and rp[1] == lo + n
            np.testing.assert_array_equal(col, np.arange(n, dtype=np.int32))
            assert np.array_equal(val.view(np.int64), (a[i] * b).view(np.int64))  # one product each
        # every row pointer
        full = hsmu_gb.c_csr64()
        full.M, full.N, full.nnz = n, n, 0
        full.row_ptr = C.desc.row_ptr
        rp = np.empty(n + 1, np.int64)
        assert hsmu_gb.load_library().hsmu_csr64_download(ctypes.byref(full), rp.ctypes.data, None, None,
                                                         None) == 0
        np.testing.assert_array_equal(rp, np.arange(n + 1, dtype=np.int64) * n)
    finally:
        C.free()
