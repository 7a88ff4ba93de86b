"""GPU parity: the engine (through the C ABI) against the host Gustavson oracle.

Structure (row_ptr, col) must be identical; values are compared bit for bit
(the engine adds products in the oracle's order) and, as the stated bar,
within 1e-12 relative (scaled by sum |a||b| where terms cancel).
"""
import numpy as np
import pytest

import oracle
from conftest import assert_csr_equal
from hsmu_gb import gen

pytestmark = pytest.mark.gpu


def run(engine, A, B, **kw):
    import hsmu_gb

    dA = hsmu_gb.DeviceCSR.from_host(A)
    dB = dA if B is A else hsmu_gb.DeviceCSR.from_host(B)
    C = engine.spgemm(dA, dB, **kw)
    out = C.to_host()
    C.free()
    out.check()
    return out


def check(engine, A, B, **kw):
    C = run(engine, A, B, **kw)
    ref = oracle.spgemm(A, B, with_abs=True)
    assert_csr_equal(C, ref[:3], absv=ref[3])
    return C


@pytest.mark.parametrize("side", [64, 256])
def test_laplacian_AA(engine, side):
    A = gen.laplacian2d(side, seed=0)
    C = check(engine, A, A)
    if side == 256:  # the measured workload itself
        assert C.nnz == 846852


@pytest.mark.parametrize("side", [6, 12])
def test_stencil27_AA(engine, side):
    A = gen.stencil27(side, 3, seed=1)
    check(engine, A, A)


@pytest.mark.parametrize("scale", [10, 12, 14])
def test_rmat_AA(engine, scale):
    A = gen.rmat(scale, 16, seed=2)
    check(engine, A, A)


@pytest.mark.parametrize("scale", [10, 13])
def test_rmat_AAt(engine, scale):
    A = gen.rmat(scale, 16, seed=2)
    check(engine, A, gen.transpose(A))


def test_rectangular_random(engine):
    A = gen.poisson_random(3000, 12, seed=5, ncols=50000)
    B = gen.poisson_random(50000, 6, seed=6, ncols=70000)
    check(engine, A, B)


def test_chunked_wide_rows(engine):
    # C rows spanning more than one 4096-tile chunk (N > 262144 columns)
    A = gen.poisson_random(400, 40, seed=7, ncols=2000)
    B = gen.poisson_random(2000, 60, seed=8, ncols=1_200_000)
    check(engine, A, B)


def test_multiwindow_dense_rows(engine):
    # rows with > 1024 entries inside a narrow tile span: several windows per row
    rng = np.random.default_rng(9)
    n = 6000
    rows, cols = [], []
    for i in range(n):
        c0 = (i * 7) % (n - 1500)
        cs = np.arange(c0, c0 + 1200, 1 + (i % 3))
        rows.append(np.full(cs.size, i))
        cols.append(cs)
    key = np.unique(np.concatenate(rows).astype(np.int64) * n + np.concatenate(cols))
    rp, col = gen._from_coo_sorted_unique(n, n, key)
    B = gen.CSR(n, n, rp, col, rng.uniform(-1, 1, col.size))
    A = gen.poisson_random(300, 6, seed=10, ncols=n)
    check(engine, A, B)


def test_empty_and_degenerate(engine):
    # empty rows in A and B, an all-empty matrix, single entries
    A = gen.poisson_random(5000, 0.7, seed=11, ncols=4000)
    B = gen.poisson_random(4000, 0.9, seed=12, ncols=6000)
    check(engine, A, B)
    Z = gen.CSR(100, 4000, np.zeros(101, np.int32), np.zeros(0, np.int32), np.zeros(0))
    C = run(engine, Z, B)
    assert C.nnz == 0 and C.M == 100 and C.N == 6000
    one = gen.CSR(1, 1, np.array([0, 1], np.int32), np.array([0], np.int32), np.array([3.0]))
    C = run(engine, one, one)
    assert C.nnz == 1 and C.val[0] == 9.0


@pytest.mark.parametrize("ncols", [1, 63, 1000, 4095])
def test_narrow_outputs(engine, ncols):
    # B->N < 4096: the reference's separate small-matrix path; here the same engine
    A = gen.poisson_random(3000, 6, seed=ncols, ncols=2000)
    B = gen.poisson_random(2000, min(5, ncols), seed=ncols + 1, ncols=ncols)
    check(engine, A, B)


def test_output_beyond_int32_reported(engine):
    # a 50,000 x 1 column times a 1 x 50,000 row: nnz(C) = 2.5e9 does not fit int32 CSR; the count
    # pass finds it and the call fails with HSMU_ERR_OVERFLOW before allocating C (tiny inputs)
    import hsmu_gb

    n = 50_000
    col = gen.CSR(n, 1, np.arange(n + 1, dtype=np.int32), np.zeros(n, np.int32), np.ones(n))
    row = gen.CSR(1, n, np.array([0, n], np.int32), np.arange(n, dtype=np.int32), np.ones(n))
    with pytest.raises(hsmu_gb.HsmuError) as e:
        run(engine, col, row)
    assert e.value.status == 4  # HSMU_ERR_OVERFLOW
    # the engine stays usable afterwards
    check(engine, gen.laplacian2d(16, seed=0), gen.laplacian2d(16, seed=0))


def test_cancellation_kept(engine):
    # (1 1) * (1 -1)^T cancels to 0.0; the entry stays (symbolic structure)
    A = gen.CSR(1, 2, np.array([0, 2], np.int32), np.array([0, 1], np.int32), np.array([1.0, 1.0]))
    B = gen.CSR(2, 1, np.array([0, 1, 2], np.int32), np.array([0, 0], np.int32), np.array([1.0, -1.0]))
    C = run(engine, A, B)
    assert C.nnz == 1 and C.col[0] == 0 and C.val[0] == 0.0


def test_deterministic_bitwise(engine):
    A = gen.rmat(12, 16, seed=3, lo=-1.0, hi=1.0)
    C1 = run(engine, A, A)
    C2 = run(engine, A, A)
    assert np.array_equal(C1.val.view(np.int64), C2.val.view(np.int64))


def test_validation_rejects_unsorted(engine):
    import hsmu_gb

    A = gen.laplacian2d(16)
    B = gen.laplacian2d(16)
    B.col = B.col.copy()
    B.col[1], B.col[2] = B.col[2], B.col[1]
    with pytest.raises(hsmu_gb.HsmuError) as ei:
        run(engine, A, B, validate=True)
    assert ei.value.status == 5
    A2 = gen.laplacian2d(16)
    A2.col = A2.col.copy()
    A2.col[3] = A2.col[4]  # duplicate column
    with pytest.raises(hsmu_gb.HsmuError) as ei:
        run(engine, A2, gen.laplacian2d(16), validate=True)
    assert ei.value.status == 5


def host_tiles(B):
    """Reference tiles of B computed with numpy (tile = col >> 6)."""
    rows = np.repeat(np.arange(B.M), np.diff(B.row_ptr))
    t = (B.col >> 6).astype(np.int64)
    key = rows.astype(np.int64) * (B.N // 64 + 1) + t
    first = np.ones(B.nnz, dtype=bool)
    first[1:] = key[1:] != key[:-1]
    starts = np.flatnonzero(first)
    tile_col = t[starts].astype(np.int32)
    bits = np.left_shift(np.uint64(1), (B.col & 63).astype(np.uint64))
    mask = np.bitwise_or.reduceat(bits, starts) if B.nnz else np.zeros(0, np.uint64)
    tile_ptr = np.zeros(B.M + 1, dtype=np.int32)
    np.cumsum(np.bincount(rows[starts], minlength=B.M), out=tile_ptr[1:])
    return tile_ptr, tile_col, mask.astype(np.uint64), starts.astype(np.int32)


@pytest.mark.parametrize("which", ["lap", "rmat", "wide"])
def test_btiles_conversion(engine, which):
    import hsmu_gb

    B = {"lap": lambda: gen.laplacian2d(64),
         "rmat": lambda: gen.rmat(12, 16, seed=2),
         "wide": lambda: gen.poisson_random(300, 90, seed=13, ncols=100000)}[which]()
    dB = hsmu_gb.DeviceCSR.from_host(B)
    bt = hsmu_gb.BTiles(engine, dB)
    got = bt.arrays()
    ref = host_tiles(B)
    assert bt.ntiles == ref[1].size
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)
    # reuse of the converted B gives the same product
    A = gen.poisson_random(B.M, 5, seed=14, ncols=B.M)
    dA = hsmu_gb.DeviceCSR.from_host(A)
    C1 = engine.spgemm(dA, dB).to_host()
    C2 = engine.spgemm(dA, dB, tiles=bt).to_host()
    assert np.array_equal(C1.row_ptr, C2.row_ptr) and np.array_equal(C1.col, C2.col)
    assert np.array_equal(C1.val.view(np.int64), C2.val.view(np.int64))
    bt.free()


def test_stats(engine):
    A = gen.laplacian2d(128)
    import hsmu_gb

    dA = hsmu_gb.DeviceCSR.from_host(A)
    C = engine.spgemm(dA, dA, stats=True)
    st = engine.last_stats
    assert st["products"] == gen.products(A, A)
    assert st["nnz_c"] == C.nnz
    assert st["windows"] >= 0 and st["ms_total"] > 0 and st["launches"] >= 9


def test_integer_pipe_multiply_selftest():
    import hsmu_gb

    assert hsmu_gb.selftest_dmul(1 << 24, seed=7) == 0


@pytest.mark.parametrize("arith", [0, 2])
def test_arith_modes_identical(engine, arith):
    # FP64-pipe multiply (0) and integer-pipe multiply (2) give the same bits
    for A in (gen.stencil27(8, 3, seed=1), gen.rmat(12, 16, seed=2, lo=-1.0, hi=1.0)):
        C = run(engine, A, A, arith=arith)
        rp, col, val = oracle.spgemm(A, A)
        assert np.array_equal(C.val.view(np.int64), val.view(np.int64))


FMA_CASES = {
    "lap64": lambda: (gen.laplacian2d(64, seed=0),) * 2,
    "st27_12": lambda: (gen.stencil27(12, 3, seed=1),) * 2,
    "rmat13": lambda: (gen.rmat(13, 16, seed=2, lo=-1.0, hi=1.0),) * 2,
    "rmat12T": lambda: (lambda A: (A, gen.transpose(A)))(gen.rmat(12, 16, seed=3)),
    "chunked": lambda: (gen.poisson_random(200, 30, seed=9, ncols=5000),
                        gen.poisson_random(5000, 400, seed=10, ncols=3_000_000)),
    "multiwindow": lambda: (gen.poisson_random(64, 200, seed=11, ncols=4000),
                            gen.poisson_random(4000, 40, seed=12, ncols=20000)),
}


@pytest.mark.parametrize("name", sorted(FMA_CASES))
def test_fma_mode(engine, name):
    # fused multiply-add mode: bit-identical to the oracle's fma accumulation
    # in the same order, and within the stated 1e-12 bar of the rounded-product
    # arithmetic of the reference
    import hsmu_gb

    A, B = FMA_CASES[name]()
    C = run(engine, A, B, arith=hsmu_gb.ARITH_FMA)
    rp, col, val = oracle.spgemm(A, B, fma=True)
    np.testing.assert_array_equal(C.row_ptr.astype(np.int64), rp)
    np.testing.assert_array_equal(C.col, col)
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))
    ref = oracle.spgemm(A, B, with_abs=True)
    assert_csr_equal(C, ref[:3], absv=ref[3], exact=False)


def test_invalid_arith_rejected(engine):
    import hsmu_gb

    A = gen.laplacian2d(8, seed=0)
    with pytest.raises(hsmu_gb.HsmuError):
        run(engine, A, A, arith=3)


@pytest.mark.parametrize("case", ["rmat15", "rmat14T", "chunked"])
def test_tile_store_and_or_walk_give_the_same_bits(engine, case):
    # the large rows' structure from the count pass's stored tiles, or from a second
    # OR walk over B's tiles: identical output
    import hsmu_gb

    if case == "rmat15":
        A = B = gen.rmat(15, 16, seed=2)
    elif case == "rmat14T":
        A = gen.rmat(14, 16, seed=3)
        B = gen.transpose(A)
    else:
        A = gen.poisson_random(400, 40, seed=7, ncols=2000)
        B = gen.poisson_random(2000, 60, seed=8, ncols=1_200_000)
    dA = hsmu_gb.DeviceCSR.from_host(A)
    dB = dA if B is A else hsmu_gb.DeviceCSR.from_host(B)
    C1 = engine.spgemm(dA, dB, stats=True).to_host()
    assert engine.last_stats["windows"] > 0
    C2 = engine.spgemm(dA, dB, tile_store=False).to_host()
    np.testing.assert_array_equal(C1.row_ptr, C2.row_ptr)
    np.testing.assert_array_equal(C1.col, C2.col)
    assert np.array_equal(C1.val.view(np.int64), C2.val.view(np.int64))
    rp, col, val = oracle.spgemm(A, B)
    np.testing.assert_array_equal(C1.col, col)
    assert np.array_equal(C1.val.view(np.int64), val.view(np.int64))
