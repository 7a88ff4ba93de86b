"""Batched persistent engine (hsmu_batch_*) and the device AMG generators.

The batch must give, product by product, exactly what the oracle gives (the
same summation order), through plain launches, CUDA-graph replays and after
autotuning, for rows of every width: thread rows, warp rows, and wide rows
(more than 512 entries or a column span of more than 512 64-column tiles) that
the launch's wide-row phase writes one column window at a time."""
import numpy as np
import pytest

import oracle
from hsmu_gb import gen

pytestmark = pytest.mark.gpu


def host(d):
    return d.to_host()


@pytest.mark.parametrize("side", [1, 2, 5, 8, 13])
def test_device_generators_match_host(side):
    import hsmu_gb

    A = host(hsmu_gb.gen_poisson7(side))
    ref = gen.poisson7(side)
    np.testing.assert_array_equal(A.row_ptr, ref.row_ptr)
    np.testing.assert_array_equal(A.col, ref.col)
    np.testing.assert_array_equal(A.val, ref.val)
    dP, dPt = hsmu_gb.gen_aggregation(side)
    P, Pt = host(dP), host(dPt)
    Pr = gen.aggregation_prolongator(side)
    np.testing.assert_array_equal(P.row_ptr, Pr.row_ptr)
    np.testing.assert_array_equal(P.col, Pr.col)
    T = gen.transpose(Pr)
    np.testing.assert_array_equal(Pt.row_ptr, T.row_ptr)
    np.testing.assert_array_equal(Pt.col, T.col)
    assert P.N == Pt.M == ((side + 1) // 2) ** 3


def galerkin_oracle(A, P, Pt):
    rp, col, val = oracle.spgemm(A, P)
    AP = gen.CSR(A.M, P.N, rp.astype(np.int32), col, val)
    return oracle.spgemm(Pt, AP)


def test_galerkin_batch_matches_oracle(engine):
    import hsmu_gb

    sides = [3, 16, 5, 24, 9, 2, 31]
    As, Ps, Pts = [], [], []
    for s in sides:
        As.append(hsmu_gb.gen_poisson7(s))
        P, Pt = hsmu_gb.gen_aggregation(s)
        Ps.append(P)
        Pts.append(Pt)
    b = hsmu_gb.Batch(engine, hsmu_gb.BATCH_GALERKIN, As, Ps, Pts)
    for launch in ("execute", "graph", "graph"):
        b.execute() if launch == "execute" else b.graph_launch()
        b.status()
        for p, s in enumerate(sides):
            C = host(b.result(p))
            rp, col, val = galerkin_oracle(host(As[p]), host(Ps[p]), host(Pts[p]))
            np.testing.assert_array_equal(C.row_ptr, rp.astype(np.int32))
            np.testing.assert_array_equal(C.col, col)
            assert np.array_equal(C.val.view(np.int64), val.view(np.int64))
    tiny, grid, ms = b.autotune()
    assert 0 < tiny <= 32 and grid > 0 and ms > 0
    b.graph_launch()
    b.status()
    C = host(b.result(3))
    rp, col, val = galerkin_oracle(host(As[3]), host(Ps[3]), host(Pts[3]))
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))


def test_product_batch_matches_plain(engine):
    import hsmu_gb

    mats = [gen.laplacian2d(40, seed=1), gen.poisson_random(3000, 3, seed=2, ncols=3000),
            gen.stencil27(7, 3, seed=3), gen.laplacian2d(9, seed=4)]
    dA = [hsmu_gb.DeviceCSR.from_host(m) for m in mats]
    b = hsmu_gb.Batch(engine, hsmu_gb.BATCH_PRODUCT, dA, dA)
    for tiny in (0, 8, 32):  # 0: every row through the warp path
        b.set_params(tiny)
        b.execute()
        b.status()
        for p, m in enumerate(mats):
            C = host(b.result(p))
            rp, col, val = oracle.spgemm(m, m)
            np.testing.assert_array_equal(C.row_ptr, rp.astype(np.int32))
            np.testing.assert_array_equal(C.col, col)
            assert np.array_equal(C.val.view(np.int64), val.view(np.int64))


def test_galerkin_batch_fma_mode(engine):
    # fused multiply-add accumulation: the oracle's fma restatement, bit for bit
    import hsmu_gb

    sides = [4, 11, 20]
    As = [hsmu_gb.gen_poisson7(s) for s in sides]
    PPt = [hsmu_gb.gen_aggregation(s) for s in sides]
    b = hsmu_gb.Batch(engine, hsmu_gb.BATCH_GALERKIN, As, [p for p, _ in PPt], [t for _, t in PPt],
                      arith=hsmu_gb.ARITH_FMA)
    b.graph_launch()
    b.status()
    for p in range(len(sides)):
        A, P, Pt = host(As[p]), host(PPt[p][0]), host(PPt[p][1])
        rp, col, val = oracle.spgemm(A, P, fma=True)
        AP = gen.CSR(A.M, P.N, rp.astype(np.int32), col, val)
        rp, col, val = oracle.spgemm(Pt, AP, fma=True)
        C = host(b.result(p))
        np.testing.assert_array_equal(C.col, col)
        assert np.array_equal(C.val.view(np.int64), val.view(np.int64))


@pytest.mark.parametrize("tiny", [0, 16, 32])
def test_galerkin_batch_wide_intermediate_rows(engine, tiny):
    # A*P rows with up to ~60 products: the intermediate round's rows go through
    # the warp path as well as the thread path (tiny 0: every row through the warp path)
    import hsmu_gb

    cases = [(1500, 40.0, 200, 1), (800, 25.0, 90, 2), (64, 3.0, 10, 3)]
    As, Ps, Pts, host_ops = [], [], [], []
    for n, lam, nc, seed in cases:
        A = gen.poisson_random(n, lam, seed=seed)
        P = gen.poisson_random(n, 1.5, seed=seed + 100, ncols=nc)
        Pt = gen.transpose(P)
        host_ops.append((A, P, Pt))
        As.append(hsmu_gb.DeviceCSR.from_host(A))
        Ps.append(hsmu_gb.DeviceCSR.from_host(P))
        Pts.append(hsmu_gb.DeviceCSR.from_host(Pt))
    b = hsmu_gb.Batch(engine, hsmu_gb.BATCH_GALERKIN, As, Ps, Pts)
    b.set_params(tiny)
    for _ in range(2):  # the intermediate is rewritten on every launch
        b.execute()
        b.status()
        for p, (A, P, Pt) in enumerate(host_ops):
            C = host(b.result(p))
            rp, col, val = galerkin_oracle(A, P, Pt)
            np.testing.assert_array_equal(C.row_ptr, rp.astype(np.int32))
            np.testing.assert_array_equal(C.col, col)
            assert np.array_equal(C.val.view(np.int64), val.view(np.int64))


def check_products(b, want):
    for p, (rp, col, val) in enumerate(want):
        C = host(b.result(p))
        np.testing.assert_array_equal(C.row_ptr, rp.astype(np.int32))
        np.testing.assert_array_equal(C.col, col)
        assert np.array_equal(C.val.view(np.int64), val.view(np.int64)), "product %d" % p


@pytest.mark.parametrize("tiny", [0, 32])
def test_product_batch_wide_rows(engine, tiny):
    # R-MAT scale 12 A*A (1,719 rows of more than 512 entries, up to 2,878), a product whose
    # rows span up to ~4,700 tiles with ~100 products each, and small products between them
    import hsmu_gb

    rm = gen.rmat(12, 16, seed=2)
    L = gen.poisson_random(2000, 20.0, seed=5, ncols=2000)
    R = gen.poisson_random(2000, 5.0, seed=6, ncols=300000)
    lap = gen.laplacian2d(30, seed=1)
    pairs = [(lap, lap), (rm, rm), (L, R), (lap, lap), (rm, rm)]
    b = hsmu_gb.Batch(engine, hsmu_gb.BATCH_PRODUCT, [hsmu_gb.DeviceCSR.from_host(x) for x, _ in pairs],
                      [hsmu_gb.DeviceCSR.from_host(y) for _, y in pairs])
    b.set_params(tiny)
    want = [oracle.spgemm(x, y) for x, y in pairs]
    for launch in ("execute", "graph", "graph"):
        b.execute() if launch == "execute" else b.graph_launch()
        b.status()
        check_products(b, want)
    b.close()


def test_product_batch_more_wide_rows_than_the_list(engine):
    # 40 copies of R-MAT 12 A*A: 68,760 wide rows, more than the launch lists (65,536), so
    # the rest are written in place by the warps that counted them
    import hsmu_gb

    rm = gen.rmat(12, 16, seed=2)
    d = hsmu_gb.DeviceCSR.from_host(rm)
    b = hsmu_gb.Batch(engine, hsmu_gb.BATCH_PRODUCT, [d] * 40, [d] * 40)
    b.graph_launch()
    b.status()
    want = oracle.spgemm(rm, rm)
    check_products(b, [want] * 40)
    b.close()


def test_galerkin_batch_wide_rows_in_both_products(engine):
    # A*P rows of ~600 products over 40,000 columns (span ~625 tiles, ~595 entries) and
    # Pt*(AP) rows of ~900 products: wide rows in the first and in the second product
    import hsmu_gb

    A = gen.poisson_random(2000, 20.0, seed=7, ncols=2000)
    P = gen.poisson_random(2000, 30.0, seed=8, ncols=40000)
    Pt = gen.transpose(P)
    lap = gen.laplacian2d(20, seed=2)
    lapP = gen.poisson_random(lap.M, 1.0, seed=9, ncols=50)
    ops = [(A, P, Pt), (lap, lapP, gen.transpose(lapP))]
    dev = hsmu_gb.DeviceCSR.from_host
    b = hsmu_gb.Batch(engine, hsmu_gb.BATCH_GALERKIN, [dev(a) for a, _, _ in ops], [dev(x) for _, x, _ in ops],
                      [dev(t) for _, _, t in ops])
    want = [galerkin_oracle(*o) for o in ops]
    for _ in range(2):
        b.graph_launch()
        b.status()
        check_products(b, want)
    b.close()


def test_product_batch_degenerate_products(engine):
    # a product without rows, one whose rows are all empty, a 1x1 product, one row past a
    # tile of 32, and rows whose A entries all point at empty B rows, in one launch
    import hsmu_gb

    def csr(M, N, rows):
        rp = np.zeros(M + 1, np.int32)
        col, val = [], []
        for i, r in enumerate(rows):
            for c, v in r:
                col.append(c)
                val.append(v)
            rp[i + 1] = len(col)
        rp[len(rows) + 1:] = len(col)
        return gen.CSR(M, N, rp, np.array(col, np.int32), np.array(val, np.float64))

    empty_rows_B = csr(6, 9, [[(1, 2.0)], [], [(3, -1.0), (8, 0.5)], [], [], [(0, 1.5)]])
    pairs = [
        (csr(0, 10, []), gen.poisson_random(10, 3.0, seed=1)),
        (csr(50, 40, []), gen.poisson_random(40, 3.0, seed=2, ncols=30)),
        (csr(1, 1, [[(0, 2.0)]]), csr(1, 1, [[(0, 3.0)]])),
        (gen.poisson_random(33, 4.0, seed=3), gen.poisson_random(33, 4.0, seed=4)),
        (csr(4, 6, [[(1, 1.0), (3, 2.0)], [(4, 1.0)], [(0, 1.0), (1, 1.0)], []]), empty_rows_B),
    ]
    dev = hsmu_gb.DeviceCSR.from_host
    b = hsmu_gb.Batch(engine, hsmu_gb.BATCH_PRODUCT, [dev(x) for x, _ in pairs], [dev(y) for _, y in pairs])
    want = [oracle.spgemm(x, y) for x, y in pairs]
    for _ in range(2):
        b.graph_launch()
        b.status()
        check_products(b, want)
    b.close()
