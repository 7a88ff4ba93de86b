"""Parity at the stated workload sizes, through the C ABI.

The products of the measured configurations are too large to compare in full
on the host (R-MAT scale 18 A*A: 1.28e9 entries; R-MAT scale 20: ~9.7e9), so
each is checked through
  * every row pointer against the oracle's exact symbolic count (a
    size-independent check of the whole structure), and
  * sampled rows -- random blocks of consecutive rows plus the rows with the
    most products, which take the large-row window path (the reference's
    bin-13 dense accumulator, src/external/spECK/dense_acc.cu:122-243) --
    against the host Gustavson oracle: columns identical, values bit for bit
    and within 1e-12 * max(|c|, sum |a||b|).
Only the sampled rows are copied back from the device.
"""
import functools

import numpy as np
import pytest

import oracle
from hsmu_gb import gen
from oracle import sampled

pytestmark = pytest.mark.gpu


@functools.lru_cache(maxsize=None)
def rmat18():
    return gen.rmat(18, 16, seed=2)


@functools.lru_cache(maxsize=None)
def rmat20():
    return gen.rmat(20, 16, seed=3)


def dev(A):
    import hsmu_gb

    return hsmu_gb.DeviceCSR.from_host(A)


def check_product(C, A, B, rp=None):
    """every row pointer against the oracle's counts, then sampled rows"""
    rp = C.row_ptr_host() if rp is None else rp
    cnt = oracle.symbolic(A, B)
    want = np.zeros(A.M + 1, dtype=np.int64)
    np.cumsum(cnt, out=want[1:])
    np.testing.assert_array_equal(rp.astype(np.int64), want)
    rows = sampled.sample_rows(A, B)
    res = sampled.check_rows(C.rows_to_host(rows, row_ptr=rp), A, B, rows)
    assert res["bitwise"], res
    return res


def test_rmat18_AA_full_size(engine):
    A = rmat18()
    dA = dev(A)
    C = engine.spgemm(dA, dA, stats=True)
    assert engine.last_stats["products"] == 2930477084
    assert C.nnz == 1280410128
    res = check_product(C, A, A)
    assert res["rows"] > 1500
    C.free()


def test_rmat18_AAt_full_size(engine):
    A = rmat18()
    dA = dev(A)
    dAt = engine.transpose(dA)
    At = gen.transpose(A)
    C = engine.spgemm(dA, dAt)
    check_product(C, A, At)
    C.free()


def test_stencil27_40_dof3_full_size(engine):
    A = gen.stencil27(40, 3, seed=1)
    dA = dev(A)
    C = engine.spgemm(dA, dA)
    assert C.nnz == 65712456
    check_product(C, A, A)
    C.free()


def test_laplacian_256_full(engine):
    # the whole product of the smallest workload, every entry
    A = gen.laplacian2d(256, seed=0)
    dA = dev(A)
    C = engine.spgemm(dA, dA).to_host()
    rp, col, val = oracle.spgemm(A, A)
    np.testing.assert_array_equal(C.row_ptr.astype(np.int64), rp)
    np.testing.assert_array_equal(C.col, col)
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))


def test_rmat20_int64_full_size(engine):
    # the R-MAT scale-20 evaluation product in one int64 CSR (~9.7e9 entries, ~116 GB on
    # the device), computed by hsmu_spgemm64 in row panels
    A = rmat20()
    dA = dev(A)
    C = engine.spgemm64(dA, dA)
    assert C.nnz > np.iinfo(np.int32).max
    check_product(C, A, A)
    C.free()


def rmat20_panels(A, max_products=1.9e9):
    """row cuts of at most max_products products each (the learned-scheduler evaluation)"""
    cum = np.concatenate(([0], np.cumsum(sampled.row_products(A, A))))
    cuts = [0]
    while cuts[-1] < A.M:
        nxt = int(np.searchsorted(cum, cum[cuts[-1]] + max_products, side="right")) - 1
        cuts.append(max(nxt, cuts[-1] + 1) if nxt < A.M else A.M)
    return cuts


@pytest.mark.parametrize("which", [0, -1])
def test_rmat20_panel_learned_and_plain(engine, which):
    # one row panel of the R-MAT scale-20 evaluation through the learned path and the
    # plain path: identical output, and sampled rows against the oracle
    import hsmu_gb
    import torch
    from hsmu_gb import learned

    A = rmat20()
    cuts = rmat20_panels(A)
    k = which % (len(cuts) - 1)
    r0, r1 = cuts[k], cuts[k + 1]
    dA = dev(A)
    Ap = hsmu_gb.DeviceCSR(hsmu_gb.c_csr(r1 - r0, A.N, A.nnz, 0, dA.desc.row_ptr + 4 * r0, dA.desc.col,
                                         dA.desc.val), keep=dA)
    hp = gen.CSR(r1 - r0, A.N, (A.row_ptr[r0:r1 + 1] - A.row_ptr[r0]).astype(np.int32),
                 A.col[A.row_ptr[r0]:A.row_ptr[r1]], A.val[A.row_ptr[r0]:A.row_ptr[r1]])
    params, margin, _ = learned.load()
    Cl = engine.spgemm_learned(Ap, dA, torch.from_numpy(params).cuda(), margin)
    Cp = engine.spgemm(Ap, dA)
    rp_l, rp_p = Cl.row_ptr_host(), Cp.row_ptr_host()
    np.testing.assert_array_equal(rp_l, rp_p)
    rows = sampled.sample_rows(hp, A)
    got_l = Cl.rows_to_host(rows, row_ptr=rp_l)
    got_p = Cp.rows_to_host(rows, row_ptr=rp_p)
    for x, y in zip(got_l, got_p):
        assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8))
    res = sampled.check_rows(got_p, hp, A, rows)
    assert res["bitwise"], res
    Cl.free()
    Cp.free()


def test_amg512_batch_sampled_products(engine):
    # the 512-product Galerkin batch at its stated sizes (sides uniform in [16, 96], seed 4):
    # 16 sampled products, among them the largest and the smallest grid, against the oracle
    import hsmu_gb

    sides = np.random.default_rng(4).integers(16, 97, size=512)
    As, Ps, Pts = [], [], []
    for sd in sides:
        As.append(hsmu_gb.gen_poisson7(int(sd)))
        P, Pt = hsmu_gb.gen_aggregation(int(sd))
        Ps.append(P)
        Pts.append(Pt)
    b = hsmu_gb.Batch(engine, hsmu_gb.BATCH_GALERKIN, As, Ps, Pts)
    b.graph_launch()
    b.status()
    pick = set(np.random.default_rng(11).choice(512, size=14, replace=False).tolist())
    pick |= {int(np.argmax(sides)), int(np.argmin(sides))}
    for p in sorted(pick):
        A, P, Pt = As[p].to_host(), Ps[p].to_host(), Pts[p].to_host()
        rp, col, val = oracle.spgemm(A, P)
        AP = gen.CSR(A.M, P.N, rp.astype(np.int32), col, val)
        rp, col, val = oracle.spgemm(Pt, AP)
        C = b.result(p).to_host()
        np.testing.assert_array_equal(C.row_ptr.astype(np.int64), rp)
        np.testing.assert_array_equal(C.col, col)
        assert np.array_equal(C.val.view(np.int64), val.view(np.int64)), "product %d (side %d)" % (p, sides[p])
    b.close()
